"""The oracle restatement pinned against the reference's own Boxcar and Cluster outputs
(tests/golden, generated by tests/golden/make_golden.py from the compiled reference)."""
import numpy as np
import pytest


@pytest.mark.parametrize("var", ["scalar", "avx2"])
@pytest.mark.parametrize("iqr", [0, 1])
def test_boxcar_matches_reference_golden(oracle, golden, var, iqr):
    g = golden["boxcar"]
    key = f"mxS_{var}_iqr{iqr}"
    if key not in g:
        pytest.skip("fixture variant not generated on this machine")
    S, W = oracle.boxcar_run(g["tim"], g["vwn"], iqr=bool(iqr), avx2_tail=(var == "avx2"))
    np.testing.assert_array_equal(S, g[key])
    np.testing.assert_array_equal(W, g[f"mxwn_{var}_iqr{iqr}"])


def test_boxcar_golden_edge_rows(golden):
    g = golden["boxcar"]
    # var <= 0 row stays all zero (boxcar.cpp:242)
    assert not g["mxS_scalar_iqr0"][1].any() and not g["mxwn_scalar_iqr0"][1].any()
    # the AVX2 build leaves tail samples of every width unvisited (boxcar.cpp:264-279)
    assert not np.array_equal(g["mxS_scalar_iqr0"], g["mxS_avx2_iqr0"])


def _cases(golden):
    z = golden["cluster"]
    for k in range(int(z["ncase"])):
        p = z[f"c{k}_params"]
        yield k, z[f"c{k}_points"], p, z[f"c{k}_out"]


def test_cluster_matches_reference_golden(oracle, golden):
    for k, pts, p, ref in _cases(golden):
        out, _ = oracle.cluster(pts, p[0], p[1], p[4], p[3], p[2], p[7], int(p[9]), int(p[10]),
                                bool(p[11]), int(p[5]))
        assert len(out) == len(ref), k
        for f in ("idm", "isamp", "wn", "S"):
            np.testing.assert_array_equal(out[f], ref[f], err_msg=f"case {k} field {f}")


def test_oracle_vs_live_reference(oracle):
    """Where the reference tree is present, compare against freshly compiled reference code on
    new random inputs as well."""
    if not oracle.ref_available("scalar"):
        pytest.skip("reference tree not present")
    rng = np.random.default_rng(5)
    vwn = oracle.width_ladder(1e-4, 0.02, 0.2, 1e-4)
    for n in (97, 640, 2049):
        tim = rng.normal(0, 5, (5, n)).astype(np.float32)
        w = vwn[vwn < n // 2]
        for var in ("scalar", "avx2"):
            if not oracle.ref_available(var):
                continue
            for iqr in (False, True):
                a = oracle.ref_boxcar_run(tim, w, iqr, var)
                b = oracle.boxcar_run(tim, w, iqr, avx2_tail=var == "avx2")
                np.testing.assert_array_equal(a[0], b[0])
                np.testing.assert_array_equal(a[1], b[1])


def test_width_ladder_known_values(oracle):
    # 64 us, minw 1e-4, maxw 0.05, snrloss 0.1: 30 widths from 2 to 741 samples
    v = oracle.width_ladder(1e-4, 0.05, 0.1, 64e-6)
    assert len(v) == 30 and v[0] == 2 and v[-1] == 741
    assert (np.diff(v) >= 1).all()


def test_kadane_definition(oracle):
    assert oracle.kadane([1, -2, 3, 4, -1, 2]) == (8.0, 2, 5)
    assert oracle.kadane([-3, -1, -2]) == (-1.0, 1, 1)          # all negative: best element
    assert oracle.kadane([2, -2, 2]) == (2.0, 0, 0)             # tie: earliest window kept
    assert oracle.kadane([0, 0, 5]) == (5.0, 0, 2)              # zero sum does not restart


def test_skzap_moments_match_numpy(oracle):
    """Channel skewness/kurtosis of the oracle against a float64 numpy evaluation."""
    rng = np.random.default_rng(4)
    raw = np.clip(np.round(rng.normal(128, 12, (3000, 64))), 0, 255).astype(np.uint8)
    raw[:, 5] = 77                                               # constant channel
    raw[:, 9] = (128 + 40 * np.sin(np.arange(3000) / 7.0)).astype(np.uint8)  # sinusoid
    sk, ku = oracle.sk_moments(raw)
    v = raw.astype(np.float64)
    d = v - v.mean(0)
    m2, m3, m4 = (d ** 2).mean(0), (d ** 3).mean(0), (d ** 4).mean(0)
    with np.errstate(invalid="ignore", divide="ignore"):
        rsk = np.where(m2 > 0, m3 / m2 ** 1.5, 0.0)
        rku = np.where(m2 > 0, m4 / m2 ** 2 - 3.0, 0.0)
    np.testing.assert_allclose(sk, rsk, atol=1e-9)
    np.testing.assert_allclose(ku, rku, atol=1e-9)
    mask = oracle.skzap(raw, 4.0)
    assert mask[9] == 1 and mask.sum() <= 3
    assert not oracle.skzap(raw, 0.0).any()       # threshold <= 0 disables the filter
