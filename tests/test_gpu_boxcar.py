"""GPU boxcar (txg_boxcar, the Boxcar::run boundary) against the oracle and the reference's
golden outputs."""
import numpy as np
import pytest

from gpu_util import assert_boxcar_close, assert_cands_close

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("var", ["scalar", "avx2"])
def test_boxcar_golden(tx, golden, var):
    g = golden["boxcar"]
    if f"mxS_{var}_iqr0" not in g:
        pytest.skip("variant not in fixture")
    for iqr in (0, 1):
        S, W, c = tx.boxcar(g["tim"], g["vwn"], iqr=bool(iqr), avx2_tail=var == "avx2", thre=7.0)
        assert_boxcar_close(g["tim"], g["vwn"], S, W, g[f"mxS_{var}_iqr{iqr}"],
                            g[f"mxwn_{var}_iqr{iqr}"], iqr=bool(iqr))


@pytest.mark.parametrize("n", [17, 1000, 4097, 15625, 40000])
def test_boxcar_random_vs_oracle(tx, oracle, n):
    rng = np.random.default_rng(n)
    ndm = 12
    tim = rng.normal(0, 20, (ndm, n)).astype(np.float32)
    tim[0, n // 3: n // 3 + 5] += 300
    tim[3] = 1.0
    vwn = oracle.width_ladder(1e-4, 0.05, 0.1, 64e-6)
    vwn = vwn[vwn < max(3, n // 2)]
    for iqr in (False, True):
        for avx in (False, True):
            Sr, Wr = oracle.boxcar_run(tim, vwn, iqr, avx)
            S, W, c = tx.boxcar(tim, vwn, iqr=iqr, avx2_tail=avx, thre=4.0)
            assert_boxcar_close(tim, vwn, S, W, Sr, Wr, iqr=iqr)
            assert_cands_close(c, oracle.threshold_scan(Sr, Wr, 4.0), 4.0)


def test_boxcar_candidates_only(tx, oracle):
    rng = np.random.default_rng(7)
    tim = rng.normal(0, 1, (40, 3000)).astype(np.float32)
    tim[10:14, 1500:1510] += 6
    vwn = oracle.width_ladder(1e-4, 0.02, 0.1, 1e-4)
    _, _, c = tx.boxcar(tim, vwn, thre=6.0, dense=False)
    Sr, Wr = oracle.boxcar_run(tim, vwn)
    assert_cands_close(c, oracle.threshold_scan(Sr, Wr, 6.0), 6.0)
    assert len(c) > 0


def test_boxcar_overflow_reported(tx):
    tim = np.zeros((4, 1000), np.float32)
    tim[:, ::2] = 50.0
    with pytest.raises(tx.TxgError) as e:
        tx.boxcar(tim, [1, 2], thre=0.1, cand_capacity=10)
    assert e.value.status == tx.ERR_OVERFLOW


def test_boxcar_rejects_bad_arguments(tx):
    with pytest.raises(tx.TxgError) as e:
        tx.boxcar(np.zeros((2, 10), np.float32), [])
    assert e.value.status == tx.ERR_ARG


@pytest.mark.parametrize("n", [62496, 100003])
def test_boxcar_long_rows_vs_oracle(tx, oracle, n):
    """Rows longer than one CTA's shared memory (16 us sampling, 1 s blocks) run on the
    segmented kernels: same agreement with the oracle as short rows."""
    rng = np.random.default_rng(n)
    ndm = 5
    tim = rng.normal(0, 20, (ndm, n)).astype(np.float32)
    tim[0, n // 3: n // 3 + 40] += 200
    tim[2, n - 30:] += 400   # near the row end, inside the last segment's halo
    tim[4] = 2.0             # var = 0 row
    vwn = oracle.width_ladder(1e-4, 0.01, 0.1, 16e-6)
    for iqr in (False, True):
        for avx in (False, True):
            Sr, Wr = oracle.boxcar_run(tim, vwn, iqr, avx)
            S, W, c = tx.boxcar(tim, vwn, iqr=iqr, avx2_tail=avx, thre=5.0)
            assert_boxcar_close(tim, vwn, S, W, Sr, Wr, iqr=iqr)
            assert_cands_close(c, oracle.threshold_scan(Sr, Wr, 5.0), 5.0)


@pytest.mark.parametrize("n", [1000, 15625, 40000])
def test_boxcar_segmented_equals_single_cta(tx, oracle, n, monkeypatch):
    """The segmented kernels rebuild the single-CTA kernel's running sum chunk by chunk, so on
    rows that fit both they give bit-identical S, widths and candidates."""
    rng = np.random.default_rng(n + 1)
    tim = rng.normal(0, 20, (9, n)).astype(np.float32)
    tim[1, n // 2: n // 2 + 9] += 250
    vwn = oracle.width_ladder(1e-4, 0.05, 0.1, 64e-6)
    vwn = vwn[vwn < max(3, n // 2)]
    for iqr in (False, True):
        for avx in (False, True):
            monkeypatch.delenv("TXG_BOXCAR_SEGMENTED", raising=False)
            S1, W1, c1 = tx.boxcar(tim, vwn, iqr=iqr, avx2_tail=avx, thre=4.0)
            monkeypatch.setenv("TXG_BOXCAR_SEGMENTED", "1")
            S2, W2, c2 = tx.boxcar(tim, vwn, iqr=iqr, avx2_tail=avx, thre=4.0)
            monkeypatch.delenv("TXG_BOXCAR_SEGMENTED")
            np.testing.assert_array_equal(S1, S2)
            np.testing.assert_array_equal(W1, W2)
            np.testing.assert_array_equal(np.sort(c1, order=["idm", "isamp"]),
                                          np.sort(c2, order=["idm", "isamp"]))


@pytest.mark.parametrize("n", [3000, 62496])
def test_boxcar_candidates_same_with_and_without_dense(tx, oracle, n):
    """Without dense output the search keeps only the largest S per sample and finds the width
    of each point above the threshold afterwards: the candidate list equals the tracked
    search's bit for bit (single-CTA and segmented rows, moment and IQR statistics)."""
    rng = np.random.default_rng(n + 3)
    tim = rng.normal(0, 20, (12, n)).astype(np.float32)
    tim[3, n // 4: n // 4 + 30] += 300
    tim[7, n - 20:] += 500
    tim[9, :50] += 400
    tim[11] = 5.0
    vwn = oracle.width_ladder(1e-4, 0.02, 0.1, 64e-6)
    key = ["idm", "isamp"]
    for iqr in (False, True):
        for thre in (3.0, -1.0):  # a negative threshold keeps every sample, S = 0 ones included
            _, _, c1 = tx.boxcar(tim, vwn, iqr=iqr, thre=thre)
            _, _, c2 = tx.boxcar(tim, vwn, iqr=iqr, thre=thre, dense=False)
            assert len(c1) > 100
            np.testing.assert_array_equal(np.sort(c1, order=key), np.sort(c2, order=key))
