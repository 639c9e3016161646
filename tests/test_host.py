"""Host-side logic of the product library (no GPU needed): exports, planning tables,
width ladder, clustering, ddplan parsing."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            names |= set(re.findall(r"^\s*(?:int|void|int32_t|const char \*)\s*\**(txg_\w+)\s*\(",
                                    src, re.M))
    return names


def test_library_exports_every_declared_symbol(tx):
    names = declared_symbols()
    assert len(names) >= 20
    L = tx.load_library()
    for n in names:
        assert hasattr(L, n), n
    assert set(tx.EXPORTS) == names
    assert L.txg_version() == 1


def test_strerror(tx):
    L = tx.load_library()
    assert L.txg_strerror(0) == b"ok"
    assert b"overflow" in L.txg_strerror(-4)


def test_width_ladder_equals_oracle(tx, oracle):
    for minw, maxw, loss, ts in [(1e-4, 0.05, 0.1, 64e-6), (1e-4, 0.05, 0.1, 76e-6),
                                 (1e-4, 0.05, 0.1, 304e-6), (5e-3, 0.1, 0.3, 1e-3),
                                 (1e-6, 0.01, 0.05, 16e-6)]:
        np.testing.assert_array_equal(tx.width_ladder(minw, maxw, loss, ts),
                                      oracle.width_ladder(minw, maxw, loss, ts))


def test_plan_tables_equal_oracle(tx, oracle):
    from transientx_gb300 import synth
    w = synth.nchan4096_rfi(nsamples=1 << 16)
    w1 = synth.nchan256_single(nsamples=1 << 16)
    for wl in (w, w1):
        for r, sp in enumerate(wl.rows):
            info, d1, d2, ss, vwn = tx.describe_row(wl.rows, r, wl.fil.nchans, wl.fil.tsamp,
                                                    wl.fil.freqs, wl.ndump)
            f = oracle.downsample_freqs(wl.fil.freqs, sp.fd)
            dd = oracle.Dedisp(f, wl.fil.tsamp * sp.td, wl.ndump // sp.td, sp.dms, sp.ddm,
                               sp.ndm, sp.overlap, info.nsub, info.dm_group)
            od1, od2, oss, _ = dd.tables()
            oi = dd.info()
            np.testing.assert_array_equal(d1, od1)
            np.testing.assert_array_equal(d2, od2)
            np.testing.assert_array_equal(ss, oss)
            assert (info.offset, info.maxd1, info.maxd2, info.noverlap) == \
                (oi.offset, oi.maxd1, oi.maxd2, oi.noverlap)
            np.testing.assert_array_equal(
                vwn, oracle.width_ladder(sp.minw, sp.maxw, sp.snrloss, wl.fil.tsamp * sp.td))


def test_plan_rejects_bad_rows(tx):
    from transientx_gb300 import SinglePulse, TxgError
    f = 1500.0 - np.arange(64.0)
    with pytest.raises(TxgError):
        tx.describe_row([SinglePulse(td=3, ndm=10)], 0, 64, 1e-4, f, 1000)   # 1000 % 3 != 0
    with pytest.raises(TxgError):
        tx.describe_row([SinglePulse(dms=-1.0, ndm=10)], 0, 64, 1e-4, f, 1000)
    with pytest.raises(TxgError):
        tx.describe_row([SinglePulse(ndm=10, rfilist=[["mask", "0", "2"]])], 0, 64, 1e-4, f, 1000)
    with pytest.raises(TxgError):
        tx.describe_row([SinglePulse(ndm=10, rfilist=[["clip", "2", "2"]])], 0, 64, 1e-4, f, 1000)
    for op in (["mask", "2", "2"], ["kadaneT", "4", "2"], ["zero"]):
        tx.describe_row([SinglePulse(ndm=10, rfilist=[op])], 0, 64, 1e-4, f, 1000)


def test_product_cluster_matches_reference_golden(tx, golden):
    z = golden["cluster"]
    for k in range(int(z["ncase"])):
        p, pts, ref = z[f"c{k}_params"], z[f"c{k}_points"], z[f"c{k}_out"]
        c = np.zeros(len(pts), tx.CAND_DTYPE)
        for f in ("idm", "isamp", "wn", "S"):
            c[f] = pts[f]
        out = tx.cluster(c, p[0], p[1], p[4], p[3], p[2], p[7], int(p[9]), int(p[10]),
                         bool(p[11]), int(p[5]))
        assert len(out) == len(ref), k
        for f in ("idm", "isamp", "wn", "S"):
            np.testing.assert_array_equal(out[f], ref[f], err_msg=f"case {k} {f}")


def test_product_cluster_matches_oracle_random(tx, oracle):
    rng = np.random.default_rng(3)
    for trial in range(30):
        n = int(rng.integers(0, 3000))
        idm = np.sort(rng.integers(0, 300, n))
        isamp = rng.integers(0, 5000, n)
        order = np.lexsort((isamp, idm))
        c = np.zeros(n, tx.CAND_DTYPE)
        c["idm"], c["isamp"] = idm[order], isamp[order]
        c["wn"] = rng.integers(1, 40, n)
        c["S"] = rng.uniform(7, 30, n).astype(np.float32)
        args = (0.0, 0.25, 1500.0, 1100.0, 1e-4, float(rng.choice([0, 2e-3, 1e-2])),
                int(rng.choice([1, 10, 100])), int(rng.choice([0, 3, 30])), bool(trial % 2), 39)
        a = tx.cluster(c, *args)
        oc = np.zeros(n, oracle.CAND_DTYPE)
        for f in ("idm", "isamp", "wn", "S"):
            oc[f] = c[f]
        b, _ = oracle.cluster(oc, *args)
        assert len(a) == len(b)
        for f in ("idm", "isamp", "wn", "S"):
            np.testing.assert_array_equal(a[f], b[f])


def test_product_cluster_edge_geometry(tx, oracle):
    """Component search (DM-row sweep, or the grid when many DM rows lie within one radius)
    against the oracle's breadth-first growth: radii at multiples of the DM and sample steps,
    many tied S values, input in arbitrary order, tiny DM steps."""
    rng = np.random.default_rng(11)
    for trial in range(160):
        n = int(rng.integers(1, 2500))
        idm = rng.integers(0, int(rng.choice([5, 60, 400])), n)
        isamp = rng.integers(0, int(rng.choice([50, 400, 4000])), n)
        _, u = np.unique(idm * 100000 + isamp, return_index=True)
        idm, isamp = idm[u], isamp[u]
        n = len(idm)
        order = np.lexsort((isamp, idm)) if trial % 4 else rng.permutation(n)
        c = np.zeros(n, tx.CAND_DTYPE)
        c["idm"], c["isamp"] = idm[order], isamp[order]
        c["wn"] = rng.integers(1, 9, n)
        c["S"] = np.round(rng.uniform(7, 12, n), 1).astype(np.float32)
        tsamp, ddm = 1e-4, float(rng.choice([1e-6, 0.01, 0.05, 0.1, 0.5]))
        step = oracle.dmdelay(ddm, 1500.0, 1200.0) * 0.5
        radius = float(rng.choice([1.5 * tsamp, 3 * tsamp, step, 2 * step, np.hypot(step, tsamp),
                                   1e-3, 3e-3]))
        args = (0.0, ddm, 1500.0, 1200.0, tsamp, radius, int(rng.choice([1, 7, 100, 100000])),
                int(rng.choice([0, 2, 5, 30])), bool(trial % 2), 8)
        a = tx.cluster(c, *args)
        oc = np.zeros(n, oracle.CAND_DTYPE)
        for f in ("idm", "isamp", "wn", "S"):
            oc[f] = c[f]
        b, _ = oracle.cluster(oc, *args)
        assert len(a) == len(b), trial
        for f in ("idm", "isamp", "wn", "S"):
            np.testing.assert_array_equal(a[f], b[f], err_msg=f"trial {trial} {f}")


def test_parse_ddplan(tx):
    text = "# td fd dms ddm ndm snrloss maxwidth(s)\n1 1 0.0 0.1 3344 0.1 0.1 zdot\n" \
           "2 1 334.4 0.2 1255 0.1 0.1 kadaneF 8 4\n"
    rows = tx.parse_ddplan(text)
    assert len(rows) == 2
    assert (rows[0].td, rows[0].dms, rows[0].ddm, rows[0].ndm, rows[0].maxw) == (1, 0.0, 0.1, 3344, 0.1)
    assert rows[0].rfilist == [["zdot"]]
    # later rows keep earlier options, as parse() reuses one SinglePulse (singlepulse.cpp:407-455)
    assert rows[1].rfilist == [["zdot"], ["kadaneF", "8", "4"]]
    assert [r.id for r in rows] == [1, 2]


def test_no_device_is_reported(tx):
    """Without a GPU the compute entry points fail with a status instead of falling back."""
    import ctypes
    try:
        n = ctypes.c_int()
        has = ctypes.CDLL("libcudart.so").cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except OSError:
        has = False
    if has:
        pytest.skip("a device is present")
    from transientx_gb300 import TxgError, boxcar
    with pytest.raises(TxgError) as e:
        boxcar(np.zeros((2, 64), np.float32), [2, 3])
    assert e.value.status == tx.ERR_NODEVICE


@pytest.mark.parametrize("descending", [True, False])
def test_stage1_delays_grow_with_the_group(tx, descending):
    """The stage-1 kernels size each subband's shared-memory window by the last coarse-DM
    group's delays: every delay is >= 0, never decreases from one group to the next, and the
    last group holds each channel's largest (and maxd1 is the largest overall).  Stage 2 sizes
    a chunk's subband window by its first and last fine DM's offsets, so the subband delays
    never decrease with the DM either.  Checked for bands in either frequency order, partial
    last groups and DM ranges starting above 0."""
    from transientx_gb300 import SinglePulse, synth
    rng = np.random.default_rng(5)
    for C, fhi, flo, ts, dms, ddm, ndm, G in [(4096, 1712.0, 856.0, 76e-6, 0.0, 0.1, 5000, 0),
                                                (256, 1500.0, 1244.0, 64e-6, 0.0, 0.5, 2000, 0),
                                                (8192, 1800.0, 1200.0, 16e-6, 700.0, 0.5, 2000, 0),
                                                (100, 400.0, 300.0, 1e-3, 3.0, 0.37, 77, 5),
                                                (33, 1400.0, 1390.0, 1e-4, 0.0, 2.0, 9, 4)]:
        f = synth.band(C, fhi, flo)
        if not descending:
            f = f[::-1].copy()
        sp = SinglePulse(dms=dms, ddm=ddm, ndm=ndm, dm_group=G, nsub=int(rng.integers(0, 2)) * 8)
        info, d1, d2 = tx.describe_row([sp], 0, C, ts, f, 4096)[:3]
        assert (d2 >= 0).all() and (np.diff(d2, axis=0) >= 0).all()
        assert info.maxd2 == d2.max()
        assert (d1 >= 0).all()
        assert (np.diff(d1, axis=0) >= 0).all(), (C, descending)
        np.testing.assert_array_equal(d1[-1], d1.max(axis=0))
        assert info.maxd1 == d1.max()


def test_missing_library_fails_loudly(tx, tmp_path):
    """Without the CUDA library the package refuses to run (ImportError naming the file and
    that there is no CPU fallback); it never substitutes another implementation."""
    missing = str(tmp_path / "libtxgpu.so")
    saved = tx._lib
    tx._lib = None
    try:
        with pytest.raises(ImportError, match="no CPU fallback"):
            tx.load_library(missing)
    finally:
        tx._lib = saved


def test_oracle_planner_equals_host_planner(tx, oracle):
    """The oracle's own subband plan (what the CPU baseline uses without the product library)
    gives the nsub and DM group that the library's host planner picks, on every benchmarked
    row and on both channel counts of the many-beam workload."""
    from transientx_gb300 import synth
    cases = []
    for name in ("nchan256_n1M_dm1000", "nchan4096_n2M_rfi_dm3000", "nchan8192_n8M_dm5000"):
        wl = synth.WORKLOADS[name](nsamples=1 << 16)
        cases.append((wl.rows, wl.fil.nchans, wl.fil.tsamp, wl.fil.freqs, wl.ndump))
    wl = synth.WORKLOADS["nchan4096_n2M_rfi_dm3000"](nsamples=1 << 16)
    for C in (1024, 2048):
        cases.append((wl.rows, C, wl.fil.tsamp, synth.band(C, 1712.0, 856.0), wl.ndump))
    for rows, C, tsamp, f, ndump in cases:
        for r, sp in enumerate(rows):
            info = tx.describe_row(rows, r, C, tsamp, f, ndump)[0]
            assert oracle.plan_row(f, tsamp, sp.td, sp.fd, sp.ddm, sp.ndm, sp.nsub,
                                   sp.dm_group) == (info.nsub, info.dm_group), (C, r)


def test_new_entry_points_refuse_bad_handles_and_rows(tx):
    """txg_reset_beam, txg_push_block_f32, txg_get_launch_shape and txg_get_row_timing refuse a
    null handle with TXG_ERR_ARG before touching any device (a host without a GPU runs this)."""
    import ctypes
    L = tx.load_library()
    i32 = ctypes.c_int32()
    buf = np.zeros(16, np.float32)
    assert L.txg_reset_beam(None, 0) == tx.ERR_ARG
    assert L.txg_push_block_f32(None, 0, buf.ctypes.data, 1) == tx.ERR_ARG
    assert L.txg_get_launch_shape(None, 0, ctypes.byref(i32), ctypes.byref(i32),
                                  ctypes.byref(i32)) == tx.ERR_ARG
    assert L.txg_get_row_timing(None, 0, None, None, 0) == tx.ERR_ARG
