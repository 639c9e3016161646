"""Full per-block chain on the GPU (txg_create / txg_push_block) against the oracle's
SinglePulse::run restatement, block by block: preprocessed data and kadaneF windows
bit-exact, dedispersed series bit-exact on the FP32 path, boxcar S within 1e-4."""
import numpy as np
import pytest

from gpu_util import assert_boxcar_close, assert_cands_close

pytestmark = pytest.mark.gpu


def small_workload(seed=21, nsamples=4096 * 6):
    from transientx_gb300 import SinglePulse, synth
    tsamp, C = 256e-6, 128
    f = synth.band(C, 1500.0, 1200.0)
    rng = np.random.default_rng(seed)
    T = nsamples * tsamp
    sines = [(int(c), float(rng.uniform(10, 30)), float(rng.uniform(0.02, 0.2)), 0.3)
             for c in rng.choice(C, 6, replace=False)]
    imps = [(float(rng.uniform(0, T)), int(rng.integers(1, 20)), 20.0) for _ in range(3)]
    pulses = [(0.3 * T, 60.0, 3e-3, 25.0), (0.55 * T, 150.0, 1e-3, 15.0),
              (0.75 * T, 300.0, 8e-3, 30.0)]
    fil = synth.Filterbank(C, tsamp, f, nsamples, seed, pulses=pulses, sines=sines, impulses=imps)
    rfi = [["kadaneF", "8", "4"], ["zdot"]]
    rows = [SinglePulse(td=1, fd=1, dms=0.0, ddm=1.0, ndm=200, maxw=0.05, rfilist=rfi,
                        widthlimit=0.02, bswidth=0.1, nsub=16),
            SinglePulse(td=2, fd=2, dms=200.0, ddm=2.0, ndm=100, maxw=0.05, rfilist=rfi,
                        widthlimit=0.02, bswidth=0.0, nsub=8, overlap=0.1)]
    return fil, rows, 4096


def oracle_rows(oracle, rows, fil, ndump, tx, avx2=False, zapthre=4.0):
    out = []
    for r, sp in enumerate(rows):
        info = tx.describe_row(rows, r, fil.nchans, fil.tsamp, fil.freqs, ndump)[0]
        row = oracle.make_row(td=sp.td, fd=sp.fd, bswidth=sp.bswidth, rfi=sp.rfilist,
                              threKadaneF=sp.threKadaneF, widthlimit=sp.widthlimit, dms=sp.dms,
                              ddm=sp.ddm, ndm=sp.ndm, overlap=sp.overlap, nsub=info.nsub,
                              group=info.dm_group, minw=sp.minw, maxw=sp.maxw,
                              snrloss=sp.snrloss, iqr=sp.iqr, thre=sp.thre, avx2_tail=avx2,
                              zapthre=zapthre, threMask=sp.threMask,
                              threKadaneT=sp.threKadaneT, bandlimitKT=sp.bandlimitKT)
        out.append(oracle.SinglePulseRow(row, fil.freqs, fil.tsamp, ndump))
    return out


@pytest.mark.parametrize("avx2,zapthre", [(False, 4.0), (True, 4.0), (False, 0.0)])
def test_pipeline_fp32_matches_oracle(tx, oracle, avx2, zapthre):
    fil, rows, ndump = small_workload()
    flags = tx.FLAG_DENSE | tx.FLAG_KEEP_SERIES | (tx.FLAG_AVX2_TAIL if avx2 else 0)
    orows = oracle_rows(oracle, rows, fil, ndump, tx, avx2, zapthre)
    nblk = fil.nsamples // ndump
    ngated = 0
    with tx.Search(rows, fil.nchans, fil.tsamp, fil.freqs, ndump, flags=flags,
                   zapthre=zapthre) as s:
        for b in range(nblk):
            raw = fil.generate(b * ndump, ndump)
            s.push_block(raw)
            s.sync()
            for r, o in enumerate(orows):
                gated = o.run(raw)
                if zapthre > 0:
                    np.testing.assert_array_equal(s.mask(), o.mask())
                info = s.row_info(r)
                assert bool(info.gated) == gated and info.counter == o.info().counter
                np.testing.assert_array_equal(s.block(r), o.block(), err_msg=f"block {b} row {r}")
                zr = s.zap_ranges(0, r)
                np.testing.assert_array_equal(zr, o.zap_ranges(0))
                if not gated:
                    continue
                ngated += 1
                tim = s.timdata(r)
                np.testing.assert_array_equal(tim, o.timdata(), err_msg=f"tim block {b} row {r}")
                S, W = s.dense(r)
                vwn = o.widths()
                assert_boxcar_close(tim, vwn, S, W, o.mxS(), o.mxwn())
                ref = oracle.threshold_scan(o.mxS(), o.mxwn(), rows[r].thre)
                assert_cands_close(s.candidates(r), ref, rows[r].thre)
    assert ngated >= 4


EDGE_CASES = {
    # name: (nchans, tsamp, ndump, row keyword arguments)
    "tiny_one_dm": (16, 256e-6, 64, dict(td=1, fd=1, dms=30.0, ddm=1.0, ndm=1, maxw=0.002,
                                          rfilist=[["zdot"]], bswidth=0.005)),
    "odd_channels_fd3": (33, 256e-6, 768, dict(td=2, fd=3, dms=0.0, ddm=2.0, ndm=40, maxw=0.01,
                                               rfilist=[["kadaneF", "3", "2"], ["zdot"]],
                                               widthlimit=0.005, bswidth=0.05)),
    "ragged_kadane_cells": (96, 128e-6, 1000, dict(td=1, fd=1, dms=10.0, ddm=0.5, ndm=64, maxw=0.01,
                                                   rfilist=[["kadaneF", "7", "5"]], widthlimit=0.003,
                                                   bswidth=0.02, nsub=8)),
    "one_width": (64, 256e-6, 512, dict(td=1, fd=1, dms=0.0, ddm=1.0, ndm=32, minw=2.5e-4,
                                        maxw=3e-4, bswidth=0.0)),
}


@pytest.mark.parametrize("name", list(EDGE_CASES))
def test_edge_geometries_match_oracle(tx, oracle, name):
    """Edge geometries: a 64-sample block with one DM, 33 channels downsampled by 3 (the staged
    unpack), kadaneF cells that do not divide the block, a one-width ladder.  Blocks, zap
    windows and series bit-exact, boxcar within the tolerance, every block."""
    from transientx_gb300 import SinglePulse, synth
    C, tsamp, ndump, kw = EDGE_CASES[name]
    f = synth.band(C, 1500.0, 1300.0)
    T = 12 * ndump * tsamp
    fil = synth.Filterbank(C, tsamp, f, 12 * ndump, 13, pulses=[(0.6 * T, 40.0, 4 * tsamp, 30.0)],
                           sines=[(C // 3, 20.0, 0.01, 0.2)])
    rows = [SinglePulse(**kw)]
    flags = tx.FLAG_DENSE | tx.FLAG_KEEP_SERIES
    o = oracle_rows(oracle, rows, fil, ndump, tx)[0]
    ngated = 0
    with tx.Search(rows, C, tsamp, f, ndump, flags=flags, zapthre=4.0) as s:
        for b in range(12):
            raw = fil.generate(b * ndump, ndump)
            s.push_block(raw)
            s.sync()
            gated = o.run(raw)
            assert bool(s.row_info(0).gated) == gated
            np.testing.assert_array_equal(s.block(0), o.block(), err_msg=f"{name} block {b}")
            for q, op in enumerate(rows[0].rfilist):
                if op[0] == "kadaneF":
                    np.testing.assert_array_equal(s.zap_ranges(q, 0), o.zap_ranges(q))
            if not gated:
                continue
            ngated += 1
            tim = s.timdata(0)
            np.testing.assert_array_equal(tim, o.timdata(), err_msg=f"{name} tim {b}")
            S, W = s.dense(0)
            assert_boxcar_close(tim, o.widths(), S, W, o.mxS(), o.mxwn())
            ref = oracle.threshold_scan(o.mxS(), o.mxwn(), rows[0].thre)
            assert_cands_close(s.candidates(0), ref, rows[0].thre)
    assert ngated >= 1


RFI_LISTS = {
    "mask": [["mask", "4", "2"]],
    "mask11": [["mask", "1", "1"]],
    "kadaneT": [["kadaneT", "2", "2"]],
    "zero": [["zero"]],
    "all": [["kadaneF", "8", "4"], ["mask", "2", "4"], ["kadaneT", "4", "4"], ["zero"], ["zdot"]],
}


@pytest.mark.parametrize("name", list(RFI_LISTS))
def test_rfi_options_match_oracle(tx, oracle, name):
    """mask / kadaneT / zero rfilist entries: preprocessed block, zapped windows and the
    dedispersed series bit-exact against the oracle, every block; each entry must fire."""
    fil, rows, ndump = small_workload()
    for sp in rows:
        sp.rfilist = [list(op) for op in RFI_LISTS[name]]
    flags = tx.FLAG_KEEP_SERIES
    orows = oracle_rows(oracle, rows, fil, ndump, tx)
    fired = {}
    with tx.Search(rows, fil.nchans, fil.tsamp, fil.freqs, ndump, flags=flags, zapthre=4.0) as s:
        for b in range(fil.nsamples // ndump):
            raw = fil.generate(b * ndump, ndump)
            s.push_block(raw)
            s.sync()
            for r, o in enumerate(orows):
                gated = o.run(raw)
                np.testing.assert_array_equal(s.block(r), o.block(), err_msg=f"{name} block {b} row {r}")
                for q, op in enumerate(rows[r].rfilist):
                    if op[0] in ("mask", "kadaneT", "kadaneF"):
                        zr = s.zap_ranges(q, r)
                        np.testing.assert_array_equal(zr, o.zap_ranges(q), err_msg=f"{name} {op}")
                        hit = zr[0, 0] if op[0] == "mask" else int((zr[:, 0] >= 0).sum() + (zr[:, 2] >= 0).sum())
                        fired[op[0]] = fired.get(op[0], 0) + int(hit)
                if gated:
                    np.testing.assert_array_equal(s.timdata(r), o.timdata(), err_msg=f"{name} tim {b} {r}")
    for op in RFI_LISTS[name]:
        if op[0] in ("mask", "kadaneT"):
            assert fired.get(op[0], 0) > 0, (name, op, fired)


def test_zdot_long_rows_match_oracle(tx, oracle):
    """Long blocks (45056 samples, zdot only): the preprocessed block equals the oracle's bit
    for bit."""
    from transientx_gb300 import SinglePulse, synth
    C, ndump = 32, 45056
    f = synth.band(C, 1500.0, 1200.0)
    fil = synth.Filterbank(C, 64e-6, f, 2 * ndump, 5, sines=[(3, 20.0, 0.01, 0.5)])
    rows = [SinglePulse(td=1, fd=1, dms=0.0, ddm=1.0, ndm=8, maxw=0.01, rfilist=[["zdot"]],
                        bswidth=0.05)]
    orow = oracle_rows(oracle, rows, fil, ndump, tx)[0]
    with tx.Search(rows, C, fil.tsamp, f, ndump, flags=tx.FLAG_KEEP_SERIES, zapthre=4.0) as s:
        for b in range(2):
            raw = fil.generate(b * ndump, ndump)
            s.push_block(raw)
            s.sync()
            orow.run(raw)
            np.testing.assert_array_equal(s.block(0), orow.block(), err_msg=f"block {b}")


@pytest.mark.parametrize("nchans,td,fd", [(128, 1, 1), (128, 3, 2), (256, 2, 16), (100, 2, 5),
                                          (96, 4, 3)])
def test_unpack_paths_match_oracle(tx, oracle, nchans, td, fd):
    """Unpack + downsample: the 16-byte path (channels a multiple of 16, fd dividing 16) and
    the staged fallback give the oracle's preprocessed block exactly, with the channel zap."""
    from transientx_gb300 import SinglePulse, synth
    ndump = 1536 * td
    f = synth.band(nchans, 1500.0, 1200.0)
    fil = synth.Filterbank(nchans, 256e-6, f, 3 * ndump, 7,
                           sines=[(5, 25.0, 0.03, 0.0), (nchans - 3, 30.0, 0.01, 1.0)])
    rows = [SinglePulse(td=td, fd=fd, dms=0.0, ddm=1.0, ndm=16, maxw=0.02, bswidth=0.0)]
    orow = oracle_rows(oracle, rows, fil, ndump, tx, zapthre=3.0)[0]
    with tx.Search(rows, nchans, fil.tsamp, f, ndump, flags=tx.FLAG_KEEP_SERIES, zapthre=3.0) as s:
        for blk in range(3):
            raw = fil.generate(blk * ndump, ndump)
            s.push_block(raw)
            s.sync()
            orow.run(raw)
            np.testing.assert_array_equal(s.mask(), orow.mask())
            np.testing.assert_array_equal(s.block(0), orow.block(), err_msg=f"block {blk}")


def test_beams_of_one_handle_equal_separate_handles(tx):
    """nbeams > 1: each beam keeps its own history, ring and candidates; two beams of one
    handle give exactly what two one-beam handles give (beams pushed interleaved)."""
    from transientx_gb300 import synth
    fil, rows, ndump = small_workload()
    fil2 = synth.Filterbank(fil.nchans, fil.tsamp, fil.freqs, fil.nsamples, 99,
                            pulses=[(0.4 * fil.nsamples * fil.tsamp, 120.0, 2e-3, 30.0)])
    flags = tx.FLAG_KEEP_SERIES | tx.FLAG_DENSE
    with tx.Search(rows, fil.nchans, fil.tsamp, fil.freqs, ndump, nbeams=2, flags=flags) as m, \
            tx.Search(rows, fil.nchans, fil.tsamp, fil.freqs, ndump, flags=flags) as a, \
            tx.Search(rows, fil.nchans, fil.tsamp, fil.freqs, ndump, flags=flags) as b:
        ngated = 0
        for blk in range(fil.nsamples // ndump):
            r0, r1 = fil.generate(blk * ndump, ndump), fil2.generate(blk * ndump, ndump)
            m.push_block(r0, beam=0)
            m.push_block(r1, beam=1)
            a.push_block(r0)
            b.push_block(r1)
            m.sync(), a.sync(), b.sync()
            for r in range(len(rows)):
                for beam, single in ((0, a), (1, b)):
                    assert m.row_info(r, beam).gated == single.row_info(r).gated
                    np.testing.assert_array_equal(m.block(r, beam), single.block(r))
                    if single.row_info(r).gated:
                        ngated += 1
                        np.testing.assert_array_equal(m.timdata(r, beam), single.timdata(r))
                        np.testing.assert_array_equal(m.candidates(r, beam), single.candidates(r))
        assert ngated > 0


def test_skzap_catches_sinusoids(tx, oracle):
    fil, rows, ndump = small_workload()
    sines = sorted(c for c, _, _, _ in fil.sines)
    with tx.Search(rows[:1], fil.nchans, fil.tsamp, fil.freqs, ndump, zapthre=4.0) as s:
        for b in range(2):
            raw = fil.generate(b * ndump, ndump)
            s.push_block(raw)
            s.sync()
            m = s.mask()
            np.testing.assert_array_equal(m, oracle.skzap(raw, 4.0))
            assert m[sines].all()


def test_kadane_fires_on_rfi(tx, oracle):
    fil, rows, ndump = small_workload()
    with tx.Search(rows[:1], fil.nchans, fil.tsamp, fil.freqs, ndump,
                   flags=tx.FLAG_KEEP_SERIES, zapthre=0.0) as s:
        s.push_block(fil.generate(0, ndump))
        s.sync()
        zr = s.zap_ranges(0)
    assert (zr[:, 0] >= 0).any(), "the sinusoid channels should be zapped"


@pytest.mark.parametrize("prec,bound", [("fp16", 4e-3), ("bf16", 3e-2)])
def test_reduced_precision_series(tx, prec, bound):
    """BF16/FP16 storage of the subband series: dedispersed series stay close to FP32.  Each
    stored subband sample carries a relative rounding error of at most 2^-9 (bf16) or 2^-12
    (fp16); summed over 8-16 subbands that bounds the worst sample at a few percent (bf16) or
    a few 1e-3 (fp16) of the series' standard deviation."""
    fil, rows, ndump = small_workload()
    flags = tx.FLAG_KEEP_SERIES
    with tx.Search(rows, fil.nchans, fil.tsamp, fil.freqs, ndump, flags=flags) as a, \
            tx.Search(rows, fil.nchans, fil.tsamp, fil.freqs, ndump, flags=flags,
                      precision=prec) as b:
        for blk in range(4):
            raw = fil.generate(blk * ndump, ndump)
            a.push_block(raw)
            b.push_block(raw)
        a.sync()
        b.sync()
        for r in range(len(rows)):
            ta, tb = a.timdata(r), b.timdata(r)
            scale = ta.std(axis=1, keepdims=True)
            err = np.abs(ta - tb) / scale
            assert err.max() < bound, (prec, r, err.max())


def test_bounded_wait_gives_up_and_context_stays_usable(tx):
    """A barrier that never completes: the kernel's bounded wait runs out after the limit and
    reports TXG_ERR_TIMEOUT; the context keeps working (a completing copy, then a search)."""
    import time
    assert tx.selftest_wait(False, 500) == tx.OK
    t0 = time.perf_counter()
    assert tx.selftest_wait(True, 200) == tx.ERR_TIMEOUT
    assert 0.15 < time.perf_counter() - t0 < 10.0
    assert tx.selftest_wait(False, 500) == tx.OK
    fil, rows, ndump = small_workload()
    with tx.Search(rows, fil.nchans, fil.tsamp, fil.freqs, ndump) as s:
        for b in range(2):
            s.push_block(fil.generate(b * ndump, ndump))
        s.sync()


def test_result_ready_polls_without_waiting(tx):
    """txg_result_ready: None with nothing waiting; after sync every waiting block is ready and
    pops in push order with the same results as a blocking pop."""
    fil, rows, ndump = small_workload()
    with tx.Search(rows, fil.nchans, fil.tsamp, fil.freqs, ndump, flags=tx.FLAG_CLUSTER) as s:
        assert s.result_ready(0) is None
        n = fil.nsamples // ndump
        for b in range(n):
            s.push_block(fil.generate(b * ndump, ndump))
            while s.result_ready(0):
                s.pop_result(0)
        s.sync()
        counters = []
        while True:
            r = s.result_ready(0)
            if r is None:
                break
            assert r is True
            counters.append(s.pop_result(0)[0].counter)
        assert counters == sorted(counters) and len(counters) >= 1
        assert s.pop_result(0) is None


def test_candidate_overflow_is_reported(tx):
    fil, rows, ndump = small_workload()
    rows = [rows[0]]
    rows[0].thre = -1e9  # every point passes
    with tx.Search(rows, fil.nchans, fil.tsamp, fil.freqs, ndump, cand_capacity=1000) as s:
        for blk in range(3):
            s.push_block(fil.generate(blk * ndump, ndump))
        rc = s.sync(allow_overflow=True)
        assert rc == tx.ERR_OVERFLOW
        assert len(s.candidates(0)) == 1000


def test_device_pointer_input_matches_host_input(tx):
    import ctypes
    fil, rows, ndump = small_workload()
    cudart = ctypes.CDLL("libcudart.so")
    raw = fil.generate(0, 3 * ndump)
    dptr = ctypes.c_void_p()
    assert cudart.cudaMalloc(ctypes.byref(dptr), ctypes.c_size_t(raw.nbytes)) == 0
    try:
        assert cudart.cudaMemcpy(dptr, raw.ctypes.data, ctypes.c_size_t(raw.nbytes), 1) == 0
        with tx.Search(rows, fil.nchans, fil.tsamp, fil.freqs, ndump,
                       flags=tx.FLAG_KEEP_SERIES) as a, \
                tx.Search(rows, fil.nchans, fil.tsamp, fil.freqs, ndump,
                          flags=tx.FLAG_KEEP_SERIES) as b:
            for blk in range(3):
                a.push_block(raw[blk * ndump:(blk + 1) * ndump])
                b.push_block_device(dptr.value + blk * ndump * fil.nchans)
            a.sync()
            b.sync()
            for r in range(len(rows)):
                np.testing.assert_array_equal(a.timdata(r), b.timdata(r))
    finally:
        cudart.cudaFree(dptr)


def _peak_errors(S_gpu, W_gpu, S_ref, thre, tol):
    """Relative S/N error at every point above threshold in the FP64 reference, and whether the
    brightest point of each DM row (the peak a cluster would report) is the same sample, or a
    sample the reference scores within tol of its maximum (a tie at that precision)."""
    sel = S_ref > thre
    rel = np.abs(S_gpu[sel] - S_ref[sel]) / S_ref[sel] if sel.any() else np.zeros(0)
    rows = np.nonzero(sel.any(axis=1))[0]
    same_peak = []
    for r in rows:
        a, b = int(np.argmax(S_gpu[r])), int(np.argmax(S_ref[r]))
        same_peak.append(a == b or S_ref[r, a] >= S_ref[r, b] * (1 - tol))
    return rel, np.array(same_peak, bool)


@pytest.mark.parametrize("prec,bound", [("fp32", 1e-4), ("fp16", 1e-3), ("bf16", None)])
def test_snr_error_against_fp64_oracle(tx, oracle, prec, bound):
    """S/N at every point above threshold against the FP64 reference (dedispersion sums and
    boxcar statistics in double): FP32 within 1e-4, FP16 storage within 1e-3, BF16 reported."""
    fil, rows, ndump = small_workload()
    rows = [rows[0]]
    orow = oracle_rows(oracle, rows, fil, ndump, tx, zapthre=4.0)[0]
    info = tx.describe_row(rows, 0, fil.nchans, fil.tsamp, fil.freqs, ndump)[0]
    r64 = oracle.make_row(td=rows[0].td, fd=rows[0].fd, bswidth=rows[0].bswidth,
                          rfi=rows[0].rfilist, widthlimit=rows[0].widthlimit, dms=rows[0].dms,
                          ddm=rows[0].ddm, ndm=rows[0].ndm, nsub=info.nsub, group=info.dm_group,
                          maxw=rows[0].maxw, thre=rows[0].thre, zapthre=4.0, fp64=True)
    o64 = oracle.SinglePulseRow(r64, fil.freqs, fil.tsamp, ndump)
    worst, npts = 0.0, 0
    with tx.Search(rows, fil.nchans, fil.tsamp, fil.freqs, ndump, precision=prec,
                   flags=tx.FLAG_DENSE, zapthre=4.0) as s:
        for b in range(fil.nsamples // ndump):
            raw = fil.generate(b * ndump, ndump)
            s.push_block(raw)
            s.sync()
            if not o64.run(raw):
                continue
            S, W = s.dense(0)
            rel, same = _peak_errors(S, W, o64.mxS(), rows[0].thre, bound or 0.0)
            npts += len(rel)
            if len(rel):
                worst = max(worst, float(rel.max()))
            if bound is not None:
                assert same.all(), f"{prec}: a row's peak moved"
    assert npts > 0, "the injected pulses should give points above threshold"
    print(f"{prec}: {npts} points above threshold, max relative S/N error {worst:.2e}")
    if bound is not None:
        assert worst <= bound, (prec, worst)


@pytest.mark.parametrize("prec,pinned,nbeams", [("fp32", False, 1), ("fp32", True, 1),
                                                ("fp16", False, 1), ("fp32", False, 2)])
def test_streamed_blocks_equal_synced_blocks(tx, prec, pinned, nbeams):
    """Blocks pushed back to back (the device runs up to three blocks ahead, the rows of a
    block run on their own streams, candidate slots are reused while earlier blocks are still
    being clustered, beams interleave) give, block by block, the same points and clusters as
    pushing one block and waiting for it.  Pinned inputs are copied asynchronously, so each
    block keeps its own buffer until the sync."""
    import torch
    fil, rows, ndump = small_workload()
    nblk = fil.nsamples // ndump
    raws = [fil.generate(b * ndump, ndump) for b in range(nblk)]
    if pinned:
        bufs = [torch.empty(r.shape, dtype=torch.uint8, pin_memory=True) for r in raws]
        for t, r in zip(bufs, raws):
            t.numpy()[...] = r
        inputs = [t.numpy() for t in bufs]
    else:
        inputs = raws

    def drain(s, beam, out):
        for r in range(len(rows)):
            while True:
                got = s.pop_result(r, beam)
                if got is None:
                    break
                res, pts, cl = got
                out[r].append((res.counter, res.gated, pts, cl))

    kw = dict(flags=tx.FLAG_CLUSTER, precision=prec)
    ref = [[] for _ in rows]
    with tx.Search(rows, fil.nchans, fil.tsamp, fil.freqs, ndump, **kw) as a:
        for raw in raws:
            a.push_block(raw)
            a.sync()
            drain(a, 0, ref)
    streamed = [[[] for _ in rows] for _ in range(nbeams)]
    with tx.Search(rows, fil.nchans, fil.tsamp, fil.freqs, ndump, nbeams=nbeams, **kw) as b:
        for x in inputs:
            for beam in range(nbeams):
                b.push_block(x, beam=beam)
        b.sync()
        for beam in range(nbeams):
            drain(b, beam, streamed[beam])
    npts = 0
    for beam in range(nbeams):
        for r in range(len(rows)):
            assert len(ref[r]) == len(streamed[beam][r]) == nblk
            for blk, (u, v) in enumerate(zip(ref[r], streamed[beam][r])):
                where = f"beam {beam} row {r} block {blk}"
                assert u[:2] == v[:2], where
                np.testing.assert_array_equal(u[2], v[2], err_msg=where + " points")
                np.testing.assert_array_equal(u[3], v[3], err_msg=where + " clusters")
                npts += len(u[2])
    assert npts > 0, "the injected pulses should give points above threshold"


@pytest.mark.parametrize("prec", ["fp32", "fp16"])
def test_reset_beam_equals_fresh_handle(tx, prec):
    """A beam that searched one file and is reset (txg_reset_beam) gives, block for block, the
    series, points and clusters that a fresh handle gives for the next file, while the other
    beam of the handle is unaffected; the first file's last results stay poppable."""
    from transientx_gb300 import synth
    fil, rows, ndump = small_workload()
    other = synth.Filterbank(fil.nchans, fil.tsamp, fil.freqs, fil.nsamples, 77,
                             pulses=[(0.6 * fil.nsamples * fil.tsamp, 120.0, 2e-3, 25.0)])
    nblk = fil.nsamples // ndump
    flags = tx.FLAG_KEEP_SERIES
    with tx.Search(rows, fil.nchans, fil.tsamp, fil.freqs, ndump, nbeams=2, precision=prec,
                   flags=flags) as s, \
            tx.Search(rows, fil.nchans, fil.tsamp, fil.freqs, ndump, precision=prec,
                      flags=flags) as fresh:
        for b in range(3):  # a first, partial file on beam 0
            s.push_block(fil.generate(b * ndump, ndump), beam=0)
        s.reset_beam(0)
        first = True
        ngated = 0
        for b in range(nblk):
            raw = other.generate(b * ndump, ndump)
            s.push_block(raw, beam=0)
            s.push_block(raw, beam=1)
            fresh.push_block(raw)
            s.sync()
            fresh.sync()
            if first:  # the first file's three blocks, then the new file's first block
                for r in range(len(rows)):
                    counters = []
                    while True:
                        out = s.pop_result(r, beam=0, points=False)
                        if out is None:
                            break
                        counters.append(out[0].counter)
                    N = s.row_info(r).ndump
                    assert counters == [N, 2 * N, 3 * N, N], counters
                first = False
            for r in range(len(rows)):
                a, f = s.row_info(r, beam=0), fresh.row_info(r)
                assert (a.counter, a.gated) == (f.counter, f.gated)
                if not f.gated:
                    continue
                ngated += 1
                np.testing.assert_array_equal(s.timdata(r, beam=0), fresh.timdata(r))
                np.testing.assert_array_equal(s.candidates(r, beam=0), fresh.candidates(r))
                np.testing.assert_array_equal(s.candidates(r, beam=1), fresh.candidates(r))
                np.testing.assert_array_equal(s.cluster(r, beam=0), fresh.cluster(r))
        assert ngated >= 4


def test_float_blocks_match_oracle(tx, oracle):
    """txg_push_block_f32: preprocessed float blocks (non-integer values, as PreprocessLite
    hands them to SinglePulse::run) give the oracle's float chain bit for bit: downsampled and
    equalized block, zap windows and dedispersed series; boxcar S within 1e-4."""
    fil, rows, ndump = small_workload()
    orows = oracle_rows(oracle, rows, fil, ndump, tx, zapthre=0.0)
    flags = tx.FLAG_DENSE | tx.FLAG_KEEP_SERIES
    ngated = 0
    with tx.Search(rows, fil.nchans, fil.tsamp, fil.freqs, ndump, flags=flags,
                   zapthre=4.0) as s:
        for b in range(fil.nsamples // ndump):
            raw = fil.generate(b * ndump, ndump)
            blk = ((raw.astype(np.float32) - np.float32(128.0)) / np.float32(12.3)
                   + np.float32(0.37)).astype(np.float32)
            s.push_block_f32(blk)
            s.sync()
            for r, o in enumerate(orows):
                gated = o.run_f32(blk)
                assert bool(s.row_info(r).gated) == gated
                np.testing.assert_array_equal(s.block(r), o.block(), err_msg=f"block {b} row {r}")
                np.testing.assert_array_equal(s.zap_ranges(0, r), o.zap_ranges(0))
                if not gated:
                    continue
                ngated += 1
                tim = s.timdata(r)
                np.testing.assert_array_equal(tim, o.timdata(), err_msg=f"tim block {b} row {r}")
                S, W = s.dense(r)
                assert_boxcar_close(tim, o.widths(), S, W, o.mxS(), o.mxwn())
    assert ngated >= 4
