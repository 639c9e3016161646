"""Parity at the sizes of the benchmarked configurations, through the same launch shapes the
bench uses: the 256-channel one-row search (2000 DMs, 16 subbands, 15625-sample blocks) and
each ddplan row of the 4096-channel RFI workload (5000/5000/3000 DMs at td 1/2/4, 128/128/256
subbands, 13156-sample blocks, kadaneF 8 4 + zdot, channel zap), each pushed from a start
block chosen so that an injected pulse of the row's DM range arrives in the first gated block,
until two blocks are gated.

Every block: channel-zap mask, preprocessed block and kadaneF windows bit-exact against the
oracle; every gated block: dedispersed series bit-exact, dense S within 1e-4*max(1,|S|)
(widths equal except ties within that), the production (non-dense) path's points above the
threshold equal to the oracle's scan except within 1e-4 of the threshold, and the clustered
candidate list (Cluster::run on those points, cluster.cpp:63-161) equal to the oracle's
clustering of its own points.  The reduced-precision paths are held against the FP64 oracle
on the heaviest row."""
import numpy as np
import pytest

from gpu_util import REL, assert_boxcar_close, assert_cands_close
from test_gpu_pipeline import oracle_rows

pytestmark = pytest.mark.gpu

CASES = {  # name: (workload, row)
    "nchan256_row0": ("nchan256_n1M_dm1000", 0),
    "nchan4096_row0": ("nchan4096_n2M_rfi_dm3000", 0),
    "nchan4096_row1": ("nchan4096_n2M_rfi_dm3000", 1),
    "nchan4096_row2": ("nchan4096_n2M_rfi_dm3000", 2),
    # a 1024-channel beam of the 64-beam job (64 subbands, DM groups of 8/8/7)
    "beams64_nchan1024_row0": ("beams64:1024", 0),
    "beams64_nchan1024_row2": ("beams64:1024", 2),
    # 8192 channels at 16 us: 62 496-sample rows (the segmented boxcar) and the td-16 row
    "nchan8192_row0": ("nchan8192_n8M_dm5000", 0),
    "nchan8192_row4": ("nchan8192_n8M_dm5000", 4),
}
ZAPTHRE = 4.0  # the bench's PreprocessLite channel-zap threshold
NGATED = 2


def _workload(name):
    """A single-beam workload, or "beams64:<C>": the 64-beam job's first beam of C channels
    that carries a pulse in every row's DM range, as a single-beam workload."""
    from transientx_gb300 import synth
    if not name.startswith("beams64:"):
        return synth.WORKLOADS[name]()
    C = int(name.split(":")[1])
    job = synth.beams64()
    ranges = [(sp.dms, sp.dms + sp.ndm * sp.ddm) for sp in job.rows]
    fil = next(f for f in job.beams if f.nchans == C and
               all(any(lo <= p[1] < hi for p in f.pulses) for lo, hi in ranges))
    return synth.Workload(name, fil, job.rows, job.ndump)


def plan_blocks(tx, wl, r):
    """(first raw block, blocks to push, first gated block) for row r: the earliest-arriving
    injected pulse inside the row's DM range lands in the first gated block."""
    sp = wl.rows[r]
    fil = wl.fil
    info = tx.describe_row(wl.rows, r, fil.nchans, fil.tsamp, fil.freqs, wl.ndump)[0]
    N, off, td = info.ndump, info.offset, sp.td
    k_gate = -(-(off - info.noverlap + N) // N) - 1
    lo, hi = sp.dms, sp.dms + sp.ndm * sp.ddm
    pulses = sorted(p for p in fil.pulses if lo <= p[1] < hi)
    s0 = 0
    if pulses:
        t_p = pulses[0][0] / fil.tsamp
        s0 = max(0, int((t_p - td * (k_gate * N - off)) // wl.ndump))
    return s0, k_gate + NGATED, k_gate


def _points_equal(a, b):
    ka = [(int(x["idm"]), int(x["isamp"])) for x in a]
    kb = [(int(x["idm"]), int(x["isamp"])) for x in b]
    return ka == kb


def _assert_clusters_equal(c_gpu, c_ref, what):
    assert len(c_gpu) == len(c_ref), f"{what}: {len(c_gpu)} vs {len(c_ref)} clusters"
    for f in ("idm", "isamp", "wn"):
        np.testing.assert_array_equal(np.asarray(c_gpu[f], np.int64),
                                      np.asarray(c_ref[f], np.int64), err_msg=f"{what}: {f}")
    S_g, S_r = np.asarray(c_gpu["S"], np.float64), np.asarray(c_ref["S"], np.float64)
    assert np.all(np.abs(S_g - S_r) <= REL * np.maximum(1.0, np.abs(S_r))), what


@pytest.mark.parametrize("case", list(CASES))
def test_benchmark_configuration_matches_oracle(tx, oracle, case):
    wname, r = CASES[case]
    wl = _workload(wname)
    fil, sp = wl.fil, wl.rows[r]
    rows = [sp]
    s0, nblk, k_gate = plan_blocks(tx, wl, r)
    o = oracle_rows(oracle, rows, fil, wl.ndump, tx, zapthre=ZAPTHRE)[0]
    vwn = o.widths()
    info0 = tx.describe_row(rows, 0, fil.nchans, fil.tsamp, fil.freqs, wl.ndump)[0]
    ngated, nclusters = 0, 0
    with tx.Search(rows, fil.nchans, fil.tsamp, fil.freqs, wl.ndump,
                   flags=tx.FLAG_DENSE | tx.FLAG_KEEP_SERIES, zapthre=ZAPTHRE) as dense, \
            tx.Search(rows, fil.nchans, fil.tsamp, fil.freqs, wl.ndump, zapthre=ZAPTHRE) as prod:
        assert (dense.row_info(0).nsub, dense.row_info(0).dm_group) == \
            (info0.nsub, info0.dm_group)
        for b in range(nblk):
            raw = fil.generate((s0 + b) * wl.ndump, wl.ndump)
            dense.push_block(raw)
            prod.push_block(raw)
            dense.sync()
            prod.sync()
            gated = o.run(raw)
            where = f"{case} block {b}"
            assert gated == (b >= k_gate) == bool(dense.row_info(0).gated), where
            np.testing.assert_array_equal(dense.mask(), o.mask(), err_msg=where)
            np.testing.assert_array_equal(dense.block(0), o.block(), err_msg=where)
            for q, op in enumerate(sp.rfilist):
                if op[0] == "kadaneF":
                    np.testing.assert_array_equal(dense.zap_ranges(q, 0), o.zap_ranges(q),
                                                  err_msg=where)
            if not gated:
                continue
            ngated += 1
            tim = dense.timdata(0)
            np.testing.assert_array_equal(tim, o.timdata(), err_msg=where)
            S, W = dense.dense(0)
            S_ref, W_ref = o.mxS(), o.mxwn()
            assert_boxcar_close(tim, vwn, S, W, S_ref, W_ref)
            ref_pts = oracle.threshold_scan(S_ref, W_ref, sp.thre)
            pts = prod.candidates(0)
            assert_cands_close(pts, ref_pts, sp.thre)
            assert_cands_close(dense.candidates(0), ref_pts, sp.thre)
            # Cluster::run: the product's clustering of its points equals the oracle's
            # clustering (pinned against the reference's Cluster::run) of the same points,
            # and, where the point lists agree, of the oracle's own points
            i = prod.row_info(0)
            args = (i.dms, i.ddm, i.fmax, i.fmin, i.tsamp, sp.radius_smearing, sp.maxncand,
                    sp.minpts, sp.remove_cand_with_maxwidth, i.maxwn)
            c_gpu = prod.cluster(0)
            ref_in = np.zeros(len(pts), oracle.CAND_DTYPE)
            for f in ("idm", "isamp", "wn", "S"):
                ref_in[f] = pts[f]
            c_same, _ = oracle.cluster(ref_in, *args)
            _assert_clusters_equal(c_gpu, c_same, where + " (same points)")
            if _points_equal(pts, ref_pts):
                c_ref, _ = oracle.cluster(ref_pts, *args)
                _assert_clusters_equal(c_gpu, c_ref, where + " (oracle points)")
            nclusters += len(c_gpu)
    assert ngated == NGATED
    assert nclusters > 0, "the injected pulse should give at least one candidate"


@pytest.mark.parametrize("prec,bound", [("fp16", 1e-3), ("bf16", None), ("fp32", 1e-4)])
def test_benchmark_row0_snr_against_fp64_oracle(tx, oracle, prec, bound):
    """The 4096-channel workload's heaviest row (td 1, 5000 DMs) with 16-bit subband storage:
    S/N of every point above the threshold and of every reported candidate against the FP64
    oracle (dedispersion sums and boxcar statistics in double).  FP16 within 1e-3 relative,
    FP32 within 1e-4; BF16 is reported.  The candidates' (DM, sample) indices are the FP64
    oracle's except where two members of a cluster score within the bound of each other."""
    wl = _workload("nchan4096_n2M_rfi_dm3000")
    fil, sp = wl.fil, wl.rows[0]
    rows = [sp]
    s0, nblk, k_gate = plan_blocks(tx, wl, 0)
    info = tx.describe_row(rows, 0, fil.nchans, fil.tsamp, fil.freqs, wl.ndump)[0]
    r64 = oracle.make_row(td=sp.td, fd=sp.fd, bswidth=sp.bswidth, rfi=sp.rfilist,
                          threKadaneF=sp.threKadaneF, widthlimit=sp.widthlimit, dms=sp.dms,
                          ddm=sp.ddm, ndm=sp.ndm, overlap=sp.overlap, nsub=info.nsub,
                          group=info.dm_group, minw=sp.minw, maxw=sp.maxw, snrloss=sp.snrloss,
                          thre=sp.thre, zapthre=ZAPTHRE, fp64=True)
    o64 = oracle.SinglePulseRow(r64, fil.freqs, fil.tsamp, wl.ndump)
    worst_pt, worst_cand, npts, ncand, moved = 0.0, 0.0, 0, 0, 0
    with tx.Search(rows, fil.nchans, fil.tsamp, fil.freqs, wl.ndump, precision=prec,
                   flags=tx.FLAG_DENSE, zapthre=ZAPTHRE) as s:
        for b in range(nblk):
            raw = fil.generate((s0 + b) * wl.ndump, wl.ndump)
            s.push_block(raw)
            s.sync()
            if not o64.run(raw):
                continue
            S, W = s.dense(0)
            S64 = o64.mxS()
            sel = S64 > sp.thre
            rel = np.abs(S[sel] - S64[sel]) / S64[sel]
            npts += int(sel.sum())
            worst_pt = max(worst_pt, float(rel.max()) if rel.size else 0.0)
            i = s.row_info(0)
            args = (i.dms, i.ddm, i.fmax, i.fmin, i.tsamp, sp.radius_smearing, sp.maxncand,
                    sp.minpts, sp.remove_cand_with_maxwidth, i.maxwn)
            c_gpu = s.cluster(0)
            c64, _ = oracle.cluster(oracle.threshold_scan(S64, o64.mxwn(), sp.thre), *args)
            for c in c_gpu:
                ref = float(S64[c["idm"], c["isamp"]])
                e = abs(float(c["S"]) - ref) / ref
                worst_cand = max(worst_cand, e)
                ncand += 1
            # indices: every FP64 candidate peak is a GPU candidate peak, or the GPU reports
            # a peak whose FP64 score ties it within the bound
            tol = bound if bound is not None else 1e-2
            peaks = {(int(c["idm"]), int(c["isamp"])) for c in c_gpu}
            for c in c64:
                k = (int(c["idm"]), int(c["isamp"]))
                if k in peaks:
                    continue
                moved += 1
                near = [S64[p] for p in peaks if abs(p[0] - k[0]) <= 64 and abs(p[1] - k[1]) <= 4096]
                if bound is not None:
                    assert near and max(near) >= float(c["S"]) * (1 - 2 * tol), \
                        f"{prec}: FP64 candidate {k} S={c['S']} has no GPU counterpart"
    print(f"{prec}: {npts} points, max rel S/N error {worst_pt:.2e}; {ncand} candidates, "
          f"max rel error {worst_cand:.2e}; {moved} FP64 peaks reported at a tied member")
    assert npts > 0 and ncand > 0
    if bound is not None:
        assert worst_pt <= bound, (prec, worst_pt)
        assert worst_cand <= bound, (prec, worst_cand)
