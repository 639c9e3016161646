"""bench.py's accounting, on the CPU: the stage-1 shared-memory loads it reports follow the
resident stage-1 kernel's thread-set structure (16 sets of 4 coarse-DM groups per CTA, groups
past the end repeating the last delay, a reload only where the delay changes), and the
kernel count per block follows run_block's launch sequence."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def loads_by_sets(d1, sets=16, gpt=4):
    """Window loads per output sample, walking chunks, sets and groups as k_stage1r does."""
    ng, C = d1.shape
    gpc = sets * gpt
    loads = 0
    for g0 in range(0, ng, gpc):
        gn = min(gpc, ng - g0)
        for gs in range(sets):
            prev = None
            for i in range(gpt):
                g = gs * gpt + i
                d = d1[g0 + (g if g < gn else gn - 1)]
                loads += C if prev is None else int((d != prev).sum())
                prev = d
    return loads


@pytest.mark.parametrize("ng,C", [(1, 7), (5, 33), (64, 16), (70, 64), (313, 128)])
def test_stage1_loads_follow_the_thread_sets(ng, C):
    rng = np.random.default_rng(ng * 1000 + C)
    steps = (rng.random((ng, C)) < 0.35).astype(np.int32)   # delays grow by 0 or 1 per group
    d1 = np.cumsum(steps, axis=0, dtype=np.int32)
    assert bench.stage1_window_loads(d1) == loads_by_sets(d1)


def test_stage1_loads_on_the_bench_workload():
    import transientx_gb300 as tx
    from transientx_gb300 import synth
    wl = synth.WORKLOADS["nchan4096_n2M_rfi_dm3000"](nsamples=1 << 16)
    for r in range(len(wl.rows)):
        info, d1 = tx.describe_row(wl.rows, r, wl.fil.nchans, wl.fil.tsamp, wl.fil.freqs,
                                   wl.ndump)[:2]
        n = bench.stage1_window_loads(d1)
        assert n == loads_by_sets(d1)
        # neighbouring groups share most delays: about half a load per addition
        assert 0.4 < n / d1.size < 0.6, (r, n / d1.size)
        smem = bench.class_smem_bytes(info, 4, d1)
        assert smem[2] == 4.0 * info.ndump * n


def test_kernels_per_block_follow_run_block():
    import transientx_gb300 as tx
    from transientx_gb300 import synth
    wl = synth.WORKLOADS["nchan4096_n2M_rfi_dm3000"](nsamples=1 << 16)
    for r, sp in enumerate(wl.rows):
        info = tx.describe_row(wl.rows, r, wl.fil.nchans, wl.fil.tsamp, wl.fil.freqs, wl.ndump)[0]
        # unpack, equalize parameters, baseline (colmean, smooth, apply), kadaneF 3, zdot 4,
        # stage 1; gated blocks add stage 2 and the boxcar (rows under 51 200 samples)
        assert bench.launches_per_block(sp, info, False) == 13
        assert bench.launches_per_block(sp, info, True) == 15
        assert bench.launches_per_block(sp, info, True, "fp16") == 15
    # the profiled 20-block command: 80 pushes, 194 gated row-blocks -> 3748 kernels
    assert 80 * bench.SKZAP_LAUNCHES + 240 * 13 + 194 * 2 == 3748


@pytest.mark.parametrize("workload", ["beams64_nchan1024_4096", "nchan4096_n2M_rfi_dm3000"])
def test_reference_arm_prints_its_line(workload):
    """`bench.py --impl reference` (the oracle port on the host cores, no GPU): one JSON line
    with the contract's keys, the same metric as the GPU arm, zero host-device bytes; it
    plans with the oracle's own rule and never loads the product library."""
    import json
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    probe = ("import runpy, sys; sys.argv = ['bench.py'] + sys.argv[1:]; "
             "runpy.run_path('bench.py', run_name='__main__'); "
             "maps = open('/proc/self/maps').read(); "
             "assert 'libtxgpu' not in maps, 'the reference arm loaded the product library'")
    r = subprocess.run([sys.executable, "-c", probe, "--impl", "reference", "--workload",
                        workload, "--steps", "1", "--warmup", "0"], capture_output=True,
                       text=True, timeout=900, cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "DM-trial samples/s"
    assert d["unit"] == d["metric"] and d["higher_is_better"] is True and d["value"] > 0
    assert d["steps"] == 1 and d["warmup"] == 0 and d["n_gpus"] == 1
    assert d["config"]["workload"] == workload
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_alu_roofline_of_the_bench_workload():
    """The FP32-operation roofline bench.py adds beside the HBM and shared-memory ones, on the
    class times of a full FP32 bench (2 steps of 159 blocks, rows serialised): stage 1 adds at
    a quarter of the 152 x 128 lanes x 2070 MHz peak; the line serialises to JSON."""
    import json
    import transientx_gb300 as tx
    from transientx_gb300 import synth
    wl = synth.WORKLOADS["nchan4096_n2M_rfi_dm3000"](nsamples=1 << 16)
    cls_ms = np.array([67.3, 328.9, 904.7, 645.5, 431.1])
    nblk, tsteps = 159, 2
    op_total = [0.0] * 5
    for r in range(len(wl.rows)):
        info = tx.describe_row(wl.rows, r, wl.fil.nchans, wl.fil.tsamp, wl.fil.freqs, wl.ndump)[0]
        ob = bench.class_fp32_ops(info)
        for c in (2, 3, 4):
            op_total[c] += ob[c] * tsteps * nblk
    alu = bench.alu_roofline(op_total, cls_ms, 2070.0)
    json.dumps(alu)
    assert abs(alu["peak"] - 152 * 128 * 2.07e9 / 1e12) < 1e-9
    assert set(alu["classes"]) == {"stage1", "stage2", "boxcar"}
    assert 0.15 < alu["classes"]["stage1"]["frac"] < 0.35
    for v in alu["classes"].values():
        assert 0.0 < v["frac"] < 1.0


def test_profiled_stage1_traffic_matches_the_algorithmic_bytes():
    """The DRAM traffic per stage-1 launch that bench.py reports (an ncu capture scaled to the
    three rows' launches) is the algorithmic stage-1 bytes of those launches within 10 %:
    each channel window crosses DRAM once and each subband sample is written once."""
    import transientx_gb300 as tx
    from transientx_gb300 import synth
    wl = synth.WORKLOADS["nchan4096_n2M_rfi_dm3000"](nsamples=1 << 16)
    for prec, elem in (("fp32", 4), ("fp16", 2)):
        alg = []
        for r, sp in enumerate(wl.rows):
            info = tx.describe_row(wl.rows, r, wl.fil.nchans, wl.fil.tsamp, wl.fil.freqs,
                                   wl.ndump)[0]
            alg.append(bench.class_bytes(info, sp, wl.fil.nchans, wl.ndump, 0, elem)[2])
        measured = bench.profiled_traffic("nchan4096_n2M_rfi_dm3000", prec, "stage1")[0]
        ratio = measured / (sum(alg) / len(alg))
        assert 0.9 < ratio < 1.1, (prec, ratio)


def test_lane_schedule_walks_every_beam_in_order():
    """Lanes of one channel count take that count's beams in job order, push each beam's
    blocks from 0 consecutively and reset exactly when they change beam; the job's beams are
    all started, in order, before any starts again."""
    from transientx_gb300 import synth
    job = synth.beams64()
    ids = list(range(len(job.beams)))
    lanes, bps = 3, 2
    per_chan = max(sum(job.nblocks(b) for b in ids if job.beams[b].nchans == C)
                   for C in (1024, 4096))
    nsteps = (3 * per_chan) // (2 * lanes * bps)  # about one and a half passes over the job
    chans, steps = bench.lane_schedule(job, ids, lanes, nsteps, bps)
    assert chans == [1024, 4096]
    for C in chans:
        order = [b for b in ids if job.beams[b].nchans == C]
        starts, prev = [], {}
        for st in steps:
            for c, lane, b, k, reset in st:
                if c != C:
                    continue
                assert job.beams[b].nchans == C and k < job.nblocks(b)
                p = prev.get(lane)
                if p is None or p[0] != b or k == 0:
                    assert k == 0 and reset == (p is not None), (lane, b, k, p)
                    starts.append(b)
                else:
                    assert k == p[1] + 1 and not reset
                prev[lane] = (b, k)
        assert len(starts) > len(order), "the schedule should run through the job"
        assert starts == (order * (len(starts) // len(order) + 1))[:len(starts)]


def test_pipeline_bytes_of_the_rfi_workload():
    """The pipeline roofline's algorithmic bytes per block of the 4096-channel workload (FP32):
    the raw block three times (RFI filters on) plus each row's subband series written and read
    once: 7.3 GB per block, halved series in 16-bit storage."""
    import transientx_gb300 as tx
    from transientx_gb300 import synth
    wl = synth.WORKLOADS["nchan4096_n2M_rfi_dm3000"](nsamples=1 << 16)
    infos = [tx.describe_row(wl.rows, r, wl.fil.nchans, wl.fil.tsamp, wl.fil.freqs, wl.ndump)[0]
             for r in range(len(wl.rows))]
    raw = 4096 * wl.ndump
    series = sum(2 * i.nsub * i.ngroup * i.ndump for i in infos)
    assert bench.b_alg_block(infos, wl.rows, 4096, wl.ndump, 4, 10) == 3 * raw + 4 * series + 160
    assert bench.b_alg_block(infos, wl.rows, 4096, wl.ndump, 2, 0) == 3 * raw + 2 * series
    assert 7.1e9 < bench.b_alg_block(infos, wl.rows, 4096, wl.ndump, 4, 0) < 7.5e9
