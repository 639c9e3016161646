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
        assert bench.launches_per_block(sp, info, True, "fp16") == 16
    # the profiled 20-block command: 80 pushes, 194 gated row-blocks -> 3748 kernels
    assert 80 * bench.SKZAP_LAUNCHES + 240 * 13 + 194 * 2 == 3748
