"""Benchmark: DM-trial samples/s of the single-pulse search (unpack -> RFI -> subband
dedispersion over the ddplan -> boxcar + threshold) on one GB300 per rank.

A step is one pass of every ddplan row over a whole synthetic filterbank (all its blocks).
`value` times the device work with the input already resident in HBM (txg_push_block_device);
`e2e` times the public host-pointer call (txg_push_block from pinned host memory, H2D inside
the timed region) plus the per-block candidate read-back and host clustering.  Ranks are
independent beams (weak scaling, no collective on the data path).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

ELEM = {"fp32": 4, "bf16": 2, "fp16": 2}
# DRAM read+write bytes per launch of the dominant class from one ncu capture of this workload
# (profiles/traffic_nchan4096_n2M_rfi_dm3000.md: mean over the three ddplan rows' launches)
PROFILED_TRAFFIC = {("nchan4096_n2M_rfi_dm3000", "fp32", "stage1"): 1285.2e6,
                    ("nchan4096_n2M_rfi_dm3000", "fp16", "stage1"): 607.5e6}
ZAPTHRE = 4.0  # PreprocessLite skewness/kurtosis channel-zap threshold (transientx_fil default)


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="nchan4096_n2M_rfi_dm3000")
    ap.add_argument("--nsamples", type=int, default=0, help="override the file length")
    ap.add_argument("--precision", choices=["fp32", "bf16", "fp16"], default="fp32")
    ap.add_argument("--replot", type=int, default=0,
                    help="time the replot chain on this many 4096-channel candidates instead")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-blocks", type=int, default=2, help="timed oracle blocks (CPU baseline)")
    ap.add_argument("--rows", default="", help="comma-separated ddplan rows to keep (profiling)")
    ap.add_argument("--ndm", type=int, default=0, help="override ndm of every row (profiling)")
    return ap.parse_args()


# ---- clocks during the timed region -------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index, self.rows, self.proc = index, [], None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.rows)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---- algorithmic bytes per kernel class (per launch, per row) ----------------------------
def class_bytes(info, sp, nchans_raw, ndump_raw, ncand, elem):
    """Bytes a perfect implementation must move for one launch of each class:
    unpack: raw uint8 in + float block out; preprocess: read+write the block once (16-bit
    precisions: plus its FP16 copy out); stage 1: block in (FP32, or its FP16 copy) + subband
    series out; stage 2: subband series in + dedispersed out; boxcar: dedispersed series in +
    16-byte candidates out."""
    C, N = info.nchans, info.ndump
    block = 4.0 * C * N
    block_in = float(elem) * C * N
    series = float(elem) * info.nsub * info.ngroup * N
    pre = 2 * block + (block_in if elem == 2 else 0.0)
    return [nchans_raw * ndump_raw + block, pre, block_in + series,
            series + 4.0 * info.ndm * info.nsamples, 4.0 * info.ndm * info.nsamples + 16 * ncand]


RFI_LAUNCHES = {"kadaneF": 3, "kadaneT": 3, "zdot": 4, "zero": 2, "mask": 10}
BOXCAR_ROW_MAX = 51200  # samples of a dedispersed row one boxcar CTA holds; longer rows: 2 kernels


SMEM_BYTES_PER_CLK = 128  # shared-memory bytes one SM delivers per clock
NSM = 152


S1_SETS, S1_GPT = 16, 4  # default stage-1 shapes: 16 thread sets of 4 coarse-DM groups per CTA


def stage1_window_loads(d1):
    """Window elements stage 1 loads per output sample, summed over channels and thread sets,
    at the default launch shapes: a thread set loads a channel's window values for its first
    group and again wherever the delay differs from the previous group's (groups past the end
    repeat the last delay)."""
    ng, C = d1.shape
    gpc = S1_SETS * S1_GPT
    nch = (ng + gpc - 1) // gpc
    pad = np.concatenate([d1, np.repeat(d1[-1:], nch * gpc - ng, axis=0)]).reshape(-1, S1_GPT, C)
    return int(pad.shape[0] * C + (pad[:, 1:] != pad[:, :-1]).sum())


def class_smem_bytes(info, elem, d1):
    """Shared-memory bytes one launch of the classes bound by shared memory loads: stage 1 one
    window element per sample for each delay change within a thread set's groups (the loads
    the kernel makes; additions are C x ngroup x N), stage 2 one window element per addition
    (nsub x ndm x (N + noverlap)), the boxcar two running-sum values per (sample, width).
    Other classes: None."""
    return [None, None, float(elem) * info.ndump * stage1_window_loads(d1),
            float(elem) * info.nsub * info.ndm * info.nsamples,
            8.0 * info.ndm * info.nsamples * info.nwidths]


FP32_LANES_PER_SM = 128  # FP32 operations one SM issues per clock (4 partitions x 32 lanes)


def class_fp32_ops(info):
    """FP32 operations of one launch of the compute classes, one per lane instruction of the
    algorithm: stage 1 one add per (channel, coarse DM, sample), stage 2 one add per (subband,
    DM, output sample), the boxcar 3 per (DM, sample) for the statistics and running sum plus
    4 per (DM, sample, width): subtract, multiply, compare, select.  Other classes: None."""
    return [None, None, float(info.nchans) * info.ngroup * info.ndump,
            float(info.nsub) * info.ndm * info.nsamples,
            float(info.ndm) * info.nsamples * (3 + 4 * info.nwidths)]


def alu_roofline(op_total, cls_ms, sm_mhz):
    """FP32 operations per second of stage 1, stage 2 and the boxcar against 152 SMs x 128
    lanes x the SM clock (one operation per lane per clock)."""
    peak = NSM * FP32_LANES_PER_SM * float(sm_mhz) * 1e6 / 1e12
    classes = {}
    for c, name in ((2, "stage1"), (3, "stage2"), (4, "boxcar")):
        if float(cls_ms[c]) > 0 and op_total[c]:
            a = float(op_total[c]) / (float(cls_ms[c]) / 1e3) / 1e12
            classes[name] = {"achieved": a, "frac": a / peak}
    return {"unit": "Top/s", "peak": peak,
            "peak_basis": f"{NSM} SMs x {FP32_LANES_PER_SM} FP32 lanes x median SM clock",
            "basis": "stage 1 one add per (channel, coarse DM, sample), stage 2 one add per "
                     "(subband, DM, sample), boxcar 3 per (DM, sample) + 4 per (DM, sample, "
                     "width)", "classes": classes}


def launches_per_block(sp, info, gated, precision="fp32"):
    """Kernels one block launches for one ddplan row (txg_api.cu run_block)."""
    n = 2  # unpack, equalize parameters
    n += 3 if sp.bswidth > 0 else 1  # colmean, smooth, equalize+baseline apply | apply
    if sp.zaplist:
        n += 1
    for op in sp.rfilist:
        n += RFI_LAUNCHES[op[0]]
    if precision != "fp32":
        n += 1  # FP16 copy of the block
    n += 1  # stage 1
    if gated:
        n += 1 + (2 if info.nsamples > BOXCAR_ROW_MAX else 1)  # stage 2, boxcar
    return n


SKZAP_LAUNCHES = 3  # per block, all rows: moments, statistics, outlier selection


# ---- reference arm / CPU baseline: the oracle port on the host cores ------------------------
def cpu_reference(wl, steps, warmup, timed_blocks=None, nthreads=0):
    """Oracle restatement of the path (oracle/txoracle.c) on the machine's host cores, row 0 of the
    workload (its heaviest ddplan row): warm the row until it is gated, then time one block
    per step.  Returns (value, seconds per step, sample description, cores)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    import transientx_gb300 as tx
    O.build(ref=False)
    cores = nthreads or os.cpu_count()
    O.lib().txo_set_threads(cores)
    sp = wl.rows[0]
    info = tx.describe_row(wl.rows, 0, wl.fil.nchans, wl.fil.tsamp, wl.fil.freqs, wl.ndump)[0]
    row = O.make_row(td=sp.td, fd=sp.fd, bswidth=sp.bswidth, rfi=sp.rfilist,
                     threKadaneF=sp.threKadaneF, widthlimit=sp.widthlimit, dms=sp.dms,
                     ddm=sp.ddm, ndm=sp.ndm, overlap=sp.overlap, nsub=info.nsub,
                     group=info.dm_group, minw=sp.minw, maxw=sp.maxw, snrloss=sp.snrloss,
                     thre=sp.thre, zapthre=ZAPTHRE)
    orow = O.SinglePulseRow(row, wl.fil.freqs, wl.fil.tsamp, wl.ndump)
    b = 0
    while True:  # fill the DM-delay history (not timed)
        raw = wl.fil.generate(b * wl.ndump, wl.ndump)
        b += 1
        if orow.run(raw):
            break
    n = (timed_blocks if timed_blocks else steps + warmup)
    times = []
    for k in range(n):
        raw = wl.fil.generate(b * wl.ndump, wl.ndump)
        b += 1
        t = time.perf_counter()
        assert orow.run(raw)
        times.append(time.perf_counter() - t)
    timed = times[warmup:] if not timed_blocks else times
    per = float(np.mean(timed))
    work = info.ndm * info.nsamples
    sample = (f"row 0 of {wl.name} (td={sp.td}, {sp.ndm} DMs, {info.nchans} channels, "
              f"{info.ndump}-sample blocks): {len(timed)} gated blocks timed after "
              f"{b - len(times)} history blocks")
    return work / per, per, sample, cores


def run_reference(args, wl):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    value, per, sample, cores = cpu_reference(wl, args.steps, args.warmup)
    line = {"metric": "DM-trial samples/s", "value": value, "unit": "DM-trial samples/s",
            "impl": "reference", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": per * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": wl.name, "sample": "one gated block of ddplan row 0 per step"},
            "cpu_baseline": {"value": value, "unit": "DM-trial samples/s", "cores": cores,
                             "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "DM-trial samples/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---- our arm ------------------------------------------------------------------------------
def run_ours(args, wl):
    import torch
    import transientx_gb300 as tx
    import transientx_gb300.shard  # noqa: F401

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    fil = wl.fil
    if world > 1:  # each rank searches its own beam
        fil.seed = fil.seed + rank
    nblk = fil.nsamples // wl.ndump
    host = torch.empty((nblk * wl.ndump, fil.nchans), dtype=torch.uint8, pin_memory=True)
    fil.generate(0, nblk * wl.ndump, out=host.numpy())
    dev = host.to("cuda", non_blocking=False)
    base = dev.data_ptr()
    blk_bytes = wl.ndump * fil.nchans

    def make_search(flags):
        return tx.Search(wl.rows, fil.nchans, fil.tsamp, fil.freqs, wl.ndump,
                         precision=args.precision, flags=flags, zapthre=ZAPTHRE)

    # the headline pass: the rows of a block run concurrently, each on its own stream
    s = make_search(0)
    infos = [s.row_info(r) for r in range(len(wl.rows))]
    stream = torch.cuda.ExternalStream(s.stream())

    def drain(stats):
        for r in range(len(wl.rows)):
            while True:
                out = s.pop_result(r, points=False)
                if out is None:
                    break
                res = out[0]
                if res.gated:
                    stats["work"] += infos[r].ndm * infos[r].nsamples
                    stats["ncand"][r] += res.npoints
                    stats["gated"][r] += 1
                    stats["launches"] += launches_per_block(wl.rows[r], infos[r], True, args.precision)
                else:
                    stats["launches"] += launches_per_block(wl.rows[r], infos[r], False, args.precision)

    def new_stats():
        return {"work": 0, "ncand": [0] * len(wl.rows), "gated": [0] * len(wl.rows),
                "launches": 0, "d2h": 0}

    def step_device(stats):
        for b in range(nblk):
            s.push_block_device(base + b * blk_bytes)
            stats["launches"] += SKZAP_LAUNCHES if ZAPTHRE > 0 else 0
            drain(stats)
        s.sync(allow_overflow=True)
        drain(stats)

    for _ in range(args.warmup):
        step_device(new_stats())
    stats = new_stats()
    clocks = ClockSampler(local)
    barrier()
    clocks.start()
    t_host = time.perf_counter()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step_device(stats)
    e1.record(stream)
    barrier()
    t_host = time.perf_counter() - t_host
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    s.close()
    # per-class device times: a second pass of the same workload with TXG_FLAG_TIMING, under
    # which the rows run one after another so that each class's event span holds its own
    # kernels only (concurrent rows share the GPU)
    s = make_search(tx.FLAG_TIMING)
    step_device(new_stats())  # gates every row
    s.timing()  # reset the per-class accumulators
    tsteps = min(args.steps, 2)
    tstats = new_stats()
    for _ in range(tsteps):
        step_device(tstats)
    cls_ms, cls_n = s.timing()
    if dist is not None:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    work_total = stats["work"] * world
    value = work_total / (ms / 1e3)

    # dominant kernel class and its roofline
    names = ["unpack", "preprocess", "stage1", "stage2", "boxcar"]
    top = int(np.argmax(cls_ms))
    nb_total = [0.0] * 5
    for r, (sp, info) in enumerate(zip(wl.rows, infos)):
        nblocks_r = tstats["gated"][r]  # every timed block is gated after the warm-up
        ncand_avg = tstats["ncand"][r] / max(1, tstats["gated"][r])
        cb = class_bytes(info, sp, fil.nchans, wl.ndump, ncand_avg, ELEM[args.precision])
        for c in range(5):
            nb_total[c] += cb[c] * (tsteps * nblk if c < 3 else nblocks_r)
    sm_total = [0.0] * 5
    op_total = [0.0] * 5
    for r, (sp, info) in enumerate(zip(wl.rows, infos)):
        d1 = tx.describe_row(wl.rows, r, fil.nchans, fil.tsamp, fil.freqs, wl.ndump)[1]
        sb = class_smem_bytes(info, ELEM[args.precision], d1)
        ob = class_fp32_ops(info)
        for c in (2, 3, 4):
            sm_total[c] += sb[c] * (tsteps * nblk if c < 3 else tstats["gated"][r])
            op_total[c] += ob[c] * (tsteps * nblk if c < 3 else tstats["gated"][r])
    peak, peak_kind = measured_peaks()
    achieved = nb_total[top] / (cls_ms[top] / 1e3) / 1e9
    roof = {"bound": "hbm", "kernel": names[top], "achieved": achieved, "peak": peak,
            "unit": "GB/s", "frac": achieved / peak,
            "traffic": PROFILED_TRAFFIC.get((wl.name, args.precision, names[top])),
            "traffic_source": ("profiles/traffic_nchan4096_n2M_rfi_dm3000.md (ncu, bytes per launch)"
                               if (wl.name, args.precision, names[top]) in PROFILED_TRAFFIC else None),
            "peak_source": peak_kind,
            "class_timing": f"CUDA events per kernel class, second pass of {tsteps} steps with "
                            "the rows serialised (TXG_FLAG_TIMING)",
            "class_ms": {names[c]: float(cls_ms[c]) for c in range(5)},
            "class_launches": {names[c]: int(cls_n[c]) for c in range(5)},
            "class_algorithmic_GBps": {names[c]: (nb_total[c] / (cls_ms[c] / 1e3) / 1e9
                                                   if cls_ms[c] > 0 else None) for c in range(5)}}
    if top in (2, 3, 4) and cls_ms[top] > 0:
        # the dedispersion and boxcar kernels are bound by shared-memory bandwidth, not HBM
        sm_clk = (clk or {}).get("sm_mhz") or 2070.0
        sm_peak = NSM * SMEM_BYTES_PER_CLK * sm_clk * 1e6 / 1e12
        sm_ach = sm_total[top] / (cls_ms[top] / 1e3) / 1e12
        roof["smem"] = {"achieved": sm_ach, "peak": sm_peak, "unit": "TB/s", "frac": sm_ach / sm_peak,
                        "peak_basis": f"{NSM} SMs x {SMEM_BYTES_PER_CLK} B/clock x median SM clock",
                        "basis": "window elements loaded: stage 1 one per sample for each delay "
                                 "change within a thread set's coarse-DM groups (default shapes), "
                                 "stage 2 one per addition; two running-sum loads per sample and "
                                 "width (boxcar)"}

    roof["alu"] = alu_roofline(op_total, cls_ms, (clk or {}).get("sm_mhz") or 2070.0)

    s.close()
    e2e = None
    if not args.no_e2e:
        # the public host-pointer path: pinned host blocks, H2D inside the timed region, and
        # Cluster::run on every block inside the library while the device runs ahead
        s = tx.Search(wl.rows, fil.nchans, fil.tsamp, fil.freqs, wl.ndump,
                      precision=args.precision, flags=tx.FLAG_CLUSTER, zapthre=ZAPTHRE)
        hpin = host.numpy()

        def pop_all(st, wait=True):
            # while streaming, only blocks whose clustering is done are popped (a streaming
            # consumer polls; the pushing thread never waits on host clustering)
            for r in range(len(wl.rows)):
                while True:
                    if not wait and not s.result_ready(r):
                        break
                    out = s.pop_result(r, points=False)
                    if out is None:
                        break
                    res, _, cl = out
                    st["d2h"] += 8 + 16 * res.npoints
                    if res.gated:
                        st["work"] += infos[r].ndm * infos[r].nsamples
                        st["clusters"] += len(cl)

        def step_host(st):
            for b in range(nblk):
                s.push_block(hpin[b * wl.ndump:(b + 1) * wl.ndump])
                pop_all(st, wait=False)
            s.sync(allow_overflow=True)
            pop_all(st)

        step_host({"work": 0, "d2h": 0, "clusters": 0})
        st = {"work": 0, "d2h": 0, "clusters": 0}
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step_host(st)
        barrier()
        wall = time.perf_counter() - t0
        wall = tx.shard.max_over_ranks(wall, dist)
        e2e = {"value": st["work"] * world / wall, "unit": "DM-trial samples/s",
               "h2d_bytes_per_step": nblk * blk_bytes,
               "d2h_bytes_per_step": st["d2h"] // max(1, args.steps),
               "clusters_per_step": st["clusters"] / max(1, args.steps),
               "includes": "H2D from pinned host memory, candidate read-back, Cluster::run per "
                           "block, every block's results popped (as they become ready, the rest "
                           "after the step's sync)"}
        s.close()

    if rank != 0:
        return
    cpu = None
    if not args.no_cpu:
        v, per, sample, cores = cpu_reference(wl, 0, 0, timed_blocks=args.cpu_blocks)
        cpu = {"value": v, "unit": "DM-trial samples/s", "cores": cores, "kind": "port",
               "sample": sample}
    line = {"metric": "DM-trial samples/s", "value": value, "unit": "DM-trial samples/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if args.precision == "fp32" else
            f"{args.precision} storage, f32 accumulate", "data": "synthetic",
            "config": {"workload": wl.name, "nchans": fil.nchans, "tsamp": fil.tsamp,
                       "nsamples": nblk * wl.ndump, "ndump": wl.ndump, "nblocks": nblk,
                       "rows": [[sp.td, sp.dms, sp.ddm, sp.ndm] for sp in wl.rows],
                       "nsub": [i.nsub for i in infos], "dm_group": [i.dm_group for i in infos],
                       "precision": args.precision, "parallelism": f"beam-per-gpu x{world}",
                       "l2": "inputs larger than L2 (raw file %.1f GB)" % (host.numel() / 1e9)},
            "clocks": clk, "e2e": e2e, "gpu_launches": stats["launches"],
            "roofline": roof, "cpu_baseline": cpu,
            "work_per_step": stats["work"] / args.steps, "host_wall_s": t_host}
    print(json.dumps(line), flush=True)


def run_replot(args):
    """Replot chain throughput: one batch of candidates through transientx_gb300.replot (host
    buffers in, results out) per step, wall time."""
    import transientx_gb300 as tx
    from transientx_gb300 import synth
    cands = synth.replot_candidates(args.replot)
    for _ in range(args.warmup):
        tx.replot(cands)
    ts = []
    for _ in range(args.steps):
        t = time.perf_counter()
        r = tx.replot(cands)
        ts.append(time.perf_counter() - t)
    per = float(np.median(ts))
    line = {"metric": "replot candidates/s", "value": args.replot / per, "unit": "candidates/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": per * 1e3,
            "higher_is_better": True, "data": "synthetic",
            "config": {"workload": "replot_nchan4096", "candidates": args.replot,
                       "shape": list(cands[0]["data"].shape), "tbin": cands[0]["tbin"],
                       "dm": cands[0]["dm"], "width": cands[0]["width"]},
            "ms_per_candidate": per * 1e3 / args.replot,
            "first": {"snr": r[0]["snr"], "dm_maxsnr": r[0]["dm_maxsnr"], "maxtid": r[0]["maxtid"]}}
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    if args.replot:
        run_replot(args)
        return
    from transientx_gb300 import synth
    make = synth.WORKLOADS[args.workload]
    wl = make(nsamples=args.nsamples) if args.nsamples else make()
    if args.rows:
        keep = [int(r) for r in args.rows.split(",")]
        wl.rows = [wl.rows[r] for r in keep]
        wl.name += "_rows" + "-".join(map(str, keep))
    if args.ndm:
        for sp in wl.rows:
            sp.ndm = args.ndm
        wl.name += f"_ndm{args.ndm}"
    if args.impl == "reference":
        run_reference(args, wl)
    else:
        run_ours(args, wl)


if __name__ == "__main__":
    main()
