"""Benchmark: DM-trial samples/s of the single-pulse search (unpack -> RFI -> subband
dedispersion over the ddplan -> boxcar + threshold) on one GB300 per rank.

Default workload: 64 beams of uneven length (2^19-2^22 samples) and channel count (1024 or
4096), searched with one three-row ddplan to DM 3000.  The beams do not fit the GPU together
(each holds about 11 GB of 16-bit subband history, 22 GB in FP32), so they run through lanes:
each lane of a handle (one handle per channel count) searches its beam block by block and
takes the next beam of the job when its beam ends (txg_reset_beam).  A step is
--blocks-per-step blocks of every lane; the timed steps are a window of the job's lane
schedule after --preroll blocks per lane (enough to fill every row's DM-delay history) and
the warm-up steps.  `value` is the mixed-precision (16-bit subband storage, FP32
accumulation), batched rate with the window's raw blocks resident in HBM
(txg_push_block_device); `fp32_same_config` is the plain FP32 path (one lane per channel
count) on the same job, and the FP32 path at the same lanes.  `e2e` times the public
host-pointer call (txg_push_block from pinned host memory, H2D inside the timed region) with
the per-block candidate read-back and host clustering.

Single-beam workloads (--workload nchan4096_n2M_rfi_dm3000 etc.): a step is one pass of every
ddplan row over the whole synthetic filterbank.  Ranks are independent beams (weak scaling,
no collective on the data path).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload NAME] [--precision fp32|fp16|bf16]
"""
from __future__ import annotations

import argparse
import collections
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
ZAPTHRE = 4.0  # PreprocessLite skewness/kurtosis channel-zap threshold (transientx_fil default)
DEFAULT_WORKLOAD = "beams64_nchan1024_4096"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD)
    ap.add_argument("--nsamples", type=int, default=0, help="override the file length")
    ap.add_argument("--precision", choices=["fp32", "bf16", "fp16"], default=None,
                    help="subband storage (default: fp16 for the many-beam job, else fp32)")
    ap.add_argument("--lanes", type=int, default=4, help="beams in flight per channel count")
    ap.add_argument("--blocks-per-step", type=int, default=2)
    ap.add_argument("--preroll", type=int, default=16, help="blocks per lane before warm-up")
    ap.add_argument("--replot", type=int, default=0,
                    help="time the replot chain on this many 4096-channel candidates instead")
    ap.add_argument("--replot-pageable", action="store_true",
                    help="replot: pageable host buffers instead of page-locked ones")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp32", action="store_true", help="skip the FP32 same-job passes")
    ap.add_argument("--cpu-blocks", type=int, default=1, help="timed oracle blocks per row")
    ap.add_argument("--rows", default="", help="comma-separated ddplan rows to keep (profiling)")
    ap.add_argument("--ndm", type=int, default=0, help="override ndm of every row (profiling)")
    a = ap.parse_args()
    if a.precision is None:
        a.precision = "fp16" if a.workload in JOBS_NAMES else "fp32"
    return a


JOBS_NAMES = ("beams64_nchan1024_4096", "beams16_nchan8192_dm5000")


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
    unpack: raw uint8 in + float block out; preprocess: read+write the block once; stage 1:
    the FP32 block in + subband series out (elem bytes per element); stage 2: subband series
    in + dedispersed out; boxcar: dedispersed series in + 16-byte candidates out."""
    C, N = info.nchans, info.ndump
    block = 4.0 * C * N
    series = float(elem) * info.nsub * info.ngroup * N
    return [nchans_raw * ndump_raw + block, 2 * block, block + series,
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
    FP32 window element per sample for each delay change within a thread set's groups (the
    loads the kernel makes; additions are C x ngroup x N), stage 2 one ring element (elem
    bytes) per addition (nsub x ndm x (N + noverlap)), the boxcar two running-sum values per
    (sample, width).  Other classes: None."""
    return [None, None, 4.0 * info.ndump * stage1_window_loads(d1),
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
    n += 1  # stage 1
    if gated:
        n += 1 + (2 if info.nsamples > BOXCAR_ROW_MAX else 1)  # stage 2, boxcar
    return n


SKZAP_LAUNCHES = 3  # per block, all rows: moments, statistics, outlier selection




def b_alg_block(info_rows, rows, nchans_raw, ndump_raw, elem, ncand):
    """Algorithmic HBM bytes of one block of one beam, the pipeline roofline's numerator:
    the raw 8-bit block read once, read twice more when an RFI filter runs (the second and
    third passes), each row's stage-1 subband series written and read once
    (2 x nsub x coarse DMs x samples x element bytes), 16 bytes per candidate point;
    dedispersed series, running sums and dense S planes stay on chip (zero)."""
    raw = float(nchans_raw) * ndump_raw
    b = raw
    if any(sp.rfilist for sp in rows):
        b += 2.0 * raw
    for info in info_rows:
        b += 2.0 * info.nsub * info.ngroup * info.ndump * elem
    return b + 16.0 * ncand


def profiled_traffic(workload, precision, cls):
    """DRAM bytes per launch of a kernel class from the ncu summaries' data file, or None."""
    p = os.path.join(ROOT, "profiles", "dram_traffic.json")
    if not os.path.exists(p):
        return None, None
    for e in json.load(open(p))["entries"]:
        if (e["workload"], e["precision"], e["class"]) == (workload, precision, cls):
            return float(e["bytes_per_launch"]), "profiles/" + e["summary"]
    return None, None


# ---- reference arm / CPU baseline: the oracle port on the host cores ------------------------
def cpu_reference(beams, rows, ndump, steps, warmup, wname, nthreads=0):
    """Oracle restatement of the path (oracle/txoracle.c) on the host cores, planned by the
    oracle's own subband rule (no product code): for each beam given (one per channel count
    of the workload), every ddplan row is run until gated (not timed), then each step times
    one gated block of every row of every beam.  Returns (value, seconds per step, sample
    description, cores)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    O.build(ref=False)
    cores = nthreads or os.cpu_count()
    O.lib().txo_set_threads(cores)
    units = []  # (row object, filterbank, next block, work per gated block)
    for fil in beams:
        for sp in rows:
            nsub, group = O.plan_row(fil.freqs, fil.tsamp, sp.td, sp.fd, sp.ddm, sp.ndm,
                                     sp.nsub, sp.dm_group)
            row = O.make_row(td=sp.td, fd=sp.fd, bswidth=sp.bswidth, rfi=sp.rfilist,
                             threKadaneF=sp.threKadaneF, widthlimit=sp.widthlimit, dms=sp.dms,
                             ddm=sp.ddm, ndm=sp.ndm, overlap=sp.overlap, nsub=nsub, group=group,
                             minw=sp.minw, maxw=sp.maxw, snrloss=sp.snrloss, thre=sp.thre,
                             zapthre=ZAPTHRE)
            o = O.SinglePulseRow(row, fil.freqs, fil.tsamp, ndump)
            b = 0
            while True:  # fill the DM-delay history (not timed)
                b += 1
                if o.run(fil.generate((b - 1) * ndump, ndump)):
                    break
            i = o.info()
            units.append([o, fil, b, i.ndm * i.nout])
    per_step, work = [], 0
    for k in range(steps + warmup):
        t = 0.0
        for u in units:
            o, fil, b, w = u
            raw = fil.generate(b * ndump, ndump)
            t0 = time.perf_counter()
            assert o.run(raw)
            t += time.perf_counter() - t0
            u[2] += 1
            if k >= warmup:
                work += w
        if k >= warmup:
            per_step.append(t)
    per = float(np.mean(per_step))
    chans = "/".join(str(f.nchans) for f in beams)
    sample = (f"{wname}: one gated block ({ndump} samples) of each of the {len(rows)} ddplan "
              f"rows of one {chans}-channel beam per step, {steps} steps timed after the "
              f"DM-delay history was filled; oracle port, own subband plan, {cores} threads")
    return work / sum(per_step), per, sample, cores


def reference_beams(args):
    """(beams, rows, ndump, name) the CPU baseline runs: one beam of each channel count of
    the many-beam job, or the single-beam workload itself."""
    from transientx_gb300 import synth
    if args.workload in JOBS_NAMES:
        job = synth.JOBS[args.workload]()
        seen, beams = set(), []
        for f in job.beams:
            if f.nchans not in seen:
                seen.add(f.nchans)
                beams.append(f)
        return beams, job.rows, job.ndump, job.name
    wl = make_workload(args)
    return [wl.fil], wl.rows, wl.ndump, wl.name


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    beams, rows, ndump, name = reference_beams(args)
    value, per, sample, cores = cpu_reference(beams, rows, ndump, args.steps, args.warmup, name)
    line = {"metric": "DM-trial samples/s", "value": value, "unit": "DM-trial samples/s",
            "impl": "reference", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": per * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": name, "sample": "one gated block of every ddplan row of one "
                                                   "beam per channel count, per step"},
            "cpu_baseline": {"value": value, "unit": "DM-trial samples/s", "cores": cores,
                             "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "DM-trial samples/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---- our arm ------------------------------------------------------------------------------
def run_single(args, wl):
    """One beam: a step is every ddplan row over every block of the filterbank."""
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
                         precision=args.precision, flags=flags | tx.FLAG_AUTOTUNE,
                         zapthre=ZAPTHRE)

    # the headline pass: the rows of a block run concurrently, each on its own stream
    s = make_search(0)
    infos = [s.row_info(r) for r in range(len(wl.rows))]
    shapes = [list(s.launch_shape(r)) for r in range(len(wl.rows))]
    stream = torch.cuda.ExternalStream(s.stream())

    def drain(stats):
        for r in range(len(wl.rows)):
            while True:
                out = s.pop_result(r, points=False)
                if out is None:
                    break
                res = out[0]
                stats["overflow"] += int(res.overflow)
                if res.gated:
                    stats["work"] += infos[r].ndm * infos[r].nsamples
                    stats["ncand"][r] += res.npoints
                    stats["gated"][r] += 1
                    stats["launches"] += launches_per_block(wl.rows[r], infos[r], True, args.precision)
                else:
                    stats["launches"] += launches_per_block(wl.rows[r], infos[r], False, args.precision)

    def new_stats():
        return {"work": 0, "ncand": [0] * len(wl.rows), "gated": [0] * len(wl.rows),
                "launches": 0, "d2h": 0, "overflow": 0}

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
            "traffic": profiled_traffic(wl.name, args.precision, names[top])[0],
            "traffic_source": profiled_traffic(wl.name, args.precision, names[top])[1],
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
    ncand_blk = sum(stats["ncand"]) / max(1, args.steps * nblk)
    balg = b_alg_block(infos, wl.rows, fil.nchans, wl.ndump, ELEM[args.precision], ncand_blk)
    pipe = balg * nblk * world / (ms / args.steps / 1e3) / 1e9
    roof["pipeline"] = {"achieved": pipe, "frac": pipe / peak, "unit": "GB/s",
                        "bytes_per_block": balg,
                        "basis": "raw block once (+2 passes with RFI filters) + every row's "
                                 "subband series written and read once + 16 B per point, per "
                                 "block, over the headline pass's CUDA-event time"}

    s.close()
    e2e = None
    if not args.no_e2e:
        # the public host-pointer path: pinned host blocks, H2D inside the timed region, and
        # Cluster::run on every block inside the library while the device runs ahead
        s = make_search(tx.FLAG_CLUSTER)
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
                    st["overflow"] += int(res.overflow)
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

        step_host({"work": 0, "d2h": 0, "clusters": 0, "overflow": 0})
        st = {"work": 0, "d2h": 0, "clusters": 0, "overflow": 0}
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
               "overflow_blocks": st["overflow"],
               "includes": "H2D from pinned host memory, candidate read-back, Cluster::run per "
                           "block, every block's results popped (as they become ready, the rest "
                           "after the step's sync)"}
        s.close()

    if rank != 0:
        return
    cpu = None
    if not args.no_cpu:
        v, per, sample, cores = cpu_reference([wl.fil], wl.rows, wl.ndump, args.cpu_blocks, 0,
                                              wl.name)
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
                       "precision": args.precision, "launch_shapes": shapes,
                       "parallelism": f"beam-per-gpu x{world}",
                       "l2": "inputs larger than L2 (raw file %.1f GB)" % (host.numel() / 1e9)},
            "clocks": clk, "e2e": e2e, "gpu_launches": stats["launches"],
            "roofline": roof, "cpu_baseline": cpu,
            "work_per_step": stats["work"] / args.steps, "host_wall_s": t_host,
            "overflow_blocks": stats["overflow"]}
    print(json.dumps(line), flush=True)


# ---- the many-beam job ---------------------------------------------------------------------
def lane_schedule(job, beam_ids, lanes, nsteps, bps):
    """The blocks each lane pushes, step by step.  Per channel count, `lanes` lanes take the
    job's beams of that count in order; a lane whose beam has no block left takes the next
    beam (resetting the lane first); when the beams run out the lanes start over.  Returns
    (channel counts, steps); a step lists (nchans, lane, beam, block, reset) items."""
    chans = sorted({job.beams[b].nchans for b in beam_ids})
    order = {C: [b for b in beam_ids if job.beams[b].nchans == C] for C in chans}
    queues = {C: collections.deque(order[C]) for C in chans}
    state = {C: [None] * lanes for C in chans}
    steps = []
    for _ in range(nsteps):
        items = []
        for _k in range(bps):
            for C in chans:
                for lane in range(lanes):
                    cur = state[C][lane]
                    reset = False
                    if cur is None or cur[1] >= job.nblocks(cur[0]):
                        if not queues[C]:
                            queues[C].extend(order[C])
                        reset = cur is not None
                        cur = state[C][lane] = [queues[C].popleft(), 0]
                    items.append((C, lane, cur[0], cur[1], reset))
                    cur[1] += 1
        steps.append(items)
    return chans, steps


class BlockCache:
    """Raw 8-bit blocks of the job's beams (seeded, time-major), generated on demand and kept
    for the later passes up to `limit` bytes."""

    def __init__(self, job, limit=24e9):
        self.job, self.d, self.limit, self.bytes = job, {}, limit, 0

    def get(self, beam, blk):
        k = (beam, blk)
        if k in self.d:
            return self.d[k]
        a = self.job.beams[beam].generate(blk * self.job.ndump, self.job.ndump)
        if self.bytes + a.nbytes <= self.limit:
            self.d[k] = a
            self.bytes += a.nbytes
        return a


class WindowInputs:
    """The raw blocks of a run of steps, contiguous in pinned host memory and, for the
    device-resident pass, copied to HBM before the timed region."""

    def __init__(self, torch, cache, steps, device):
        items = [it for st in steps for it in st]
        sizes = [cache.job.ndump * it[0] for it in items]
        self.offsets = np.concatenate([[0], np.cumsum(sizes)])[:-1].astype(np.int64)
        self.host = torch.empty(int(sum(sizes)), dtype=torch.uint8, pin_memory=True)
        hv = self.host.numpy()
        for it, o, n in zip(items, self.offsets, sizes):
            hv[o:o + n] = cache.get(it[2], it[3]).reshape(-1)
        self.dev = self.host.to(device) if device is not None else None
        self.nbytes = int(sum(sizes))
        self.k = 0

    def next_host(self, C, ndump):
        o = int(self.offsets[self.k])
        self.k += 1
        return self.host.numpy()[o:o + ndump * C].reshape(ndump, C)

    def next_dev(self):
        o = int(self.offsets[self.k])
        self.k += 1
        return self.dev.data_ptr() + o


class Lanes:
    """One handle per channel count, `lanes` beams each, all searching the job's ddplan."""

    def __init__(self, tx, job, chans, lanes, precision, flags):
        self.job, self.lanes, self.precision = job, lanes, precision
        self.s, self.infos = {}, {}
        f0 = job.beams[0]
        for C in chans:
            freqs = next(f.freqs for f in job.beams if f.nchans == C)
            s = tx.Search(job.rows, C, f0.tsamp, freqs, job.ndump,
                          nbeams=lanes, precision=precision, flags=flags | tx.FLAG_AUTOTUNE,
                          zapthre=ZAPTHRE)
            self.s[C] = s
            self.infos[C] = [s.row_info(r) for r in range(len(job.rows))]
            self.shapes = getattr(self, "shapes", {})
            self.shapes[C] = [list(s.launch_shape(r)) for r in range(len(job.rows))]

    def push(self, item, data=None, dev=None):
        C, lane, _beam, _blk, reset = item
        s = self.s[C]
        if reset:
            s.reset_beam(lane)
        if dev is not None:
            s.push_block_device(dev, beam=lane)
        else:
            s.push_block(data, beam=lane)

    def drain(self, st, wait):
        """Pop every harvested block (only those whose clustering is done unless `wait`)."""
        rows = self.job.rows
        for C, s in self.s.items():
            for lane in range(self.lanes):
                for r in range(len(rows)):
                    while True:
                        if not wait and not s.result_ready(r, beam=lane):
                            break
                        out = s.pop_result(r, beam=lane, points=False)
                        if out is None:
                            break
                        res, _, cl = out
                        info = self.infos[C][r]
                        st["overflow"] += int(res.overflow)
                        st["d2h"] += 8 + 16 * res.npoints
                        st["launches"] += launches_per_block(rows[r], info, bool(res.gated),
                                                             self.precision)
                        if res.gated:
                            st["work"] += info.ndm * info.nsamples
                            st["ncand"][(C, r)] += res.npoints
                            st["gated"][(C, r)] += 1
                            st["clusters"] += len(cl)

    def sync(self):
        for s in self.s.values():
            s.sync(allow_overflow=True)

    def close(self):
        for s in self.s.values():
            s.close()
        self.s = {}


def h2d_rates(torch, window):
    """Host-to-device rate of each block of the page-locked window, timed with CUDA events
    just before the timed pass that pushes them (outside it).  On the GB300 machines the rate
    of page-locked memory differs between allocations and over time (3-20 GB/s for some
    blocks, about 210 GB/s for others, whatever the device is doing), which bounds the e2e
    rate of jobs whose blocks are large."""
    hv = window.host.numpy()
    ends = list(window.offsets[1:]) + [window.nbytes]
    sizes = [int(e) - int(o) for o, e in zip(window.offsets, ends)]
    try:
        scratch = torch.empty(max(sizes), dtype=torch.uint8, device="cuda")
    except torch.cuda.OutOfMemoryError:
        return {"unmeasured": "no device memory for a block-sized scratch beside the lanes"}
    evs = []
    for o, n in zip(window.offsets, sizes):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        scratch[:n].copy_(torch.from_numpy(hv[int(o):int(o) + n]), non_blocking=True)
        e1.record()
        evs.append((n, e0, e1))
    torch.cuda.synchronize()
    r = sorted(n / (a.elapsed_time(b) / 1e3) / 1e9 for n, a, b in evs)
    del scratch
    torch.cuda.empty_cache()
    return {"blocks": len(r), "min_GBps": round(r[0], 1), "median_GBps": round(r[len(r) // 2], 1),
            "max_GBps": round(r[-1], 1)}


def new_stats():
    return {"work": 0, "launches": 0, "overflow": 0, "d2h": 0, "clusters": 0, "pushed": 0,
            "blocks": collections.Counter(), "ncand": collections.Counter(),
            "gated": collections.Counter()}


def run_lanes(torch, L, cache, steps, t_first, window, dev_inputs, stream, clocks=None):
    """Push steps[:t_first] untimed (pageable host blocks, staged by the library), drain,
    then push steps[t_first:] from the window (device pointers or pinned host blocks) between
    two CUDA events; every block's results are popped as they become ready and the rest after
    the final sync.  Returns (milliseconds of the timed steps, their statistics)."""
    junk = new_stats()
    for st in steps[:t_first]:
        for it in st:
            L.push(it, data=cache.get(it[2], it[3]))
        L.drain(junk, wait=False)
    L.sync()
    L.drain(junk, wait=True)
    stats = new_stats()
    if not dev_inputs:
        stats["h2d_window"] = h2d_rates(torch, window)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    window.k = 0
    if clocks is not None:
        clocks.start()
    t_host = time.perf_counter()
    torch.cuda.nvtx.range_push("timed")  # lets a profiler capture the timed launches alone
    e0.record(stream)
    for st in steps[t_first:]:
        for it in st:
            if dev_inputs:
                L.push(it, dev=window.next_dev())
            else:
                L.push(it, data=window.next_host(it[0], L.job.ndump))
            stats["blocks"][it[0]] += 1
            stats["pushed"] += 1
            stats["launches"] += SKZAP_LAUNCHES if ZAPTHRE > 0 else 0
        L.drain(stats, wait=False)
    L.sync()
    L.drain(stats, wait=True)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.nvtx.range_pop()
    stats["host_s"] = time.perf_counter() - t_host
    if clocks is not None:
        stats["clocks"] = clocks.stop()
    return e0.elapsed_time(e1), stats


def class_times(tx, job, chans, lanes, precision, cache, steps, t_first, ntimed):
    """Per-kernel-class CUDA-event times of `ntimed` steps of the schedule (after the same
    untimed steps as the headline): TXG_FLAG_TIMING serialises each handle's rows, and the
    handles take turns, so each class's event span holds its own kernels only."""
    L = Lanes(tx, job, chans, lanes, precision, tx.FLAG_TIMING)
    junk = new_stats()
    for st in steps[:t_first]:
        for it in st:
            L.push(it, data=cache.get(it[2], it[3]))
        L.drain(junk, wait=False)
    L.sync()
    L.drain(junk, wait=True)
    for s in L.s.values():
        s.timing()  # reset the accumulators, the handle's and each row's
        for r in range(len(job.rows)):
            s.row_timing(r)
    stats = new_stats()
    for st in steps[t_first:t_first + ntimed]:
        for C in chans:
            for it in st:
                if it[0] == C:
                    L.push(it, data=cache.get(it[2], it[3]))
                    stats["blocks"][C] += 1
            L.s[C].sync(allow_overflow=True)
        L.drain(stats, wait=True)
    cls = {C: L.s[C].timing() for C in chans}
    rows = {C: [L.s[C].row_timing(r) for r in range(len(job.rows))] for C in chans}
    L.close()
    return cls, rows, stats


def run_batch(args):
    import torch
    import transientx_gb300 as tx
    from transientx_gb300 import shard, synth

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

    job = synth.JOBS[args.workload]()
    mine = shard.beams_for_rank(len(job.beams), rank, world)  # independent beams per rank
    bps, P, W, K = args.blocks_per_step, args.preroll, args.warmup, args.steps
    t_first = (P + bps - 1) // bps + W  # untimed steps: pre-roll, then warm-up
    nsteps = t_first + K
    cache = BlockCache(job)
    stream = torch.cuda.current_stream()
    names = ["unpack", "preprocess", "stage1", "stage2", "boxcar"]
    elem = ELEM[args.precision]

    shapes = {}

    def measure(lanes, precision, dev_inputs, flags=0, clocks=None):
        chans, steps = lane_schedule(job, mine, lanes, nsteps, bps)
        window = WindowInputs(torch, cache, steps[t_first:], "cuda" if dev_inputs else None)
        L = Lanes(tx, job, chans, lanes, precision, flags)
        barrier()
        ms, st = run_lanes(torch, L, cache, steps, t_first, window, dev_inputs, stream, clocks)
        infos = L.infos
        shapes.update(L.shapes)
        L.close()
        nbytes = window.nbytes
        del window
        torch.cuda.empty_cache()
        return ms, st, chans, steps, infos, nbytes

    # headline: mixed precision, batched lanes, inputs resident in HBM
    ms, stats, chans, steps, infos, win_bytes = measure(args.lanes, args.precision, True,
                                                        clocks=ClockSampler(local))
    clk = stats["clocks"]
    ms = shard.max_over_ranks(ms, dist, "cuda")
    work = shard.sum_over_ranks(stats["work"], dist, "cuda")
    value = work / (ms / 1e3)

    # per-class times and the roofline of the dominant class
    cls, cls_rows, tst = class_times(tx, job, chans, args.lanes, args.precision, cache, steps,
                                     t_first, min(K, 2))
    cls_ms = [sum(float(cls[C][0][c]) for C in chans) for c in range(5)]
    cls_n = [sum(int(cls[C][1][c]) for C in chans) for c in range(5)]
    nb, sm, op = [0.0] * 5, [0.0] * 5, [0.0] * 5
    f0 = job.beams[0]
    for C in chans:
        freqs = next(f.freqs for f in job.beams if f.nchans == C)
        for r, sp in enumerate(job.rows):
            info = infos[C][r]
            g = tst["gated"][(C, r)]
            ncand = tst["ncand"][(C, r)] / max(1, g)
            cb = class_bytes(info, sp, C, job.ndump, ncand, elem)
            d1 = tx.describe_row(job.rows, r, C, f0.tsamp, freqs, job.ndump)[1]
            sb = class_smem_bytes(info, elem, d1)
            ob = class_fp32_ops(info)
            for c in range(5):
                n = tst["blocks"][C] if c < 3 else g
                nb[c] += cb[c] * n
                if c >= 2:
                    sm[c] += sb[c] * n
                    op[c] += ob[c] * n
    top = int(np.argmax(cls_ms))
    peak, peak_kind = measured_peaks()
    achieved = nb[top] / (cls_ms[top] / 1e3) / 1e9
    traffic, tsrc = profiled_traffic(job.name, args.precision, names[top])
    sm_clk = (clk or {}).get("sm_mhz") or 2070.0
    roof = {"bound": "hbm", "kernel": names[top], "achieved": achieved, "peak": peak,
            "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
            "traffic_source": tsrc, "peak_source": peak_kind,
            "class_timing": f"CUDA events per kernel class over {min(K, 2)} steps of the same "
                            "schedule, rows serialised (TXG_FLAG_TIMING), handles in turn",
            "class_ms": {names[c]: cls_ms[c] for c in range(5)},
            "class_launches": {names[c]: cls_n[c] for c in range(5)},
            "class_algorithmic_GBps": {names[c]: (nb[c] / (cls_ms[c] / 1e3) / 1e9
                                                   if cls_ms[c] > 0 else None) for c in range(5)}}
    if top in (2, 3, 4):
        sm_peak = NSM * SMEM_BYTES_PER_CLK * sm_clk * 1e6 / 1e12
        sm_ach = sm[top] / (cls_ms[top] / 1e3) / 1e12
        roof["smem"] = {"achieved": sm_ach, "peak": sm_peak, "unit": "TB/s",
                        "frac": sm_ach / sm_peak,
                        "peak_basis": f"{NSM} SMs x {SMEM_BYTES_PER_CLK} B/clock x median SM clock"}
    roof["alu"] = alu_roofline(op, cls_ms, sm_clk)
    # per ddplan row (stage): its serialised class times, DM-trial rate and rooflines
    per_row = []
    for r, sp in enumerate(job.rows):
        rms = [sum(float(cls_rows[C][r][0][c]) for C in chans) for c in range(5)]
        work_r, nbr, balg_r = 0.0, [0.0] * 5, 0.0
        for C in chans:
            info = infos[C][r]
            g = tst["gated"][(C, r)]
            work_r += g * info.ndm * info.nsamples
            cb = class_bytes(info, sp, C, job.ndump, tst["ncand"][(C, r)] / max(1, g), elem)
            for c in range(5):
                nbr[c] += cb[c] * (tst["blocks"][C] if c < 3 else g)
            balg_r += tst["blocks"][C] * 2.0 * info.nsub * info.ngroup * info.ndump * elem
        tot = sum(rms)
        topr = int(np.argmax(rms))
        gbps = [nbr[c] / (rms[c] / 1e3) / 1e9 if rms[c] > 0 else None for c in range(5)]
        per_row.append({
            "row": r, "td": sp.td, "dms": sp.dms, "ddm": sp.ddm, "ndm": sp.ndm,
            "class_ms": {names[c]: rms[c] for c in range(5)},
            "dm_trial_samples_per_s": work_r / (tot / 1e3) if tot > 0 else None,
            "dominant": names[topr],
            "dominant_hbm_frac": gbps[topr] / peak if gbps[topr] else None,
            "class_algorithmic_GBps": {names[c]: gbps[c] for c in range(5)},
            "subband_series_frac": balg_r / (tot / 1e3) / 1e9 / peak if tot > 0 else None})
    row_sum = [sum(pr["class_ms"][names[c]] for pr in per_row) for c in range(5)]
    roof["per_row_sums_match"] = all(abs(row_sum[c] - cls_ms[c]) <= 1e-3 * max(1.0, cls_ms[c])
                                     for c in range(5))
    roof["per_row"] = per_row
    roof["per_row_basis"] = ("the class-timing pass's CUDA-event times per ddplan row (rows "
                             "serialised); dominant_hbm_frac = that class's algorithmic bytes / "
                             "its time / peak; subband_series_frac = the row's stage-1 series "
                             "written and read once / the row's time / peak")
    balg = 0.0
    for C in chans:
        rows_info = infos[C]
        nc = sum(stats["ncand"][(C, r)] for r in range(len(job.rows)))
        balg += stats["blocks"][C] * b_alg_block(rows_info, job.rows, C, job.ndump, elem, 0.0)
        balg += 16.0 * nc
    balg = shard.sum_over_ranks(balg, dist, "cuda")
    pipe = balg / (ms / 1e3) / 1e9
    roof["pipeline"] = {"achieved": pipe, "frac": pipe / peak, "unit": "GB/s",
                        "bytes_per_step": balg / K,
                        "basis": "per pushed block: raw block once (+2 passes with RFI filters) "
                                 "+ every row's subband series written and read once + 16 B "
                                 "per point, over the headline's CUDA-event time"}

    # the same job in FP32: plain (one lane per channel count) and at the same lanes
    fp32 = None
    if not args.no_fp32:
        fp32 = {}
        for key, lanes in (("plain", 1), ("batched", args.lanes)):
            m32, s32, *_ = measure(lanes, "fp32", True)
            m32 = shard.max_over_ranks(m32, dist, "cuda")
            w32 = shard.sum_over_ranks(s32["work"], dist, "cuda")
            fp32[key] = {"value": w32 / (m32 / 1e3), "lanes_per_nchans": lanes,
                         "ms_per_step": m32 / K}
        fp32["ratio_vs_plain"] = value / fp32["plain"]["value"]
        fp32["ratio_vs_batched"] = value / fp32["batched"]["value"]

    e2e = None
    if not args.no_e2e:
        ms_e, st_e, *_ = measure(args.lanes, args.precision, False, tx.FLAG_CLUSTER)
        wall = shard.max_over_ranks(st_e["host_s"], dist, "cuda")
        we = shard.sum_over_ranks(st_e["work"], dist, "cuda")
        e2e = {"value": we / wall, "unit": "DM-trial samples/s",
               "h2d_bytes_per_step": win_bytes // K,
               "d2h_bytes_per_step": st_e["d2h"] // K,
               "clusters_per_step": st_e["clusters"] / K, "overflow_blocks": st_e["overflow"],
               "h2d_window": st_e["h2d_window"],
               "includes": "H2D from pinned host memory, candidate read-back and Cluster::run "
                           "of every block inside the library, every block's results popped "
                           "(as they become ready, the rest after the final sync); host wall "
                           "time"}

    if rank != 0:
        return
    cpu = None
    if not args.no_cpu:
        beams, rows, ndump, name = reference_beams(args)
        v, per, sample, cores = cpu_reference(beams, rows, ndump, args.cpu_blocks, 0, name)
        cpu = {"value": v, "unit": "DM-trial samples/s", "cores": cores, "kind": "port",
               "sample": sample}
    lens = [job.beams[b].nsamples for b in range(len(job.beams))]
    nchan_count = collections.Counter(f.nchans for f in job.beams)
    line = {"metric": "DM-trial samples/s", "value": value, "unit": "DM-trial samples/s",
            "n_gpus": world, "steps": K, "warmup": W, "ms_per_step": ms / K,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if args.precision == "fp32" else
            f"{args.precision} subband storage, f32 accumulate",
            "data": "synthetic",
            "config": {"workload": job.name, "beams": len(job.beams),
                       "nchans": {str(k): v for k, v in sorted(nchan_count.items())},
                       "nsamples_range": [min(lens), max(lens)], "tsamp": f0.tsamp,
                       "ndump": job.ndump, "job_blocks": sum(job.nblocks(b) for b in mine),
                       "lanes_per_nchans": args.lanes, "blocks_per_step": bps,
                       "beam_blocks_per_step": stats["pushed"] / K,
                       "preroll_blocks_per_lane": P,
                       "timed_window": f"steps {t_first}..{nsteps - 1} of the job's lane "
                                       "schedule",
                       "rows": [[sp.td, sp.dms, sp.ddm, sp.ndm] for sp in job.rows],
                       "nsub": {str(C): [i.nsub for i in infos[C]] for C in chans},
                       "dm_group": {str(C): [i.dm_group for i in infos[C]] for C in chans},
                       "precision": args.precision,
                       "launch_shapes": {str(C): shapes.get(C) for C in chans},
                       "launch_shapes_basis": "[stage-1 shape, stage-2 variant, stage-2 KB] per "
                                              "row, autotuned at txg_create (last pass)",
                       "parallelism": f"{args.lanes} lanes per channel count x beams sharded "
                                      f"over {world} rank(s)",
                       "l2": "inputs larger than L2 (timed raw blocks %.1f GB)" % (win_bytes / 1e9)},
            "clocks": clk, "e2e": e2e, "gpu_launches": stats["launches"],
            "roofline": roof, "cpu_baseline": cpu, "fp32_same_config": fp32,
            "work_per_step": work / K, "overflow_blocks": stats["overflow"]}
    print(json.dumps(line), flush=True)


def run_replot(args):
    """Replot chain throughput: one batch of candidates through transientx_gb300.replot (host
    buffers in, results out) per step, wall time."""
    import transientx_gb300 as tx
    from transientx_gb300 import synth
    cands = synth.replot_candidates(args.replot)
    if not args.replot_pageable:
        # page-locked host buffers: the cut data crosses to the device at full copy bandwidth
        import torch
        keep = []
        for c in cands:
            t = torch.empty(c["data"].shape, dtype=torch.float32, pin_memory=True)
            t.numpy()[:] = c["data"]
            keep.append(t)
            c["data"] = t.numpy()
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
                       "host_buffers": "pageable" if args.replot_pageable else "pinned",
                       "shape": list(cands[0]["data"].shape), "tbin": cands[0]["tbin"],
                       "dm": cands[0]["dm"], "width": cands[0]["width"]},
            "ms_per_candidate": per * 1e3 / args.replot,
            "first": {"snr": r[0]["snr"], "dm_maxsnr": r[0]["dm_maxsnr"], "maxtid": r[0]["maxtid"]}}
    print(json.dumps(line), flush=True)


def make_workload(args):
    """A single-beam workload with the --nsamples/--rows/--ndm overrides applied."""
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
    return wl


def main():
    args = parse_args()
    if args.replot:
        run_replot(args)
    elif args.impl == "reference":
        run_reference(args)
    elif args.workload in JOBS_NAMES:
        run_batch(args)
    else:
        run_single(args, make_workload(args))


if __name__ == "__main__":
    main()
