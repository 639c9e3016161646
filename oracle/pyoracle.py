"""ctypes bindings for the CPU oracle (libtxoracle.so) and for the reference's own
Boxcar/Cluster compiled in place (oracle/_ref/libtxref_*.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` and by the
CPU-baseline leg of bench.py, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# The TransientX source tree whose boxcar.cpp, cluster.cpp and candidate.cpp are compiled in
# place (read-only) comes from the caller of build() or from TXREF_TREE; without one (a machine
# without the reference) only the oracle itself is built and the tests that need the
# reference's own code skip.

f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")

RFI_KADANEF = 1
RFI_ZDOT = 2
RFI_MASK = 3
RFI_KADANET = 4
RFI_ZERO = 5


def build(ref: bool = True, tree: str | None = None) -> None:
    """Compile the oracle; with `ref`, also the reference harness from the TransientX source
    tree `tree` (default: the TXREF_TREE environment variable) when one is given."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    tree = tree or os.environ.get("TXREF_TREE")
    if ref and tree:
        if not os.path.isdir(os.path.join(tree, "src", "singlepulse")):
            raise FileNotFoundError(f"TXREF_TREE={tree!r} is not a TransientX source tree "
                                    "(no src/singlepulse)")
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={tree}"], check=True)


class Cand(C.Structure):
    _fields_ = [("idm", C.c_int64), ("isamp", C.c_int64), ("wn", C.c_int32), ("S", C.c_float)]


CAND_DTYPE = np.dtype([("idm", "<i8"), ("isamp", "<i8"), ("wn", "<i4"), ("S", "<f4")])
assert CAND_DTYPE.itemsize == C.sizeof(Cand)


class DedispInfo(C.Structure):
    _fields_ = [
        ("nchan", C.c_int), ("nsub", C.c_int), ("group", C.c_int), ("ngroup", C.c_int),
        ("ndm", C.c_long), ("ndump", C.c_long), ("maxd1", C.c_long), ("maxd2", C.c_long),
        ("noverlap", C.c_long), ("offset", C.c_long), ("ring", C.c_long), ("nout", C.c_long),
        ("counter", C.c_long), ("tsamp", C.c_double), ("fmax", C.c_double),
        ("fmin", C.c_double),
    ]


class Row(C.Structure):
    _fields_ = [
        ("td", C.c_int), ("fd", C.c_int), ("bswidth", C.c_float), ("nrfi", C.c_int),
        ("rfi_kind", C.c_int * 8), ("rfi_td", C.c_int * 8), ("rfi_fd", C.c_int * 8),
        ("nzap", C.c_int), ("zap", (C.c_double * 2) * 16), ("threKadaneF", C.c_float),
        ("widthlimit", C.c_double), ("dms", C.c_double), ("ddm", C.c_double),
        ("ndm", C.c_long), ("overlap", C.c_double), ("nsub", C.c_int), ("group", C.c_int),
        ("minw", C.c_float), ("maxw", C.c_float), ("snrloss", C.c_float), ("iqr", C.c_int),
        ("avx2_tail", C.c_int), ("thre", C.c_float), ("zapthre", C.c_float), ("fp64", C.c_int),
        ("threMask", C.c_float), ("threKadaneT", C.c_float), ("bandlimitKT", C.c_double),
    ]


def make_row(**kw) -> Row:
    r = Row()
    r.td, r.fd = kw.get("td", 1), kw.get("fd", 1)
    r.bswidth = kw.get("bswidth", 0.0)
    rfi = kw.get("rfi", [])
    r.nrfi = len(rfi)
    for i, op in enumerate(rfi):
        if op[0] == "kadaneF":
            r.rfi_kind[i], r.rfi_td[i], r.rfi_fd[i] = RFI_KADANEF, int(op[1]), int(op[2])
        elif op[0] == "zdot":
            r.rfi_kind[i], r.rfi_td[i], r.rfi_fd[i] = RFI_ZDOT, 1, 1
        elif op[0] == "mask":
            r.rfi_kind[i], r.rfi_td[i], r.rfi_fd[i] = RFI_MASK, int(op[1]), int(op[2])
        elif op[0] == "kadaneT":
            r.rfi_kind[i], r.rfi_td[i], r.rfi_fd[i] = RFI_KADANET, int(op[1]), int(op[2])
        elif op[0] == "zero":
            r.rfi_kind[i], r.rfi_td[i], r.rfi_fd[i] = RFI_ZERO, 1, 1
        else:
            raise ValueError(f"unsupported rfi op {op}")
    zap = kw.get("zap", [])
    r.nzap = len(zap)
    for i, (a, b) in enumerate(zap):
        r.zap[i][0], r.zap[i][1] = a, b
    r.threKadaneF = kw.get("threKadaneF", 7.0)
    r.widthlimit = kw.get("widthlimit", 50e-3)
    r.dms, r.ddm, r.ndm = kw["dms"], kw["ddm"], kw["ndm"]
    r.overlap = kw.get("overlap", 0.0)
    r.nsub, r.group = kw["nsub"], kw["group"]
    r.minw, r.maxw, r.snrloss = kw.get("minw", 1e-4), kw["maxw"], kw.get("snrloss", 0.1)
    r.iqr = int(kw.get("iqr", False))
    r.avx2_tail = int(kw.get("avx2_tail", False))
    r.thre = kw.get("thre", 7.0)
    r.zapthre = kw.get("zapthre", -1.0)
    r.threMask = kw.get("threMask", 10.0)
    r.threKadaneT = kw.get("threKadaneT", 7.0)
    r.bandlimitKT = kw.get("bandlimitKT", 10.0)
    r.fp64 = int(kw.get("fp64", False))
    return r


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    path = os.path.join(HERE, "libtxoracle.so")
    if not os.path.exists(path):
        build(ref=False)
    L = C.CDLL(path)
    L.txo_dmdelay.restype = C.c_double
    L.txo_dmdelay.argtypes = [C.c_double] * 3
    L.txo_width_ladder.restype = C.c_int
    L.txo_width_ladder.argtypes = [C.c_float, C.c_float, C.c_float, C.c_double, i32p, C.c_int]
    L.txo_kadane.restype = C.c_float
    L.txo_kadane.argtypes = [f32p, C.c_long, C.POINTER(C.c_long), C.POINTER(C.c_long)]
    L.txo_red32.restype = C.c_double
    L.txo_red32.argtypes = [f32p, C.c_void_p, C.c_long, C.c_int]
    L.txo_unpack_downsample.argtypes = [u8p, C.c_long, C.c_int, C.c_int, C.c_int, f32p, C.c_long,
                                        C.c_void_p]
    L.txo_sk_moments.argtypes = [u8p, C.c_long, C.c_int, f64p, f64p]
    L.txo_skzap.restype = C.c_int
    L.txo_skzap.argtypes = [u8p, C.c_long, C.c_int, C.c_float, u8p]
    L.txo_sp_mask.restype = C.POINTER(C.c_uint8)
    L.txo_sp_mask.argtypes = [C.c_void_p]
    L.txo_downsample_freqs.argtypes = [f64p, C.c_int, C.c_int, f64p]
    L.txo_equalize.argtypes = [f32p, C.c_int, C.c_long, C.c_long, C.c_void_p]
    L.txo_baseline.argtypes = [f32p, C.c_int, C.c_long, C.c_long, C.c_long, C.c_void_p]
    L.txo_zap_channels.argtypes = [f32p, C.c_int, C.c_long, C.c_long, f64p, f64p, C.c_int]
    L.txo_kadaneF.restype = C.c_int
    L.txo_kadaneF.argtypes = [f32p, C.c_int, C.c_long, C.c_long, C.c_int, C.c_int, C.c_float,
                              C.c_long, i32p]
    L.txo_zdot.argtypes = [f32p, C.c_int, C.c_long, C.c_long]
    L.txo_kadaneT.restype = C.c_int
    L.txo_kadaneT.argtypes = [f32p, C.c_int, C.c_long, C.c_long, C.c_int, C.c_int, C.c_float,
                              C.c_long, i32p]
    L.txo_mask.restype = C.c_int
    L.txo_mask.argtypes = [f32p, C.c_int, C.c_long, C.c_long, C.c_int, C.c_int, C.c_float, f32p]
    L.txo_zero.argtypes = [f32p, C.c_int, C.c_long, C.c_long, C.c_void_p]
    L.txo_sp_dedisp.restype = C.c_void_p
    L.txo_sp_dedisp.argtypes = [C.c_void_p]
    L.txo_dedisp_subdata.restype = C.c_int
    L.txo_dedisp_subdata.argtypes = [C.c_void_p, C.c_long, f32p]
    L.txo_cand_band.argtypes = [f32p, C.c_int, C.c_long, i32p, f64p, C.c_long, C.c_int,
                                C.POINTER(C.c_float), C.POINTER(C.c_float)]
    L.txo_boxcar_match.argtypes = [f32p, C.c_long, i32p, C.c_int, C.c_int, C.c_int, f32p, i32p]
    L.txo_boxcar_run.argtypes = [f32p, C.c_long, C.c_long, i32p, C.c_int, C.c_int, C.c_int,
                                 f32p, i32p]
    L.txo_threshold_scan.restype = C.c_long
    L.txo_threshold_scan.argtypes = [f32p, i32p, C.c_long, C.c_long, C.c_float, C.c_void_p,
                                     C.c_long]
    L.txo_cluster.restype = C.c_long
    L.txo_cluster.argtypes = [C.c_void_p, C.c_long, C.c_double, C.c_double, C.c_double,
                              C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int,
                              C.c_int, C.c_void_p, C.c_void_p]
    L.txo_dedisp_create.restype = C.c_void_p
    L.txo_dedisp_create.argtypes = [C.c_int, f64p, C.c_double, C.c_long, C.c_double,
                                    C.c_double, C.c_long, C.c_double, C.c_int, C.c_int]
    L.txo_dedisp_destroy.argtypes = [C.c_void_p]
    L.txo_dedisp_get_info.argtypes = [C.c_void_p, C.POINTER(DedispInfo)]
    L.txo_dedisp_tables.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.txo_dedisp_run.restype = C.c_int
    L.txo_dedisp_run.argtypes = [C.c_void_p, f32p, C.c_long]
    L.txo_dedisp_timdata.restype = C.POINTER(C.c_float)
    L.txo_dedisp_timdata.argtypes = [C.c_void_p]
    L.txo_sp_create.restype = C.c_void_p
    L.txo_sp_create.argtypes = [C.POINTER(Row), C.c_int, f64p, C.c_double, C.c_long]
    L.txo_sp_destroy.argtypes = [C.c_void_p]
    L.txo_sp_run.restype = C.c_int
    L.txo_sp_run.argtypes = [C.c_void_p, u8p]
    L.txo_sp_run_f32.restype = C.c_int
    L.txo_sp_run_f32.argtypes = [C.c_void_p, f32p]
    L.txo_sp_nwidths.restype = C.c_int
    L.txo_sp_nwidths.argtypes = [C.c_void_p, i32p, C.c_int]
    L.txo_sp_dedisp_info.argtypes = [C.c_void_p, C.POINTER(DedispInfo)]
    L.txo_sp_block.restype = C.POINTER(C.c_float)
    L.txo_sp_block.argtypes = [C.c_void_p, C.POINTER(C.c_long), C.POINTER(C.c_int),
                               C.POINTER(C.c_long)]
    L.txo_sp_zap_ranges.restype = C.POINTER(C.c_int32)
    L.txo_sp_zap_ranges.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int)]
    L.txo_sp_timdata.restype = C.POINTER(C.c_float)
    L.txo_sp_timdata.argtypes = [C.c_void_p]
    L.txo_sp_mxS.restype = C.POINTER(C.c_float)
    L.txo_sp_mxS.argtypes = [C.c_void_p]
    L.txo_sp_mxwn.restype = C.POINTER(C.c_int)
    L.txo_sp_mxwn.argtypes = [C.c_void_p]
    L.txo_sp_freqs.argtypes = [C.c_void_p, f64p]
    L.txo_set_threads.argtypes = [C.c_int]
    _lib = L
    return L


# ---- thin numpy wrappers -------------------------------------------------------------------

def dmdelay(dm, fh, fl):
    return lib().txo_dmdelay(dm, fh, fl)


# ---- subband plan: the oracle's own choice of subband count and DM group -------------------
# The reference leaves both to XLibs' SubbandDedispersion; this rule defines them for the
# oracle and for the CPU baseline, which must not take its plan from the product library.

def _subband_edges(freqs, nsub):
    """First channel of each subband (channels j with j*nsub/C = s) and the highest and lowest
    frequency of each."""
    C_ = len(freqs)
    start = [(s * C_ + nsub - 1) // nsub for s in range(nsub + 1)]
    fref = [max(freqs[start[s]:start[s + 1]]) for s in range(nsub)]
    flow = [min(freqs[start[s]:start[s + 1]]) for s in range(nsub)]
    return start, fref, flow


def plan_group(freqs, nsub, tsamp, ddm, ndm):
    """Largest DM group whose smearing within a subband stays within one sample:
    group*ddm/2 * max_s dmdelay(1, fref_s, flow_s) <= tsamp, rounded down to a multiple of 8
    when at least 8, between 1 and ndm."""
    _, fref, flow = _subband_edges(freqs, nsub)
    kmax = max(dmdelay(1.0, h, l) for h, l in zip(fref, flow))
    if not ddm * kmax > 0.0:
        return int(min(max(ndm, 1), 1 << 30))
    g = np.floor(2.0 * tsamp / (ddm * kmax))
    if g >= 8.0:
        g = np.floor(g / 8.0) * 8.0
    return int(min(max(g, 1.0), float(ndm)))


def plan_nsub(freqs, tsamp, ddm, ndm):
    """The power of two (<= C) minimising the additions per output sample,
    C*ceil(ndm/group) + nsub*ndm; ties go to the smaller count."""
    C_ = len(freqs)
    best, bestcost, p = 1, None, 1
    while p <= C_:
        g = plan_group(freqs, p, tsamp, ddm, ndm)
        cost = float(C_) * float((ndm + g - 1) // g) + float(p) * float(ndm)
        if bestcost is None or cost < bestcost:
            best, bestcost = p, cost
        p *= 2
    return best


def plan_row(freqs_raw, tsamp_raw, td, fd, ddm, ndm, nsub=0, group=0):
    """(nsub, group) of one ddplan row on the td x fd downsampled channels: the given values
    where positive, else the rule above."""
    f = downsample_freqs(np.asarray(freqs_raw, np.float64), fd)
    tsamp = tsamp_raw * td
    ns = min(nsub, len(f)) if nsub > 0 else plan_nsub(f, tsamp, ddm, ndm)
    g = min(group, ndm) if group > 0 else plan_group(f, ns, tsamp, ddm, ndm)
    return ns, g


def width_ladder(minw, maxw, snrloss, tsamp, cap=256):
    out = np.zeros(cap, np.int32)
    n = lib().txo_width_ladder(minw, maxw, snrloss, tsamp, out, cap)
    return out[:n].copy()


def kadane(y):
    y = np.ascontiguousarray(y, np.float32)
    s, e = C.c_long(), C.c_long()
    b = lib().txo_kadane(y, len(y), C.byref(s), C.byref(e))
    return float(np.float32(b)), s.value, e.value


def red32(x, y=None, mode=0):
    x = np.ascontiguousarray(x, np.float32)
    yp = None
    if y is not None:
        y = np.ascontiguousarray(y, np.float32)
        yp = y.ctypes.data
    return lib().txo_red32(x, yp, len(x), mode)


def unpack_downsample(raw, td=1, fd=1, mask=None):
    raw = np.ascontiguousarray(raw, np.uint8)
    n0, nchan = raw.shape
    x = np.zeros((nchan // fd, n0 // td), np.float32)
    m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
    lib().txo_unpack_downsample(raw, n0, nchan, td, fd, x, x.shape[1],
                                None if m is None else m.ctypes.data)
    return x


def sk_moments(raw):
    raw = np.ascontiguousarray(raw, np.uint8)
    sk = np.zeros(raw.shape[1], np.float64)
    ku = np.zeros(raw.shape[1], np.float64)
    lib().txo_sk_moments(raw, raw.shape[0], raw.shape[1], sk, ku)
    return sk, ku


def skzap(raw, thr):
    raw = np.ascontiguousarray(raw, np.uint8)
    mask = np.zeros(raw.shape[1], np.uint8)
    lib().txo_skzap(raw, raw.shape[0], raw.shape[1], thr, mask)
    return mask


def downsample_freqs(f, fd):
    f = np.ascontiguousarray(f, np.float64)
    out = np.zeros(len(f) // fd, np.float64)
    lib().txo_downsample_freqs(f, len(f), fd, out)
    return out


def equalize(x):
    x = np.array(x, np.float32, order="C", copy=True)
    live = np.zeros(x.shape[0], np.uint8)
    lib().txo_equalize(x, x.shape[0], x.shape[1], x.shape[1], live.ctypes.data)
    return x, live


def baseline(x, nw, live=None):
    x = np.array(x, np.float32, order="C", copy=True)
    live = np.ones(x.shape[0], np.uint8) if live is None else np.ascontiguousarray(live, np.uint8)
    lib().txo_baseline(x, x.shape[0], x.shape[1], x.shape[1], nw, live.ctypes.data)
    return x


def kadaneF(x, tdk, fdk, thr, wnlimit):
    x = np.array(x, np.float32, order="C", copy=True)
    ranges = np.zeros((x.shape[0] // fdk, 4), np.int32)
    lib().txo_kadaneF(x, x.shape[0], x.shape[1], x.shape[1], tdk, fdk, thr, wnlimit, ranges)
    return x, ranges


def kadaneT(x, tdk, fdk, thr, bwlimit):
    x = np.array(x, np.float32, order="C", copy=True)
    ranges = np.zeros((x.shape[1] // tdk, 4), np.int32)
    n = lib().txo_kadaneT(x, x.shape[0], x.shape[1], x.shape[1], tdk, fdk, thr, bwlimit, ranges)
    return x, ranges, n


def mask(x, tdk, fdk, thr):
    """Returns (x, number of zapped pixels, [Q1, Q3, lo, hi])."""
    x = np.array(x, np.float32, order="C", copy=True)
    q = np.zeros(4, np.float32)
    n = lib().txo_mask(x, x.shape[0], x.shape[1], x.shape[1], tdk, fdk, thr, q)
    return x, n, q


def zero(x, live=None):
    x = np.array(x, np.float32, order="C", copy=True)
    live = np.ones(x.shape[0], np.uint8) if live is None else np.ascontiguousarray(live, np.uint8)
    lib().txo_zero(x, x.shape[0], x.shape[1], x.shape[1], live.ctypes.data)
    return x


def cand_band(sub, sub_start, fsub, isamp, wn):
    """fl, fh of one candidate from the [nsub][nout] subband sums of its DM."""
    sub = np.ascontiguousarray(sub, np.float32)
    fl, fh = C.c_float(), C.c_float()
    lib().txo_cand_band(sub, sub.shape[0], sub.shape[1], np.ascontiguousarray(sub_start, np.int32),
                        np.ascontiguousarray(fsub, np.float64), isamp, wn, C.byref(fl), C.byref(fh))
    return np.float32(fl.value), np.float32(fh.value)


def zdot(x):
    x = np.array(x, np.float32, order="C", copy=True)
    lib().txo_zdot(x, x.shape[0], x.shape[1], x.shape[1])
    return x


def boxcar_run(tim, vwn, iqr=False, avx2_tail=False):
    tim = np.ascontiguousarray(tim, np.float32)
    ndm, n = tim.shape
    vwn = np.ascontiguousarray(vwn, np.int32)
    mxS = np.zeros((ndm, n), np.float32)
    mxwn = np.zeros((ndm, n), np.int32)
    lib().txo_boxcar_run(tim, ndm, n, vwn, len(vwn), int(iqr), int(avx2_tail), mxS, mxwn)
    return mxS, mxwn


def threshold_scan(mxS, mxwn, thre):
    mxS = np.ascontiguousarray(mxS, np.float32)
    mxwn = np.ascontiguousarray(mxwn, np.int32)
    cnt = lib().txo_threshold_scan(mxS, mxwn, mxS.shape[0], mxS.shape[1], thre, None, 0)
    out = np.zeros(cnt, CAND_DTYPE)
    lib().txo_threshold_scan(mxS, mxwn, mxS.shape[0], mxS.shape[1], thre, out.ctypes.data, cnt)
    return out


def cluster(cands, dms, ddm, fmax, fmin, tsamp, radius, maxncand, minpts, drop, maxwn):
    cands = np.ascontiguousarray(cands, CAND_DTYPE)
    out = np.zeros(max(len(cands), 1), CAND_DTYPE)
    sizes = np.zeros(max(len(cands), 1), np.int32)
    n = lib().txo_cluster(cands.ctypes.data, len(cands), dms, ddm, fmax, fmin, tsamp, radius,
                          maxncand, minpts, int(drop), maxwn, out.ctypes.data, sizes.ctypes.data)
    return out[:n].copy(), sizes[:n].copy()


class Dedisp:
    """Streaming two-stage subband dedispersion (oracle)."""

    def __init__(self, freqs, tsamp, ndump, dms, ddm, ndm, overlap, nsub, group):
        f = np.ascontiguousarray(freqs, np.float64)
        self.h = lib().txo_dedisp_create(len(f), f, tsamp, ndump, dms, ddm, ndm, overlap, nsub,
                                         group)
        if not self.h:
            raise ValueError("invalid dedispersion parameters")
        self.nchan = len(f)
        self.ndm = ndm

    def info(self) -> DedispInfo:
        i = DedispInfo()
        lib().txo_dedisp_get_info(self.h, C.byref(i))
        return i

    def tables(self):
        i = self.info()
        d1 = np.zeros((i.ngroup, i.nchan), np.int32)
        d2 = np.zeros((i.ndm, i.nsub), np.int32)
        ss = np.zeros(i.nsub + 1, np.int32)
        fr = np.zeros(i.nsub, np.float64)
        lib().txo_dedisp_tables(self.h, d1.ctypes.data, d2.ctypes.data, ss.ctypes.data,
                                fr.ctypes.data)
        return d1, d2, ss, fr

    def run(self, x):
        x = np.ascontiguousarray(x, np.float32)
        return bool(lib().txo_dedisp_run(self.h, x, x.shape[1]))

    def timdata(self):
        i = self.info()
        p = lib().txo_dedisp_timdata(self.h)
        return np.ctypeslib.as_array(p, shape=(i.ndm, i.nout)).copy()

    def __del__(self):
        if getattr(self, "h", None):
            lib().txo_dedisp_destroy(self.h)
            self.h = None


class SinglePulseRow:
    """One ddplan row of the SinglePulse::run chain (oracle)."""

    def __init__(self, row: Row, freqs, tsamp, ndump):
        f = np.ascontiguousarray(freqs, np.float64)
        self.row = row
        self.h = lib().txo_sp_create(C.byref(row), len(f), f, tsamp, ndump)
        if not self.h:
            raise ValueError("invalid row parameters")
        self.nchan_raw = len(f)

    def run(self, raw) -> bool:
        raw = np.ascontiguousarray(raw, np.uint8)
        return bool(lib().txo_sp_run(self.h, raw))

    def run_f32(self, block) -> bool:
        """A preprocessed float block [ndump][nchan] (no channel zap)."""
        block = np.ascontiguousarray(block, np.float32)
        return bool(lib().txo_sp_run_f32(self.h, block))

    def info(self) -> DedispInfo:
        i = DedispInfo()
        lib().txo_sp_dedisp_info(self.h, C.byref(i))
        return i

    def widths(self):
        out = np.zeros(256, np.int32)
        n = lib().txo_sp_nwidths(self.h, out, 256)
        return out[:n].copy()

    def block(self):
        ldx, nch, n = C.c_long(), C.c_int(), C.c_long()
        p = lib().txo_sp_block(self.h, C.byref(ldx), C.byref(nch), C.byref(n))
        a = np.ctypeslib.as_array(p, shape=(nch.value, ldx.value))
        return a[:, : n.value].copy()

    def mask(self):
        p = lib().txo_sp_mask(self.h)
        return np.ctypeslib.as_array(p, shape=(self.nchan_raw,)).copy()

    def zap_ranges(self, irfi):
        nrows = C.c_int()
        p = lib().txo_sp_zap_ranges(self.h, irfi, C.byref(nrows))
        if not p:
            return None
        return np.ctypeslib.as_array(p, shape=(nrows.value, 4)).copy()

    def subdata(self, idm):
        i = self.info()
        out = np.zeros((i.nsub, i.nout), np.float32)
        assert lib().txo_dedisp_subdata(lib().txo_sp_dedisp(self.h), idm, out) == 0
        return out

    def timdata(self):
        i = self.info()
        return np.ctypeslib.as_array(lib().txo_sp_timdata(self.h), shape=(i.ndm, i.nout)).copy()

    def mxS(self):
        i = self.info()
        return np.ctypeslib.as_array(lib().txo_sp_mxS(self.h), shape=(i.ndm, i.nout)).copy()

    def mxwn(self):
        i = self.info()
        return np.ctypeslib.as_array(lib().txo_sp_mxwn(self.h), shape=(i.ndm, i.nout)).copy()

    def freqs(self):
        i = self.info()
        out = np.zeros(i.nchan, np.float64)
        lib().txo_sp_freqs(self.h, out)
        return out

    def __del__(self):
        if getattr(self, "h", None):
            lib().txo_sp_destroy(self.h)
            self.h = None


# ---- the reference's own code, compiled in place (only where the reference tree exists) -----

_ref = {}


def ref_available(variant="scalar") -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", f"libtxref_{variant}.so"))


def ref_lib(variant="scalar") -> C.CDLL:
    if variant in _ref:
        return _ref[variant]
    L = C.CDLL(os.path.join(HERE, "_ref", f"libtxref_{variant}.so"))
    L.ref_boxcar_run.restype = C.c_int
    L.ref_boxcar_run.argtypes = [f32p, C.c_long, C.c_long, i32p, C.c_int, C.c_int, f32p, i32p,
                                 C.c_int]
    L.ref_replot.restype = C.c_int
    L.ref_replot.argtypes = [C.c_void_p, C.c_int, C.c_long, C.c_double, C.c_void_p, C.c_double,
                             C.c_double, C.c_int, C.c_void_p, C.c_void_p, C.c_float, C.c_void_p,
                             C.c_int, C.c_int, C.c_float, C.c_int, C.c_int, C.c_int, C.c_int,
                             C.c_void_p, C.c_long, C.POINTER(C.c_long), C.POINTER(C.c_int),
                             C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_double),
                             C.POINTER(C.c_double), C.c_void_p, C.c_long, C.POINTER(C.c_int)]
    L.ref_candidate_rfi.restype = C.c_int
    L.ref_candidate_rfi.argtypes = [f32p, C.c_int, C.c_long, C.c_double, C.c_float, C.c_int,
                                    C.c_int, C.c_int, C.c_float, C.c_int, C.c_void_p]
    L.ref_candidate_downsample.restype = C.c_int
    L.ref_candidate_downsample.argtypes = [f32p, C.c_int, C.c_long, C.c_void_p, C.c_int, C.c_int,
                                           C.c_void_p, C.c_void_p]
    L.ref_dmdelay.restype = C.c_double
    L.ref_dmdelay.argtypes = [C.c_double, C.c_double, C.c_double]
    L.ref_cluster_run.restype = C.c_long
    L.ref_cluster_run.argtypes = [f32p, i32p, C.c_long, C.c_long, C.c_double, C.c_double,
                                  C.c_double, C.c_double, C.c_double, C.c_int, C.c_float,
                                  C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_long,
                                  i64p, i64p, i32p, f32p, C.c_long]
    _ref[variant] = L
    return L


def ref_replot(data, freqs, tbin, dm, width, zdot=False, kadane=None, clip=None, zapthre=3.0,
               zap=(), fd=1, snrloss=0.1, nwidth=20, pow2bin=False, nopt=False, upto=12,
               variant="scalar"):
    """The reference's Candidate chain of replot_fil on one candidate ([nchan][nbin] float):
    returns data after step `upto` (1..12) and, after step 12, snr, width, dm_maxsnr, mjd (from
    mjd_start 0) and the S/N map."""
    L = ref_lib(variant)
    data = np.ascontiguousarray(data, np.float32)
    nchan, nbin = data.shape
    freqs = np.ascontiguousarray(freqs, np.float64)
    out = np.zeros(nchan * nbin, np.float32)
    nb, nc, nd = C.c_long(), C.c_int(), C.c_int()
    snr, wid, dmx, mjd = C.c_float(), C.c_float(), C.c_double(), C.c_double()
    smap = np.zeros(4 * nchan * nbin + 64, np.float32)
    kad = (C.c_int * 3)(*kadane) if kadane else None
    clp = (C.c_int * 3)(*clip) if clip else None
    z = np.ascontiguousarray(np.array(zap, np.float64).reshape(-1), np.float64)
    L.ref_replot(data.ctypes.data, nchan, nbin, C.c_double(tbin), freqs.ctypes.data, C.c_double(dm),
                 C.c_double(width), int(zdot), kad, clp, C.c_float(zapthre),
                 z.ctypes.data if z.size else None, z.size // 2, fd, C.c_float(snrloss), nwidth,
                 int(pow2bin), int(nopt), upto, out.ctypes.data, out.size, C.byref(nb), C.byref(nc),
                 C.byref(snr), C.byref(wid), C.byref(dmx), C.byref(mjd), smap.ctypes.data, smap.size,
                 C.byref(nd))
    res = {"data": out[:nc.value * nb.value].reshape(nc.value, nb.value), "nbin": nb.value,
           "nchan": nc.value}
    if upto >= 12:
        res.update(snr=np.float32(snr.value), width=np.float32(wid.value), dm_maxsnr=dmx.value,
                   mjd=mjd.value, ndm=nd.value, snrmap=smap[:nd.value * nb.value].reshape(nd.value, nb.value))
    return res


def ref_zdot(x, variant="scalar"):
    """The reference's Candidate::zdot (candidate.cpp:831-897) on a [nchan][nbin] block."""
    x = np.array(x, np.float32, order="C")
    ref_lib(variant).ref_candidate_rfi(x, x.shape[0], x.shape[1], 1.0, 1.0, 0, 1, 1, 0.0, 1, None)
    return x


def ref_kadaneF(x, td, fd, threshold, nwidth, width, tbin, variant="scalar"):
    """The reference's Candidate::get_stats + normalize + kadaneF(td, fd, threshold, nwidth)
    (candidate.cpp:429-567, 710-829) on a [nchan][nbin] block: (normalised block, result)."""
    x = np.array(x, np.float32, order="C")
    pre = np.zeros_like(x)
    ref_lib(variant).ref_candidate_rfi(x, x.shape[0], x.shape[1], tbin, width, 1, td, fd,
                                       threshold, nwidth, pre.ctypes.data)
    return pre, x


def ref_downsample(x, freqs, td, fd, variant="scalar"):
    """The reference's Candidate::downsample(td, fd) (candidate.cpp:381-427) on a [nchan][nbin]
    block and its channel frequencies."""
    x = np.ascontiguousarray(x, np.float32)
    f = np.ascontiguousarray(freqs, np.float64)
    nc, nb = x.shape[0] // fd, x.shape[1] // td
    out = np.zeros((nc, nb), np.float32)
    fout = np.zeros(nc, np.float64)
    ref_lib(variant).ref_candidate_downsample(x, x.shape[0], x.shape[1], f.ctypes.data, td, fd,
                                              out.ctypes.data, fout.ctypes.data)
    return out, fout


def ref_boxcar_run(tim, vwn, iqr=False, variant="scalar", nthreads=4):
    tim = np.ascontiguousarray(tim, np.float32)
    ndm, n = tim.shape
    vwn = np.ascontiguousarray(vwn, np.int32)
    mxS = np.zeros((ndm, n), np.float32)
    mxwn = np.zeros((ndm, n), np.int32)
    ref_lib(variant).ref_boxcar_run(tim, ndm, n, vwn, len(vwn), int(iqr), mxS, mxwn, nthreads)
    return mxS, mxwn


def ref_cluster_run(mxS, mxwn, dms, ddm, tsamp, fmin, fmax, maxwn, thre, radius, kvalue,
                    maxncand, minpts, drop, counter=1, variant="scalar"):
    mxS = np.ascontiguousarray(mxS, np.float32)
    mxwn = np.ascontiguousarray(mxwn, np.int32)
    ndm, n = mxS.shape
    cap = max(int(maxncand), 1)
    idm = np.zeros(cap, np.int64)
    isamp = np.zeros(cap, np.int64)
    wn = np.zeros(cap, np.int32)
    S = np.zeros(cap, np.float32)
    m = ref_lib(variant).ref_cluster_run(mxS, mxwn, ndm, n, dms, ddm, tsamp, fmin, fmax, maxwn,
                                         thre, radius, kvalue, maxncand, minpts, int(drop),
                                         counter, idm, isamp, wn, S, cap)
    out = np.zeros(max(m, 0), CAND_DTYPE)
    out["idm"], out["isamp"], out["wn"], out["S"] = idm[:m], isamp[:m], wn[:m], S[:m]
    return out
