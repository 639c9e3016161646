"""transientx_gb300 -- GB300 (sm_103a) implementation of TransientX's per-block single-pulse
search, driven through the C ABI of include/transientx_gb300.h.

The Python layer mirrors the reference's host interface for this path:
  * ``SinglePulse`` carries the per-ddplan-row configuration members of the reference class
    (include/singlepulse.h:95-133) and ``parse_ddplan`` reads the ddplan text format of
    parse() (src/singlepulse/singlepulse.cpp:407-463);
  * ``Search`` owns one handle: ``push_block`` is one iteration of the transientx_fil block
    loop (dedisperse_fil.cpp:319-337) over all ddplan rows, ``candidates`` yields the
    S > thre points Cluster::run consumes, ``cluster`` runs the clustering;
  * ``boxcar`` is Boxcar::run over caller-supplied dedispersed series.
All compute runs in the CUDA library; importing this module without it raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libtxgpu.so")

OK = 0
ERR_ARG, ERR_NOMEM, ERR_CUDA, ERR_OVERFLOW = -1, -2, -3, -4
ERR_TIMEOUT, ERR_STATE, ERR_NODEVICE, ERR_UNSUPPORTED = -5, -6, -7, -8
RFI_KADANEF, RFI_ZDOT, RFI_MASK, RFI_KADANET, RFI_ZERO = 1, 2, 3, 4, 5
PREC_FP32, PREC_BF16, PREC_FP16 = 0, 1, 2
FLAG_AVX2_TAIL, FLAG_DENSE, FLAG_KEEP_SERIES, FLAG_TIMING, FLAG_CLUSTER = 1, 2, 4, 8, 16
FLAG_AUTOTUNE = 32
PRECISIONS = {"fp32": PREC_FP32, "bf16": PREC_BF16, "fp16": PREC_FP16}


class TxgError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(msg)
        self.status = status


class txg_row(C.Structure):
    _fields_ = [
        ("td", C.c_int32), ("fd", C.c_int32), ("bswidth", C.c_float), ("nrfi", C.c_int32),
        ("rfi_kind", C.c_int32 * 8), ("rfi_td", C.c_int32 * 8), ("rfi_fd", C.c_int32 * 8),
        ("nzap", C.c_int32), ("zap", (C.c_double * 2) * 16), ("threKadaneF", C.c_float),
        ("widthlimit", C.c_double), ("dms", C.c_double), ("ddm", C.c_double),
        ("ndm", C.c_int64), ("overlap", C.c_double), ("minw", C.c_float), ("maxw", C.c_float),
        ("snrloss", C.c_float), ("iqr", C.c_int32), ("thre", C.c_float), ("nsub", C.c_int32),
        ("dm_group", C.c_int32), ("radius_smearing", C.c_double), ("maxncand", C.c_int32),
        ("minpts", C.c_int32), ("drop", C.c_int32), ("threMask", C.c_float),
        ("threKadaneT", C.c_float), ("pad", C.c_int32), ("bandlimitKT", C.c_double),
    ]


class txg_replot_opts(C.Structure):
    _fields_ = [("zdot", C.c_int32), ("kadane", C.c_int32 * 3), ("clip", C.c_int32 * 3),
                ("zapthre", C.c_float), ("nzap", C.c_int32), ("zap", (C.c_double * 2) * 16),
                ("fd", C.c_int32), ("snrloss", C.c_float), ("nwidth", C.c_int32),
                ("pow2bin", C.c_int32), ("nopt", C.c_int32), ("upto", C.c_int32)]


class txg_replot_cand(C.Structure):
    _fields_ = [("data", C.c_void_p), ("nchan", C.c_int32), ("nbin", C.c_int64),
                ("tbin", C.c_double), ("frequencies", C.c_void_p), ("dm", C.c_double),
                ("width", C.c_float)]


class txg_replot_result(C.Structure):
    _fields_ = [("snr", C.c_float), ("width", C.c_float), ("dm_maxsnr", C.c_double),
                ("maxtid", C.c_int64), ("nbin", C.c_int64), ("nchan", C.c_int32),
                ("ndm", C.c_int32), ("dms", C.c_double), ("ddm", C.c_double)]


class txg_result(C.Structure):
    _fields_ = [("counter", C.c_int64), ("gated", C.c_int32), ("overflow", C.c_int32),
                ("npoints", C.c_int64), ("nclusters", C.c_int64)]


class txg_plan(C.Structure):
    _fields_ = [
        ("nchans", C.c_int32), ("tsamp", C.c_double), ("frequencies", C.POINTER(C.c_double)),
        ("ndump", C.c_int64), ("nrows", C.c_int32), ("rows", C.POINTER(txg_row)),
        ("nbeams", C.c_int32), ("precision", C.c_int32), ("flags", C.c_int32),
        ("cand_capacity", C.c_int64), ("zapthre", C.c_float),
    ]


class txg_row_info(C.Structure):
    _fields_ = [
        ("nchans", C.c_int32), ("nsub", C.c_int32), ("dm_group", C.c_int32),
        ("ngroup", C.c_int32), ("nwidths", C.c_int32), ("maxwn", C.c_int32),
        ("ndm", C.c_int64), ("ndump", C.c_int64), ("noverlap", C.c_int64), ("offset", C.c_int64),
        ("nsamples", C.c_int64), ("counter", C.c_int64), ("maxd1", C.c_int64),
        ("maxd2", C.c_int64), ("tsamp", C.c_double), ("dms", C.c_double), ("ddm", C.c_double),
        ("fmin", C.c_double), ("fmax", C.c_double), ("gated", C.c_int32), ("pad", C.c_int32),
    ]


CAND_DTYPE = np.dtype([("idm", "<i4"), ("isamp", "<i4"), ("wn", "<i4"), ("S", "<f4")])

# every symbol include/transientx_gb300.h declares
EXPORTS = [
    "txg_create", "txg_destroy", "txg_push_block", "txg_push_block_device", "txg_sync",
    "txg_get_row_info", "txg_get_candidates", "txg_get_dense", "txg_get_timdata",
    "txg_get_block", "txg_get_zap_ranges", "txg_get_tables", "txg_width_ladder", "txg_boxcar",
    "txg_cluster", "txg_get_timing", "txg_get_stream", "txg_strerror", "txg_version",
    "txg_describe_row", "txg_pop_result", "txg_get_mask", "txg_kadaneF_noalloc",
    "txg_get_subdata", "txg_cand_band", "txg_replot", "txg_get_timdata_q", "txg_result_ready",
    "txg_selftest_wait", "txg_reset_beam", "txg_push_block_f32", "txg_get_launch_shape",
    "txg_get_row_timing",
]

_lib: Optional[C.CDLL] = None
vp = C.c_void_p


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Load the CUDA library (built in-tree by ``transientx_gb300._build``)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with `python -m transientx_gb300._build` "
                          "(there is no CPU fallback)")
    L = C.CDLL(path)
    L.txg_version.restype = C.c_int32
    L.txg_strerror.restype = C.c_char_p
    L.txg_strerror.argtypes = [C.c_int32]
    L.txg_create.argtypes = [C.POINTER(txg_plan), C.POINTER(vp)]
    L.txg_destroy.argtypes = [vp]
    L.txg_destroy.restype = None
    L.txg_push_block.argtypes = [vp, C.c_int32, vp, C.c_int64]
    L.txg_push_block_device.argtypes = [vp, C.c_int32, vp, C.c_int64]
    L.txg_sync.argtypes = [vp]
    L.txg_reset_beam.argtypes = [vp, C.c_int32]
    L.txg_push_block_f32.argtypes = [vp, C.c_int32, vp, C.c_int64]
    L.txg_get_row_timing.argtypes = [vp, C.c_int32, vp, vp, C.c_int32]
    L.txg_get_launch_shape.argtypes = [vp, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                       C.POINTER(C.c_int32)]
    L.txg_get_row_info.argtypes = [vp, C.c_int32, C.c_int32, C.POINTER(txg_row_info)]
    L.txg_get_candidates.argtypes = [vp, C.c_int32, C.c_int32, vp, C.c_int64,
                                     C.POINTER(C.c_int64)]
    L.txg_get_dense.argtypes = [vp, C.c_int32, C.c_int32, vp, vp]
    L.txg_get_timdata.argtypes = [vp, C.c_int32, C.c_int32, C.c_int64, C.c_int64, vp]
    L.txg_get_block.argtypes = [vp, C.c_int32, C.c_int32, vp]
    L.txg_get_zap_ranges.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, vp, C.c_int64]
    L.txg_get_tables.argtypes = [vp, C.c_int32, vp, vp, vp, vp]
    L.txg_width_ladder.argtypes = [C.c_float, C.c_float, C.c_float, C.c_double, vp, C.c_int32]
    L.txg_boxcar.argtypes = [vp, C.c_int64, C.c_int64, vp, C.c_int32, C.c_int32, C.c_int32,
                             C.c_float, vp, vp, vp, C.c_int64, C.POINTER(C.c_int64)]
    L.txg_cluster.argtypes = [vp, C.c_int64, C.c_double, C.c_double, C.c_double, C.c_double,
                              C.c_double, C.c_double, C.c_int32, C.c_int32, C.c_int32,
                              C.c_int32, vp, C.c_int64, C.POINTER(C.c_int64)]
    L.txg_get_timing.argtypes = [vp, vp, vp, C.c_int32]
    L.txg_get_stream.argtypes = [vp, C.POINTER(vp)]
    L.txg_get_mask.argtypes = [vp, C.c_int32, vp]
    L.txg_get_subdata.argtypes = [vp, C.c_int32, C.c_int32, C.c_int64, vp]
    L.txg_get_timdata_q.argtypes = [vp, C.c_int32, C.c_int32, C.c_int64, C.c_int64, C.c_int64,
                                    C.c_int32, C.c_float, C.c_float, vp]
    L.txg_replot.argtypes = [C.POINTER(txg_replot_opts), C.POINTER(txg_replot_cand), C.c_int64,
                             C.POINTER(txg_replot_result), vp, C.c_int64, vp, C.c_int64]
    L.txg_cand_band.argtypes = [vp, C.c_int32, C.c_int32, vp, C.c_int64, vp, vp]
    L.txg_kadaneF_noalloc.argtypes = [vp, C.c_int64, C.c_int32, C.c_int64, C.c_int32, C.c_int32,
                                      C.c_float, C.c_int64, vp, vp]
    L.txg_pop_result.argtypes = [vp, C.c_int32, C.c_int32, C.POINTER(txg_result), vp, C.c_int64,
                                 vp, C.c_int64]
    L.txg_result_ready.argtypes = [vp, C.c_int32, C.c_int32, C.POINTER(C.c_int32)]
    L.txg_selftest_wait.argtypes = [C.c_int32, C.c_int32]
    L.txg_describe_row.argtypes = [C.POINTER(txg_plan), C.c_int32, C.POINTER(txg_row_info), vp,
                                   vp, vp, vp]
    _lib = L
    return L


def _check(rc: int, what: str = "") -> None:
    if rc != OK:
        msg = load_library().txg_strerror(rc).decode()
        raise TxgError(rc, f"{what}: {msg}" if what else msg)


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


# ---- configuration mirror --------------------------------------------------------------

@dataclass
class Boxcar:
    """The public members of the reference's Boxcar (include/boxcar.h:31-43) for one (row,
    beam) after its last block, as Search.boxcar fills them: mxS / mxwn are the dense
    [ndm][nsamples] planes when the plan has FLAG_DENSE, else None; gated is what Boxcar::run
    returned (boxcar.cpp:160-161)."""
    counter: int = 0
    tsamp: float = 0.0
    nsamples: int = 0
    dms: float = 0.0
    ddm: float = 0.0
    ndm: int = 0
    maxwn: int = 0
    fmin: float = 0.0
    fmax: float = 0.0
    mxS: Optional[np.ndarray] = None
    mxwn: Optional[np.ndarray] = None
    gated: bool = False

    def dump2txt(self, fname: str) -> None:
        """mxS as text, one line per DM trial, each value printed "%f " (boxcar.cpp:473-489)."""
        if self.mxS is None:
            raise TxgError(ERR_STATE, "dump2txt: no dense mxS (plan without FLAG_DENSE)")
        with open(fname, "w") as f:
            for row in np.asarray(self.mxS, np.float32).reshape(self.ndm, self.nsamples):
                f.write("".join("%f " % v for v in row) + "\n")


@dataclass
class SinglePulse:
    """Configuration of one ddplan row, with the member names of the reference's SinglePulse
    (include/singlepulse.h:95-133) and its defaults (src/singlepulse/singlepulse.cpp:18-65,
    CLI defaults of src/singlepulse/dedisperse_fil.cpp:54-99 where the CLI sets them)."""
    td: int = 1
    fd: int = 1
    bswidth: float = 0.1
    zaplist: List[Tuple[float, float]] = field(default_factory=list)
    rfilist: List[List[str]] = field(default_factory=list)
    widthlimit: float = 50e-3
    threKadaneF: float = 7.0
    threMask: float = 10.0
    threKadaneT: float = 7.0
    bandlimitKT: float = 10.0
    dms: float = 0.0
    ddm: float = 1.0
    ndm: int = 200
    overlap: float = 0.0
    minw: float = 1e-4
    maxw: float = 0.02
    snrloss: float = 0.1
    iqr: bool = False
    thre: float = 7.0
    radius_smearing: float = 1e-3
    kvalue: int = 2
    maxncand: int = 100
    minpts: int = 5
    remove_cand_with_maxwidth: bool = False
    nsub: int = 0
    dm_group: int = 0
    id: int = 1

    def to_c(self) -> txg_row:
        r = txg_row()
        r.td, r.fd, r.bswidth = self.td, self.fd, self.bswidth
        if len(self.rfilist) > 8 or len(self.zaplist) > 16:
            raise ValueError("at most 8 rfilist and 16 zaplist entries")
        r.nrfi = len(self.rfilist)
        for i, op in enumerate(self.rfilist):
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
                raise TxgError(ERR_UNSUPPORTED, f"rfilist entry {op[0]!r} is not implemented")
        r.nzap = len(self.zaplist)
        for i, (a, b) in enumerate(self.zaplist):
            r.zap[i][0], r.zap[i][1] = a, b
        r.threKadaneF, r.widthlimit = self.threKadaneF, self.widthlimit
        r.threMask, r.threKadaneT, r.bandlimitKT = self.threMask, self.threKadaneT, self.bandlimitKT
        r.dms, r.ddm, r.ndm, r.overlap = self.dms, self.ddm, self.ndm, self.overlap
        r.minw, r.maxw, r.snrloss = self.minw, self.maxw, self.snrloss
        r.iqr, r.thre = int(self.iqr), self.thre
        r.nsub, r.dm_group = self.nsub, self.dm_group
        r.radius_smearing, r.maxncand = self.radius_smearing, self.maxncand
        r.minpts, r.drop = self.minpts, int(self.remove_cand_with_maxwidth)
        return r


def _rfi_opts(tokens: Sequence[str], sp: SinglePulse) -> None:
    i = 0
    while i < len(tokens):
        t = tokens[i]
        if t in ("mask", "kadaneF", "kadaneT"):
            sp.rfilist.append([t, tokens[i + 1], tokens[i + 2]])
            i += 3
        elif t == "zap":
            sp.zaplist.append((float(tokens[i + 1]), float(tokens[i + 2])))
            i += 3
        elif t in ("zero", "zdot"):
            sp.rfilist.append([t])
            i += 1
        else:
            i += 1


def parse_ddplan(text: str, base: Optional[SinglePulse] = None) -> List[SinglePulse]:
    """ddplan rows ``td fd dms ddm ndm snrloss maxw [rfi options]``; lines not starting with a
    digit are skipped and each row inherits the rfi options of earlier rows, as parse() does
    (singlepulse.cpp:407-456)."""
    import copy
    sp = copy.deepcopy(base) if base is not None else SinglePulse()
    rows, ident = [], 0
    for line in text.splitlines():
        line = line.strip()
        if not line or not line[0].isdigit():
            continue
        p = line.split()
        sp.td, sp.fd = int(p[0]), int(p[1])
        sp.dms, sp.ddm, sp.ndm = float(p[2]), float(p[3]), int(p[4])
        sp.snrloss, sp.maxw = float(p[5]), float(p[6])
        _rfi_opts(p[7:], sp)
        ident += 1
        sp.id = ident
        rows.append(copy.deepcopy(sp))
    return rows


def width_ladder(minw: float, maxw: float, snrloss: float, tsamp: float) -> np.ndarray:
    out = np.zeros(256, np.int32)
    n = load_library().txg_width_ladder(minw, maxw, snrloss, tsamp, _ptr(out), 256)
    return out[:n].copy()


def _make_plan(rows, nchans, tsamp, freqs, ndump, nbeams, precision, flags, cand_capacity,
               zapthre=0.0):
    crows = (txg_row * len(rows))(*[r.to_c() for r in rows])
    plan = txg_plan()
    plan.nchans, plan.tsamp = nchans, tsamp
    plan.frequencies = freqs.ctypes.data_as(C.POINTER(C.c_double))
    plan.ndump, plan.nrows, plan.rows = ndump, len(rows), crows
    plan.nbeams, plan.precision, plan.flags = nbeams, PRECISIONS[precision], flags
    plan.cand_capacity = cand_capacity
    plan.zapthre = zapthre
    return plan, crows


def describe_row(rows: Sequence[SinglePulse], row: int, nchans: int, tsamp: float,
                 frequencies: Sequence[float], ndump: int):
    """Host-only planning of one ddplan row: (info, d1, d2, sub_start, vwn)."""
    freqs = np.ascontiguousarray(frequencies, np.float64)
    plan, crows = _make_plan(rows, nchans, tsamp, freqs, ndump, 1, "fp32", 0, 0)
    info = txg_row_info()
    L = load_library()
    _check(L.txg_describe_row(C.byref(plan), row, C.byref(info), None, None, None, None),
           "describe_row")
    d1 = np.zeros((info.ngroup, info.nchans), np.int32)
    d2 = np.zeros((info.ndm, info.nsub), np.int32)
    ss = np.zeros(info.nsub + 1, np.int32)
    vwn = np.zeros(info.nwidths, np.int32)
    _check(L.txg_describe_row(C.byref(plan), row, C.byref(info), _ptr(d1), _ptr(d2), _ptr(ss),
                              _ptr(vwn)), "describe_row")
    return info, d1, d2, ss, vwn


# ---- handle ------------------------------------------------------------------------------

class Search:
    """One handle: all ddplan rows of ``rows`` for ``nbeams`` beams of the same format."""

    def __init__(self, rows: Sequence[SinglePulse], nchans: int, tsamp: float,
                 frequencies: Sequence[float], ndump: int, nbeams: int = 1,
                 precision: str = "fp32", flags: int = 0, cand_capacity: int = 0,
                 zapthre: float = 4.0):
        """zapthre: skewness/kurtosis channel-zap threshold in IQR units, the --zapthre of
        transientx_fil (default 4, dedisperse_fil.cpp:56); <= 0 disables it."""
        L = load_library()
        self.rows = list(rows)
        self.nchans, self.tsamp, self.ndump, self.nbeams = nchans, tsamp, ndump, nbeams
        self._freqs = np.ascontiguousarray(frequencies, np.float64)
        if len(self._freqs) != nchans:
            raise ValueError("need one frequency per channel")
        plan, self._crows = _make_plan(self.rows, nchans, tsamp, self._freqs, ndump, nbeams,
                                       precision, flags, cand_capacity, zapthre)
        self.zapthre = zapthre
        self.cap = cand_capacity if cand_capacity > 0 else 1 << 20
        self.flags = flags
        h = vp()
        _check(L.txg_create(C.byref(plan), C.byref(h)), "txg_create")
        self.h = h

    def close(self) -> None:
        if getattr(self, "h", None):
            load_library().txg_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def push_block(self, raw: np.ndarray, beam: int = 0) -> None:
        raw = np.ascontiguousarray(raw, np.uint8)
        if raw.shape != (self.ndump, self.nchans):
            raise ValueError(f"block must be [{self.ndump}][{self.nchans}] uint8")
        rc = load_library().txg_push_block(self.h, beam, _ptr(raw), self.ndump)
        if rc not in (OK, ERR_OVERFLOW):
            _check(rc, "txg_push_block")

    def push_block_f32(self, block: np.ndarray, beam: int = 0) -> None:
        """One preprocessed float block [ndump][nchans] (txg_push_block_f32)."""
        blk = np.ascontiguousarray(block, np.float32)
        if blk.shape != (self.ndump, self.nchans):
            raise ValueError(f"block must be [{self.ndump}][{self.nchans}] float32")
        rc = load_library().txg_push_block_f32(self.h, beam, _ptr(blk), self.ndump)
        if rc not in (OK, ERR_OVERFLOW):
            _check(rc, "push_block_f32")

    def push_block_device(self, dev_ptr: int, beam: int = 0) -> None:
        rc = load_library().txg_push_block_device(self.h, beam, int(dev_ptr), self.ndump)
        if rc not in (OK, ERR_OVERFLOW):
            _check(rc, "txg_push_block_device")

    def sync(self, allow_overflow: bool = False) -> int:
        rc = load_library().txg_sync(self.h)
        if rc == ERR_OVERFLOW and allow_overflow:
            return rc
        _check(rc, "txg_sync")
        return rc

    def reset_beam(self, beam: int = 0) -> None:
        """Begin a new observation on `beam` (txg_reset_beam): the next block pushed is the
        first of a new file; blocks queued before belong to the previous one."""
        _check(load_library().txg_reset_beam(self.h, beam), "reset_beam")

    def row_info(self, row: int = 0, beam: int = 0) -> txg_row_info:
        info = txg_row_info()
        _check(load_library().txg_get_row_info(self.h, beam, row, C.byref(info)), "row_info")
        return info

    def candidates(self, row: int = 0, beam: int = 0) -> np.ndarray:
        L = load_library()
        n = C.c_int64()
        L.txg_get_candidates(self.h, beam, row, None, 0, C.byref(n))
        kept = min(n.value, self.cap)
        out = np.zeros(kept, CAND_DTYPE)
        rc = L.txg_get_candidates(self.h, beam, row, _ptr(out), kept, C.byref(n))
        if rc not in (OK, ERR_OVERFLOW):
            _check(rc, "candidates")
        return out

    def result_ready(self, row: int = 0, beam: int = 0) -> Optional[bool]:
        """Whether pop_result would return without waiting on host clustering; None when no
        block of (beam,row) is waiting."""
        L = load_library()
        ready = C.c_int32(0)
        rc = L.txg_result_ready(self.h, beam, row, C.byref(ready))
        if rc == ERR_STATE:
            return None
        _check(rc)
        return bool(ready.value)

    def pop_result(self, row: int = 0, beam: int = 0, points: bool = True):
        """Oldest unread block of (beam,row) as (result, points, clusters), or None.  Clusters
        are filled when the plan has FLAG_CLUSTER."""
        L = load_library()
        res = txg_result()
        buf = getattr(self, "_popbuf", None)
        if buf is None:
            buf = self._popbuf = np.zeros(self.cap, CAND_DTYPE)
            self._clbuf = np.zeros(1 << 12, CAND_DTYPE)
        rc = L.txg_pop_result(self.h, beam, row, C.byref(res), _ptr(buf) if points else None,
                              len(buf) if points else 0, _ptr(self._clbuf), len(self._clbuf))
        if rc == ERR_STATE:
            return None
        if rc not in (OK, ERR_OVERFLOW):
            _check(rc, "pop_result")
        pts = buf[:min(res.npoints, self.cap)].copy() if points else None
        cl = self._clbuf[:min(res.nclusters, len(self._clbuf))].copy()
        return res, pts, cl

    def boxcar(self, row: int = 0, beam: int = 0) -> Boxcar:
        """Boxcar's members for the row's last block; the dense planes with FLAG_DENSE."""
        i = self.row_info(row, beam)
        b = Boxcar(counter=i.counter, tsamp=i.tsamp, nsamples=i.nsamples, dms=i.dms, ddm=i.ddm,
                   ndm=i.ndm, maxwn=i.maxwn, fmin=i.fmin, fmax=i.fmax, gated=bool(i.gated))
        if self.flags & FLAG_DENSE:
            b.mxS, b.mxwn = self.dense(row, beam)
        return b

    def dense(self, row: int = 0, beam: int = 0) -> Tuple[np.ndarray, np.ndarray]:
        i = self.row_info(row, beam)
        mxS = np.zeros((i.ndm, i.nsamples), np.float32)
        mxwn = np.zeros((i.ndm, i.nsamples), np.int32)
        _check(load_library().txg_get_dense(self.h, beam, row, _ptr(mxS), _ptr(mxwn)), "dense")
        return mxS, mxwn

    def timdata(self, row: int = 0, beam: int = 0, idm0: int = 0, count: int = -1) -> np.ndarray:
        i = self.row_info(row, beam)
        count = i.ndm - idm0 if count < 0 else count
        out = np.zeros((count, i.nsamples), np.float32)
        _check(load_library().txg_get_timdata(self.h, beam, row, idm0, count, _ptr(out)),
               "timdata")
        return out

    def timdata_q(self, row: int = 0, beam: int = 0, idm0: int = 0, count: int = -1,
                  nsamp: int = 0, nbits: int = 8, mean: float = 0.0, std: float = 3.0) -> np.ndarray:
        """Quantised dedispersed series of the last block ([count][nsamp] uint8 / uint16 /
        float32; nsamp 0 = ndump, the non-overlapping part)."""
        i = self.row_info(row, beam)
        count = i.ndm - idm0 if count < 0 else count
        nsamp = i.ndump if nsamp <= 0 else nsamp
        dt = {8: np.uint8, 16: np.uint16, 32: np.float32}[nbits]
        out = np.zeros((count, nsamp), dt)
        _check(load_library().txg_get_timdata_q(self.h, beam, row, idm0, count, nsamp, nbits, mean,
                                                std, _ptr(out)), "timdata_q")
        return out

    def subdata(self, idm: int, row: int = 0, beam: int = 0) -> np.ndarray:
        """SubbandDedispersion::get_subdata of the last block: [nsub][nsamples] subband sums."""
        i = self.row_info(row, beam)
        out = np.zeros((i.nsub, i.nsamples), np.float32)
        _check(load_library().txg_get_subdata(self.h, beam, row, idm, _ptr(out)), "subdata")
        return out

    def cand_band(self, cands: np.ndarray, row: int = 0, beam: int = 0):
        """fl, fh of the .cands line for each candidate (idm, isamp, wn, S) of the last block."""
        c = np.ascontiguousarray(cands, CAND_DTYPE)
        fl = np.zeros(len(c), np.float32)
        fh = np.zeros(len(c), np.float32)
        _check(load_library().txg_cand_band(self.h, beam, row, _ptr(c), len(c), _ptr(fl),
                                            _ptr(fh)), "cand_band")
        return fl, fh

    def block(self, row: int = 0, beam: int = 0) -> np.ndarray:
        i = self.row_info(row, beam)
        out = np.zeros((i.nchans, i.ndump), np.float32)
        _check(load_library().txg_get_block(self.h, beam, row, _ptr(out)), "block")
        return out

    def mask(self, beam: int = 0) -> np.ndarray:
        out = np.zeros(self.nchans, np.uint8)
        _check(load_library().txg_get_mask(self.h, beam, _ptr(out)), "mask")
        return out

    def zap_ranges(self, irfi: int, row: int = 0, beam: int = 0) -> np.ndarray:
        """kadaneF: [nchans/fd][4] sample windows; kadaneT: [ndump/td][4] channel bands;
        mask: [1][4] with the number of zapped pixels first."""
        i = self.row_info(row, beam)
        op = self.rows[row].rfilist[irfi]
        if op[0] == "mask":
            n = 1
        elif op[0] == "kadaneT":
            n = i.ndump // int(op[1])
        else:
            n = i.nchans // int(op[2])
        out = np.zeros((n, 4), np.int32)
        _check(load_library().txg_get_zap_ranges(self.h, beam, row, irfi, _ptr(out), out.size),
               "zap_ranges")
        return out

    def tables(self, row: int = 0):
        i = self.row_info(row)
        d1 = np.zeros((i.ngroup, i.nchans), np.int32)
        d2 = np.zeros((i.ndm, i.nsub), np.int32)
        ss = np.zeros(i.nsub + 1, np.int32)
        vwn = np.zeros(i.nwidths, np.int32)
        _check(load_library().txg_get_tables(self.h, row, _ptr(d1), _ptr(d2), _ptr(ss),
                                             _ptr(vwn)), "tables")
        return d1, d2, ss, vwn

    def timing(self) -> Tuple[np.ndarray, np.ndarray]:
        ms = np.zeros(8, np.float64)
        n = np.zeros(8, np.int64)
        k = load_library().txg_get_timing(self.h, _ptr(ms), _ptr(n), 8)
        return ms[:k], n[:k]

    def row_timing(self, row: int) -> Tuple[np.ndarray, np.ndarray]:
        """Per-class device time of one ddplan row since the last call (FLAG_TIMING)."""
        ms = np.zeros(8, np.float64)
        n = np.zeros(8, np.int64)
        k = load_library().txg_get_row_timing(self.h, row, _ptr(ms), _ptr(n), 8)
        if k < 0:
            _check(k, "row_timing")
        return ms[:k], n[:k]

    def launch_shape(self, row: int = 0) -> Tuple[int, int, int]:
        """(stage-1 shape, stage-2 variant, stage-2 KB) the row runs with
        (txg_get_launch_shape; with FLAG_AUTOTUNE, the fastest timed at creation)."""
        a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
        _check(load_library().txg_get_launch_shape(self.h, row, C.byref(a), C.byref(b),
                                                   C.byref(c)), "launch_shape")
        return a.value, b.value, c.value

    def stream(self) -> int:
        s = vp()
        _check(load_library().txg_get_stream(self.h, C.byref(s)), "stream")
        return s.value or 0

    def cluster(self, row: int = 0, beam: int = 0, cands: Optional[np.ndarray] = None):
        """Cluster<double>::run on this row's last block (cluster.cpp:63-161)."""
        sp = self.rows[row]
        i = self.row_info(row, beam)
        if cands is None:
            cands = self.candidates(row, beam)
        return cluster(cands, i.dms, i.ddm, i.fmax, i.fmin, i.tsamp, sp.radius_smearing,
                       sp.maxncand, sp.minpts, sp.remove_cand_with_maxwidth, i.maxwn)


def selftest_wait(never_complete: bool, limit_ms: int = 200) -> int:
    """The bounded device wait of the shared-memory copies, on a copy that completes or on a
    barrier that never completes (then TXG_ERR_TIMEOUT after limit_ms); returns the status."""
    return int(load_library().txg_selftest_wait(1 if never_complete else 0, int(limit_ms)))


def boxcar(tim: np.ndarray, vwn: Sequence[int], iqr: bool = False, avx2_tail: bool = False,
           thre: float = 7.0, dense: bool = True, cand_capacity: int = 1 << 20):
    """Boxcar::run (boxcar.cpp:158-296) on the GPU over caller-supplied series [ndm][n]."""
    tim = np.ascontiguousarray(tim, np.float32)
    ndm, n = tim.shape
    vwn = np.ascontiguousarray(vwn, np.int32)
    mxS = np.zeros((ndm, n), np.float32) if dense else None
    mxwn = np.zeros((ndm, n), np.int32) if dense else None
    cands = np.zeros(cand_capacity, CAND_DTYPE)
    nc = C.c_int64()
    rc = load_library().txg_boxcar(_ptr(tim), ndm, n, _ptr(vwn), len(vwn), int(iqr),
                                   FLAG_AVX2_TAIL if avx2_tail else 0, thre,
                                   _ptr(mxS) if dense else None, _ptr(mxwn) if dense else None,
                                   _ptr(cands), cand_capacity, C.byref(nc))
    _check(rc, "txg_boxcar")
    return mxS, mxwn, cands[: nc.value].copy()


def cluster(cands: np.ndarray, dms: float, ddm: float, fmax: float, fmin: float, tsamp: float,
            radius_smearing: float, maxncand: int, minpts: int, drop: bool,
            maxwn: int) -> np.ndarray:
    """Cluster<double>::run (cluster.cpp:63-161): the reported (idm, isamp, wn, S) list."""
    cands = np.ascontiguousarray(cands, CAND_DTYPE)
    out = np.zeros(max(maxncand, 1), CAND_DTYPE)
    n = C.c_int64()
    _check(load_library().txg_cluster(_ptr(cands) if len(cands) else None, len(cands), dms, ddm,
                                      fmax, fmin, tsamp, radius_smearing, maxncand, minpts,
                                      int(drop), maxwn, _ptr(out), len(out), C.byref(n)),
           "txg_cluster")
    return out[: n.value].copy()


def replot(cands, zdot: bool = False, kadane=None, clip=None, zapthre: float = 3.0, zap=(),
           fd: int = 1, snrloss: float = 0.1, nwidth: int = 20, pow2bin: bool = False,
           nopt: bool = False, upto: int = 0, maps: bool = False, data: bool = False):
    """The replot_fil chain (replot_fil.cpp:409-457) on the GPU for a batch of candidates, each a
    dict with data [nchan][nbin] float32, tbin, frequencies, dm, width (s).  Returns a list of
    dicts (snr, width, dm_maxsnr, maxtid, nbin, nchan, ndm, dms, ddm), with the S/N map and/or
    the final data when asked."""
    L = load_library()
    o = txg_replot_opts()
    o.zdot = int(zdot)
    for i, v in enumerate(kadane or (0, 0, 0)):
        o.kadane[i] = int(v)
    for i, v in enumerate(clip or (0, 0, 0)):
        o.clip[i] = int(v)
    o.zapthre = zapthre
    o.nzap = len(zap)
    for i, (a, b) in enumerate(zap):
        o.zap[i][0], o.zap[i][1] = a, b
    o.fd, o.snrloss, o.nwidth, o.pow2bin, o.nopt, o.upto = fd, snrloss, nwidth, int(pow2bin), int(nopt), upto
    keep = []
    arr = (txg_replot_cand * len(cands))()
    for k, c in enumerate(cands):
        d = np.ascontiguousarray(c["data"], np.float32)
        f = np.ascontiguousarray(c["frequencies"], np.float64)
        keep += [d, f]
        arr[k].data, arr[k].nchan, arr[k].nbin = d.ctypes.data, d.shape[0], d.shape[1]
        arr[k].tbin, arr[k].frequencies = c["tbin"], f.ctypes.data
        arr[k].dm, arr[k].width = c["dm"], c["width"]
    res = (txg_replot_result * len(cands))()
    total = sum(np.asarray(c["data"]).size for c in cands)
    mapcap = sum(int(2 ** np.ceil(np.log2(max(2, np.asarray(c["data"]).shape[0])))) *
                 np.asarray(c["data"]).shape[1] for c in cands)
    smap = np.zeros(mapcap if maps else 0, np.float32)
    dout = np.zeros(total if data else 0, np.float32)
    _check(L.txg_replot(C.byref(o), arr, len(cands), res, _ptr(smap) if maps else None, smap.size,
                        _ptr(dout) if data else None, dout.size), "replot")
    out, pm, pd = [], 0, 0
    for r in res:
        d = {k: getattr(r, k) for k, _ in txg_replot_result._fields_}
        if maps and d["ndm"] > 0:
            cnt = d["ndm"] * d["nbin"]
            d["snrmap"] = smap[pm:pm + cnt].reshape(d["ndm"], d["nbin"])
            pm += cnt
        if data:
            cnt = d["nchan"] * d["nbin"]
            d["data"] = dout[pd:pd + cnt].reshape(d["nchan"], d["nbin"])
            pd += cnt
        out.append(d)
    return out
