"""Seeded synthetic 8-bit filterbanks (time-major [t][chan] uint8) and the search workloads
they feed: Gaussian noise N(128, 12^2) clipped to 0..255, dispersed boxcar pulses, narrow-band
sinusoids and zero-DM impulses, all drawn from a seed so any block can be regenerated."""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import SinglePulse

PKG = os.path.dirname(os.path.abspath(__file__))


class _Pulse(C.Structure):
    _fields_ = [("t0", C.c_double), ("dm", C.c_double), ("width", C.c_double), ("snr", C.c_double)]


class _Sine(C.Structure):
    _fields_ = [("chan", C.c_int32), ("amp", C.c_double), ("period", C.c_double),
                ("phase", C.c_double)]


class _Imp(C.Structure):
    _fields_ = [("t0", C.c_double), ("nsamp", C.c_int64), ("amp", C.c_double)]


class _Cfg(C.Structure):
    _fields_ = [("nchan", C.c_int32), ("tsamp", C.c_double), ("freqs", C.POINTER(C.c_double)),
                ("mean", C.c_double), ("sigma", C.c_double), ("seed", C.c_uint64),
                ("npulse", C.c_int32), ("pulses", C.POINTER(_Pulse)), ("nsine", C.c_int32),
                ("sines", C.POINTER(_Sine)), ("nimp", C.c_int32), ("imps", C.POINTER(_Imp))]


_lib = None


def _synth_lib():
    global _lib
    if _lib is None:
        path = os.path.join(PKG, "libtxsynth.so")
        if not os.path.exists(path):
            from ._build import build
            build()
        _lib = C.CDLL(path)
        _lib.txs_generate.restype = C.c_int
        _lib.txs_generate.argtypes = [C.POINTER(_Cfg), C.c_int64, C.c_int64, C.c_void_p, C.c_int]
    return _lib


@dataclass
class Filterbank:
    nchans: int
    tsamp: float
    freqs: np.ndarray
    nsamples: int
    seed: int
    pulses: List[tuple] = field(default_factory=list)   # (t0 s, dm, width s, snr)
    sines: List[tuple] = field(default_factory=list)    # (chan, amp sigma, period s, phase)
    impulses: List[tuple] = field(default_factory=list)  # (t0 s, nsamp, amp sigma)
    mean: float = 128.0
    sigma: float = 12.0

    def generate(self, t0: int, n: int, out: Optional[np.ndarray] = None,
                 nthreads: int = 0) -> np.ndarray:
        """Samples [t0, t0+n) as uint8 [n][nchans]."""
        if out is None:
            out = np.empty((n, self.nchans), np.uint8)
        assert out.shape == (n, self.nchans) and out.dtype == np.uint8 and out.flags.c_contiguous
        freqs = np.ascontiguousarray(self.freqs, np.float64)
        P = (_Pulse * max(1, len(self.pulses)))(*[_Pulse(*p) for p in self.pulses])
        S = (_Sine * max(1, len(self.sines)))(*[_Sine(*s) for s in self.sines])
        I = (_Imp * max(1, len(self.impulses)))(*[_Imp(*i) for i in self.impulses])
        cfg = _Cfg(self.nchans, self.tsamp, freqs.ctypes.data_as(C.POINTER(C.c_double)),
                   self.mean, self.sigma, self.seed, len(self.pulses), P, len(self.sines), S,
                   len(self.impulses), I)
        rc = _synth_lib().txs_generate(C.byref(cfg), t0, n, out.ctypes.data, nthreads)
        if rc != 0:
            raise RuntimeError("synthetic generation failed")
        return out


def band(nchans: int, fhi: float, flo: float) -> np.ndarray:
    """Channel centres of a band [flo, fhi] in descending order (sigproc fch1/foff style)."""
    foff = -(fhi - flo) / nchans
    return fhi + foff * (np.arange(nchans) + 0.5)


def seglen_ndump(tsamp: float, tds: List[int], seglen: float = 1.0) -> int:
    """Block length of transientx_fil: (int)(seglen/tsamp)/td_lcm*td_lcm (dedisperse_fil.cpp:244)."""
    import math
    lcm = 1
    for t in tds:
        lcm = lcm * t // math.gcd(lcm, t)
    return int(int(np.float32(seglen) / tsamp) // lcm * lcm)


@dataclass
class Workload:
    name: str
    fil: Filterbank
    rows: List[SinglePulse]
    ndump: int


def nchan256_single(seed: int = 1, nsamples: int = 1 << 20) -> Workload:
    """1 beam, 256 channels, fch1 1500 MHz, foff -1 MHz, 64 us, 2^20 samples of uint8 noise with
    pulses at DM 100/350/800 (1/4/16 ms, S/N 10-30); one ddplan row DM 0-1000 step 0.5,
    16 subbands, maxw 0.05 s, thre 7, no RFI."""
    tsamp = 64e-6
    freqs = 1500.0 - np.arange(256, dtype=np.float64)
    T = nsamples * tsamp
    pulses = [(0.2 * T, 100.0, 1e-3, 10.0), (0.45 * T, 350.0, 4e-3, 20.0),
              (0.7 * T, 800.0, 16e-3, 30.0)]
    fil = Filterbank(256, tsamp, freqs, nsamples, seed, pulses=pulses)
    sp = SinglePulse(td=1, fd=1, dms=0.0, ddm=0.5, ndm=2000, snrloss=0.1, maxw=0.05, thre=7.0,
                     nsub=16, bswidth=0.1)
    return Workload("nchan256_n1M_dm1000", fil, [sp], seglen_ndump(tsamp, [1]))


def nchan4096_rfi(seed: int = 2, nsamples: int = 1 << 21) -> Workload:
    """4096 channels 856-1712 MHz, 76 us, 2^21 samples, seeded noise; 5% of channels carry
    10-30 sigma sinusoids (period 2-200 ms), zero-DM impulses (1-50 samples, 20 sigma) at a
    Poisson rate of 1/s, twelve pulses DM 50-2500, width 0.1-20 ms, S/N 8-40.  Three ddplan
    rows to DM 3000 with td 1/2/4 and rfilist kadaneF 8 4, zdot."""
    rng = np.random.default_rng(seed)
    tsamp, C_ = 76e-6, 4096
    freqs = band(C_, 1712.0, 856.0)
    T = nsamples * tsamp
    chans = rng.choice(C_, size=int(0.05 * C_), replace=False)
    sines = [(int(c), float(rng.uniform(10, 30)), float(rng.uniform(2e-3, 0.2)),
              float(rng.uniform(0, 2 * np.pi))) for c in chans]
    nimp = rng.poisson(T)
    imps = [(float(rng.uniform(0, T)), int(rng.integers(1, 51)), 20.0) for _ in range(nimp)]
    pulses = [(float(t0), float(dm), float(w), float(s)) for t0, dm, w, s in zip(
        np.sort(rng.uniform(0.05 * T, 0.9 * T, 12)), rng.uniform(50, 2500, 12),
        np.exp(rng.uniform(np.log(1e-4), np.log(2e-2), 12)), rng.uniform(8, 40, 12))]
    fil = Filterbank(C_, tsamp, freqs, nsamples, seed, pulses=pulses, sines=sines, impulses=imps)
    rfi = [["kadaneF", "8", "4"], ["zdot"]]
    rows = [
        SinglePulse(td=1, fd=1, dms=0.0, ddm=0.1, ndm=5000, snrloss=0.1, maxw=0.05, rfilist=rfi, id=1),
        SinglePulse(td=2, fd=1, dms=500.0, ddm=0.2, ndm=5000, snrloss=0.1, maxw=0.05, rfilist=rfi, id=2),
        SinglePulse(td=4, fd=1, dms=1500.0, ddm=0.5, ndm=3000, snrloss=0.1, maxw=0.05, rfilist=rfi, id=3),
    ]
    return Workload("nchan4096_n2M_rfi_dm3000", fil, rows, seglen_ndump(tsamp, [1, 2, 4]))


def nchan8192_dm5000(seed: int = 5, nsamples: int = 1 << 23) -> Workload:
    """One beam of an 8192-channel search-mode observation: 1200-1800 MHz, 16 us, 2^23 samples (134 s),
    RFI as the 4096-channel workload (5% sinusoid channels, zero-DM impulses at 1/s), bursts of
    32 us-5 ms at DM 10-5000 and S/N 8-30.  Five ddplan rows to DM 5000 with td 1/2/4/8/16,
    maxw 0.01 s, rfilist kadaneF 8 4, zdot; 1 s blocks (62496 samples at td 1)."""
    rng = np.random.default_rng(seed)
    tsamp, C_ = 16e-6, 8192
    freqs = band(C_, 1800.0, 1200.0)
    T = nsamples * tsamp
    chans = rng.choice(C_, size=int(0.05 * C_), replace=False)
    sines = [(int(c), float(rng.uniform(10, 30)), float(rng.uniform(2e-3, 0.2)),
              float(rng.uniform(0, 2 * np.pi))) for c in chans]
    nimp = rng.poisson(T)
    imps = [(float(rng.uniform(0, T)), int(rng.integers(1, 51)), 20.0) for _ in range(nimp)]
    pulses = [(float(t0), float(dm), float(w), float(s)) for t0, dm, w, s in zip(
        np.sort(rng.uniform(0.05 * T, 0.9 * T, 12)), rng.uniform(10, 5000, 12),
        np.exp(rng.uniform(np.log(32e-6), np.log(5e-3), 12)), rng.uniform(8, 30, 12))]
    fil = Filterbank(C_, tsamp, freqs, nsamples, seed, pulses=pulses, sines=sines, impulses=imps)
    rfi = [["kadaneF", "8", "4"], ["zdot"]]
    rows = [
        SinglePulse(td=1, dms=0.0, ddm=0.05, ndm=2000, maxw=0.01, rfilist=rfi, id=1),
        SinglePulse(td=2, dms=100.0, ddm=0.1, ndm=2000, maxw=0.01, rfilist=rfi, id=2),
        SinglePulse(td=4, dms=300.0, ddm=0.2, ndm=2000, maxw=0.01, rfilist=rfi, id=3),
        SinglePulse(td=8, dms=700.0, ddm=0.5, ndm=2000, maxw=0.01, rfilist=rfi, id=4),
        SinglePulse(td=16, dms=1700.0, ddm=1.0, ndm=3300, maxw=0.01, rfilist=rfi, id=5),
    ]
    return Workload("nchan8192_n8M_dm5000", fil, rows, seglen_ndump(tsamp, [1, 2, 4, 8, 16]))


@dataclass
class BeamJob:
    """Many independent beams searched with one ddplan: the beams differ in length and channel
    count; every beam has its own seeded filterbank."""
    name: str
    beams: List[Filterbank]
    rows: List[SinglePulse]
    ndump: int

    def nblocks(self, b: int) -> int:
        return self.beams[b].nsamples // self.ndump


def beams64(seed: int = 4, nbeams: int = 64) -> BeamJob:
    """64 beams of uneven length: 2^U(19,22) samples (log-uniform, seeded), 1024 or 4096
    channels (seeded coin) over 856-1712 MHz at 76 us, uint8 Gaussian noise (mean 128, sigma
    12) with 0-5 injected pulses per beam (DM 20-3000, width 0.1-30 ms log-uniform, S/N 8-50).
    Beam b uses seed + b.  The ddplan is the 4096-channel workload's (three rows to DM 3000
    with td 1/2/4, rfilist kadaneF 8 4, zdot), so both channel counts share the block length
    (13156 samples, 1 s)."""
    rng = np.random.default_rng(seed)
    tsamp = 76e-6
    lens = np.round(2.0 ** rng.uniform(19.0, 22.0, nbeams)).astype(np.int64)
    chans = np.where(rng.random(nbeams) < 0.5, 1024, 4096)
    beams = []
    for b in range(nbeams):
        T = float(lens[b]) * tsamp
        k = int(rng.integers(0, 6))
        pulses = [(float(t0), float(dm), float(w), float(sn)) for t0, dm, w, sn in zip(
            np.sort(rng.uniform(0.05 * T, 0.9 * T, k)), rng.uniform(20.0, 3000.0, k),
            np.exp(rng.uniform(np.log(1e-4), np.log(3e-2), k)), rng.uniform(8.0, 50.0, k))]
        C_ = int(chans[b])
        beams.append(Filterbank(C_, tsamp, band(C_, 1712.0, 856.0), int(lens[b]), seed + b,
                                pulses=pulses))
    rows = nchan4096_rfi(nsamples=1 << 16).rows
    return BeamJob("beams64_nchan1024_4096", beams, rows, seglen_ndump(tsamp, [1, 2, 4]))


def beams16_nchan8192(seed: int = 5, nbeams: int = 16, nsamples: int = 1 << 23) -> BeamJob:
    """16 beams of an 8192-channel search-mode observation at 16 us (1200-1800 MHz), 2^23
    samples each: the single-beam 8192-channel workload's RFI (5% sinusoid channels, zero-DM
    impulses at 1/s) and bursts (32 us-5 ms, DM 10-5000, S/N 8-30), beam b seeded seed + b;
    the five-row ddplan to DM 5000 with td 1/2/4/8/16 and maxw 0.01 s."""
    beams = [nchan8192_dm5000(seed=seed + b, nsamples=nsamples).fil for b in range(nbeams)]
    wl = nchan8192_dm5000(seed=seed, nsamples=1 << 16)
    return BeamJob("beams16_nchan8192_dm5000", beams, wl.rows, wl.ndump)


def replot_candidates(n: int, nchan: int = 4096, seed: int = 9, dm: float = 500.0,
                      width: float = 2e-3, tbin: float = 76e-6, nwidth: int = 20):
    """Candidates as replot_fil cuts them (replot_fil.cpp:300-306): nbin = (delay across the
    band + 2*nw*width)/tbin samples of integer-valued noise of 4096 channels 1712-856 MHz with
    a dispersed pulse, one dict per candidate for transientx_gb300.replot."""
    f = band(nchan, 1712.0, 856.0)
    k = 4.148741601e3
    dly = k * dm * (1.0 / f.min() ** 2 - 1.0 / f.max() ** 2)
    nbin = int((dly + 2 * nwidth * width) / tbin)
    wb = max(1, int(width / tbin))
    out = []
    for c in range(n):
        rng = np.random.default_rng(seed + c)
        x = np.round(rng.normal(100.0, 10.0, (nchan, nbin))).astype(np.float32)
        t0 = 0.4 * nbin * tbin
        for j in range(nchan):
            i0 = int((t0 + k * dm * (1.0 / f[j] ** 2 - 1.0 / f.max() ** 2)) / tbin) % nbin
            x[j, i0:i0 + wb] += 3.0
        out.append({"data": x, "frequencies": f, "tbin": tbin, "dm": dm, "width": width})
    return out


WORKLOADS = {"nchan256_n1M_dm1000": nchan256_single, "nchan4096_n2M_rfi_dm3000": nchan4096_rfi,
             "nchan8192_n8M_dm5000": nchan8192_dm5000}
# workloads of many beams (BeamJob)
JOBS = {"beams64_nchan1024_4096": beams64, "beams16_nchan8192_dm5000": beams16_nchan8192}
