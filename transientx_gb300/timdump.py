"""Dedispersed-series dump (--savetim, --format, --nbits, --mean, --std of transientx_fil:
dedisperse_fil.cpp:95-99, singlepulse.cpp:228,237-238,339-340): one file per DM trial, appended
block by block with the non-overlapping ndump samples of each gated block.

Formats: ``sigproc`` (a SIGPROC time-series header, data_type 2, then nbits 8/16/32 samples)
and ``presto`` (32-bit float .dat plus the .inf text description written at close; the
reference forces 32 bits for presto, singlepulse.cpp:228).  The reference's default
``pulsarx`` layout is defined in XLibs, whose source is not in the reference tree, and is not
written here.  Quantisation follows ``Search.timdata_q``: each block's series standardised by
its own mean and standard deviation, then z*std + mean.
"""
import os
import struct
from typing import List, Optional

import numpy as np


def _kw(f, key: str) -> None:
    b = key.encode()
    f.write(struct.pack("<i", len(b)) + b)


def _kv(f, key: str, value, kind: str) -> None:
    _kw(f, key)
    if kind == "s":
        b = str(value).encode()
        f.write(struct.pack("<i", len(b)) + b)
    elif kind == "i":
        f.write(struct.pack("<i", int(value)))
    else:
        f.write(struct.pack("<d", float(value)))


def write_sigproc_header(f, source_name: str, refdm: float, fch1: float, nbits: int,
                         tstart: float, tsamp: float, rawdatafile: str = "") -> None:
    _kw(f, "HEADER_START")
    _kv(f, "rawdatafile", rawdatafile, "s")
    _kv(f, "source_name", source_name, "s")
    _kv(f, "data_type", 2, "i")
    _kv(f, "refdm", refdm, "d")
    _kv(f, "fch1", fch1, "d")
    _kv(f, "nchans", 1, "i")
    _kv(f, "nbits", nbits, "i")
    _kv(f, "nifs", 1, "i")
    _kv(f, "tstart", tstart, "d")
    _kv(f, "tsamp", tsamp, "d")
    _kw(f, "HEADER_END")


def read_sigproc_header(path: str):
    """Keywords of a SIGPROC header written by this module and the offset of its data."""
    ints = {"data_type", "nchans", "nbits", "nifs"}
    strs = {"rawdatafile", "source_name"}
    out = {}
    with open(path, "rb") as f:
        def word():
            n = struct.unpack("<i", f.read(4))[0]
            return f.read(n).decode()
        assert word() == "HEADER_START"
        while True:
            k = word()
            if k == "HEADER_END":
                break
            if k in strs:
                out[k] = word()
            elif k in ints:
                out[k] = struct.unpack("<i", f.read(4))[0]
            else:
                out[k] = struct.unpack("<d", f.read(8))[0]
        out["data_offset"] = f.tell()
    return out


class TimDumper:
    """One ddplan row's dedispersed series, DMs idm0..idm0+count-1, into
    ``<rootname>_DM<dm>.tim`` (sigproc) or ``.dat``/``.inf`` (presto)."""

    def __init__(self, rootname: str, info, idm0: int = 0, count: Optional[int] = None,
                 fmt: str = "sigproc", nbits: int = 8, mean: float = 0.0, std: float = 3.0,
                 tstart: float = 0.0, source_name: str = "", fch1: float = 0.0,
                 freqs: Optional[np.ndarray] = None):
        if fmt not in ("sigproc", "presto"):
            raise ValueError("formats: sigproc, presto (the pulsarx layout is not available)")
        self.fmt = fmt
        self.nbits = 32 if fmt == "presto" else nbits
        self.mean, self.std = mean, std
        self.info = info
        self.idm0 = idm0
        self.count = info.ndm - idm0 if count is None else count
        self.tstart, self.source_name, self.fch1 = tstart, source_name, fch1
        self.freqs = None if freqs is None else np.asarray(freqs, np.float64)
        self.nwritten = 0
        self.paths: List[str] = []
        self.files = []
        for k in range(self.count):
            dm = info.dms + (idm0 + k) * info.ddm
            base = f"{rootname}_DM{dm:.2f}"
            path = base + (".tim" if fmt == "sigproc" else ".dat")
            f = open(path, "wb")
            if fmt == "sigproc":
                write_sigproc_header(f, source_name, dm, fch1, self.nbits, tstart, info.tsamp)
            self.paths.append(path)
            self.files.append(f)

    def push(self, search, row: int, beam: int = 0) -> bool:
        """Append the last block of (beam, row) if it produced output; returns whether it did."""
        if not search.row_info(row, beam).gated:
            return False
        q = search.timdata_q(row, beam, self.idm0, self.count, nsamp=self.info.ndump,
                             nbits=self.nbits, mean=self.mean, std=self.std)
        for k, f in enumerate(self.files):
            f.write(q[k].tobytes())
        self.nwritten += q.shape[1]
        return True

    def close(self) -> None:
        for f in self.files:
            f.close()
        if self.fmt == "presto":
            for k, path in enumerate(self.paths):
                self._write_inf(path[:-4], self.info.dms + (self.idm0 + k) * self.info.ddm)
        self.files = []

    def _write_inf(self, base: str, dm: float) -> None:
        """PRESTO's .inf description of a .dat time series."""
        f = self.freqs
        lo = float(f.min()) if f is not None else 0.0
        nch = len(f) if f is not None else 1
        chbw = float(abs(f[1] - f[0])) if f is not None and len(f) > 1 else 0.0
        lines = [
            ("Data file name without suffix", os.path.basename(base)),
            ("Telescope used", "unknown"),
            ("Instrument used", "unknown"),
            ("Object being observed", self.source_name or "unknown"),
            ("J2000 Right Ascension (hh:mm:ss.ssss)", "00:00:00.0000"),
            ("J2000 Declination     (dd:mm:ss.ssss)", "00:00:00.0000"),
            ("Data observed by", "unknown"),
            ("Epoch of observation (MJD)", "%.15f" % self.tstart),
            ("Barycentered?           (1=yes, 0=no)", "0"),
            ("Number of bins in the time series", "%d" % self.nwritten),
            ("Width of each time series bin (sec)", "%.15g" % self.info.tsamp),
            ("Any breaks in the data? (1=yes, 0=no)", "0"),
            ("Type of observation (EM band)", "Radio"),
            ("Beam diameter (arcsec)", "0"),
            ("Dispersion measure (cm-3 pc)", "%.12g" % dm),
            ("Central freq of low channel (Mhz)", "%.12g" % lo),
            ("Total bandwidth (Mhz)", "%.12g" % (chbw * nch)),
            ("Number of channels", "%d" % nch),
            ("Channel bandwidth (Mhz)", "%.12g" % chbw),
            ("Data analyzed by", "transientx_gb300"),
        ]
        with open(base + ".inf", "w") as out:
            for k, v in lines:
                out.write(" %-39s=  %s\n" % (k, v))
            out.write(" Any additional notes:\n    dedispersed time series\n\n")

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
