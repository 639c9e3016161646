"""The .cands output of transientx_fil: CandPlot::plot (src/singlepulse/candplot.cpp:32-433)
appends one line per reported candidate of a block to ``<rootname>_<tstart>_<beam>.cands``.

Per line (candplot.cpp:423-433), tab-separated: beam, running candidate number, MJD of the
candidate (15 decimals), DM (2), width in ms (2), S/N (1), fl and fh in MHz (0), the name of
the candidate plot (``<rootname>_<block MJD>_<beam>_<kk>_<id>.png``, kk = rank of the
candidate in the block by S/N), the ddplan row id (two digits) and the input file name.
Candidates of a block are taken in descending S/N, ties in candidate-list order (the stable
argsort of candplot.h:27-35).  The plot itself is not produced by this library.
"""
from typing import List, Optional, Sequence

import numpy as np

from . import CAND_DTYPE


class CandsWriter:
    """Formats (and optionally appends) the .cands lines of one beam of one observation.

    ``tstart`` is the observation start MJD; ``beam`` the beam label (obsinfo "Beam");
    ``fname`` the input file name written in the last column.  The running number continues
    across blocks and rows, like CandPlot::num_cand."""

    def __init__(self, rootname: str, tstart: float, beam: str = "0", fname: str = "",
                 path: Optional[str] = None):
        self.rootname, self.tstart, self.beam, self.fname = rootname, float(tstart), str(beam), fname
        self.num_cand = 0
        self.path = path

    @property
    def filename(self) -> str:
        """``<rootname>_<tstart, 10 decimals>_<beam>.cands`` (candplot.cpp:420)."""
        return f"{self.rootname}_{self.tstart:.10f}_{self.beam}.cands"

    def format_block(self, clusters: np.ndarray, counter: int, offset: int, ndump: int,
                     tsamp: float, dms: float, ddm: float, fl: Sequence[float],
                     fh: Sequence[float], row_id: int) -> List[str]:
        """Lines for the reported candidates ``clusters`` (idm, isamp, wn, S) of one block of a
        row whose Boxcar counter is ``counter`` (row geometry: offset, ndump after td, tsamp
        after td, dms, ddm); fl/fh per candidate from ``Search.cand_band``."""
        c = np.asarray(clusters, CAND_DTYPE)
        order = sorted(range(len(c)), key=lambda k: -float(c["S"][k]))  # stable: ties keep order
        s_id = f"{row_id:02d}"
        bmjd = self.tstart + (-offset + counter - ndump) * tsamp / 86400.0
        lines = []
        for iidx, k in enumerate(order):
            idm, isamp, wn = int(c["idm"][k]), int(c["isamp"][k]), int(c["wn"][k])
            snr = float(np.float32(c["S"][k]))
            mjd = self.tstart + (-offset + counter - ndump + isamp) * tsamp / 86400.0
            basename = f"{self.rootname}_{bmjd:.10f}_{self.beam}_{iidx + 1:02d}_{s_id}"
            self.num_cand += 1
            lines.append(f"{self.beam}\t{self.num_cand}\t{mjd:.15f}\t{dms + idm * ddm:.2f}\t"
                         f"{wn * tsamp * 1000:.2f}\t{snr:.1f}\t{float(fl[k]):.0f}\t"
                         f"{float(fh[k]):.0f}\t{basename}.png\t{s_id}\t{self.fname}\n")
        return lines

    def block(self, search, row: int, clusters: np.ndarray, row_id: int, beam: int = 0) -> List[str]:
        """Lines for one block straight from a ``Search`` after ``sync`` (the row's last
        block), appended to the file when the writer has a ``path`` directory."""
        if len(clusters) == 0:
            return []
        info = search.row_info(row, beam)
        fl, fh = search.cand_band(clusters, row, beam)
        lines = self.format_block(clusters, info.counter, info.offset, info.ndump, info.tsamp,
                                  info.dms, info.ddm, fl, fh, row_id)
        if self.path is not None:
            import os
            with open(os.path.join(self.path, self.filename), "a") as f:
                f.writelines(lines)
        return lines
