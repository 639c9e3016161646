"""Golden fixtures for the replot chain: the reference's own Candidate class
(src/singlepulse/candidate.cpp, compiled in place by `make -C oracle ref` against the stub
headers of oracle/refshim) run by oracle/ref_replot.cpp in the order of replot_fil
(src/singlepulse/replot_fil.cpp:409-457) on seeded candidates.

Run from the repository root where the reference tree exists:
    python tests/golden/make_golden_replot.py
Writes tests/golden/replot.npz: the candidates' inputs (integer-valued, as filterbank sums are)
and, per option set, the results, one candidate's S/N map and final data, and that
candidate's data after every step of the fullest option set.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import pyoracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
NW = 20

# option sets of replot_fil: name -> keyword arguments of pyoracle.ref_replot
CASES = {
    "default": {},
    "full": {"zdot": True, "kadane": (2, 2, 7), "clip": (2, 2, 10), "fd": 2, "zap": [(1440.0, 1452.0)]},
    "nopt": {"nopt": True},
    "pow2": {"pow2bin": True, "nwidth": 10, "snrloss": 0.2},
}


def candidates(seed=31):
    """(frequencies, tbin, dm, width, injected S/N per channel) of three candidates; nbin as
    replot_fil sizes the cut: (delay across the band + 2*nw*width)/tbin."""
    rng = np.random.default_rng(seed)
    specs = [(1500.0 - 4.0 * np.arange(32), 128e-6, 150.0, 2e-3, 6.0, None),
             (1300.0 + 3.0 * np.arange(48), 128e-6, 60.0, 1e-3, 8.0, 7),
             (1600.0 - 5.0 * np.arange(24), 64e-6, 200.0, 5e-4, 10.0, None)]
    out = []
    for f, tbin, dm, width, amp, rfi in specs:
        f = f.astype(np.float64)
        dly = abs(O.dmdelay(dm, f[0], f[-1]))
        nbin = int((dly + 2 * NW * width) / tbin)
        x = rng.normal(100.0, 10.0, (len(f), nbin))
        t0 = 0.35 * nbin * tbin
        fmax = f.max()
        for j in range(len(f)):
            i0 = int(round((t0 + O.dmdelay(dm, fmax, f[j])) / tbin)) % nbin
            wb = max(1, int(width / tbin))
            x[j, i0:i0 + wb] += amp * 10.0 / np.sqrt(wb)
        if rfi is not None:
            x[rfi] += 60.0 * np.sin(np.arange(nbin) * 0.3)
        x = np.clip(np.round(x), 0, 255).astype(np.float32)
        out.append({"data": x, "frequencies": f, "tbin": tbin, "dm": dm, "width": np.float32(width)})
    return out


def main():
    O.build(ref=True)
    cands = candidates()
    z = {}
    for k, c in enumerate(cands):
        z[f"c{k}_data"] = c["data"].astype(np.int16)
        z[f"c{k}_freqs"] = c["frequencies"]
        z[f"c{k}_meta"] = np.array([c["tbin"], c["dm"], c["width"]], np.float64)
    for name, opts in CASES.items():
        for k, c in enumerate(cands):
            r = O.ref_replot(c["data"], c["frequencies"], c["tbin"], c["dm"], float(c["width"]), **opts)
            z[f"{name}_c{k}_res"] = np.array([r["snr"], r["width"], r["dm_maxsnr"], r["mjd"],
                                              r["nbin"], r["nchan"], r["ndm"]], np.float64)
            if k == 1:
                z[f"{name}_c{k}_snrmap"] = r["snrmap"]
                z[f"{name}_c{k}_data"] = r["data"]
    for upto in range(1, 12):
        c = cands[1]
        r = O.ref_replot(c["data"], c["frequencies"], c["tbin"], c["dm"], float(c["width"]),
                         upto=upto, **CASES["full"])
        z[f"full_c1_step{upto}"] = r["data"]
    np.savez_compressed(os.path.join(OUT, "replot.npz"), **z)
    print("wrote", os.path.join(OUT, "replot.npz"))


if __name__ == "__main__":
    main()
