"""Generate golden fixtures by running the reference's own Boxcar (src/singlepulse/boxcar.cpp)
and Cluster<double> (src/singlepulse/cluster.cpp), compiled in place from the reference tree
by oracle/Makefile (`make -C oracle ref`), on seeded inputs.

Run from the repository root where the reference tree exists (TXREF_TREE names it when it is
not at its usual mount point):
    python tests/golden/make_golden.py
Writes tests/golden/boxcar.npz and tests/golden/cluster.npz.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import pyoracle as O  # noqa: E402
from __graft_entry__ import reference_tree  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def boxcar_inputs(seed=11, ndm=8, n=1500):
    rng = np.random.default_rng(seed)
    tim = rng.normal(3.0, 30.0, (ndm, n)).astype(np.float32)
    tim[1, :] = 7.0                                   # var == 0: boxcar.cpp:242 skips the row
    tim[2, 600:640] += 120.0                          # a wide pulse
    tim[3, 100] += 400.0                              # a one-sample spike
    tim[4] = np.round(tim[4] / 10.0) * 10.0           # many equal values: IQR ties, width ties
    tim[5, -3:] += 300.0                              # signal in the AVX2 tail region
    tim[6] *= 1e-3                                    # small magnitudes
    tim[7, 200:1300] += np.linspace(0, 50, 1100, dtype=np.float32)  # slow drift
    vwn = O.width_ladder(1e-4, 0.05, 0.1, 64e-6)
    vwn = vwn[vwn < n // 2].astype(np.int32)
    return tim, vwn


def main():
    O.build(ref=True, tree=reference_tree())
    assert O.ref_available("scalar"), "reference harness not built (set TXREF_TREE to the reference tree)"
    tim, vwn = boxcar_inputs()
    out = {"tim": tim, "vwn": vwn}
    variants = ["scalar"] + (["avx2"] if O.ref_available("avx2") else [])
    for var in variants:
        for iqr in (0, 1):
            S, W = O.ref_boxcar_run(tim, vwn, iqr=bool(iqr), variant=var)
            out[f"mxS_{var}_iqr{iqr}"] = S
            out[f"mxwn_{var}_iqr{iqr}"] = W
    np.savez_compressed(os.path.join(OUT, "boxcar.npz"), **out)

    rng = np.random.default_rng(12)
    cases = []
    for c in range(16):
        ndm, n = 48, 2500
        mxS = np.abs(rng.normal(0, 2.5, (ndm, n))).astype(np.float32)
        for _ in range(int(rng.integers(2, 14))):
            j, i = int(rng.integers(0, ndm)), int(rng.integers(0, n))
            mxS[max(0, j - 4):j + 4, max(0, i - 25):i + 25] += np.float32(rng.uniform(4, 25))
        mxwn = rng.integers(1, 60, (ndm, n)).astype(np.int32)
        p = dict(dms=float(rng.choice([0.0, 12.5])), ddm=float(rng.choice([0.1, 0.5])),
                 tsamp=float(rng.choice([64e-6, 1e-4])), fmin=1200.0, fmax=1500.0, maxwn=59,
                 thre=7.0, radius=float(rng.choice([0.0, 1e-3, 4e-3])), kvalue=2,
                 maxncand=int(rng.choice([1, 5, 20, 100])), minpts=int(rng.choice([0, 5, 50, 400])),
                 drop=bool(c % 3 == 0))
        mxwn[mxS > 20] = 59                           # some maximum-width points for --drop
        res = O.ref_cluster_run(mxS, mxwn, **p)
        cases.append((mxS, mxwn, p, res))
    arrs = {}
    for k, (mxS, mxwn, p, res) in enumerate(cases):
        # clustering only consumes the row-major S > thre points (cluster.cpp:91-112)
        arrs[f"c{k}_points"] = O.threshold_scan(mxS, mxwn, p["thre"])
        arrs[f"c{k}_params"] = np.array([p["dms"], p["ddm"], p["tsamp"], p["fmin"], p["fmax"],
                                         p["maxwn"], p["thre"], p["radius"], p["kvalue"],
                                         p["maxncand"], p["minpts"], int(p["drop"])], np.float64)
        arrs[f"c{k}_out"] = res
    arrs["ncase"] = np.array(len(cases))
    np.savez_compressed(os.path.join(OUT, "cluster.npz"), **arrs)
    print("wrote", os.path.join(OUT, "boxcar.npz"), os.path.join(OUT, "cluster.npz"))


if __name__ == "__main__":
    main()
