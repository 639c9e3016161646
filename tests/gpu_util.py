"""Comparison helpers shared by the GPU parity tests."""
import numpy as np

REL = 1e-4  # S/N agreement bound for the FP32 path (relative, floor 1)


def width_scores(tim, vwn, mean, var):
    """S for every width at every sample, in float64, from one series (boxcar.cpp:244-262)."""
    n = len(tim)
    c = np.cumsum(tim.astype(np.float64) - mean)
    out = np.full((len(vwn), n), -np.inf)
    for k, wn in enumerate(vwn):
        wl, wh = wn // 2 + 1, (wn - 1) // 2
        i = np.arange(wl, n - wh)
        out[k, i] = (c[i + wh] - c[i - wl]) / np.sqrt(wn * var)
    return out


def row_stats(t, iqr):
    """mean and variance as Boxcar::match forms them (boxcar.cpp:204-227)."""
    if not iqr:
        return t.mean(), t.var()
    s = np.sort(t.astype(np.float32))
    n = len(s)
    q1, q2, q3 = s[n // 4], s[n // 2], s[n - 1 - n // 4]
    return float(q2), (float(q3 - q1) / 1.349) ** 2


def assert_boxcar_close(tim, vwn, S_gpu, W_gpu, S_ref, W_ref, rel=REL, iqr=False):
    """S within rel*max(1,|S|); widths equal except where the two widths' scores tie within
    that bound."""
    tol = rel * np.maximum(1.0, np.abs(S_ref))
    bad = np.abs(S_gpu - S_ref) > tol
    assert not bad.any(), f"{bad.sum()} S values differ, worst {np.abs(S_gpu - S_ref)[bad].max()}"
    diff = W_gpu != W_ref
    if diff.any():
        rows = np.unique(np.nonzero(diff)[0])
        for r in rows:
            t = tim[r].astype(np.float64)
            sc = width_scores(t, vwn, *row_stats(t, iqr))
            idx = np.nonzero(diff[r])[0]
            lut = {int(w): k for k, w in enumerate(vwn)}
            for i in idx:
                a, b = int(W_gpu[r, i]), int(W_ref[r, i])
                sa = sc[lut[a], i] if a in lut else 0.0
                sb = sc[lut[b], i] if b in lut else 0.0
                assert abs(sa - sb) <= 2 * rel * max(1.0, abs(S_ref[r, i])), \
                    f"row {r} sample {i}: width {a} vs {b} ({sa} vs {sb})"


def assert_cands_close(c_gpu, c_ref, thre, rel=REL):
    """Same (idm, isamp) sets except points whose S lies within rel (relative) of the
    threshold in either list; S of the common points within rel*max(1,|S|)."""
    a = {(int(x["idm"]), int(x["isamp"])): float(x["S"]) for x in c_gpu}
    b = {(int(x["idm"]), int(x["isamp"])): float(x["S"]) for x in c_ref}
    band = rel * max(1.0, thre)
    for k in set(a) ^ set(b):
        s = a.get(k, b.get(k))
        assert abs(s - thre) <= band, f"point {k} S={s} not within {rel} of the threshold"
    for k in set(a) & set(b):
        assert abs(a[k] - b[k]) <= rel * max(1.0, abs(b[k])), f"point {k}: S {a[k]} vs {b[k]}"
    # the reported order is row-major (Cluster::run scan order)
    keys = [(int(x["idm"]), int(x["isamp"])) for x in c_gpu]
    assert keys == sorted(keys)
