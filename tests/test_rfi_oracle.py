"""The oracle's mask, kadaneT and zero RFI entries (their XLibs sources are not in the
reference tree; the definitions are restated in oracle/txoracle.c): properties on planted
outliers, a broadband burst and dead channels."""
import numpy as np


def _noise(C=64, N=2048, seed=0):
    return np.random.default_rng(seed).standard_normal((C, N)).astype(np.float32)


def _seq_ds(x, tdk, fdk):
    """Sum-downsample in the oracle's order (fd outer, td inner, float32 from 0)."""
    C, N = x.shape
    cds, nds = C // fdk, N // tdk
    d = np.zeros((cds, nds), np.float32)
    for k in range(fdk):
        for t in range(tdk):
            d += x[k:cds * fdk:fdk, t:nds * tdk:tdk]
    return d


def test_mask_quartiles_and_zapped_cells(oracle):
    x = _noise()
    x[10:12, 400:404] += 30.0
    x[40:42, 1000:1004] -= 30.0
    y, nz, q = oracle.mask(x, 4, 2, 3.0)
    d = _seq_ds(x, 4, 2)
    s = np.sort(d.ravel())
    n = s.size
    assert q[0] == s[n // 4] and q[1] == s[n - 1 - n // 4]
    r = np.float32(q[1] - q[0])
    assert q[2] == np.float32(q[0] - np.float32(3.0) * r)
    assert q[3] == np.float32(q[1] + np.float32(3.0) * r)
    out = (d < q[2]) | (d > q[3])
    assert nz == out.sum() and nz >= 2
    zapped = np.repeat(np.repeat(out, 2, axis=0), 4, axis=1)
    np.testing.assert_array_equal(y[zapped], 0.0)
    np.testing.assert_array_equal(y[~zapped], x[~zapped])
    assert (y[10:12, 400:404] == 0).all() and (y[40:42, 1000:1004] == 0).all()


def test_mask_high_threshold_zaps_nothing(oracle):
    x = _noise(seed=1)
    y, nz, _ = oracle.mask(x, 2, 2, 1e6)
    assert nz == 0
    np.testing.assert_array_equal(y, x)


def test_kadaneT_zaps_broadband_burst_only(oracle):
    x = _noise(seed=2)
    x[8:56, 700:704] += 3.0
    y, r, n = oracle.kadaneT(x, 4, 2, 49.0, 10)
    assert r[175, 0] >= 0 and r[175, 0] <= 8 and r[175, 1] >= 56
    assert (y[r[175, 0]:r[175, 1], 700:704] == 0).all()
    # nothing else clears the threshold on pure noise
    assert n == int((r[:, 0] >= 0).sum() + (r[:, 2] >= 0).sum())
    assert (r[:, 0] >= 0).sum() <= 2


def test_kadaneT_band_limit_blocks_narrow_bands(oracle):
    x = _noise(seed=3)
    x[20:24, 300:304] += 20.0   # bright, 2 downsampled channels (the best band grows a little)
    _, r, _ = oracle.kadaneT(x, 4, 2, 49.0, 1)
    wn = (r[75, 1] - r[75, 0]) // 2
    assert r[75, 0] >= 0 and wn < 16
    _, r2, _ = oracle.kadaneT(x, 4, 2, 49.0, wn)   # band must be wider than the limit
    assert r2[75, 0] < 0


def test_zero_removes_the_live_channel_mean(oracle):
    x = _noise(seed=4)
    live = np.ones(x.shape[0], np.uint8)
    live[[5, 17]] = 0
    x[[5, 17]] = 0.0
    z = oracle.zero(x, live)
    assert np.abs(z[live == 1].mean(axis=0)).max() < 1e-6
    np.testing.assert_array_equal(z[[5, 17]], 0.0)
    # a one-sample baseline is the same filter
    np.testing.assert_array_equal(z, oracle.baseline(x, 1, live))
