"""The oracle's main-path zdot, kadaneF and downsample (oracle/txoracle.c, the restatements the
GPU kernels equal bit for bit) against the reference's own Candidate::zdot, Candidate::kadaneF
and Candidate::downsample (src/singlepulse/candidate.cpp:381-427, 710-897, compiled in place
with oracle/ref_rfi.cpp), the in-tree code the main path's XLibs RFI::zdot / RFI::kadaneF /
Downsample are restated from.  Both sides use the project's kadane<float>
(oracle/refshim/utils.h: XLibs' version is not in the tree).  Downsample: bit-exact, samples
and averaged frequencies.

kadaneF: bit-exact on the normalised block Candidate::kadaneF sees, with the main path's
squared threshold and the window limit Candidate computes.  zdot: the oracle folds its sums
in FP32 runs of 32 with FP64 accumulators (the GPU's order) where Candidate adds sequentially
in FP64, so values agree within 2e-5 of the block's largest magnitude (observed: 5e-7)."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def ref(oracle):
    if not oracle.ref_available("scalar"):
        pytest.skip("reference tree not present")
    return oracle


def _block(C, n, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(3.0, 2.0, (C, n)).astype(np.float32)
    x[min(5, C - 1)] = 7.0                                # a constant channel (std 0 -> 1)
    x[:, n // 10:n // 10 + 10] += 5.0                     # a broadband burst
    x[:: max(1, C // 8), :] += np.float32(2.0) * np.sin(np.arange(n) / 9.0).astype(np.float32)
    return x


@pytest.mark.parametrize("C,n,seed", [(64, 1000, 1), (128, 4096, 2), (33, 517, 3), (1, 64, 4)])
def test_zdot_follows_candidate_zdot(ref, C, n, seed):
    x = _block(C, n, seed)
    a = ref.ref_zdot(x)
    b = ref.zdot(x)
    scale = max(1.0, float(np.abs(a).max()))
    assert float(np.abs(a - b).max()) <= 2e-5 * scale


@pytest.mark.parametrize("td,fd,thr,nwidth,width,tbin", [(8, 4, 7.0, 2, 0.004, 0.001),
                                                        (1, 1, 5.0, 1, 0.01, 0.001),
                                                        (4, 1, 6.0, 3, 0.002, 0.0005),
                                                        (2, 8, 4.0, 1, 0.0015, 0.00025)])
@pytest.mark.parametrize("C,n,seed", [(64, 1000, 1), (128, 4096, 2), (40, 517, 3)])
def test_kadaneF_equals_candidate_kadaneF(ref, C, n, seed, td, fd, thr, nwidth, width, tbin):
    rng = np.random.default_rng(seed)
    y = rng.normal(0.0, 1.0, (C, n)).astype(np.float32)
    y[3, n // 5:n // 5 + n // 8] += 2.0                   # a long positive excursion
    y[7, n // 20:n // 20 + 40] -= 3.0                     # a negative one
    y[8:16, n // 2:n // 2 + 100] += 1.5                   # several channels at once
    pre, want = ref.ref_kadaneF(y, td, fd, thr, nwidth, width, tbin)
    # Candidate::kadaneF's limit (candidate.cpp:748): int(nwidth*width / tbin / td), the product
    # in float, the divisions in double
    wnlimit = int(float(np.float32(nwidth * np.float32(width))) / tbin / td)
    got, ranges = ref.kadaneF(pre, td, fd, np.float32(thr) * np.float32(thr), wnlimit)
    np.testing.assert_array_equal(got, want)
    assert (ranges[:, ::2] >= 0).any(), "the planted excursions should be zapped"
    assert not np.array_equal(want, pre)


@pytest.mark.parametrize("C,n0,td,fd", [(64, 1000, 1, 1), (64, 1000, 2, 1), (128, 4096, 4, 2),
                                        (33, 517, 3, 4), (256, 2048, 16, 8)])
def test_downsample_equals_candidate_downsample(ref, C, n0, td, fd):
    """The unpack + sum-downsample of the oracle (time-major uint8 in, channel-major float out)
    and its frequency averaging against Candidate::downsample on the same samples."""
    rng = np.random.default_rng(C + n0 + td)
    raw = np.clip(np.round(rng.normal(128, 20, (n0, C))), 0, 255).astype(np.uint8)
    freqs = 1500.0 - np.arange(C) * 0.390625 + rng.uniform(-1e-3, 1e-3, C)
    want, fwant = ref.ref_downsample(raw.T.astype(np.float32), freqs, td, fd)
    got = ref.unpack_downsample(raw, td, fd)
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(ref.downsample_freqs(freqs, fd), fwant)


def test_dmdelay_equals_candidate_dmdelay(ref):
    """The oracle's dispersion delay against Candidate::dmdelay, bit for bit (the product's
    delay tables equal the oracle's, tests/test_host.py)."""
    rng = np.random.default_rng(9)
    L = ref.ref_lib("scalar")
    for _ in range(200):
        dm = float(rng.uniform(0, 5000))
        fl, fh = sorted(rng.uniform(100, 3000, 2))
        want = L.ref_dmdelay(dm, fh, fl)
        assert ref.dmdelay(dm, fh, fl) == want


def test_zdot_degenerate_blocks(ref):
    """Constant channels (std 0 -> 1, candidate.cpp:850) everywhere make the zero-DM series 0
    and the fit's determinant 0 (no fit, candidate.cpp:886); one channel makes the series the
    channel itself."""
    flat = np.tile(np.arange(8, dtype=np.float32)[:, None] * 3.0, (1, 100))
    np.testing.assert_array_equal(ref.zdot(flat), ref.ref_zdot(flat))
    one = np.random.default_rng(2).normal(0, 1, (1, 333)).astype(np.float32)
    a, b = ref.ref_zdot(one), ref.zdot(one)
    assert float(np.abs(a - b).max()) <= 2e-5 * max(1.0, float(np.abs(a).max()))
