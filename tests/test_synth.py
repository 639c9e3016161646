"""Synthetic filterbank generator: determinism, noise statistics, injections."""
import numpy as np

from transientx_gb300 import synth


def test_deterministic_and_blockwise():
    w = synth.nchan256_single(nsamples=1 << 14)
    a = w.fil.generate(0, 4096)
    b = w.fil.generate(0, 4096)
    np.testing.assert_array_equal(a, b)
    c = w.fil.generate(1000, 500)
    np.testing.assert_array_equal(a[1000:1500], c)


def test_noise_statistics():
    fil = synth.Filterbank(64, 1e-4, 1500.0 - np.arange(64.0), 1 << 15, seed=9)
    x = fil.generate(0, 1 << 15).astype(np.float64)
    assert abs(x.mean() - 128.0) < 0.05
    assert abs(x.std() - np.sqrt(144 + 1 / 12)) < 0.1


def test_pulse_is_dispersed():
    f = 1500.0 - np.arange(256.0)
    fil = synth.Filterbank(256, 64e-6, f, 1 << 14, seed=3, pulses=[(0.2, 300.0, 2e-3, 200.0)])
    quiet = synth.Filterbank(256, 64e-6, f, 1 << 14, seed=3)
    d = fil.generate(0, 1 << 14).astype(int) - quiet.generate(0, 1 << 14).astype(int)
    t_hi = np.argmax(d[:, 0].cumsum() > 0)
    t_lo = np.argmax(d[:, 255].cumsum() > 0)
    delay = 4.148741601e3 * 300 * (1 / f[255] ** 2 - 1 / f[0] ** 2) / 64e-6
    assert abs((t_lo - t_hi) - delay) < 3


def test_seglen_ndump():
    assert synth.seglen_ndump(76e-6, [1, 2, 4]) == 13156
    assert synth.seglen_ndump(64e-6, [1]) == 15625
