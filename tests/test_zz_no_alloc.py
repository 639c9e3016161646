"""txg_kadaneF_noalloc, the entry point for callers that cannot allocate device memory while
they run (real-time back ends with all memory reserved at start-up, frameworks that own the
GPU memory): it must give exactly what the allocating pipeline gives for the same kadaneF
entry, on two calls in a row that share its fixed scratch array.  This file is collected
last so a failure here cannot hide failures of the other tests."""
import ctypes

import numpy as np
import pytest

# (ldx, nchans, nsamples, td, fd): inputs the entry point must refuse before queuing anything:
# downsampled channels past the 65535 grid rows, fewer channels than fd, more samples than the
# int32 zap ranges hold, and more downsampled samples than the fixed scratch
BAD_ARGS = [
    (16, 65536, 16, 8, 1),
    (64, 3, 64, 8, 4),
    (1 << 31, 1, 1 << 31, 1 << 11, 1),
    (1 << 22, 4096, 1 << 22, 1, 1),
]


def test_kadane_noalloc_rejects_bad_sizes_before_touching_the_device(tx):
    """The size checks return TXG_ERR_ARG before any CUDA call: they hold on a host without a
    GPU, so on a GPU nothing can have been launched for these inputs."""
    L = tx.load_library()
    for ldx, C, N, td, fd in BAD_ARGS:
        rc = L.txg_kadaneF_noalloc(ctypes.c_void_p(16), ldx, C, N, td, fd, 1.0, 1,
                                   ctypes.c_void_p(16), None)
        assert rc == tx.ERR_ARG, (ldx, C, N, td, fd)


def _workload():
    from transientx_gb300 import SinglePulse, synth
    tsamp, C, ndump = 256e-6, 128, 4096
    f = synth.band(C, 1500.0, 1200.0)
    rng = np.random.default_rng(33)
    sines = [(int(c), float(rng.uniform(10, 30)), float(rng.uniform(0.05, 0.3)), 0.7)
             for c in rng.choice(C, 8, replace=False)]
    fil = synth.Filterbank(C, tsamp, f, 3 * ndump, 33, sines=sines,
                           pulses=[(0.5, 100.0, 2e-3, 30.0)])
    base = dict(td=1, fd=1, dms=0.0, ddm=1.0, ndm=64, maxw=0.02, nsub=8, widthlimit=0.02,
                bswidth=0.1)
    plain = SinglePulse(rfilist=[], **base)
    kad = SinglePulse(rfilist=[["kadaneF", "8", "4"]], **base)
    return fil, plain, kad, ndump


@pytest.mark.gpu
def test_kadane_noalloc_matches_pipeline(tx):
    cudart = ctypes.CDLL("libcudart.so")
    L = tx.load_library()
    fil, plain, kad, ndump = _workload()
    C = fil.nchans
    td, fd = 8, 4
    thr2 = float(np.float32(kad.threKadaneF) * np.float32(kad.threKadaneF))
    wnlimit = int(kad.widthlimit / (fil.tsamp * td))
    flags = tx.FLAG_KEEP_SERIES
    dx, dr = ctypes.c_void_p(), ctypes.c_void_p()
    nbytes = C * ndump * 4
    rbytes = (C // fd) * 4 * 4
    assert cudart.cudaMalloc(ctypes.byref(dx), ctypes.c_size_t(nbytes)) == 0
    assert cudart.cudaMalloc(ctypes.byref(dr), ctypes.c_size_t(rbytes)) == 0
    try:
        with tx.Search([plain], C, fil.tsamp, fil.freqs, ndump, flags=flags, zapthre=0.0) as a, \
                tx.Search([kad], C, fil.tsamp, fil.freqs, ndump, flags=flags, zapthre=0.0) as b:
            fired = 0
            for blk in range(2):  # two calls in a row through the shared scratch
                raw = fil.generate(blk * ndump, ndump)
                a.push_block(raw)
                b.push_block(raw)
                a.sync()
                b.sync()
                x_in = np.ascontiguousarray(a.block(0))       # block before kadaneF
                x_ref, r_ref = b.block(0), b.zap_ranges(0)     # the pipeline's kadaneF
                assert cudart.cudaMemcpy(dx, x_in.ctypes.data, ctypes.c_size_t(nbytes), 1) == 0
                assert cudart.cudaMemset(dr, 0x7f, ctypes.c_size_t(rbytes)) == 0
                rc = L.txg_kadaneF_noalloc(dx, ndump, C, ndump, td, fd, thr2, wnlimit, dr, None)
                assert rc == 0, L.txg_strerror(rc)
                assert cudart.cudaDeviceSynchronize() == 0
                x_out = np.empty_like(x_in)
                r_out = np.empty_like(r_ref)
                assert cudart.cudaMemcpy(x_out.ctypes.data, dx, ctypes.c_size_t(nbytes), 2) == 0
                assert cudart.cudaMemcpy(r_out.ctypes.data, dr, ctypes.c_size_t(rbytes), 2) == 0
                np.testing.assert_array_equal(r_out, r_ref)
                np.testing.assert_array_equal(x_out, x_ref)
                fired += int((r_ref[:, 0] >= 0).sum() + (r_ref[:, 2] >= 0).sum())
            assert fired > 0, "the sinusoid channels should trigger kadaneF"
        # refused sizes (proved on the host by the test above) leave x and ranges untouched
        x_keep = np.empty(C * ndump, np.float32)
        r_keep = np.empty((C // fd) * 4, np.int32)
        assert cudart.cudaMemcpy(x_keep.ctypes.data, dx, ctypes.c_size_t(nbytes), 2) == 0
        assert cudart.cudaMemcpy(r_keep.ctypes.data, dr, ctypes.c_size_t(rbytes), 2) == 0
        for ldx, nc, ns, tdb, fdb in BAD_ARGS:
            rc = L.txg_kadaneF_noalloc(dx, ldx, nc, ns, tdb, fdb, thr2, wnlimit, dr, None)
            assert rc == tx.ERR_ARG, (ldx, nc, ns, tdb, fdb)
        assert cudart.cudaDeviceSynchronize() == 0
        x_now, r_now = np.empty_like(x_keep), np.empty_like(r_keep)
        assert cudart.cudaMemcpy(x_now.ctypes.data, dx, ctypes.c_size_t(nbytes), 2) == 0
        assert cudart.cudaMemcpy(r_now.ctypes.data, dr, ctypes.c_size_t(rbytes), 2) == 0
        np.testing.assert_array_equal(x_now, x_keep)
        np.testing.assert_array_equal(r_now, r_keep)
    finally:
        cudart.cudaFree(dx)
        cudart.cudaFree(dr)
