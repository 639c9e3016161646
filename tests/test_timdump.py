"""Dedispersed-series dump: the quantised read-back (GPU) against a numpy restatement of the
same definition, and the SIGPROC / PRESTO writers."""
import os
import tempfile
from types import SimpleNamespace

import numpy as np
import pytest


def _quant(tim, nsamp, nbits, mean, std):
    x = tim[:, :nsamp].astype(np.float64)
    m = x.mean(axis=1, keepdims=True)
    v = (x * x).mean(axis=1, keepdims=True) - m * m
    sd = np.where(v > 0, np.sqrt(np.maximum(v, 0)), 1.0)
    q = ((x - m) / sd * std + mean).astype(np.float32)
    if nbits == 32:
        return q
    hi = 65535.0 if nbits == 16 else 255.0
    return np.clip(np.rint(q), 0, hi)


class _FakeSearch:
    def __init__(self, blocks):
        self.blocks, self.k = blocks, -1

    def row_info(self, row, beam=0):
        return SimpleNamespace(gated=1)

    def timdata_q(self, row, beam, idm0, count, nsamp, nbits, mean, std):
        self.k += 1
        return self.blocks[self.k][idm0:idm0 + count, :nsamp]


def test_sigproc_writer_round_trip():
    from transientx_gb300 import timdump
    info = SimpleNamespace(ndm=3, dms=10.0, ddm=0.5, tsamp=64e-6, ndump=100)
    rng = np.random.default_rng(0)
    blocks = [rng.integers(0, 255, (3, 120)).astype(np.uint8) for _ in range(2)]
    with tempfile.TemporaryDirectory() as d:
        with timdump.TimDumper(os.path.join(d, "x"), info, fmt="sigproc", nbits=8, tstart=60000.5,
                               source_name="SRC", fch1=1500.0) as w:
            s = _FakeSearch(blocks)
            w.push(s, 0)
            w.push(s, 0)
            paths = list(w.paths)
        assert [os.path.basename(p) for p in paths] == ["x_DM10.00.tim", "x_DM10.50.tim", "x_DM11.00.tim"]
        h = timdump.read_sigproc_header(paths[1])
        assert h["data_type"] == 2 and h["nbits"] == 8 and h["nchans"] == 1
        assert h["refdm"] == 10.5 and h["tsamp"] == 64e-6 and h["tstart"] == 60000.5
        assert h["source_name"] == "SRC" and h["fch1"] == 1500.0
        data = np.fromfile(paths[1], np.uint8, offset=h["data_offset"])
        np.testing.assert_array_equal(data, np.concatenate([blocks[0][1, :100], blocks[1][1, :100]]))


def test_presto_writer_inf():
    from transientx_gb300 import timdump
    info = SimpleNamespace(ndm=1, dms=57.25, ddm=1.0, tsamp=1e-4, ndump=50)
    blocks = [np.arange(60, dtype=np.float32).reshape(1, 60)]
    with tempfile.TemporaryDirectory() as d:
        w = timdump.TimDumper(os.path.join(d, "p"), info, fmt="presto", tstart=59000.25,
                              freqs=np.linspace(1500, 1200, 64))
        w.push(_FakeSearch(blocks), 0)
        w.close()
        dat = np.fromfile(os.path.join(d, "p_DM57.25.dat"), np.float32)
        np.testing.assert_array_equal(dat, np.arange(50, dtype=np.float32))
        inf = open(os.path.join(d, "p_DM57.25.inf")).read()
        assert " Number of bins in the time series      =  50\n" in inf
        assert " Dispersion measure (cm-3 pc)           =  57.25\n" in inf
        assert " Epoch of observation (MJD)             =  59000.250000000000000\n" in inf
        assert " Number of channels                     =  64\n" in inf


@pytest.mark.gpu
@pytest.mark.parametrize("nbits", [8, 16, 32])
def test_quantised_series_match_definition(tx, nbits):
    from test_gpu_pipeline import small_workload
    fil, rows, ndump = small_workload()
    with tx.Search(rows, fil.nchans, fil.tsamp, fil.freqs, ndump, flags=tx.FLAG_KEEP_SERIES) as s:
        checked = 0
        for b in range(fil.nsamples // ndump):
            s.push_block(fil.generate(b * ndump, ndump))
            s.sync()
            for r in range(len(rows)):
                info = s.row_info(r)
                if not info.gated:
                    continue
                tim = s.timdata(r)
                mean, std = (128.0, 20.0) if nbits < 32 else (0.0, 3.0)
                q = s.timdata_q(r, nbits=nbits, mean=mean, std=std)
                ref = _quant(tim, info.ndump, nbits, mean, std)
                if nbits == 32:
                    np.testing.assert_allclose(q, ref, atol=1e-4, rtol=1e-5)
                else:
                    d = np.abs(q.astype(np.int64) - ref.astype(np.int64))
                    assert d.max() <= 1 and (d > 0).mean() < 1e-3
                checked += 1
        assert checked > 0
