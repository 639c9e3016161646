"""Every dedispersion launch shape selectable through TXG_DEDISP_SHAPE gives the oracle's
dedispersed series bit for bit (FP32), including the chunked stage-1 kernel that takes
windows too large to stay resident; with 16-bit subband storage every stage-1 shape and every
stage-2 pair-kernel shape gives the default shape's series bit for bit (the same additions
in the same order)."""
import numpy as np
import pytest

from test_gpu_pipeline import oracle_rows, small_workload

pytestmark = pytest.mark.gpu

FP32_SHAPES = ["s1=16", "s1=1", "s1=11", "s1=14", "s1=-1", "s2=1", "s2=2,s2kb=36", "s2=0,s2kb=8",
               "s2=3", "s2=5"]
PAIR_SHAPES = ["s1=16", "s1=1", "s1=11", "s1=-1", "s2=1", "s2=2,s2kb=36", "s2=3", "s2=4"]


def _series(tx, rows, fil, ndump, prec="fp32"):
    out = []
    with tx.Search(rows, fil.nchans, fil.tsamp, fil.freqs, ndump, precision=prec,
                   flags=tx.FLAG_KEEP_SERIES) as s:
        for b in range(fil.nsamples // ndump):
            s.push_block(fil.generate(b * ndump, ndump))
            s.sync()
            out.append([s.timdata(r).copy() if s.row_info(r).gated else None
                        for r in range(len(rows))])
    return out


@pytest.mark.parametrize("shape", FP32_SHAPES)
def test_fp32_shapes_match_oracle(tx, oracle, shape, monkeypatch):
    fil, rows, ndump = small_workload()
    monkeypatch.setenv("TXG_DEDISP_SHAPE", shape)
    got = _series(tx, rows, fil, ndump)
    orows = oracle_rows(oracle, rows, fil, ndump, tx)
    ngated = 0
    for b, blk in enumerate(got):
        raw = fil.generate(b * ndump, ndump)
        for r, o in enumerate(orows):
            gated = o.run(raw)
            assert (blk[r] is not None) == gated
            if gated:
                ngated += 1
                np.testing.assert_array_equal(blk[r], o.timdata(), err_msg=f"{shape} block {b} row {r}")
    assert ngated >= 4


@pytest.mark.parametrize("prec", ["fp16", "bf16"])
@pytest.mark.parametrize("shape", PAIR_SHAPES)
def test_16bit_shapes_equal_default(tx, prec, shape, monkeypatch):
    fil, rows, ndump = small_workload()
    monkeypatch.delenv("TXG_DEDISP_SHAPE", raising=False)
    ref = _series(tx, rows, fil, ndump, prec)
    monkeypatch.setenv("TXG_DEDISP_SHAPE", shape)
    got = _series(tx, rows, fil, ndump, prec)
    for b, (x, y) in enumerate(zip(ref, got)):
        for r, (u, v) in enumerate(zip(x, y)):
            assert (u is None) == (v is None)
            if u is not None:
                np.testing.assert_array_equal(u, v, err_msg=f"{prec} {shape} block {b} row {r}")


@pytest.mark.parametrize("prec", ["fp32", "fp16"])
def test_autotuned_shapes_give_the_same_series(tx, prec, monkeypatch):
    """TXG_FLAG_AUTOTUNE times the candidate launch shapes at txg_create and keeps the fastest
    per row: the series are those of the default shapes bit for bit, and the reported shapes
    are among the candidates."""
    monkeypatch.delenv("TXG_DEDISP_SHAPE", raising=False)
    fil, rows, ndump = small_workload()
    ref = _series(tx, rows, fil, ndump, prec)
    with tx.Search(rows, fil.nchans, fil.tsamp, fil.freqs, ndump, precision=prec,
                   flags=tx.FLAG_KEEP_SERIES | tx.FLAG_AUTOTUNE) as s:
        for r in range(len(rows)):
            s1, s2, kb = s.launch_shape(r)
            assert s1 in (0, 13, 17, 14, 16, 10, 1)
            assert (s2, kb) in ((0, 0), (1, 0), (2, 0), (0, 36), (2, 36), (1, 24), (3, 0),
                                (4, 0), (5, 0))
        for b in range(fil.nsamples // ndump):
            s.push_block(fil.generate(b * ndump, ndump))
            s.sync()
            for r in range(len(rows)):
                if ref[b][r] is not None:
                    np.testing.assert_array_equal(s.timdata(r), ref[b][r],
                                                  err_msg=f"{prec} block {b} row {r}")
