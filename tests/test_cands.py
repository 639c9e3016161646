"""The .cands writer (CandPlot::plot, src/singlepulse/candplot.cpp:32-433): line format,
the C++ and Python writers agreeing, and (GPU) the subband data and candidate bands
against the oracle."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _clusters(rows):
    import transientx_gb300 as tx
    c = np.zeros(len(rows), tx.CAND_DTYPE)
    for k, (idm, isamp, wn, S) in enumerate(rows):
        c[k] = (idm, isamp, wn, S)
    return c


def test_line_format():
    from transientx_gb300.cands import CandsWriter
    w = CandsWriter("J1234", 60000.25, beam="3", fname="obs.fil")
    c = _clusters([(10, 100, 4, 12.34), (20, 50, 8, 30.0), (5, 7, 2, 12.34)])
    counter, offset, ndump, tsamp = 3 * 13156, 2 * 13156, 13156, 76e-6
    lines = w.format_block(c, counter, offset, ndump, tsamp, 0.0, 0.1,
                           [1000.4, 900.6, 800.0], [1200.5, 1100.2, 850.0], 1)
    assert w.filename == "J1234_60000.2500000000_3.cands"
    bmjd = 60000.25 + (-offset + counter - ndump) * tsamp / 86400.0
    assert len(lines) == 3
    # descending S/N, ties in list order: (20,50) first, then (10,100), then (5,7)
    f = lines[0].rstrip("\n").split("\t")
    assert f[0] == "3" and f[1] == "1"
    assert f[2] == "%.15f" % (60000.25 + (-offset + counter - ndump + 50) * tsamp / 86400.0)
    assert f[3] == "2.00" and f[4] == "%.2f" % (8 * tsamp * 1000) and f[5] == "30.0"
    assert f[6] == "901" and f[7] == "1100"
    assert f[8] == "J1234_%.10f_3_01_01.png" % bmjd and f[9] == "01" and f[10] == "obs.fil"
    f1 = lines[1].split("\t")
    f2 = lines[2].split("\t")
    assert f1[3] == "1.00" and f1[5] == "12.3" and f1[8].endswith("_02_01.png") and f1[1] == "2"
    assert f2[3] == "0.50" and f2[8].endswith("_03_01.png") and f2[1] == "3"
    # the running number continues with the next block
    more = w.format_block(c[:1], counter + ndump, offset, ndump, tsamp, 0.0, 0.1, [1.0], [2.0], 2)
    assert more[0].split("\t")[1] == "4" and more[0].split("\t")[9] == "02"


CPP = r'''
#include <cstdio>
#include <iostream>
#include "transientx_gb300.hpp"
int main() {
    long counter, offset, ndump; double tsamp, dms, ddm, tstart; int n, id;
    std::cin >> tstart >> counter >> offset >> ndump >> tsamp >> dms >> ddm >> id >> n;
    std::vector<txg_cand> c(n); std::vector<float> fl(n), fh(n);
    for (int k = 0; k < n; k++) std::cin >> c[k].idm >> c[k].isamp >> c[k].wn >> c[k].S >> fl[k] >> fh[k];
    txgpu::CandsWriter w("root", tstart, "7", "f.fil");
    for (const std::string &s : w.format_block(c, counter, offset, ndump, tsamp, dms, ddm, fl, fh, id))
        std::cout << s;
    std::cout << w.filename() << "\n";
}
'''


def test_cpp_writer_equals_python_writer():
    from transientx_gb300.cands import CandsWriter
    rng = np.random.default_rng(5)
    n = 40
    c = _clusters([(int(rng.integers(0, 5000)), int(rng.integers(0, 13000)),
                    int(rng.integers(1, 600)), float(np.float32(rng.uniform(7, 50)))) for _ in range(n)])
    c["S"][5] = c["S"][9]  # a tie
    fl = rng.uniform(856, 1712, n).astype(np.float32)
    fh = rng.uniform(856, 1712, n).astype(np.float32)
    args = (59876.123456789, 7 * 13156, 3 * 13156, 13156, 7.6e-05, 500.0, 0.2, 2)
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "w.cpp"), os.path.join(d, "w")
        open(src, "w").write(CPP)
        subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), src, "-o", exe],
                       check=True)
        inp = " ".join(repr(a) for a in (args[0],) + args[1:]) + f" {n}\n"
        inp += "".join(f"{int(x['idm'])} {int(x['isamp'])} {int(x['wn'])} {float(x['S']):.9g} "
                       f"{float(a):.9g} {float(b):.9g}\n" for x, a, b in zip(c, fl, fh))
        out = subprocess.run([exe], input=inp, capture_output=True, text=True, check=True).stdout
    w = CandsWriter("root", args[0], beam="7", fname="f.fil")
    expect = "".join(w.format_block(c, *args[1:7], fl, fh, args[7])) + w.filename + "\n"
    assert out == expect


@pytest.mark.gpu
def test_subdata_and_band_match_oracle(tx, oracle):
    from test_gpu_pipeline import oracle_rows, small_workload
    from transientx_gb300.cands import CandsWriter
    fil, rows, ndump = small_workload()
    orows = oracle_rows(oracle, rows, fil, ndump, tx)
    checked = 0
    with tx.Search(rows, fil.nchans, fil.tsamp, fil.freqs, ndump, flags=tx.FLAG_CLUSTER,
                   zapthre=4.0) as s:
        for b in range(fil.nsamples // ndump):
            raw = fil.generate(b * ndump, ndump)
            s.push_block(raw)
            s.sync()
            for r, o in enumerate(orows):
                if not o.run(raw):
                    continue
                info = s.row_info(r)
                _, _, _, sub_start, _ = tx.describe_row(rows, r, fil.nchans, fil.tsamp, fil.freqs, ndump)
                freqs = o.freqs()
                fsub = []
                for q in range(info.nsub):
                    acc = 0.0
                    for j in range(sub_start[q], sub_start[q + 1]):
                        acc += float(freqs[j])
                    fsub.append(acc / (sub_start[q + 1] - sub_start[q]))
                for idm in (0, info.ndm // 2, info.ndm - 1):
                    np.testing.assert_array_equal(s.subdata(idm, r), o.subdata(idm))
                cl = s.cluster(r)
                if len(cl) == 0:
                    continue
                fl, fh = s.cand_band(cl, r)
                for k in range(len(cl)):
                    sub = o.subdata(int(cl["idm"][k]))
                    efl, efh = oracle.cand_band(sub, sub_start, fsub, int(cl["isamp"][k]), int(cl["wn"][k]))
                    assert fl[k] == efl and fh[k] == efh, (b, r, k)
                w = CandsWriter("x", 60000.0)
                lines = w.format_block(cl, info.counter, info.offset, info.ndump, info.tsamp,
                                       info.dms, info.ddm, fl, fh, r + 1)
                assert len(lines) == len(cl)
                checked += len(cl)
    assert checked > 0
