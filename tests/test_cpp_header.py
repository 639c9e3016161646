"""The C++ layer (include/transientx_gb300.hpp) compiles against the C ABI and links with the
library; on a GPU it also runs a small search end to end."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

SNIPPETS = os.path.join(ROOT, "tests", "snippets")  # the C and C++ examples the integration guide quotes


def _compile(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    from transientx_gb300 import _build
    _build.build()
    src = os.path.join(SNIPPETS, "drop_in.cpp")
    exe = tmp_path / "drop_in"
    lib = os.path.join(ROOT, "transientx_gb300")
    subprocess.run(["g++", "-std=c++17", "-O2", src, "-I", os.path.join(ROOT, "include"),
                    "-L", lib, "-ltxgpu", f"-Wl,-rpath,{lib}", "-o", str(exe)], check=True)
    return exe


def test_header_compiles_and_parses(tmp_path):
    exe = _compile(tmp_path)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True,
                         cwd=tmp_path).stdout
    assert "parsed 1 rows" in out
    # Boxcar::dump2txt: one line per DM trial, "%f " per value (boxcar.cpp:473-489)
    vals = np.arange(12, dtype=np.float32) * np.float32(1.25) - np.float32(3.5)
    want = "".join("".join("%f " % v for v in vals[j * 4:(j + 1) * 4]) + "\n" for j in range(3))
    assert (tmp_path / "boxcar.txt").read_text() == want
    # the Python mirror writes the same file
    import transientx_gb300 as tx
    tx.Boxcar(ndm=3, nsamples=4, mxS=vals.reshape(3, 4)).dump2txt(str(tmp_path / "py.txt"))
    assert (tmp_path / "py.txt").read_text() == want
    with pytest.raises(tx.TxgError):
        tx.Boxcar(ndm=2, nsamples=2).dump2txt(str(tmp_path / "never.txt"))
    # without dense planes it refuses (TXG_ERR_STATE) instead of reading nothing
    assert "throws -6" in out


@pytest.mark.gpu
def test_header_end_to_end(tmp_path):
    exe = _compile(tmp_path)
    r = subprocess.run([str(exe), "run"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def _link(tmp_path, compiler, std, name, main):
    from transientx_gb300 import _build
    _build.build()
    src = os.path.join(SNIPPETS, name)
    drv = tmp_path / ("main" + os.path.splitext(name)[1])
    drv.write_text(main)
    lib = os.path.join(ROOT, "transientx_gb300")
    subprocess.run([compiler, f"-std={std}", "-Wall", "-Werror", "-Wno-unused-variable", src,
                    str(drv), "-I", os.path.join(ROOT, "include"), "-L", lib, "-ltxgpu",
                    f"-Wl,-rpath,{lib}", "-o", str(tmp_path / "snippet")], check=True)


def test_integration_c_snippet_compiles(tmp_path):
    """The C example the integration guide quotes (section 2, tests/snippets/c_api.c) compiles
    against the C header and links with the library."""
    if not shutil.which("gcc"):
        pytest.skip("no gcc")
    _link(tmp_path, "gcc", "c11", "c_api.c", "int main(void) { return 0; }\n")


def test_integration_cpp_snippet_compiles(tmp_path):
    """The C++ replacement of the block loop the integration guide quotes (section 1,
    tests/snippets/block_loop.cpp) compiles against the C++ layer, with the reference-side
    names it uses declared around it, and links with the library."""
    if not shutil.which("g++"):
        pytest.skip("no g++")
    _link(tmp_path, "g++", "c++17", "block_loop.cpp", "int main() { return 0; }\n")


def _build_fil_loop(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    from transientx_gb300 import _build
    _build.build()
    lib = os.path.join(ROOT, "transientx_gb300")
    exe = tmp_path / "fil_loop"
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror",
                    os.path.join(SNIPPETS, "fil_loop.cpp"), "-I", os.path.join(ROOT, "include"),
                    "-L", lib, "-ltxgpu", f"-Wl,-rpath,{lib}", "-o", str(exe)], check=True)
    return exe


def test_fil_loop_compiles_against_the_class_compatible_headers(tmp_path):
    """transientx_fil's block loop (dedisperse_fil.cpp:319-338), with the reference's class
    names and calls -- parse(vm, search), SinglePulse::prepare/run(DataBuffer<float>&),
    PreprocessLite, Boxcar, Cluster<double>, CandPlot -- compiles against include/compat/ and
    links with the library."""
    _build_fil_loop(tmp_path)


@pytest.mark.gpu
def test_fil_loop_finds_the_oracles_candidates(tx, oracle, tmp_path):
    """The block loop over include/compat/ on the 256-channel configuration (ddplan
    "1 1 0 0.5 2000 0.1 0.05", 16 subbands, 15625-sample blocks, from the block before the
    DM-100 pulse): every searched block's candidate list equals the oracle's float chain
    clustered by the oracle's Cluster::run rule, and the .cands file has one line each."""
    from transientx_gb300 import synth
    exe = _build_fil_loop(tmp_path)
    wl = synth.WORKLOADS["nchan256_n1M_dm1000"]()
    fil, ndump = wl.fil, wl.ndump
    s0, nblk = 12, 4
    raw = fil.generate(s0 * ndump, nblk * ndump)
    (tmp_path / "obs.raw").write_bytes(raw.tobytes())
    (tmp_path / "ddplan.txt").write_text("# td fd dms ddm ndm snrloss maxw\n"
                                         "1 1 0 0.5 2000 0.1 0.05\n")
    r = subprocess.run([str(exe), str(tmp_path / "obs.raw"), str(fil.nchans), repr(fil.tsamp),
                        repr(float(fil.freqs[0])), repr(float(fil.freqs[1] - fil.freqs[0])),
                        str(ndump), str(tmp_path / "ddplan.txt"), str(tmp_path / "obs")],
                       capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    got = {}
    for line in r.stdout.splitlines():
        if line.startswith("cand "):
            _, rid, counter, idm, isamp, wn, S = line.split()
            got.setdefault(int(counter), []).append((int(idm), int(isamp), int(wn), float(S)))
    nsub, group = oracle.plan_row(fil.freqs, fil.tsamp, 1, 1, 0.5, 2000, 16, 0)
    row = oracle.make_row(td=1, fd=1, bswidth=0.1, rfi=[], dms=0.0, ddm=0.5, ndm=2000,
                          nsub=nsub, group=group, minw=1e-4, maxw=0.05, snrloss=0.1, thre=7.0,
                          zapthre=0.0)
    o = oracle.SinglePulseRow(row, fil.freqs, fil.tsamp, ndump)
    maxwn = int(o.widths().max())
    want, ngated = {}, 0
    for b in range(nblk):
        blk = raw[b * ndump:(b + 1) * ndump].astype(np.float32)
        if not o.run_f32(blk):
            continue
        ngated += 1
        i = o.info()
        pts = oracle.threshold_scan(o.mxS(), o.mxwn(), 7.0)
        cl, _ = oracle.cluster(pts, 0.0, 0.5, i.fmax, i.fmin, i.tsamp, 1e-3, 100, 5, False, maxwn)
        want[int(i.counter)] = [(int(c["idm"]), int(c["isamp"]), int(c["wn"]), float(c["S"]))
                                for c in cl]
    assert ngated == nblk - 1
    assert sum(len(v) for v in want.values()) > 0, "the DM-100 pulse should be found"
    for counter, cl in want.items():
        g = got.get(counter, [])
        assert [c[:3] for c in g] == [c[:3] for c in cl], counter
        for a, b in zip(g, cl):
            assert abs(a[3] - b[3]) <= 1e-4 * max(1.0, abs(b[3])), (counter, a, b)
    cands = list(tmp_path.glob("obs_*.cands"))
    assert len(cands) == 1
    assert len(cands[0].read_text().splitlines()) == sum(len(v) for v in want.values())


def test_parse_and_parse_json_rows(tmp_path):
    """parse(vm, search) and parse_json(vm, config, search) of include/compat/singlepulse.h,
    instantiated over stand-ins for the options map and the JSON type
    (tests/snippets/parse_config.cpp): the fields of every row follow singlepulse.cpp:343-545
    -- radius in ms becomes seconds, a ddplan line's seven numbers override the options, the
    command-line rfi words come first, and one SinglePulse is carried down the ddplan lines
    and JSON entries, so a row keeps every earlier row's zap and rfi entries.  An rfilist entry
    of the JSON configuration takes no zap.  No GPU call is made."""
    if not shutil.which("g++"):
        pytest.skip("no g++")
    from transientx_gb300 import _build
    _build.build()
    lib = os.path.join(ROOT, "transientx_gb300")
    exe = tmp_path / "parse_config"
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-Wno-unused-variable",
                    os.path.join(SNIPPETS, "parse_config.cpp"), "-I", os.path.join(ROOT, "include"),
                    "-L", lib, "-ltxgpu", f"-Wl,-rpath,{lib}", "-o", str(exe)], check=True)
    (tmp_path / "ddplan.txt").write_text(
        "# td fd dms ddm ndm snrloss maxw\n"
        "1 1 0 0.1 5000 0.1 0.05 zap 1300 1310 kadaneT 3 5\n"
        "  2 1 500 0.2 5000 0.1 0.05 mask 4 8 zero\n"
        "\n"
        "not a row\n")
    json_rows = [
        "row 1 td 2 fd 1 dms 500 ddm 0.2 ndm 5000 snrloss 0.1 maxw 0.05 bswidth 0.2 thre 6.5 "
        "radius 0.002 minpts 3 iqr 1 nzap 1 rfi kadaneF 8 4 zdot",
        "row 2 td 4 fd 1 dms 1500 ddm 0.2 ndm 5000 snrloss 0.1 maxw 0.05 bswidth 0.2 thre 6.5 "
        "radius 0.002 minpts 3 iqr 1 nzap 2 rfi kadaneF 8 4 zdot zero"]
    out = subprocess.run([str(exe), str(tmp_path / "ddplan.txt")], capture_output=True,
                         text=True, check=True).stdout.splitlines()
    assert out == [
        "row 1 td 1 fd 1 dms 0 ddm 0.1 ndm 5000 snrloss 0.1 maxw 0.05 bswidth 0.1 thre 7 "
        "radius 0.001 minpts 5 iqr 0 nzap 2 rfi zdot kadaneF 8 4 kadaneT 3 5",
        "row 2 td 2 fd 1 dms 500 ddm 0.2 ndm 5000 snrloss 0.1 maxw 0.05 bswidth 0.1 thre 7 "
        "radius 0.001 minpts 5 iqr 0 nzap 2 rfi zdot kadaneF 8 4 kadaneT 3 5 mask 4 8 zero",
    ] + json_rows
    # without a ddplan the options make one row, id 1
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines()
    assert out == [
        "row 1 td 1 fd 1 dms 0 ddm 1 ndm 1000 snrloss 0.1 maxw 0.02 bswidth 0.1 thre 7 "
        "radius 0.001 minpts 5 iqr 0 nzap 1 rfi zdot kadaneF 8 4"] + json_rows
