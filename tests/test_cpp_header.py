"""The C++ layer (include/transientx_gb300.hpp) compiles against the C ABI and links with the
library; on a GPU it also runs a small search end to end."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

GUIDE = os.path.join(ROOT, "INTEGRATION.md")  # the integration guide with the C and C++ examples

SRC = r'''
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include "transientx_gb300.hpp"
int main(int argc, char **argv) {
    const int C = 64; const long N = 2048; const double tsamp = 256e-6;
    std::vector<double> f(C);
    for (int j = 0; j < C; j++) f[j] = 1500.0 - (j + 0.5) * 300.0 / C;
    auto rows = txgpu::parse_ddplan("# td fd dms ddm ndm snrloss maxw\n1 1 0 1 100 0.1 0.02\n");
    rows[0].nsub = 8;
    if (argc < 2) {
        std::printf("parsed %zu rows\n", rows.size());
        txgpu::Boxcar bx;                 /* Boxcar::dump2txt on host-filled planes */
        bx.ndm = 3;
        bx.nsamples = 4;
        for (int k = 0; k < 12; k++) bx.mxS.push_back(k * 1.25f - 3.5f);
        bx.dump2txt("boxcar.txt");
        txgpu::Boxcar none;
        none.ndm = 2;
        none.nsamples = 2;
        try { none.dump2txt("never.txt"); std::printf("no throw\n"); }
        catch (const txgpu::Error &e) { std::printf("throws %d\n", e.status); }
        return 0;
    }
    txgpu::Search s(rows, C, tsamp, f, N);
    std::vector<uint8_t> raw(N * C);
    unsigned long long z = 12345;
    int found = 0;
    for (int b = 0; b < 4; b++) {
        for (long t = 0; t < N; t++)
            for (int j = 0; j < C; j++) {
                double g = 0; for (int k = 0; k < 12; k++) { z = z * 6364136223846793005ULL + 1442695040888963407ULL; g += (z >> 11) * (1.0 / 9007199254740992.0); }
                double v = 128 + 12 * (g - 6);
                long tt = b * N + t;
                double d = 4.148741601e3 * 50.0 * (1.0 / (f[j] * f[j]) - 1.0 / (f[0] * f[0])) / tsamp;
                if (tt >= 5000 + std::lround(d) && tt < 5008 + std::lround(d)) v += 30;
                raw[t * C + j] = (uint8_t)std::fmin(255, std::fmax(0, std::floor(v + 0.5)));
            }
        s.run(raw.data());
        s.sync();
        if (s.info(0).gated) found += (int)s.cluster(0).size();
    }
    std::printf("clusters %d\n", found);
    return found > 0 ? 0 : 1;
}
'''


def _compile(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    from transientx_gb300 import _build
    _build.build()
    src = tmp_path / "drop_in.cpp"
    src.write_text(SRC)
    exe = tmp_path / "drop_in"
    lib = os.path.join(ROOT, "transientx_gb300")
    subprocess.run(["g++", "-std=c++17", "-O2", str(src), "-I", os.path.join(ROOT, "include"),
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


def test_integration_c_snippet_compiles(tmp_path):
    """The C example of the integration guide (section 2) compiles against the C header as
    written (its free names, freqs and block, declared around it) and links with the
    library."""
    import re
    if not shutil.which("gcc"):
        pytest.skip("no gcc")
    doc = open(GUIDE).read()
    blocks = re.findall(r"```c\n(.*?)```", doc, re.S)
    assert blocks, "the integration guide has no C example"
    body = blocks[0].replace('#include "transientx_gb300.h"', "")
    src = tmp_path / "snippet.c"
    src.write_text('#include <stdio.h>\n#include "transientx_gb300.h"\n'
                   "int run(const double *freqs, const uint8_t *block) {\n" + body +
                   "    return 0;\n}\nint main(void) { return 0; }\n")
    from transientx_gb300 import _build
    _build.build()
    lib = os.path.join(ROOT, "transientx_gb300")
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-Wno-unused-variable", str(src),
                    "-I", os.path.join(ROOT, "include"), "-L", lib, "-ltxgpu",
                    f"-Wl,-rpath,{lib}", "-o", str(tmp_path / "snippet")], check=True)


def test_integration_cpp_snippet_compiles(tmp_path):
    """The C++ replacement of the block loop in the integration guide (section 1) compiles
    against the C++ layer as written, with the reference-side names it uses (the command-line
    map, the reader, the writer and the output stream) declared around it."""
    import re
    doc = open(GUIDE).read()
    blocks = [b for b in re.findall(r"```cpp\n(.*?)```", doc, re.S) if "transientx_gb300.hpp" in b]
    assert len(blocks) == 1
    body = blocks[0].replace('#include "transientx_gb300.hpp"', "")
    prelude = r'''
#include <fstream>
#include <string>
#include "transientx_gb300.hpp"
struct OptionValue { float v; template <class T> T as() const { return (T)v; } };
struct OptionMap { OptionValue operator[](const char *) const { return {4.f}; } };
static bool read_raw_block(uint8_t *, long) { return false; }
int run(const std::string &ddplan_text, const txgpu::SinglePulse &base_row, int nchans,
        double tsamp, const std::vector<double> &frequencies, long ndump, const OptionMap &vm,
        txgpu::CandsWriter &writer, std::ofstream &cands_file) {
'''
    src = tmp_path / "snippet.cpp"
    src.write_text(prelude + body + "    return 0;\n}\nint main() { return 0; }\n")
    from transientx_gb300 import _build
    _build.build()
    lib = os.path.join(ROOT, "transientx_gb300")
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-Wno-unused-variable", str(src),
                    "-I", os.path.join(ROOT, "include"), "-L", lib, "-ltxgpu",
                    f"-Wl,-rpath,{lib}", "-o", str(tmp_path / "snippet")], check=True)
