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
