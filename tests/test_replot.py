"""The replot chain (replot_fil.cpp:409-457) on the GPU against the reference's own Candidate
class (candidate.cpp compiled in place): golden fixtures from tests/golden/make_golden_replot.py,
compared exactly -- results, S/N maps, final data and the data after every step."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from make_golden_replot import CASES  # noqa: E402


@pytest.fixture(scope="module")
def fix():
    return np.load(os.path.join(HERE, "golden", "replot.npz"))


def _cands(z):
    out = []
    for k in range(3):
        tbin, dm, width = z[f"c{k}_meta"]
        out.append({"data": z[f"c{k}_data"].astype(np.float32), "frequencies": z[f"c{k}_freqs"],
                    "tbin": float(tbin), "dm": float(dm), "width": float(np.float32(width))})
    return out


def test_fixture_reproduces_with_the_reference(fix, oracle):
    """Where the reference tree is compiled here, re-running it on the stored inputs gives the
    stored results (guards the fixture against drift)."""
    if not oracle.ref_available():
        pytest.skip("reference not compiled on this machine")
    c = _cands(fix)[1]
    for name, opts in CASES.items():
        r = oracle.ref_replot(c["data"], c["frequencies"], c["tbin"], c["dm"], c["width"], **opts)
        np.testing.assert_array_equal(r["snrmap"], fix[f"{name}_c1_snrmap"])
        np.testing.assert_array_equal(r["data"], fix[f"{name}_c1_data"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_replot_matches_reference(tx, fix, name):
    cands = _cands(fix)
    kw = dict(CASES[name])
    res = tx.replot(cands, maps=True, data=True, **kw)
    for k, r in enumerate(res):
        snr, width, dmx, mjd, nbin, nchan, ndm = fix[f"{name}_c{k}_res"]
        assert (r["nbin"], r["nchan"], r["ndm"]) == (int(nbin), int(nchan), int(ndm)), (name, k)
        assert np.float32(r["snr"]) == np.float32(snr), (name, k, r["snr"], snr)
        assert np.float32(r["width"]) == np.float32(width), (name, k)
        assert r["dm_maxsnr"] == dmx, (name, k, r["dm_maxsnr"], dmx)
        assert r["maxtid"] * cands[k]["tbin"] / 86400.0 == mjd, (name, k)
    np.testing.assert_array_equal(res[1]["snrmap"], fix[f"{name}_c1_snrmap"])
    np.testing.assert_array_equal(res[1]["data"], fix[f"{name}_c1_data"])


@pytest.mark.gpu
@pytest.mark.parametrize("upto", range(1, 12))
def test_replot_each_step_matches_reference(tx, fix, upto):
    cands = _cands(fix)
    r = tx.replot([cands[1]], upto=upto, data=True, **CASES["full"])[0]
    np.testing.assert_array_equal(r["data"], fix[f"full_c1_step{upto}"], err_msg=f"step {upto}")


@pytest.mark.gpu
def test_replot_batch_equals_single(tx, fix):
    """A batch gives each candidate what it gets alone."""
    cands = _cands(fix)
    batch = tx.replot(cands, maps=True, **CASES["full"])
    for k, c in enumerate(cands):
        one = tx.replot([c], maps=True, **CASES["full"])[0]
        assert one["snr"] == batch[k]["snr"] and one["maxtid"] == batch[k]["maxtid"]
        np.testing.assert_array_equal(one["snrmap"], batch[k]["snrmap"])


def test_replot_rejects_bad_input(tx):
    with pytest.raises(tx.TxgError):
        tx.replot([{"data": np.zeros((1, 100), np.float32), "frequencies": [1400.0], "tbin": 1e-4,
                    "dm": 10.0, "width": 1e-3}])
