"""dgc_write_data_file against the visualisation file the reference's
advection driver writes (examples/advection_2d/main.cpp:164-174), rendered by
the reference harness from the same stream statements: byte-identical text for
every golden case.  Host-only (no GPU)."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN

import dgc_gb300 as dg

CASES = sorted(p for p in glob.glob(os.path.join(GOLDEN, "ref_*_N*.npz")) if "adv1d" not in p and "stokes" not in p)


@pytest.fixture(scope="module", autouse=True)
def built():
    from dgc_gb300 import build
    build.build()


@pytest.mark.parametrize("path", CASES, ids=lambda p: os.path.basename(p)[4:-4])
def test_data_file_matches_reference_driver(path, tmp_path):
    d = np.load(path)
    out = tmp_path / "Advection2DDataFile.txt"
    dg.write_data_file(str(out), d["adv_x"], d["adv_y"], d["adv_rk4_10"], d["adv_exact_10"])
    want = bytes(d["adv_datafile"].astype(np.uint8))
    assert out.read_bytes() == want


def test_data_file_without_reference_block(tmp_path):
    out = tmp_path / "f.txt"
    dg.write_data_file(str(out), [0.5, -1.0], [2.0, 1e-20], [-0.0, 3.25])
    assert out.read_text() == "#         x         y         u\n0.5  2  -0\n-1  1e-20  3.25\n\n"


def test_data_file_bad_path_raises():
    with pytest.raises(dg.DgcError):
        dg.write_data_file("/nonexistent-dir/x.txt", [0.0], [0.0], [0.0])
