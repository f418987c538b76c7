"""Gmsh MSH 4 import / export (dgc_msh_read, dgc_msh_write) against the
reference's gmsh_importer_exporter: the reference's own .msh files read to the
vertices and triangles the reference imports, and the exporter's output
byte-identical to the reference exporter's for every golden mesh.  Host-only."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN

import dgc_gb300 as dg
from dgc_gb300 import meshes

CASES = sorted(p for p in glob.glob(os.path.join(GOLDEN, "ref_*_N*.npz")) if "adv1d" not in p and "stokes" not in p)
SOURCES = [p for p in CASES if "msh_source" in np.load(p).files]


@pytest.fixture(scope="module", autouse=True)
def built():
    from dgc_gb300 import build
    build.build()


def case_id(p):
    return os.path.basename(p)[4:-4]


@pytest.mark.parametrize("path", SOURCES, ids=case_id)
def test_import_matches_reference_importer(path, tmp_path):
    d = np.load(path)
    src = tmp_path / "mesh.msh"
    src.write_bytes(bytes(d["msh_source"]))
    m = dg.read_msh(str(src))
    assert np.array_equal(m.xy.reshape(-1), d["mesh_xy"])
    assert np.array_equal(m.cells.reshape(-1), d["mesh_cells"])


@pytest.mark.parametrize("path", CASES, ids=case_id)
def test_export_matches_reference_exporter(path, tmp_path):
    d = np.load(path)
    m = meshes.Mesh(xy=d["mesh_xy"].reshape(-1, 2), cells=d["mesh_cells"].reshape(-1, 3))
    out = tmp_path / "out.msh"
    dg.write_msh(str(out), m)
    assert out.read_bytes() == bytes(d["msh_export"])


def test_lossless_round_trip(tmp_path):
    m = meshes.jittered_square(40, 3)
    out = str(tmp_path / "j.msh")
    dg.write_msh(out, m, digits=17)
    r = dg.read_msh(out)
    assert np.array_equal(r.xy, m.xy) and np.array_equal(r.cells, m.cells)


def test_rejects_bad_files(tmp_path):
    bad = tmp_path / "bad.msh"
    bad.write_text("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n")
    with pytest.raises(dg.DgcError):
        dg.read_msh(str(bad))
    bad.write_text("$MeshFormat\n4.1 0 8\n$EndMeshFormat\n$Nodes\n1 3 1 3\n2 1 0 3\n1\n3\n2\n"
                   "0 0 0\n1 0 0\n0 1 0\n$EndNodes\n$Elements\n1 1 1 1\n2 1 2 1\n1 1 2 3\n$EndElements\n")
    with pytest.raises(dg.DgcError):   # node tags out of file order
        dg.read_msh(str(bad))
    with pytest.raises(dg.DgcError):
        dg.read_msh(str(tmp_path / "missing.msh"))
