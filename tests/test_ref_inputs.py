"""The reference's own shipped inputs, loaded by the host library (no GPU).

tests/golden/cases/ref_* hold files/cavity.neu with case-re400.txt, case-re1000.txt and
case-kn0.075.txt, and files/case-neumann.txt with its gambit physical and velocity meshes, copied
verbatim from the reference (tests/golden/make_golden.py).
"""
import os

import numpy as np
import pytest

import meso_gpu as mg
from conftest import GOLDEN
from helpers import golden_case


def test_cavity_neu_counts(tmp_path):
    """files/cavity.neu: 1717 nodes, 1928 cells (mixed quads and triangles), 3644 faces, 40 lid and
    120 wall faces."""
    c = mg.Case(golden_case("ref_re400"))
    a = c.arrays()
    assert c.ncell == 1928 and a["nface"] == 3644
    marks = np.bincount(a["face_mark"], minlength=3)
    assert int((a["face_cell"][:, 0] == a["face_cell"][:, 1]).sum()) == 160
    assert sorted(marks[1:].tolist()) == [40, 120], marks
    grid = tmp_path / "grid.plt"
    c.output_grid(str(grid))
    zone = [line for line in open(grid) if line.startswith("ZONE")][0]
    assert "N=1717," in zone and "E=1928," in zone, zone
    c.close()


@pytest.mark.parametrize("name,nv,dim", [("ref_re400", 9, 2), ("ref_re1000", 64, 2), ("ref_kn0075", 1681, 2),
                                         ("ref_neumann", 2990, 2)])
def test_reference_cases_load(name, nv, dim):
    c = mg.Case(golden_case(name))
    assert c.nv == nv and c.mesh.dim == dim
    a = c.arrays()
    # every velocity set integrates the weight function it was built for to the quadrature's accuracy
    assert np.all(a["w"] > 0.0) and np.isfinite(a["xi"]).all()
    rho, u, T, mask = c.initial_fields()
    assert np.all(rho > 0.0)
    c.close()


def test_neumann_groups_initialise_four_states():
    """case-neumann.txt sets four cell groups (RU, LU, LD, RD) to different states."""
    c = mg.Case(golden_case("ref_neumann"))
    rho, u, T, mask = c.initial_fields()
    assert sorted(set(np.round(rho, 6).tolist())) == [0.5313, 0.8, 1.0]
    assert sorted(set(np.round(T, 7).tolist())) == [1.5057406, 2.0, 2.5]
    assert c.ncell == 2216
    c.close()


def test_grid_file_matches_the_reference(tmp_path):
    """Mesh::output_grid (mesh_output.cpp:182-215) on the host against the reference's own grid.plt."""
    from test_gpu_output import _compare

    for name in ("out_shakhov_q8", "out_cdugks_q8"):
        c = mg.Case(golden_case(name))
        out = tmp_path / f"{name}.plt"
        c.output_grid(str(out))
        _compare(str(out), os.path.join(GOLDEN, "output", name, "grid.plt"))
        c.close()
