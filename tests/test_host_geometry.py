"""Host layer: case-file parsing, Gambit reader, geometry and DVS vs the reference.

geometry_*.npz were dumped by the reference itself (tests/golden/make_golden.py);
the product's host library must rebuild the same tables bit for bit.
"""
import math
import os

import numpy as np
import pytest

import cases
import meso_gpu as mg
from conftest import GOLDEN

GEOM = [f[len("geometry_"):-4] for f in os.listdir(GOLDEN) if f.startswith("geometry_")]


@pytest.mark.parametrize("name", GEOM)
def test_geometry_bit_exact(name):
    ref = np.load(os.path.join(GOLDEN, f"geometry_{name}.npz"))
    a = mg.Case(os.path.join(GOLDEN, "cases", name, "case.txt")).arrays()
    assert a["ncell"] == int(ref["ncell"]) and a["nface"] == int(ref["nface"])
    for k in ("cell_pos", "cell_vol", "cell_nbr", "lsq_w", "lsq_c", "face_cell", "face_pos", "face_area",
              "face_normal", "xi", "w", "sym"):
        assert np.array_equal(a[k], ref[k]), k
    assert a["min_cell_size"] == float(ref["min_cell_size"])
    assert a["total_volume"] == float(ref["total_volume"])
    assert a["dvs_max_magnitude"] == float(ref["dvs_max_magnitude"])


def test_quad_mesh_counts(tmp_path):
    p = cases.bgk_cavity(str(tmp_path / "c"), 8, 10)
    a = mg.Case(p).arrays()
    assert a["ncell"] == 64 and a["nface"] == 2 * 8 * 9
    # every interior face has two distinct cells; boundary faces repeat their cell
    fc = a["face_cell"]
    bnd = fc[:, 0] == fc[:, 1]
    assert bnd.sum() == 32
    assert (a["face_mark"][bnd] > 0).all() and (a["face_mark"][~bnd] == 0).all()
    assert abs(a["cell_vol"].sum() - 1.0) < 1e-14 and abs(a["total_volume"] - 1.0) < 1e-14
    # least-squares gradient is exact for a linear field on interior cells
    pos = a["cell_pos"]
    phi = 0.3 * pos[:, 0] - 1.7 * pos[:, 1] + 2.0
    for c in range(a["ncell"]):
        s, e = a["cell_nbr_ptr"][c], a["cell_nbr_ptr"][c + 1]
        if e - s < 3:
            continue
        S = np.zeros(3)
        for j in range(s, e):
            S += a["lsq_w"][j] * (phi[a["cell_nbr"][j]] - phi[c]) * a["lsq_dr"][j]
        C = a["lsq_c"][c].reshape(3, 3)
        assert np.allclose(C @ S, [0.3, -1.7, 0.0], atol=1e-10)


def test_dvs_known_answers(tmp_path):
    # D2Q9 from gh-3: weights 4/9, 1/9, 1/36 (dvs_generator.cpp:32-39 scales by 1/sqrt(pi))
    p = cases.bgk_cavity(str(tmp_path / "b"), 4, 1)
    a = mg.Case(p).arrays()
    w = np.sort(a["w"])
    assert np.allclose(w, sorted([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4), rtol=1e-15, atol=1e-16)
    # half-range Gauss-Hermite 28: sum w exp(-x^2) = sqrt(pi) per axis
    x = cases.half_range_gh(str(tmp_path / "h.dvs"), 28)
    lines = open(str(tmp_path / "h.dvs")).read().split("\n")[1:29]
    ww = np.array([float(l.split()[1]) for l in lines])
    assert abs(np.sum(ww * np.exp(-x ** 2)) - math.sqrt(math.pi)) < 1e-13
    # Newton-Cotes trapezoid 101 points on [-5,5]: composite weights
    p = cases.shakhov_cavity(str(tmp_path / "n"), "quad", 4, "nc", 101, 1.0, 0.1, 1)
    a = mg.Case(p).arrays()
    assert a["nv"] == 101 * 101 and a["tensor_n"] == 101
    w1 = a["w"][:101] / a["w"][0] * 0.05
    assert abs(a["w"].sum() - 100.0) < 1e-9
    assert np.allclose(a["xi"][:101, 0], np.linspace(-5, 5, 101), atol=1e-12)


def test_config_defaults_and_patches(tmp_path):
    d = tmp_path / "c"
    p = cases.shakhov_cavity(str(d), "quad", 4, "hgh", 8, 0.1, 0.15, 5)
    # drop optional keys: the reference's defaults apply (cdugks_shakhov.cpp:10-20)
    txt = open(p).read().replace("Pr                  0.6666666666666667\n", "").replace(
        "vhs-index           0.5\n", "")
    open(p, "w").write(txt)
    c = mg.Case(p)
    assert abs(c.params.Pr - 0.67) < 1e-15 and abs(c.params.vhs_index - 0.81) < 1e-15
    assert c.params.solver == mg.SOLVER_CDUGKS_SHAKHOV and c.params.gradient_switch == 1
    rho, u, T, mask = c.initial_fields()
    assert (rho == 1.0).all() and (T == 1.0).all() and (u == 0.0).all() and (mask == 0).all()
    m = [c.marks_ptr[i] for i in range(c.nmarks)]
    lid = [x for x in m if x.velocity[0] != 0.0][0]
    assert lid.type == mg.BC["wall"] and abs(lid.velocity[0] - 0.15) < 1e-15 and lid.temperature == 1.0


def test_malformed_inputs_raise(tmp_path):
    with pytest.raises(mg.MesoError) as e:
        mg.Case(str(tmp_path / "missing.txt"))
    assert e.value.code == mg.ERR_IO
    p = cases.bgk_cavity(str(tmp_path / "x"), 4, 1)
    open(p, "a").write("\n[mark]\nname lid\ntype no-such-boundary\n")
    with pytest.raises(mg.MesoError) as e:
        mg.Case(p)
    assert e.value.code == mg.ERR_INVALID
    p = cases.bgk_cavity(str(tmp_path / "y"), 4, 1)
    open(p, "w").write(open(p).read().replace("solver              cdugks@incompressible", "solver nope"))
    with pytest.raises(mg.MesoError):
        mg.Case(p)
