"""The rarefied-cavity workload as the reference builds it (tests/golden/workload_config2.npz: its
constructor's mesh and velocity tables, dumped by oracle/_ref/meso_ref --mesh-only) against the
product's host loader on the same generated case files, at full size (7744 cells, 15664 faces,
10201 velocities): every geometry table bit for bit, and the case settings, marks and initial fields
the CPU reference arm of bench.py reads from it without the product library."""
import os

import numpy as np

import cases
import meso_gpu as mg
import meso_oracle as mo
from conftest import GOLDEN

KEYS = ("cell_pos", "cell_vol", "cell_group", "cell_face_ptr", "cell_face", "cell_nbr_ptr", "cell_nbr", "lsq_w",
        "lsq_dr", "lsq_c", "face_cell", "face_pos", "face_area", "face_normal", "xi", "w", "sym")


def test_workload_tables_equal_the_host_loader(tmp_path):
    w = mo.Workload(os.path.join(GOLDEN, "workload_config2.npz"))
    c = mg.Case(cases.config2(str(tmp_path / "c2"), 500, "fp64"))
    a = c.arrays()
    assert (w.ncell, w.nv) == (c.ncell, c.nv) == (7744, 10201)
    for k in KEYS:
        x, y = np.asarray(a[k]).reshape(-1), np.asarray(w._a[k]).reshape(-1)
        assert x.shape == y.shape and np.array_equal(x, y), k
    assert np.array_equal(a["face_mark"], w._a["face_group"])
    assert a["min_cell_size"] == w.mesh.min_cell_size and a["total_volume"] == w.mesh.total_volume
    for f in ("dt", "R", "T0", "rho0", "mu0", "vhs_index", "Pr", "K", "gradient_switch", "limiter_switch"):
        assert getattr(c.params, f) == getattr(w.params, f), f
    for g in range(c.nmarks):
        m, n = c.marks_ptr[g], w.marks_ptr[g]
        assert (m.type, m.temperature_type, m.temperature, list(m.velocity)) == \
               (n.type, n.temperature_type, n.temperature, list(n.velocity)), g
    rho, u, T, mask = c.initial_fields()
    assert np.array_equal(rho, w.rho) and np.array_equal(u, w.u) and np.array_equal(T, w.T)
    c.close()
