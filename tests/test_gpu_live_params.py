"""Step settings changed between steps take effect at the next step (the reference re-reads its
case file's [settings] after every step, cdugks_shakhov.cpp:762), also when the step is replayed
from a captured CUDA graph.

A solve stepped with one time step and Prandtl number, then changed through meso_set_params and
stepped on, must equal the same first steps, a snapshot, and a fresh context created with the new
settings that restores the snapshot and steps on.
"""
import numpy as np
import pytest

import cases
import meso_gpu as mg


def _solver(case, precision, params=None):
    rho, u, T, mask = case.initial_fields()
    s = mg.Solver(case=case, precision=precision, mask=mask, params=params)
    s.init_macros(rho, u, T, None, 0)
    return s


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [mg.FP64, mg.FP32], ids=["fp64", "fp32"])
def test_changed_settings_apply_to_later_steps(gpu, tmp_path, precision):
    case = mg.Case(cases.shakhov_cavity(str(tmp_path / "c"), "quad", 10, "hgh", 8, 0.1, 0.15, 40))
    a = _solver(case, precision)
    a.step(10)
    snap = a.snapshot()
    p = mg.Params.from_buffer_copy(a.params)
    p.dt *= 0.8
    p.Pr = 0.7
    a.set_params(p)
    a.step(10)
    out_a, st_a = a.macros(case.ncell), a.status()
    a.close()

    p2 = mg.Params.from_buffer_copy(case.params)
    p2.dt, p2.Pr = p.dt, p.Pr
    b = _solver(case, precision, params=p2)
    b.restore(snap)
    b.step(10)
    out_b, st_b = b.macros(case.ncell), b.status()
    b.close()

    assert st_a.step == st_b.step == 20
    for k, x, y in zip(("rho", "u", "T", "q"), out_a, out_b):
        assert np.array_equal(x, y), k
    # and the change mattered: the old settings give another state
    c = _solver(case, precision)
    c.step(20)
    assert not np.array_equal(c.macros(case.ncell)[0], out_a[0])
    c.close()
