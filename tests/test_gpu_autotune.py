"""FP32 kernel-shape autotuner (meso_autotune*): picks a valid shape, remembers it
for solves of the same size, and a tuned solve keeps the FP32 accuracy bar."""
import pytest

import cases
import meso_gpu as mg
from helpers import relerr

TOL = {"rho": 2e-6, "u": 2e-5, "T": 2e-6}


@pytest.mark.gpu
def test_autotune_picks_and_remembers_a_shape(gpu, tmp_path):
    path = cases.shakhov_cavity(str(tmp_path / "t"), "quad", 16, "hgh", 28, 0.1, 0.15, 30, cfl=0.5)
    try:
        best, ms = mg.autotune(path, steps=3)
        assert ms > 0.0
        assert best.tile_cells in (24, 32, 40, 48) and best.vpl in (1, 2) and best.ngroup >= 0
        case = mg.Case(path)
        rho, u, T, mask = case.initial_fields()
        s = mg.Solver(case=case, precision=mg.FP32, mask=mask)  # shape 0: the remembered one
        assert (s.params.tile_cells, s.params.vpl, s.params.ngroup) == (best.tile_cells, best.vpl, best.ngroup)
        s.init_macros(rho, u, T, None, 0)
        s.step(30)
        a = s.macros(case.ncell)
        s.close()
        r = mg.Solver(case=case, precision=mg.FP64, mask=mask)
        r.init_macros(rho, u, T, None, 0)
        r.step(30)
        b = r.macros(case.ncell)
        r.close()
        for k, x, y in zip(("rho", "u", "T"), a, b):
            assert relerr(x, y) <= TOL[k], k
    finally:
        mg.lib().meso_autotune_forget()
