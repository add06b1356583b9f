"""Masked cells (cell_value_interp, cdugks_shakhov.cpp:697-719, 766-789): a cell that turns NaN or
T < 0 inside the mask is re-equilibrated from its neighbours instead of stopping the run, in both
the FP64 and the FP32 forms; outside the mask the run stops with MESO_ERR_NAN."""
import numpy as np
import pytest

import cases
import meso_gpu as mg


def _blowup(tmp_path):
    # CFL 30: the scheme is unstable and cells go bad within a few steps
    return cases.shakhov_cavity(str(tmp_path / "b"), "quad", 8, "hgh", 8, 0.1, 0.15, 40, cfl=30.0)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [mg.FP64, mg.FP32], ids=["fp64", "fp32"])
def test_masked_cells_are_repaired(gpu, tmp_path, prec):
    path = _blowup(tmp_path)
    case = mg.Case(path)
    rho, u, T, _ = case.initial_fields()
    s = mg.Solver(case=case, precision=prec, mask=np.ones(case.ncell, np.uint8))
    s.init_macros(rho, u, T, None, 0)
    done = s.step(4)
    st = s.status()
    assert done == 4 and st.run_state == 1
    assert st.bad_cells > 0 and st.masked_repairs > 0
    s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [mg.FP64, mg.FP32], ids=["fp64", "fp32"])
def test_unmasked_bad_cell_stops_the_run(gpu, tmp_path, prec):
    path = _blowup(tmp_path)
    case = mg.Case(path)
    rho, u, T, _ = case.initial_fields()
    s = mg.Solver(case=case, precision=prec, mask=np.zeros(case.ncell, np.uint8))
    s.init_macros(rho, u, T, None, 0)
    with pytest.raises(mg.MesoError) as e:
        s.step(40)
    assert e.value.code == mg.ERR_NAN
    st = s.status()
    assert st.run_state == 0 and st.converged == 0 and st.first_bad_cell >= 0
    s.close()
