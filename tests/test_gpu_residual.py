"""The residual check and the convergence counter of do_step (field.cpp:223-249, core.cpp:45-51,
cdugks_shakhov.cpp:729-757, cdugks.cpp:343-368).

Two cases the reference itself runs to convergence (tests/golden/*_converge.npz: run_state 0 by
convergence at the stored step): an 8x8 BGK cavity with residual-limit 1e-5 (converged at step
37800) and an 8x8 Shakhov cavity (hGH 8^2, Kn 0.1) with the default limit 1e-6 (step 1600).

* FP64: the GPU stops at the reference's step with converged = 1, its fields within 1e-12 of the
  reference's, and the residual list of its last check (the reference's print order) within 1e-4
  relative (or 1e-10 absolute) of the oracle's: the residuals are sums of |new - old| / |old| over
  cells, each term a difference of nearly equal fields (relative changes of 1e-7 and below at
  convergence), so the fields' 1e-13 differences reach them amplified by up to 1e6.
* FP32 (Shakhov): the device-side check on rho, T and u converges within two checks (200 steps)
  of the FP64 step with the same fields watched, its fields within 1e-6 of FP64's there.
"""
import os

import numpy as np
import pytest

import meso_gpu as mg
import meso_oracle as mo
from conftest import GOLDEN
from helpers import golden_case, relerr

LIMIT = {"cdugks_q8_converge": 1e-5, "shakhov_q8_converge": 1e-6}  # their residual-limit settings


def _oracle_residual(path: str, steps: int):
    case = mg.Case(path)
    rho, u, T, mask = case.initial_fields()
    o = mo.Oracle(case, 1, mask)
    o.init(rho, u, T, None, 0)
    o.step(steps)
    st = o.state()
    res = o.residual()
    o.close()
    return st, res


def _gpu(path: str, steps: int, precision: int):
    case = mg.Case(path)
    rho, u, T, mask = case.initial_fields()
    s = mg.Solver(case=case, precision=precision, mask=mask)
    s.init_macros(rho, u, T, None, 0)
    done = s.step(steps)
    st = s.status()
    out = s.macros(case.ncell)
    s.close()
    return done, st, np.array(st.residual[:st.nresidual]), out


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["cdugks_q8_converge", "shakhov_q8_converge"])
def test_fp64_converges_at_the_reference_step(gpu, name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    assert int(g["run_state"]) == 0
    path = golden_case(name)
    done, st, res, out = _gpu(path, int(g["requested"]), mg.FP64)
    assert st.step == int(g["step"]) and st.run_state == 0 and st.converged == 1, (st.step, int(g["step"]))
    for k, a in zip(("rho", "u", "T", "q"), out):
        assert relerr(a, g[k]) <= 1e-12, (k, relerr(a, g[k]))
    ost, ores = _oracle_residual(path, int(g["requested"]))
    assert ost["step"] == st.step and ost["converged"] == 1
    assert res.shape == ores.shape and res.size in (3, 6), (res, ores)
    print(name, res, ores)
    for a, b in zip(res, ores):
        assert abs(a - b) <= 1e-4 * abs(b) + 1e-10, (a, b)
        assert a <= LIMIT[name]


@pytest.mark.gpu
def test_fp32_converges_near_the_fp64_step(gpu):
    """The FP32 form's device-side check on rho, T and u (MESO_RES_RHO | T | U): the heat flux of FP32
    storage moves by about 4e-6 of itself from one check to the next (its floor under the reference's
    mean of |new - old| / |old|), so a check that watches q does not reach 1e-6 in FP32."""
    g = np.load(os.path.join(GOLDEN, "shakhov_q8_converge.npz"))
    path = golden_case("shakhov_q8_converge")
    out = {}
    for prec in (mg.FP64, mg.FP32):
        case = mg.Case(path)
        rho, u, T, mask = case.initial_fields()
        prm = case.params
        prm.residual_fields = mg.RES_RHO | mg.RES_T | mg.RES_U
        s = mg.Solver(case=case, precision=prec, mask=mask, params=prm)
        s.init_macros(rho, u, T, None, 0)
        s.step(int(g["requested"]))
        st = s.status()
        out[prec] = (st.step, st.converged, np.array(st.residual[:st.nresidual]), s.macros(case.ncell))
        s.close()
    print("fp64", out[mg.FP64][:3], "fp32", out[mg.FP32][:3])
    for prec in (mg.FP64, mg.FP32):
        assert out[prec][1] == 1
        assert np.all(out[prec][2][:4] <= 1e-6)
    assert abs(out[mg.FP32][0] - out[mg.FP64][0]) <= 200, (out[mg.FP32][0], out[mg.FP64][0])
    for k, a, b in zip(("rho", "u", "T"), out[mg.FP32][3], out[mg.FP64][3]):
        assert relerr(a, b) <= 1e-6, (k, relerr(a, b))
