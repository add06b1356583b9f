"""Defect correction of the FP32 form (meso_fp32_refine).

Every K-th step runs the plain FP64 step (the reference's arithmetic, 1e-12 of the reference) and
the FP32 step from the same state; their difference becomes a correction that the following FP32
steps add to their results (state, conservative update, heat flux), the state rounded
stochastically.  On the rarefied 16x16 cavity of test_gpu_fp32_steady.py (NC 21^2, Kn 1,
6000 steps, steady), where the plain FP32 form settles u ~1e-5 away from the FP64 steady state,
K = 10 brings it within the 1e-6 steady-state bar.
"""
import numpy as np
import pytest

import cases
import meso_gpu as mg
from helpers import relerr

STEPS = 6000


def _errs(a, b):
    return {"rho": relerr(a[0], b[0]), "u": relerr(a[1][:, 0], b[1][:, 0]), "v": relerr(a[1][:, 1], b[1][:, 1]),
            "T": relerr(a[2], b[2]), "q": relerr(a[3][:, :2], b[3][:, :2])}


def _solver(case, prec, rho, u, T, mask):
    prm = case.params
    prm.residual_interval = 0
    s = mg.Solver(case=case, precision=prec, mask=mask, params=prm)
    s.init_macros(rho, u, T, None, 0)
    return s


@pytest.mark.gpu
def test_refined_fp32_meets_the_steady_state_bar(gpu, tmp_path):
    path = cases.shakhov_cavity(str(tmp_path / "c"), "jquad", 16, "nc", 21, 1.0, 0.15, 10 ** 6, seed=0, name="c")
    case = mg.Case(path)
    rho, u, T, mask = case.initial_fields()
    out = {}
    for key in ("fp64", "fp32", "refined"):
        s = _solver(case, mg.FP64 if key == "fp64" else mg.FP32, rho, u, T, mask)
        if key == "refined":
            s.refine(10)
        s.step(STEPS - 500)
        before = s.macros(case.ncell)
        s.step(500)
        out[key] = (before, s.macros(case.ncell))
        s.close()
    f64 = out["fp64"][1]
    drift = _errs(out["fp64"][0], f64)
    e32, eref = _errs(out["fp32"][1], f64), _errs(out["refined"][1], f64)
    print("FP64 change over the last 500 steps", drift, "\nFP32", e32, "\nFP32 refined every 10 steps", eref)
    assert drift["u"] <= 1e-7  # steady state
    for k in ("rho", "u", "v", "T"):
        assert eref[k] <= 1e-6, (k, eref[k])
    assert eref["u"] <= e32["u"] / 5 and eref["v"] <= e32["v"] / 5, (eref, e32)


@pytest.mark.gpu
def test_refinement_step_is_the_fp64_step(gpu, tmp_path):
    """A refinement step continues from the FP64 step's result: the first step of a refined FP32
    solve equals the FP64 solve's first step to the FP32 rounding of the initial deviations (the
    velocity compared against the largest speed: the cross-lid component is still near zero), and
    the corrected steps after it stay at the FP32 form's transient error or below."""
    path = cases.shakhov_cavity(str(tmp_path / "c"), "jquad", 8, "nc", 21, 1.0, 0.15, 10 ** 6, seed=0, name="c")
    case = mg.Case(path)
    rho, u, T, mask = case.initial_fields()
    s64 = _solver(case, mg.FP64, rho, u, T, mask)
    s32 = _solver(case, mg.FP32, rho, u, T, mask)
    ref = _solver(case, mg.FP32, rho, u, T, mask)
    ref.refine(5)
    for k in range(12):
        for s in (s64, s32, ref):
            s.step(1)
        a, b, c = (s.macros(case.ncell) for s in (s64, s32, ref))
        e32, eref = _errs(b, a), _errs(c, a)
        if k == 0:
            speed = float(np.max(np.abs(a[1])))
            dv = float(np.max(np.abs(c[1] - a[1]))) / speed
            assert eref["rho"] <= 1e-12 and eref["T"] <= 1e-12 and dv <= 1e-9, (eref, dv)
        for key in ("rho", "u", "T"):
            assert eref[key] <= max(2.0 * e32[key], 1e-9), (k, key, eref[key], e32[key])
    for s in (s64, s32, ref):
        s.close()


@pytest.mark.gpu
def test_refine_rules(gpu, tmp_path):
    path = cases.shakhov_cavity(str(tmp_path / "c"), "jquad", 6, "nc", 21, 1.0, 0.15, 10 ** 6, seed=0, name="c")
    case = mg.Case(path)
    rho, u, T, mask = case.initial_fields()
    s64 = _solver(case, mg.FP64, rho, u, T, mask)
    with pytest.raises(mg.MesoError) as e:
        s64.refine(10)
    assert e.value.code == mg.ERR_UNSUPPORTED
    s32 = _solver(case, mg.FP32, rho, u, T, mask)
    with pytest.raises(mg.MesoError) as e:
        s32.refine(-1)
    assert e.value.code == mg.ERR_INVALID
    s32.refine(4)
    with pytest.raises(mg.MesoError) as e:
        mg.Batch([s32])
    assert e.value.code == mg.ERR_UNSUPPORTED
    # new settings keep the correction (the step constants reach the FP64 step too)
    s32.step(4)
    prm = s32.params
    prm.dt = prm.dt * 0.5
    s32.set_params(prm)
    s32.step(8)
    ref64 = _solver(case, mg.FP64, rho, u, T, mask)
    ref64.step(4)
    p64 = mg.Params.from_buffer_copy(prm)
    p64.precision = mg.FP64
    ref64.set_params(p64)
    ref64.step(8)
    e = _errs(s32.macros(case.ncell), ref64.macros(case.ncell))
    assert e["rho"] <= 1e-7 and e["T"] <= 1e-7 and e["u"] <= 1e-5, e
    ref64.close()
    # switched off, the solve steps as a plain FP32 solve again (and may join a batch)
    s32.refine(0)
    s32.step(8)
    b = mg.Batch([s32])
    b.close()
    for s in (s64, s32):
        s.close()
