"""Where the FP32-storage form's error at steady state comes from, on a rarefied cavity.

A 16x16 jittered-quad cavity, NC 21^2 velocities, Kn 1, lid 0.15 (the rarefied workload's regime,
small enough to reach steady state in seconds), 6000 steps with the residual check off:

* the FP32 form against the FP64 GPU step (itself the reference's step to 1e-12);
* the oracle (FP64) with its storage-rounding hook: after every step the stored g - g0, h - h0 are
  rounded to FP32 and nothing else changes, i.e. the FP32 form's storage rounding in isolation.

At steady state the FP32 error is that of the storage rounding: rounding the state's deviations
to FP32 every step already moves the steady fields by u ~1e-5 (relative to max |u|), because the
per-step rounding of ~6e-8 |g - g0| is integrated over the thousands of steps it takes the cavity to
settle.  The FP32 form's own error stays within twice that of the rounding alone (its FP32
arithmetic and face values add little), and both are printed; the 1e-6 steady-state bar is met by
rho and T, not by the velocity, on rarefied cavities.
"""
import os

import numpy as np
import pytest

import cases
import meso_gpu as mg
import meso_oracle as mo
from helpers import relerr

STEPS = 6000


def _errs(a, b):
    return {"rho": relerr(a[0], b[0]), "u": relerr(a[1][:, 0], b[1][:, 0]), "v": relerr(a[1][:, 1], b[1][:, 1]),
            "T": relerr(a[2], b[2])}


@pytest.mark.gpu
def test_fp32_steady_error_is_the_storage_rounding(gpu, tmp_path):
    path = cases.shakhov_cavity(str(tmp_path / "c"), "jquad", 16, "nc", 21, 1.0, 0.15, 10 ** 6, seed=0, name="c")
    case = mg.Case(path)
    rho, u, T, mask = case.initial_fields()
    out = {}
    for prec in (mg.FP64, mg.FP32):
        prm = case.params
        prm.residual_interval = 0  # every step runs
        s = mg.Solver(case=case, precision=prec, mask=mask, params=prm)
        s.init_macros(rho, u, T, None, 0)
        s.step(STEPS - 500)
        before = s.macros(case.ncell)
        s.step(500)
        out[prec] = (before, s.macros(case.ncell))
        s.close()
    prm = case.params
    prm.residual_interval = 0
    o = mo.Oracle(case, os.cpu_count() or 1, mask, params=prm)
    o.set_storage_rounding(True)
    o.init(rho, u, T, None, 0)
    o.step(STEPS)
    rounded = o.macros()
    o.close()
    f64 = out[mg.FP64][1]
    drift = _errs(out[mg.FP64][0], f64)
    e32 = _errs(out[mg.FP32][1], f64)
    eround = _errs(rounded, f64)
    print("FP64 change over the last 500 steps:", drift, "\nFP32 form:", e32, "\nFP32 storage rounding alone:",
          eround)
    assert drift["u"] <= 1e-7, drift  # steady state
    for k in e32:
        assert e32[k] <= 2.0 * eround[k], (k, e32[k], eround[k])
    assert e32["rho"] <= 1e-5 and e32["T"] <= 1e-6 and e32["u"] <= 5e-5 and e32["v"] <= 5e-5, e32
