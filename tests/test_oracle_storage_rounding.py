"""Why FP32 storage rounding moves the steady state: rounding to nearest is deterministic, so at a
(near-)steady state the same stored values are rounded the same way every step and the per-step
errors add up coherently along the slowest relaxation modes instead of averaging out.

An 8x8 jittered-quad cavity, NC 21^2 velocities, Kn 1, lid 0.15, 4000 steps (steady: the FP64
fields change by ~1e-13 over the last 500 steps), oracle only (CPU), the stored g - g0, h - h0
rounded to FP32 after every step:

* to nearest: the velocity moves by ~5e-6 of max |u|;
* stochastically (up with probability equal to the distance from the float below, a hash of cell,
  velocity and step for the draw): ~6e-8, two orders of magnitude less for the same per-step
  rounding size.

The FP32 form's own error at steady state has a second source of the same size, its FP32
arithmetic (deterministic too): with stochastic rounding applied to the update kernel's store the
GPU's steady-state velocity error stays where it was, so the product rounds to nearest.
"""
import os

import numpy as np

import cases
import meso_gpu as mg
import meso_oracle as mo
from helpers import relerr

STEPS = 4000


def test_stochastic_storage_rounding_removes_the_coherent_drift(tmp_path):
    path = cases.shakhov_cavity(str(tmp_path / "c"), "jquad", 8, "nc", 21, 1.0, 0.15, 10 ** 6, seed=0, name="c")
    case = mg.Case(path)
    rho, u, T, mask = case.initial_fields()
    out = {}
    for mode in ("fp64", "nearest", "stochastic"):
        prm = case.params
        prm.residual_interval = 0
        o = mo.Oracle(case, os.cpu_count() or 1, mask, params=prm)
        if mode != "fp64":
            o.set_storage_rounding(True, stochastic=(mode == "stochastic"))
        o.init(rho, u, T, None, 0)
        o.step(STEPS - 500)
        before = o.macros()
        o.step(500)
        out[mode] = (before, o.macros())
        o.close()
    case.close()
    ref = out["fp64"][1]
    drift = relerr(out["fp64"][0][1][:, 0], ref[1][:, 0])
    e = {m: max(relerr(out[m][1][1][:, 0], ref[1][:, 0]), relerr(out[m][1][1][:, 1], ref[1][:, 1]))
         for m in ("nearest", "stochastic")}
    print("FP64 change over the last 500 steps", drift, "velocity error", e)
    assert drift <= 1e-10
    assert e["nearest"] >= 1e-6, e
    assert e["stochastic"] <= 3e-7 and e["stochastic"] <= e["nearest"] / 20, e
