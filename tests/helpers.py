"""Helpers shared by the tests: run a case through the GPU library or the oracle."""
from __future__ import annotations

import numpy as np

import meso_gpu as mg
import meso_oracle as mo


def relerr(a, b) -> float:
    """max |a-b| / max |b| (normwise relative error; fields that pass through 0 stay meaningful)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = float(np.max(np.abs(b))) if b.size else 0.0
    if scale == 0.0:
        return float(np.max(np.abs(a))) if a.size else 0.0
    return float(np.max(np.abs(a - b))) / scale


def run_gpu(case_path: str, nsteps: int, precision: int = mg.FP64):
    case = mg.Case(case_path)
    rho, u, T, mask = case.initial_fields()
    s = mg.Solver(case=case, precision=precision, mask=mask)
    s.init_macros(rho, u, T, None, 0)
    done = s.step(nsteps)
    out = s.macros(case.ncell)
    st = s.status()
    fm = s.flux_moments(case.ncell)
    s.close()
    return dict(rho=out[0], u=out[1], T=out[2], q=out[3], done=done, step=st.step, run_state=st.run_state,
                time=st.solution_time, fm=fm)


def run_oracle(case_path: str, nsteps: int, nthreads: int = 1):
    case = mg.Case(case_path)
    rho, u, T, mask = case.initial_fields()
    o = mo.Oracle(case, nthreads, mask)
    o.init(rho, u, T, None, 0)
    done, rc = o.step(nsteps)
    r, uu, t, q = o.macros()
    st = o.state()
    fm = o.flux_moments()
    o.close()
    return dict(rho=r, u=uu, T=t, q=q, done=done, step=st["step"], run_state=st["run_state"],
                time=st["solution_time"], fm=fm, rc=rc)


def max_field_err(a: dict, b: dict, shakhov: bool) -> dict:
    keys = ["rho", "u", "T", "q"] if shakhov else ["rho", "u"]
    return {k: relerr(a[k], b[k]) for k in keys}
