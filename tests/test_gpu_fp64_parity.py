"""FP64 plain GPU step vs the reference.

Two checks per case, both at max relative error <= 1e-12 on every
macroscopic field (normwise: max|a-b| / max|b|):
  * against the reference's own outputs in tests/golden/ (same inputs),
  * against the oracle on freshly generated inputs (arbitrary step counts).
The oracle is pinned bit-exact to the reference by test_oracle_golden.py.
Cases cover the three solvers; quad, mixed quad/triangle and triangle meshes;
hGH, Newton-Cotes and Sparse velocity sets; the limiter and gradient-off
paths; pressure / farfield inlets and outlets, symmetry, slip and diffuse
walls; and the NaN monitor stopping the run at the reference's step.
"""
import os

import numpy as np
import pytest

import cases
import meso_gpu as mg
from conftest import GOLDEN
from helpers import (RESTART_GOLDENS, copy_golden_case, golden_case, golden_names, max_field_err, relerr,
                     run_gpu, run_gpu_case_initial, run_oracle)

TOL = 1e-12
THRESHOLD_SENSITIVE = {"shakhov_q8_limiter"}
# the BGK solvers have no temperature or heat flux: their T and q fields are zero on both sides
GOLDEN_NAMES = golden_names()


@pytest.mark.gpu
@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_fp64_matches_reference_outputs(gpu, name, tmp_path):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    path = golden_case(name)
    steps = int(g["requested"])
    if name in RESTART_GOLDENS:  # initial() from the first run's latest/ files (read-np-data True)
        r = run_gpu_case_initial(copy_golden_case(name, str(tmp_path / name)), steps, mg.FP64)
        assert r["step"] == int(g["step"])
        for k in ("rho", "u", "T", "q"):
            assert relerr(r[k], g[k]) <= TOL, (k, relerr(r[k], g[k]))
        return
    try:
        r = run_gpu(path, steps, mg.FP64)
    except mg.MesoError as e:
        # the reference stopped on a NaN / T<0 cell: the GPU must stop at the same step
        assert e.code == mg.ERR_NAN and int(g["run_state"]) == 0
        s = mg.Solver(path, mg.FP64)
        s.initial()
        with pytest.raises(mg.MesoError):
            s.step(steps)
        st = s.status()
        assert st.step == int(g["step"]) and st.run_state == 0 and st.bad_cells > 0
        s.close()
        return
    assert r["step"] == int(g["step"]) and r["run_state"] == int(g["run_state"])
    tol = dict.fromkeys(("rho", "u", "T", "q"), TOL)
    if name in THRESHOLD_SENSITIVE:
        # The Venkatakrishnan limiter returns 1 when |dw| <= eps (limiter.cpp:11), a jump that turns
        # 1e-16 summation-order differences into O(1e-5) field differences.  The reference run on two
        # velocity slices (its 2-rank MPI path) already differs from its 1-rank run by that much; the
        # GPU must stay inside 4x that envelope.
        o2 = run_oracle(path, steps, nthreads=2)
        tol = {k: max(TOL, 4.0 * relerr(o2[k], g[k])) for k in tol}
    for k in ("rho", "u", "T"):
        assert relerr(r[k], g[k]) <= tol[k], (k, relerr(r[k], g[k]), tol[k])
    assert q_err(r["q"], g, mg.Case(path).params.R) <= tol["q"], (q_err(r["q"], g, mg.Case(path).params.R), tol["q"])


def q_err(q, g, R: float) -> float:
    """Heat-flux error: max |q - q_ref| over max |q_ref|, where q_ref is at least 1 % of the size
    rho (R T)^(3/2) of the terms of its velocity sum.  In near-continuum cases (ref_re1000: Kn 1.8e-4)
    the heat flux itself is a thousand times smaller than its terms, and its last bits are the
    rounding of their sum."""
    scale = max(float(np.max(np.abs(g["q"]))), 0.01 * float(np.max(g["rho"])) * (R * float(np.max(g["T"]))) ** 1.5)
    return float(np.max(np.abs(np.asarray(q) - g["q"]))) / scale if scale > 0 else 0.0


CASES = [
    ("cdugks_q12", lambda d: cases.bgk_cavity(d, 12, 150), 150, False),
    ("dugks_q12", lambda d: cases.bgk_cavity(d, 12, 150, solver="dugks@incompressible"), 150, False),
    ("shakhov_m12_hgh8", lambda d: cases.shakhov_cavity(d, "mixed", 12, "hgh", 8, 0.075, 0.15, 60), 60, True),
    ("shakhov_q10_nc31", lambda d: cases.shakhov_cavity(d, "quad", 10, "nc", 31, 1.0, 0.15, 40), 40, True),
    ("channel_pressure_nc", lambda d: cases.shakhov_channel(d, "pressure", 12, 6, "nc", 21, 0.2, 40), 40, True),
    ("channel_freestream", lambda d: cases.shakhov_channel(d, "freestream", steps=40), 40, True),
]


@pytest.mark.gpu
@pytest.mark.parametrize("name,build,steps,shakhov", CASES, ids=[c[0] for c in CASES])
def test_fp64_matches_oracle(gpu, tmp_path, name, build, steps, shakhov):
    path = build(str(tmp_path / name))
    g = run_gpu(path, steps, mg.FP64)
    o = run_oracle(path, steps)
    assert g["step"] == o["step"] == steps
    errs = max_field_err(g, o, shakhov)
    assert all(v <= TOL for v in errs.values()), errs
    assert abs(g["time"] - o["time"]) <= 1e-12 * max(1.0, abs(o["time"]))
    if shakhov:
        for a, b in zip(g["fm"], o["fm"]):
            assert relerr(a, b) <= 1e-9


@pytest.mark.gpu
def test_case_context_initial_and_output(gpu, tmp_path):
    """The case-file path: meso_ctx_create_from_case + initial() + output() writes the reference's files."""
    path = cases.shakhov_cavity(str(tmp_path / "o"), "quad", 6, "hgh", 8, 0.1, 0.15, 5)
    s = mg.Solver(path, mg.FP64)
    s.initial()
    s.output()
    assert s.step(5) == 5
    s.output()
    base = tmp_path / "o" / "shakhov"
    assert (base / "grid.plt").exists() and (base / "step-5" / "data.plt").exists()
    rho = np.loadtxt(base / "latest" / "Rho")
    o = run_oracle(path, 5)
    assert relerr(rho, o["rho"]) <= 1e-12  # 18-digit text round-trips FP64
    s.close()
