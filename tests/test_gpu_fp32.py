"""FP32-storage Shakhov step vs the FP64 step on the same inputs.

The FP32 form stores and streams g, h in FP32 and keeps the moment sums, the
equilibrium inputs, the Shakhov heat flux and the wall balance in FP64 (or
compensated FP32 partials combined in FP64).  Its error is stated against the
FP64 GPU step (itself pinned to the reference at 1e-12):
  * transients (tens of steps): max relative error (normwise) <= TOL_TRANSIENT
  * steady state: <= 1e-6 on rho, u, T
"""
import numpy as np
import pytest

import cases
import meso_gpu as mg
from helpers import relerr, run_gpu

TOL_TRANSIENT = {"rho": 2e-6, "u": 2e-5, "T": 2e-6, "q": 2e-4}

CASES = [
    ("quad_hgh8_kn0.1", lambda d: cases.shakhov_cavity(d, "quad", 10, "hgh", 8, 0.1, 0.15, 60), 60),
    ("mixed_nc21_kn1", lambda d: cases.shakhov_cavity(d, "mixed", 12, "nc", 21, 1.0, 0.15, 60), 60),
    ("jquad_nc21_kn1", lambda d: cases.shakhov_cavity(d, "jquad", 12, "nc", 21, 1.0, 0.15, 60), 60),
    ("quad_d2q9_kn0.05", lambda d: cases.shakhov_cavity(d, "quad", 10, "d2q9", 3, 0.05, 0.15, 60), 60),
    ("quad_hgh28_kn0.075", lambda d: cases.shakhov_cavity(d, "quad", 12, "hgh", 28, 0.075, 0.15, 40), 40),
    # NC 51^2 = 2601 velocities: the large-set kernels (warp-per-face sums, a block per boundary face)
    ("jquad_nc51_kn1", lambda d: cases.shakhov_cavity(d, "jquad", 8, "nc", 51, 1.0, 0.15, 40, seed=4), 40),
    ("quad_nograd", lambda d: cases.shakhov_cavity(d, "quad", 10, "hgh", 8, 0.1, 0.15, 40, gradient=False), 40),
    ("channel_pressure", lambda d: cases.shakhov_channel(d, "pressure", 12, 6, "hgh", 8, 0.2, 40), 40),
    ("channel_farfield", lambda d: cases.shakhov_channel(d, "farfield", steps=40), 40),
    ("channel_freestream", lambda d: cases.shakhov_channel(d, "freestream", steps=40), 40),
]


@pytest.mark.gpu
@pytest.mark.parametrize("name,build,steps", CASES, ids=[c[0] for c in CASES])
def test_fp32_matches_fp64_transient(gpu, tmp_path, name, build, steps):
    path = build(str(tmp_path / name))
    a = run_gpu(path, steps, mg.FP32)
    b = run_gpu(path, steps, mg.FP64)
    assert a["step"] == b["step"] == steps
    errs = {k: relerr(a[k], b[k]) for k in TOL_TRANSIENT}
    print(name, errs)
    for k, tol in TOL_TRANSIENT.items():
        assert errs[k] <= tol, (k, errs[k])
    # conservation: both forms conserve total mass of a closed cavity to rounding
    if name.startswith(("quad", "mixed")):
        c = mg.Case(path)
        vol = c.arrays()["cell_vol"]
        m0 = float(np.sum(vol))
        assert abs(float(np.sum(a["rho"] * vol)) - m0) / m0 < 1e-11


@pytest.mark.gpu
def test_fp32_steady_state_within_1e6(gpu, tmp_path):
    """Steady lid-driven cavity: FP32 storage within 1e-6 of FP64 on rho, u, T."""
    path = cases.shakhov_cavity(str(tmp_path / "ss"), "quad", 10, "hgh", 8, 0.1, 0.15, 3000)
    a = run_gpu(path, 3000, mg.FP32)
    b = run_gpu(path, 3000, mg.FP64)
    errs = {k: relerr(a[k], b[k]) for k in ("rho", "u", "T", "q")}
    print("steady", errs)
    for k in ("rho", "u", "T"):
        assert errs[k] <= 1e-6, (k, errs[k])


@pytest.mark.gpu
def test_fp32_snapshot_restore_is_exact(gpu, tmp_path):
    path = cases.shakhov_cavity(str(tmp_path / "snap"), "quad", 8, "hgh", 8, 0.1, 0.15, 20)
    case = mg.Case(path)
    rho, u, T, mask = case.initial_fields()
    s = mg.Solver(case=case, precision=mg.FP32, mask=mask)
    s.init_macros(rho, u, T, None, 0)
    s.step(10)
    snap = s.snapshot()
    s.step(10)
    ref = s.macros(case.ncell)
    s.restore(snap)
    assert s.status().step == 10
    s.step(10)
    out = s.macros(case.ncell)
    for x, y in zip(out, ref):
        assert np.array_equal(x, y)
    s.close()


@pytest.mark.gpu
def test_fp32_rejects_what_it_does_not_cover(gpu, tmp_path):
    path = cases.bgk_cavity(str(tmp_path / "bgk"), 6, 5)
    with pytest.raises(mg.MesoError) as e:
        mg.Solver(path, mg.FP32)
    assert e.value.code == mg.ERR_UNSUPPORTED
    path = cases.shakhov_cavity(str(tmp_path / "lim"), "quad", 6, "hgh", 8, 0.1, 0.15, 5, limiter=True)
    with pytest.raises(mg.MesoError) as e:
        mg.Solver(path, mg.FP32)
    assert e.value.code == mg.ERR_UNSUPPORTED
