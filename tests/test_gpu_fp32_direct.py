"""The FP32-storage step against the reference's own outputs directly (no FP64 GPU step in between).

tests/golden/*.npz hold the fields the unmodified reference produced on the committed inputs; the
FP32 form runs the same cases and is measured against them with the transient bars of
test_gpu_fp32.py (rho 2e-6, u 2e-5, T 2e-6, q 2e-4, max norm relative to the field's largest
magnitude; the heat flux against max(|q|, 1 % of rho (R T)^(3/2)), the size of its terms, as in
test_gpu_fp64_parity.py).  The cases cover both velocity-set classes of the FP32 kernels: small
sets (hGH 8^2, NC 21^2, D2Q9, the reference's own NC 41^2 on +-1500 with R = 208, T = 273) and large
ones (the reference's gambit velocity mesh of 2990 points, and NC 51^2 against the oracle).
"""
import os

import numpy as np
import pytest

import cases
import meso_gpu as mg
from conftest import GOLDEN
from helpers import golden_case, relerr, run_gpu, run_oracle
from test_gpu_fp64_parity import q_err

TOL = {"rho": 2e-6, "u": 2e-5, "T": 2e-6, "q": 2e-4}

GOLDENS = ["shakhov_q8_hgh8", "shakhov_m10_nc21", "shakhov_t8_nc21", "shakhov_q8_d2q9", "shakhov_q8_nograd",
           "channel_pressure", "channel_farfield", "ref_re1000", "ref_kn0075", "ref_neumann"]


def _errs(r, g, R):
    return {"rho": relerr(r["rho"], g["rho"]), "u": relerr(r["u"], g["u"]), "T": relerr(r["T"], g["T"]),
            "q": q_err(r["q"], g, R)}


@pytest.mark.gpu
@pytest.mark.parametrize("name", GOLDENS)
def test_fp32_matches_reference_outputs(gpu, name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    path = golden_case(name)
    case = mg.Case(path)
    nv, R = case.nv, case.params.R
    case.close()
    r = run_gpu(path, int(g["requested"]), mg.FP32)
    assert r["step"] == int(g["step"]) and r["run_state"] == int(g["run_state"]) == 1
    errs = _errs(r, g, R)
    print(name, nv, errs)
    for k, tol in TOL.items():
        assert errs[k] <= tol, (name, k, errs[k])


@pytest.mark.gpu
def test_fp32_large_set_matches_oracle(gpu, tmp_path):
    """NC 51^2 (2601 velocities, the large-set kernels) on a jittered-quad cavity, 40 steps, against
    the oracle at one thread (bit-exact with the reference)."""
    path = cases.shakhov_cavity(str(tmp_path / "nc51"), "jquad", 8, "nc", 51, 1.0, 0.15, 40, seed=4)
    r = run_gpu(path, 40, mg.FP32)
    o = run_oracle(path, 40)
    errs = {"rho": relerr(r["rho"], o["rho"]), "u": relerr(r["u"], o["u"]), "T": relerr(r["T"], o["T"]),
            "q": relerr(r["q"], o["q"])}
    print(errs)
    for k, tol in TOL.items():
        assert errs[k] <= tol, (k, errs[k])
