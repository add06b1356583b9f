"""The transitional-cavity workload at its full size: 61x61 quads, half-range Gauss-Hermite 28x28
velocities (784), Shakhov, Kn 0.075, lid 0.15, CFL 0.5.

* FP64 GPU step against the oracle (all host threads, the reference's velocity-slice split) after
  500 steps: the parity bar, max relative error <= 1e-12 on rho, u, T, q.
* FP32-storage step against the FP64 GPU step after the workload's 5000 steps, on rho, T, u, v,
  qx, qy (max norm relative to the field's largest magnitude).
At CFL 0.8 (the CFL of the other workloads) the reference scheme blows up on this cavity after 140
steps (tests/golden/config3_cfl08_blowup.npz, the reference's own run): test_gpu_fp64_parity.py
checks that the FP64 GPU step stops at that step, test_cpu_evidence.py that the oracle does.
"""
import os

import pytest

import cases
import meso_gpu as mg
from helpers import relerr, run_gpu, run_oracle


@pytest.fixture(scope="module")
def config3_path(tmp_path_factory):
    return cases.config3(str(tmp_path_factory.mktemp("config3") / "c3"), 5000, "fp64")


@pytest.mark.gpu
def test_config3_fp64_500_steps_matches_oracle(gpu, config3_path):
    g = run_gpu(config3_path, 500, mg.FP64)
    o = run_oracle(config3_path, 500, os.cpu_count() or 1)
    assert g["step"] == o["step"] == 500 and g["run_state"] == o["run_state"] == 1
    errs = {k: relerr(g[k], o[k]) for k in ("rho", "u", "T", "q")}
    print(errs)
    for k, e in errs.items():
        assert e <= 1e-12, (k, e)


@pytest.mark.gpu
def test_config3_fp32_5000_steps_against_fp64(gpu, config3_path):
    a = run_gpu(config3_path, 5000, mg.FP32)
    b = run_gpu(config3_path, 5000, mg.FP64)
    assert a["step"] == b["step"] == 5000 and a["run_state"] == b["run_state"] == 1
    errs = {"rho": relerr(a["rho"], b["rho"]), "T": relerr(a["T"], b["T"]),
            "u": relerr(a["u"][:, 0], b["u"][:, 0]), "v": relerr(a["u"][:, 1], b["u"][:, 1]),
            "qx": relerr(a["q"][:, 0], b["q"][:, 0]), "qy": relerr(a["q"][:, 1], b["q"][:, 1])}
    print(errs)
    bound = {"rho": 1e-6, "T": 1e-6, "u": 1e-6, "v": 1e-6, "qx": 2e-5, "qy": 2e-5}
    for k, tol in bound.items():
        assert errs[k] <= tol, (k, errs[k])
