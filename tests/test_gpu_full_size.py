"""The rarefied-cavity workload at its full size (7744 cells x 10201 Newton-Cotes velocities).

* FP64 GPU step against the oracle (all host threads, the reference's velocity-slice split) after
  5 steps: the parity bar, max relative error <= 1e-12 on rho, u, T, q.
* FP32-storage step against the FP64 GPU step after the workload's 500 steps.  At step 500 the
  cavity is still in its transient (u changes by 7 % between steps 400 and 500), where the two
  trajectories drift apart faster than at steady state (the steady-state bar, 1e-6, is tested on a
  cavity run to steady state in test_gpu_fp32.py); measured here: rho 2.8e-7, u 3.3e-6, T 2.0e-7,
  q 2.3e-5 (max norm relative to the field's largest magnitude), bounded below with a margin of 3.
"""
import os

import pytest

import cases
import meso_gpu as mg
from helpers import relerr, run_gpu, run_oracle


@pytest.fixture(scope="module")
def config2_path(tmp_path_factory):
    return cases.config2(str(tmp_path_factory.mktemp("config2") / "c2"), 500)


@pytest.mark.gpu
def test_fp64_full_size_matches_oracle(gpu, config2_path):
    g = run_gpu(config2_path, 5, mg.FP64)
    o = run_oracle(config2_path, 5, os.cpu_count() or 1)
    assert g["step"] == o["step"] == 5
    for k in ("rho", "u", "T", "q"):
        assert relerr(g[k], o[k]) <= 1e-12, (k, relerr(g[k], o[k]))


@pytest.mark.gpu
def test_fp32_full_size_500_steps_against_fp64(gpu, config2_path):
    a = run_gpu(config2_path, 500, mg.FP32)
    b = run_gpu(config2_path, 500, mg.FP64)
    assert a["step"] == b["step"] == 500 and a["run_state"] == b["run_state"] == 1
    bound = {"rho": 1e-6, "u": 1e-5, "T": 6e-7, "q": 7e-5}
    for k, tol in bound.items():
        assert relerr(a[k], b[k]) <= tol, (k, relerr(a[k], b[k]))
