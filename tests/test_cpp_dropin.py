"""The C++ drop-in (include/meso_solver.hpp) driven by the reference's handle_solver loop
(meso-lts_gb300/apps/meso_gpu_run.cpp): golden cases reproduced through it, and its error behaviour."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import build
import meso_gpu as mg
from conftest import GOLDEN
from helpers import relerr

CASES = ["shakhov_q8_hgh8", "cdugks_q8", "dugks_q8", "channel_pressure"]


def _run(args, cwd):
    return subprocess.run([build.APP, *args], cwd=cwd, capture_output=True, text=True, timeout=600)


def test_dropin_reports_bad_input_as_invalid_argument(tmp_path):
    r = _run([str(tmp_path / "missing.txt")], str(tmp_path))
    assert r.returncode == 1 and "invalid argument" in r.stderr
    r = _run([], str(tmp_path))
    assert r.returncode == 2 and "usage" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_dropin_loop_matches_golden(gpu, tmp_path, name):
    d = tmp_path / name
    shutil.copytree(os.path.join(GOLDEN, "cases", name), d)
    out = tmp_path / "macros.bin"
    r = _run(["case.txt", "fp64", "--dump", str(out), "--fields", str(tmp_path / "f_")], str(d))
    assert r.returncode == 0, r.stderr
    raw = np.fromfile(out, dtype=np.float64)
    n, step = int(raw[0]), int(raw[1])
    rho, u = raw[3:3 + n], raw[3 + n:3 + 4 * n].reshape(n, 3)
    T, q = raw[3 + 4 * n:3 + 5 * n], raw[3 + 5 * n:3 + 8 * n].reshape(n, 3)
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    assert step == int(g["step"])
    assert relerr(rho, g["rho"]) <= 1e-12 and relerr(u, g["u"]) <= 1e-12
    if name.startswith(("shakhov", "channel")):
        assert relerr(T, g["T"]) <= 1e-12 and relerr(q, g["q"]) <= 1e-12
    # output() wrote the reference's files (case-name directory, latest/ and step data)
    assert any(os.scandir(d)), "no output written"
    # the solver's mesh and velocity-mesh views
    line = [l for l in r.stdout.splitlines() if l.startswith("cells ")][0].split()
    c = mg.Case(str(d / "case.txt"))
    assert int(line[1]) == c.ncell == n and int(line[5]) == c.nv
    vol = c.arrays()["cell_vol"]
    assert abs(float(line[7]) - float(np.sum(rho * vol))) <= 1e-12 * float(np.sum(rho * vol))
    # the Field API's text output (18 digits, a value or "x y z" per line) and heft
    assert np.array_equal(np.loadtxt(tmp_path / "f_rho.dat"), rho)
    assert np.array_equal(np.loadtxt(tmp_path / "f_u.dat"), u[:, 0])
    assert np.array_equal(np.loadtxt(tmp_path / "f_vel.dat").reshape(n, 3), u)


@pytest.mark.gpu
def test_dropin_fp32_with_refinement(gpu, tmp_path):
    """--refine K through the drop-in class (MESO::GPU::Solver::refine): the FP32 form of a golden
    Shakhov case with an FP64 defect correction every 5 steps, within the FP32 transient bars of
    the reference's outputs."""
    name = "shakhov_q8_hgh8"
    d = tmp_path / name
    shutil.copytree(os.path.join(GOLDEN, "cases", name), d)
    out = tmp_path / "macros.bin"
    r = _run(["case.txt", "fp32", "--refine", "5", "--dump", str(out)], str(d))
    assert r.returncode == 0, r.stderr
    raw = np.fromfile(out, dtype=np.float64)
    n, step = int(raw[0]), int(raw[1])
    rho, u, T = raw[3:3 + n], raw[3 + n:3 + 4 * n].reshape(n, 3), raw[3 + 4 * n:3 + 5 * n]
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    assert step == int(g["step"])
    assert relerr(rho, g["rho"]) <= 2e-6 and relerr(u, g["u"]) <= 2e-5 and relerr(T, g["T"]) <= 2e-6
