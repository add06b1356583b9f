"""Helpers shared by the tests: run a case through the GPU library or the oracle."""
from __future__ import annotations

import glob
import os
import shutil

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


GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
# goldens whose reference run starts from the files a first run wrote (read-np-data True)
RESTART_GOLDENS = ("restart_shakhov_q8", "restart_cdugks_q8")
# goldens too long for a one-thread oracle run in the CPU suite (the reference blows up after
# 25-140 steps of a 3.5-2.9 M cell-velocity case); test_cpu_evidence.py runs them on all threads
HEAVY_GOLDENS = ("config3_cfl08_blowup", "tri64_nc21_blowup")


def golden_names() -> list[str]:
    """The step goldens (the reference's fields after N steps; geometry_* and workload_* hold tables)."""
    return sorted(f[:-4] for f in os.listdir(GOLDEN_DIR)
                  if f.endswith(".npz") and not f.startswith(("geometry_", "workload_")))


def golden_case(name: str) -> str:
    """The case file of a golden (case.txt, or the reference's own case-*.txt)."""
    d = os.path.join(GOLDEN_DIR, "cases", name)
    if os.path.exists(os.path.join(d, "case.txt")):
        return os.path.join(d, "case.txt")
    found = sorted(glob.glob(os.path.join(d, "case*.txt")))
    assert len(found) == 1, (name, found)
    return found[0]


def copy_golden_case(name: str, dst: str) -> str:
    """A writable copy of a golden's case folder (runs that read or write files next to it)."""
    src = os.path.dirname(golden_case(name))
    shutil.copytree(src, dst)
    return os.path.join(dst, os.path.basename(golden_case(name)))


def read_latest(case_dir: str, case_name: str, shakhov: bool, ncell: int):
    """The latest/ text files output() writes (rho, u, T, q), as read-np-data reads them."""
    base = os.path.join(case_dir, case_name, "latest")
    rho = np.loadtxt(os.path.join(base, "Rho")).reshape(ncell)
    u = np.loadtxt(os.path.join(base, "U")).reshape(ncell, 3)
    if not shakhov:
        return rho, u, None, None
    T = np.loadtxt(os.path.join(base, "T")).reshape(ncell)
    q = np.loadtxt(os.path.join(base, "q")).reshape(ncell, 3)
    return rho, u, T, q


def case_setting(path: str, key: str, default: str | None = None) -> str | None:
    for line in open(path):
        t = line.split()
        if len(t) >= 2 and t[0] == key:
            return t[1]
    return default


def run_oracle_restart(case_path: str, nsteps: int, nthreads: int = 1):
    """The oracle from a golden's latest/ files (initial() with read-np-data True, mode 1)."""
    case = mg.Case(case_path)
    shakhov = case.params.solver == mg.SOLVER_CDUGKS_SHAKHOV
    rho, u, T, q = read_latest(os.path.dirname(case_path), case_setting(case_path, "case-name"), shakhov, case.ncell)
    o = mo.Oracle(case, nthreads)
    o.init(rho, u, T, q, 1)
    done, rc = o.step(nsteps)
    r, uu, t, qq = o.macros()
    st = o.state()
    o.close()
    return dict(rho=r, u=uu, T=t, q=qq, done=done, step=st["step"], run_state=st["run_state"],
                time=st["solution_time"], rc=rc)


def run_gpu_case_initial(case_path: str, nsteps: int, precision: int = mg.FP64):
    """The case-file path of the C ABI (meso_ctx_create_from_case + meso_initial), run from the case's
    folder as the reference runs (read-np-data and output() paths are relative to it)."""
    cwd = os.getcwd()
    os.chdir(os.path.dirname(case_path))
    try:
        s = mg.Solver(case_path, precision)
        s.initial()
        try:
            done = s.step(nsteps)
        except mg.MesoError as e:
            if e.code != mg.ERR_NAN:
                raise
            done = None
        st = s.status()
        n = mg.Case(case_path).ncell
        out = s.macros(n)
        s.close()
    finally:
        os.chdir(cwd)
    return dict(rho=out[0], u=out[1], T=out[2], q=out[3], done=done, step=st.step, run_state=st.run_state,
                time=st.solution_time, converged=st.converged, residual=np.array(st.residual[:st.nresidual]))
