"""Runs a few steps of a benchmark workload, for profiler captures.

    python meso-lts_gb300/profile_case.py [--workload config2|config3|config1|served64] [--precision fp32|fp64]
                                          [--steps N] [--phases]

Builds the workload's case files (cases.py) in a temporary directory, creates
a context, runs initial() and N steps, prints the mean device time per step.
served64 is a batch of the first 64 requests of the served stream (FP32 cavities of
sides 16-32, hGH 28^2 or NC 21^2 velocities, one velocity group per tile as the
server runs them) stepped as one batch.  --phases
also prints the mean device time of each kernel phase (kernels launched one by
one, a few more steps).
Meant to be wrapped by ncu, e.g.

    ncu --set full --clock-control none -k regex:"k32_update|k32_moments" -s 2 -c 2 \\
        python meso-lts_gb300/profile_case.py --workload config2 --steps 3
"""
from __future__ import annotations

import argparse
import os
import sys
import tempfile

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

import cases  # noqa: E402
import meso_gpu as mg  # noqa: E402


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="config2", choices=["config1", "config2", "config3", "served64"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--phases", action="store_true")
    a = ap.parse_args()
    if a.workload == "served64":
        return served_batch(a)
    with tempfile.TemporaryDirectory() as d:
        build = {"config1": lambda p: cases.config1(p, 10), "config2": lambda p: cases.config2(p, 10, a.precision),
                 "config3": lambda p: cases.config3(p, 10, a.precision)}[a.workload]
        path = build(os.path.join(d, a.workload))
        case = mg.Case(path)
        rho, u, T, mask = case.initial_fields()
        prec = mg.FP32 if a.precision == "fp32" else mg.FP64
        s = mg.Solver(case=case, precision=prec, mask=mask)
        s.init_macros(rho, u, T, None, 0)
        s.step(a.steps)
        print(f"{a.workload} {a.precision}: {case.ncell} cells x {case.nv} velocities, "
              f"{s.last_step_ms() / a.steps:.3f} ms/step, {s.last_step_launches()} launches")
        if a.phases:
            for k, v in s.phase_times(5).items():
                print(f"  {k}: {v:.4f} ms")
        s.close()
    return 0


def served_batch(a) -> int:
    with tempfile.TemporaryDirectory() as d:
        solvers, kases, work = [], [], 0
        for r in cases.config5_requests(count=64):
            case = mg.Case(cases.config5_case(os.path.join(d, f"s{r['index']}"), r, 8000))
            rho, u, T, mask = case.initial_fields()
            prm = case.params
            prm.precision = mg.FP32
            prm.ngroup = 1  # as the server runs requests that set no kernel shape
            s = mg.Solver(case=case, precision=mg.FP32, mask=mask, params=prm)
            s.init_macros(rho, u, T, None, 0)
            solvers.append(s)
            work += case.ncell * case.nv
            kases.append(case)
        b = mg.Batch(solvers)
        b.step(a.steps)
        ms = b.last_step_ms() / a.steps
        print(f"served64: 64 solves, {work} cell-velocities, {ms:.3f} ms/step, {work / ms * 1e3 / 1e9:.2f} G cell-xi/s")
        if a.phases:
            for k, v in b.phase_times(5).items():
                print(f"  {k}: {v:.4f} ms")
        b.close()
        for s in solvers:
            s.close()
        for case in kases:
            case.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
