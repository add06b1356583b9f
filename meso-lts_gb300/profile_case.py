"""Runs a few steps of a benchmark workload, for profiler captures.

    python meso-lts_gb300/profile_case.py [--workload config2|config3|config1] [--precision fp32|fp64]
                                          [--steps N]

Builds the workload's case files (cases.py) in a temporary directory, creates
a context, runs initial() and N steps, prints the mean device time per step.
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
    ap.add_argument("--workload", default="config2", choices=["config1", "config2", "config3"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--steps", type=int, default=3)
    a = ap.parse_args()
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
        s.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
