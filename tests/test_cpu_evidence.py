"""Where the reference scheme itself blows up: evidence for the two workload substitutions, on the CPU.

* The rarefied workload names a Delaunay-triangle cavity of about 8k cells.  On the triangle cavity
  that meso-lts_gb300/cases.py generates for it (7938 triangles from a seeded jittered 64x64 point
  grid, corner triangles flipped so that every cell has two non-collinear neighbours; Kn 1, lid
  0.15, CFL 0.8), the reference stops with a NaN / T < 0 cell after 25 steps even with 21x21
  Newton-Cotes velocities (tests/golden/tri64_nc21_blowup.npz, the reference's own run): its
  unlimited least-squares upwind reconstruction grows an unstable mode on these triangles.  The
  rarefied workload therefore runs on seeded jittered quadrilaterals.
* The transitional workload (61x61 quads, half-range Gauss-Hermite 28x28, Kn 0.075) at CFL 0.8
  stops after 140 steps in the reference (tests/golden/config3_cfl08_blowup.npz); it runs at CFL
  0.5.

Here the oracle (the reference's step restated in C, bit-exact with it at one thread and run here
on all host threads, the reference's velocity-slice split) must stop at the reference's step.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from helpers import golden_case, run_oracle


@pytest.mark.parametrize("name", ["tri64_nc21_blowup", "config3_cfl08_blowup"])
def test_oracle_blows_up_at_the_reference_step(name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    assert int(g["run_state"]) == 0
    o = run_oracle(golden_case(name), int(g["requested"]), os.cpu_count() or 1)
    assert o["run_state"] == 0 and o["step"] == int(g["step"]), (o["step"], int(g["step"]))
