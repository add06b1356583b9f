"""FP64 plain GPU step vs the oracle (CPU restatement of the reference step).

Bar: max relative error <= 1e-12 on every macroscopic field after N steps
(the oracle itself is pinned bit-exact to the reference binary by
test_oracle_golden.py).  Cases cover the three solvers, quad and triangle
meshes, the hGH / Newton-Cotes / Sparse velocity sets, the limiter and the
gradient-off path.
"""
import os

import pytest

import cases
import meso_gpu as mg
from helpers import max_field_err, run_gpu, run_oracle

TOL = 1e-12

CASES = [
    # id, builder kwargs, steps, shakhov?
    ("cdugks_q8", lambda d: cases.bgk_cavity(d, 8, 100), 100, False),
    ("cdugks_q8_nograd", lambda d: cases.bgk_cavity(d, 8, 60, gradient=False), 60, False),
    ("dugks_q8", lambda d: cases.bgk_cavity(d, 8, 100, solver="dugks@incompressible"), 100, False),
    ("shakhov_q8_hgh8", lambda d: cases.shakhov_cavity(d, "quad", 8, "hgh", 8, 0.1, 0.15, 40), 40, True),
    ("shakhov_t8_nc21", lambda d: cases.shakhov_cavity(d, "tri", 8, "nc", 21, 1.0, 0.15, 30), 30, True),
    ("shakhov_q8_d2q9", lambda d: cases.shakhov_cavity(d, "quad", 8, "d2q9", 3, 0.05, 0.15, 60), 60, True),
    ("shakhov_q8_limiter", lambda d: cases.shakhov_cavity(d, "quad", 8, "hgh", 8, 0.1, 0.15, 30, limiter=True), 30, True),
    ("shakhov_q8_nograd", lambda d: cases.shakhov_cavity(d, "quad", 8, "hgh", 8, 0.1, 0.15, 30, gradient=False), 30, True),
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
            assert (abs(a - b).max() <= 1e-9 * max(1.0, abs(b).max()))
