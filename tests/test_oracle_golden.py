"""Pins the oracle (oracle/meso_oracle.c) to the reference's own outputs.

tests/golden/*.npz hold the macroscopic fields the unmodified reference
solver produced on the committed inputs (tests/golden/make_golden.py).  With
one velocity slice the oracle must reproduce them bit for bit; with several
slices (the reference's DVS-parallel decomposition) to rounding of the
partial sums.
"""
import os

import numpy as np
import pytest

import meso_gpu as mg
from conftest import GOLDEN
from helpers import HEAVY_GOLDENS, RESTART_GOLDENS, golden_case, golden_names, relerr, run_oracle, run_oracle_restart

NAMES = golden_names()


def _case(name):
    return golden_case(name)


@pytest.mark.parametrize("name", [n for n in NAMES if n not in HEAVY_GOLDENS])
def test_oracle_bit_exact(name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    if name in RESTART_GOLDENS:
        o = run_oracle_restart(_case(name), int(g["requested"]))
    else:
        o = run_oracle(_case(name), int(g["requested"]))
    assert o["step"] == int(g["step"])
    assert o["run_state"] == int(g["run_state"])
    for k in ("rho", "u", "T", "q"):
        assert np.array_equal(o[k], g[k], equal_nan=True), (k, relerr(o[k], g[k]))
    assert o["time"] == float(g["time"])


@pytest.mark.parametrize("name", ["shakhov_q8_hgh8", "cdugks_q8", "channel_pressure"])
def test_oracle_sliced_velocity_set(name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    o = run_oracle(_case(name), int(g["requested"]), nthreads=3)
    assert o["step"] == int(g["step"])
    for k in ("rho", "u", "T", "q"):
        assert relerr(o[k], g[k]) <= 1e-12, k


def test_golden_inputs_load():
    for name in NAMES:
        c = mg.Case(_case(name))
        assert c.ncell > 0 and c.nv > 0
