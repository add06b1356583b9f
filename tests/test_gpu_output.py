"""output() files against the reference's own (mesh_output.cpp:182-248, field.cpp:139-173,
cdugks_shakhov.cpp:791-845, cdugks.cpp output()).

tests/golden/output/<name>/ holds what the unmodified reference wrote through output() after
initial() and after the golden's steps (tests/golden/make_golden.py): grid.plt, step-0/data.plt,
step-N/data.plt and latest/*.  The GPU library (FP64) runs the same case through the case-file path
of the C ABI and meso_output at the same two points; every file must have the same lines and
tokens, text tokens identical and numbers equal to 1e-12 of the largest magnitude in the file
(the fields' parity bar; grid coordinates and connectivity come out identical).
"""
import os
import re

import numpy as np
import pytest

import meso_gpu as mg
from conftest import GOLDEN
from helpers import case_setting, copy_golden_case

NUM = re.compile(r"^[-+]?(\d+\.?\d*|\.\d+)([eE][-+]?\d+)?$|^[-+]?(nan|inf)$", re.IGNORECASE)


def _files(root: str) -> list[str]:
    out = []
    for dp, _, fs in os.walk(root):
        for f in fs:
            out.append(os.path.relpath(os.path.join(dp, f), root))
    return sorted(out)


def _compare(a_path: str, b_path: str) -> None:
    a = open(a_path).read().split("\n")
    b = open(b_path).read().split("\n")
    assert len(a) == len(b), (a_path, len(a), len(b))
    nums_b = [float(t) for line in b for t in line.split() if NUM.match(t)]
    scale = max([abs(x) for x in nums_b if np.isfinite(x)] + [1.0])
    for i, (la, lb) in enumerate(zip(a, b)):
        ta, tb = la.split(), lb.split()
        assert len(ta) == len(tb), (a_path, i, la, lb)
        for x, y in zip(ta, tb):
            if NUM.match(y):
                assert NUM.match(x), (a_path, i, x, y)
                fx, fy = float(x), float(y)
                assert abs(fx - fy) <= 1e-12 * scale, (a_path, i, x, y)
            else:
                assert x == y, (a_path, i, x, y)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["out_shakhov_q8", "out_cdugks_q8"])
def test_output_files_match_the_reference(gpu, tmp_path, name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    path = copy_golden_case(name, str(tmp_path / name))
    cname = case_setting(path, "case-name")
    cwd = os.getcwd()
    os.chdir(os.path.dirname(path))
    try:
        s = mg.Solver(path, mg.FP64)
        s.initial()
        s.output()
        assert s.step(int(g["requested"])) == int(g["requested"])
        s.output()
        s.close()
    finally:
        os.chdir(cwd)
    ours = os.path.join(os.path.dirname(path), cname)
    ref = os.path.join(GOLDEN, "output", name)
    assert _files(ours) == _files(ref), (_files(ours), _files(ref))
    for f in _files(ref):
        _compare(os.path.join(ours, f), os.path.join(ref, f))
