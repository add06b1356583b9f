"""Batched FP32 solves (meso_batch_*): each member's result is the same as the
same solve run alone, whatever else is in the batch.

The batch runs the same kernels over a work list of every member's tiles, and
each member's velocity-group partial sums are combined in a fixed order, so
the comparison is exact (bit for bit), which is tighter than the 1e-6 the
serving tests need.
"""
import numpy as np
import pytest

import cases
import meso_gpu as mg

MEMBERS = [
    ("quad_hgh8", lambda d: cases.shakhov_cavity(d, "quad", 10, "hgh", 8, 0.1, 0.15, 50)),
    ("jquad_nc21", lambda d: cases.shakhov_cavity(d, "jquad", 14, "nc", 21, 1.0, 0.1, 50, seed=3)),
    ("quad_d2q9", lambda d: cases.shakhov_cavity(d, "quad", 12, "d2q9", 3, 0.05, 0.12, 50)),
    ("channel_pressure", lambda d: cases.shakhov_channel(d, "pressure", 12, 6, "hgh", 8, 0.2, 50)),
    # a large velocity set (NC 51^2): the batch launches the large- and small-set face kernels
    ("jquad_nc51", lambda d: cases.shakhov_cavity(d, "jquad", 8, "nc", 51, 1.0, 0.15, 50, seed=4)),
]


def _solver(path, params=None):
    case = mg.Case(path)
    rho, u, T, mask = case.initial_fields()
    s = mg.Solver(case=case, precision=mg.FP32, mask=mask, params=params)
    s.init_macros(rho, u, T, None, 0)
    return case, s


def _alone(path, nsteps, params=None):
    case, s = _solver(path, params)
    s.step(nsteps)
    out = s.macros(case.ncell)
    st = s.status()
    s.close()
    return out, st


@pytest.mark.gpu
def test_batch_members_match_alone(gpu, tmp_path):
    paths = [build(str(tmp_path / name)) for name, build in MEMBERS]
    solvers = [_solver(p) for p in paths]
    b = mg.Batch([s for _, s in solvers])
    assert b.step(30) == len(MEMBERS)
    assert b.last_step_launches() > 0
    b.step(20)
    for (name, _), path, (case, s) in zip(MEMBERS, paths, solvers):
        ref, st_ref = _alone(path, 50)
        out = s.macros(case.ncell)
        st = s.status()
        assert st.step == st_ref.step == 50, name
        assert st.solution_time == st_ref.solution_time, name
        for k, x, y in zip(("rho", "u", "T", "q"), out, ref):
            assert np.array_equal(x, y), (name, k, float(np.max(np.abs(x - y))))
    b.close()
    for _, s in solvers:
        s.close()


@pytest.mark.gpu
def test_batch_member_converges_and_stops(gpu, tmp_path):
    """Members converge (10 residual checks in a row) and stop at the same step as alone."""
    path = cases.shakhov_cavity(str(tmp_path / "conv"), "quad", 8, "hgh", 8, 0.1, 0.15, 5000)
    other = cases.shakhov_cavity(str(tmp_path / "other"), "quad", 10, "hgh", 8, 0.1, 0.15, 5000)
    p = mg.Case(path).params
    p.residual_interval = 10
    p.residual_limit = 1e-2
    p2 = mg.Case(other).params
    p2.residual_interval = 20
    p2.residual_limit = 1e-3
    p2.residual_fields = mg.RES_U  # converge on the velocity only
    ref, st_ref = _alone(path, 4000, params=p)
    ref2, st_ref2 = _alone(other, 4000, params=p2)
    assert st_ref.converged == 1 and st_ref2.converged == 1
    assert st_ref.step < st_ref2.step
    mid = (st_ref.step + st_ref2.step) // 2
    (case, s), (case2, s2) = _solver(path, params=p), _solver(other, params=p2)
    b = mg.Batch([s, s2])
    assert b.step(mid) == 1  # the first has converged, the second runs on
    st = s.status()
    assert st.converged == 1 and st.run_state == 0 and st.step == st_ref.step
    assert s2.status().step == mid
    assert b.step(4000) == 0
    st2 = s2.status()
    assert st2.converged == 1 and st2.step == st_ref2.step
    for x, y in zip(s.macros(case.ncell), ref):
        assert np.array_equal(x, y)
    for x, y in zip(s2.macros(case2.ncell), ref2):
        assert np.array_equal(x, y)
    b.close()
    s.close()
    s2.close()


@pytest.mark.gpu
def test_batch_isolates_a_failing_member(gpu, tmp_path):
    """A member that blows up stops alone; the others' results do not change."""
    bad = cases.shakhov_cavity(str(tmp_path / "bad"), "quad", 8, "hgh", 8, 0.1, 0.15, 40, cfl=30.0)
    good = cases.shakhov_cavity(str(tmp_path / "good"), "quad", 10, "hgh", 8, 0.1, 0.15, 40)
    (cb, sb), (cg, sg) = _solver(bad), _solver(good)
    b = mg.Batch([sb, sg])
    b.step(40)
    assert sb.status().run_state == 0 and sb.status().bad_cells > 0
    ref, _ = _alone(good, 40)
    for x, y in zip(sg.macros(cg.ncell), ref):
        assert np.array_equal(x, y)
    b.close()
    sb.close()
    sg.close()


@pytest.mark.gpu
def test_batch_rejects_fp64_and_double_membership(gpu, tmp_path):
    path = cases.shakhov_cavity(str(tmp_path / "c"), "quad", 6, "hgh", 8, 0.1, 0.15, 5)
    case = mg.Case(path)
    rho, u, T, mask = case.initial_fields()
    s64 = mg.Solver(case=case, precision=mg.FP64, mask=mask)
    s64.init_macros(rho, u, T, None, 0)
    with pytest.raises(mg.MesoError) as e:
        mg.Batch([s64])
    assert e.value.code == mg.ERR_UNSUPPORTED
    _, s = _solver(path)
    b = mg.Batch([s])
    with pytest.raises(mg.MesoError):
        mg.Batch([s])
    with pytest.raises(mg.MesoError):
        s.step(1)  # stepped by its batch only
    b.close()
    s.step(1)  # free again
    s.close()
    s64.close()
