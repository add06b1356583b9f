"""Served solves (meso_server_*): continuous batching gives each solve the
result it gets alone.

Requests arrive while others are on the GPU; each is admitted, stepped with
whatever else is running, and retired when it converges or reaches its
max-step.  Every result must equal the same solve run alone through
meso_step (tolerance 1e-6 relative, the FP32 form's stated bar; the batch
kernels combine each solve's partial sums in a fixed order, so the results
are in fact identical).
"""
import numpy as np
import pytest

import cases
import meso_gpu as mg
from helpers import relerr

TOL = 1e-6


def _params(path, interval, limit, fields=0):
    p = mg.Case(path).params
    p.precision = mg.FP32
    p.residual_interval = interval
    p.residual_limit = limit
    p.residual_fields = fields
    p.ngroup = 1  # the server's own choice for requests that set no kernel shape
    return p


def _alone(path, params, max_step):
    case = mg.Case(path)
    rho, u, T, mask = case.initial_fields()
    s = mg.Solver(case=case, precision=mg.FP32, mask=mask, params=params)
    s.init_macros(rho, u, T, None, 0)
    while s.status().run_state and s.status().step < max_step:
        s.step(min(50, max_step - s.status().step))
    out, st = s.macros(case.ncell), s.status()
    s.close()
    return out, st


@pytest.mark.gpu
def test_served_results_equal_alone(gpu, tmp_path):
    reqs = [
        # (case, params, max_step): converges on all fields / on U only / stops at max-step
        (cases.shakhov_cavity(str(tmp_path / "a"), "quad", 8, "hgh", 8, 0.1, 0.15, 4000), (10, 1e-2, 0), 4000),
        (cases.shakhov_cavity(str(tmp_path / "b"), "quad", 10, "hgh", 8, 0.1, 0.12, 4000), (20, 1e-3, mg.RES_U), 4000),
        (cases.shakhov_cavity(str(tmp_path / "c"), "jquad", 12, "nc", 21, 1.0, 0.1, 120, seed=5), (100, 1e-9, 0), 120),
        (cases.shakhov_cavity(str(tmp_path / "d"), "quad", 12, "d2q9", 3, 0.05, 0.1, 4000), (10, 1e-2, 0), 4000),
    ]
    srv = mg.Server(hbm_budget_bytes=8 << 30, max_members=3)
    tags = {}
    finished = {}
    # staggered arrivals: one request per poll, polls of 40 steps
    for i, (path, (ri, lim, fields), _) in enumerate(reqs):
        tags[srv.submit(path, _params(path, ri, lim, fields))] = i
        for t in srv.poll(40):
            finished[t] = srv.result(t)
    pending, running, _ = srv.counts()
    assert pending + running > 0
    for _ in range(400):
        if sum(srv.counts()[:2]) == 0:
            break
        for t in srv.poll(40):
            finished[t] = srv.result(t)
    assert len(finished) == len(reqs)
    for t, ((rho, u, T, q), st, (total, queued)) in finished.items():
        path, (ri, lim, fields), max_step = reqs[tags[t]]
        ref, st_ref = _alone(path, _params(path, ri, lim, fields), max_step)
        assert st.step == st_ref.step and st.converged == st_ref.converged, (tags[t], st.step, st_ref.step)
        assert total >= queued >= 0.0
        for k, x, y in zip(("rho", "u", "T", "q"), (rho, u, T, q), ref):
            assert relerr(x, y) <= TOL, (tags[t], k)
            assert np.array_equal(x, y), (tags[t], k)
    assert srv.device_bytes() == 0
    srv.close()


@pytest.mark.gpu
def test_server_admits_by_budget(gpu, tmp_path):
    """With room for one solve at a time, the second waits until the first has finished."""
    a = cases.shakhov_cavity(str(tmp_path / "a"), "quad", 10, "hgh", 8, 0.1, 0.15, 60)
    b = cases.shakhov_cavity(str(tmp_path / "b"), "quad", 10, "hgh", 8, 0.1, 0.15, 60)
    srv = mg.Server(hbm_budget_bytes=8 << 30, max_members=1)
    ta, tb = srv.submit(a), srv.submit(b)
    srv.poll(30)
    assert srv.counts()[:2] == (1, 1)
    done = []
    for _ in range(20):
        done += srv.poll(30)
        if len(done) == 2:
            break
    assert done == [ta, tb]
    (_, st_a, _), (_, st_b, (total_b, queued_b)) = srv.result(ta), srv.result(tb)
    assert st_a.step == st_b.step == 60
    assert queued_b > 0.0
    srv.close()
