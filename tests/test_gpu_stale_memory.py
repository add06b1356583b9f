"""No FP32 kernel reads device memory it has not written.

A solve's contexts are allocated from memory that earlier contexts (or anything
else in the process) freed.  Here the device memory a context is about to get
is first filled with NaN bit patterns (0xFF bytes) and freed; the solve must
then give exactly the result it gives on fresh memory.  The velocity sets are
chosen so that the default velocity-group split does not divide the chunk count
evenly (hGH 28^2: 13 chunks of 64 velocities), the case where a group without
chunks once left its heat-flux partials unwritten.
"""
import ctypes as C

import numpy as np
import pytest

import cases
import meso_gpu as mg


def _cudart():
    for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            return C.CDLL(name)
        except OSError:
            continue
    raise RuntimeError("libcudart not found")


def _poison(rt, sizes=(4 << 10, 16 << 10, 64 << 10, 256 << 10, 1 << 20, 4 << 20), per_size_bytes=64 << 20):
    """Allocates buffers of the given sizes (the range of a context's arrays), fills them with 0xFF
    (NaN in FP32 and FP64) and frees them, so that the next allocations are likely to get them."""
    ptrs = []
    for size in sizes:
        for _ in range(max(1, per_size_bytes // size)):
            p = C.c_void_p()
            if rt.cudaMalloc(C.byref(p), C.c_size_t(size)) != 0:
                break
            assert rt.cudaMemset(p, 0xFF, C.c_size_t(size)) == 0
            ptrs.append(p)
    assert rt.cudaDeviceSynchronize() == 0
    for p in reversed(ptrs):
        rt.cudaFree(p)


def _run(path, steps, ngroup=0):
    case = mg.Case(path)
    rho, u, T, mask = case.initial_fields()
    prm = case.params
    prm.precision = mg.FP32
    prm.ngroup = ngroup
    s = mg.Solver(case=case, precision=mg.FP32, mask=mask, params=prm)
    s.init_macros(rho, u, T, None, 0)
    s.step(steps)
    out, st = s.macros(case.ncell), s.status()
    s.close()
    return out, st


@pytest.mark.gpu
@pytest.mark.parametrize("side,dvs,nv1d", [(16, "hgh", 28), (24, "hgh", 28), (20, "nc", 21), (12, "nc", 51)])
def test_fp32_solve_independent_of_stale_memory(gpu, tmp_path, side, dvs, nv1d):
    path = cases.shakhov_cavity(str(tmp_path / "c"), "quad", side, dvs, nv1d, 0.1, 0.12, 30, cfl=0.5)
    ref, st_ref = _run(path, 30)
    rt = _cudart()
    for _ in range(2):
        _poison(rt)
        out, st = _run(path, 30)
        assert st.step == st_ref.step == 30 and st.run_state == 1
        for k, x, y in zip(("rho", "u", "T", "q"), out, ref):
            assert np.all(np.isfinite(x)), k
            assert np.array_equal(x, y), (k, float(np.max(np.abs(x - y))))


@pytest.mark.gpu
def test_served_solves_on_reused_memory_equal_alone(gpu, tmp_path):
    """Served solves admitted into memory that retired solves freed give their alone results."""
    paths = []
    for i in range(24):
        side = (16, 24)[i % 2]
        paths.append(cases.shakhov_cavity(str(tmp_path / f"r{i}"), "quad", side, "hgh", 28, 0.1 + 0.01 * i, 0.12, 60,
                                          cfl=0.5))
    # six velocity groups over the 13 chunks of hGH 28^2 (planned as five): the split that once
    # left a group without chunks
    def prm(path):
        q = mg.Case(path).params
        q.precision = mg.FP32
        q.ngroup = 6
        return q

    srv = mg.Server(hbm_budget_bytes=8 << 30, max_members=4)
    tags, got = {}, {}
    for i, p in enumerate(paths):
        tags[srv.submit(p, prm(p))] = i
        for t in srv.poll(20):
            got[tags[t]] = srv.result(t)
    for _ in range(200):
        if len(got) == len(paths):
            break
        for t in srv.poll(20):
            got[tags[t]] = srv.result(t)
    srv.close()
    assert len(got) == len(paths)
    for i, p in enumerate(paths):
        (rho, u, T, q), st, _ = got[i]
        ref, st_ref = _run(p, 60, ngroup=6)
        assert st.step == st_ref.step == 60 and st.run_state == st_ref.run_state, i
        for k, x, y in zip(("rho", "u", "T", "q"), (rho, u, T, q), ref):
            assert np.array_equal(x, y), (i, k)
