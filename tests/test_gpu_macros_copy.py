"""meso_get_macros gives the same values into page-locked and into pageable host arrays.

The macros are permuted to the caller's cell order on the device; the library copies them straight
into the caller's arrays when all of them are page-locked and through its own staging buffer
otherwise.  Both paths, and a call that asks for only some of the fields, must agree exactly, in
the original cell order of the mesh (checked against the FP64 form's values of the same state)."""
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


def _pinned(rt, n, keep):
    p = C.c_void_p()
    assert rt.cudaHostAlloc(C.byref(p), C.c_size_t(n * 8), 0) == 0
    keep.append(p)
    return np.frombuffer((C.c_double * n).from_address(p.value), dtype=np.float64)


def _ptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [mg.FP64, mg.FP32], ids=["fp64", "fp32"])
def test_macros_pinned_and_pageable_agree(gpu, tmp_path, precision):
    case = mg.Case(cases.shakhov_cavity(str(tmp_path / "c"), "jquad", 14, "hgh", 8, 0.1, 0.15, 20, seed=3))
    rho0, u0, T0, mask = case.initial_fields()
    s = mg.Solver(case=case, precision=precision, mask=mask)
    s.init_macros(rho0, u0, T0, None, 0)
    s.step(20)
    n = case.ncell
    ref = s.macros(n)  # pageable numpy arrays
    rt, keep = _cudart(), []
    try:
        pr, pu, pT, pq = _pinned(rt, n, keep), _pinned(rt, 3 * n, keep), _pinned(rt, n, keep), _pinned(rt, 3 * n, keep)
        assert mg.lib().meso_get_macros(s.handle, _ptr(pr), _ptr(pu), _ptr(pT), _ptr(pq)) == 0
        for k, a, b in zip(("rho", "u", "T", "q"), ref, (pr, pu.reshape(n, 3), pT, pq.reshape(n, 3))):
            assert np.array_equal(a, b), k
        only_T = np.zeros(n)
        assert mg.lib().meso_get_macros(s.handle, None, None, _ptr(only_T), None) == 0
        assert np.array_equal(only_T, ref[2])
    finally:
        for p in keep:
            rt.cudaFreeHost(p)
        s.close()
    # original cell order: the FP64 form of the same state, read the same way, agrees to rounding
    if precision == mg.FP32:
        d = mg.Solver(case=case, precision=mg.FP64, mask=mask)
        d.init_macros(rho0, u0, T0, None, 0)
        d.step(20)
        r64 = d.macros(n)
        d.close()
        assert np.max(np.abs(r64[0] - ref[0])) / np.max(np.abs(r64[0])) < 1e-5
