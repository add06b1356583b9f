"""ctypes loader of oracle/lib/libmeso_oracle.so -- TEST INFRASTRUCTURE.

The CPU restatement of the meso-lts step (meso_oracle.c).  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg use it, as the
results the GPU step is tested against and as the CPU baseline; it is never
part of the product path.

It takes the descriptor structs of a loaded case (anything exposing the
ctypes attributes `mesh`, `dvs`, `marks_ptr`, `nmarks`, `params`, as
meso_gpu.Case does), so the oracle and the GPU library run the same inputs.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libmeso_oracle.so")
_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} not built; run `python meso-lts_gb300/build.py`")
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        dp = C.POINTER(C.c_double)
        L.mo_create.argtypes = [vp, vp, vp, C.c_int32, vp, vp, C.c_int32, C.POINTER(vp)]
        L.mo_create.restype = C.c_int
        L.mo_destroy.argtypes = [vp]
        L.mo_destroy.restype = None
        L.mo_init.argtypes = [vp, dp, dp, dp, dp, C.c_int32]
        L.mo_init.restype = C.c_int
        L.mo_step.argtypes = [vp, C.c_int32, C.POINTER(C.c_int32)]
        L.mo_step.restype = C.c_int
        L.mo_get_macros.argtypes = [vp, dp, dp, dp, dp]
        L.mo_get_macros.restype = C.c_int
        L.mo_get_flux_moments.argtypes = [vp, dp, dp, dp]
        L.mo_get_flux_moments.restype = C.c_int
        L.mo_get_state.argtypes = [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32), dp]
        L.mo_get_state.restype = C.c_int
        L.mo_get_f.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32]
        L.mo_get_f.restype = C.c_double
        L.mo_get_residual.argtypes = [vp, dp, C.POINTER(C.c_int32)]
        L.mo_get_residual.restype = C.c_int
        L.mo_set_params.argtypes = [vp, vp]
        L.mo_set_params.restype = C.c_int
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    def __init__(self, case, nthreads: int = 1, mask: np.ndarray | None = None, params=None):
        h = C.c_void_p()
        p = params if params is not None else case.params
        mk = None if mask is None else np.ascontiguousarray(mask, np.uint8)
        rc = lib().mo_create(C.addressof(case.mesh), C.addressof(case.dvs), C.cast(case.marks_ptr, C.c_void_p),
                             case.nmarks, C.addressof(p), None if mk is None else mk.ctypes.data, nthreads,
                             C.byref(h))
        if rc:
            raise RuntimeError(f"mo_create failed ({rc})")
        self._h = h
        self.ncell = case.mesh.ncell
        self._mask = mk

    def init(self, rho, u, T=None, q=None, mode: int = 0):
        f = lambda a: None if a is None else np.ascontiguousarray(a, np.float64).reshape(-1)
        rho, u, T, q = f(rho), f(u), f(T), f(q)
        rc = lib().mo_init(self._h, _p(rho), _p(u), _p(T), _p(q), mode)
        if rc:
            raise RuntimeError(f"mo_init failed ({rc})")

    def step(self, n: int) -> tuple[int, int]:
        done = C.c_int32()
        rc = lib().mo_step(self._h, n, C.byref(done))
        return done.value, rc

    def macros(self):
        n = self.ncell
        rho, u, T, q = np.zeros(n), np.zeros(3 * n), np.zeros(n), np.zeros(3 * n)
        lib().mo_get_macros(self._h, _p(rho), _p(u), _p(T), _p(q))
        return rho, u.reshape(n, 3), T, q.reshape(n, 3)

    def flux_moments(self):
        n = self.ncell
        a, b, c = np.zeros(n), np.zeros(3 * n), np.zeros(n)
        lib().mo_get_flux_moments(self._h, _p(a), _p(b), _p(c))
        return a, b.reshape(n, 3), c

    def state(self) -> dict:
        s, r, c = C.c_int32(), C.c_int32(), C.c_int32()
        t = C.c_double()
        lib().mo_get_state(self._h, C.byref(s), C.byref(r), C.byref(c), C.byref(t))
        return dict(step=s.value, run_state=r.value, converged=c.value, solution_time=t.value)

    def residual(self) -> np.ndarray:
        """The last residual check's list, in the reference's print order."""
        a = np.zeros(8)
        n = C.c_int32()
        lib().mo_get_residual(self._h, _p(a), C.byref(n))
        return a[:n.value].copy()

    def f(self, d: int, p: int, c: int) -> float:
        return lib().mo_get_f(self._h, d, p, c)

    def set_params(self, p):
        rc = lib().mo_set_params(self._h, C.addressof(p))
        if rc:
            raise RuntimeError(f"mo_set_params failed ({rc})")

    def close(self):
        if self._h:
            lib().mo_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
