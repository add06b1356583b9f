"""meso_shakhov_moments_noalloc (the allocation-free entry point) against meso_init_macros.

meso_init_macros(mode 0) builds the equilibrium state of given rho, u, T and
stores its discrete moments as the cell macros; meso_get_macros returns them.
The allocation-free entry point gets the same state (built here in numpy) in
caller-owned device buffers and must return the same moments.  Tolerance:
1e-12 relative (max norm) on rho, u, T.  The heat flux of an equilibrium
state is a sum whose terms cancel to a small remainder, so its error is
measured against the magnitude of those terms, 1/2 sum w |c| (c^2 g + h),
at the same 1e-12.

Three calls in a row on cases of different size and velocity count check that
the shared scratch array carries nothing from one call into the next.
"""
import ctypes as C
import os

import numpy as np
import pytest

import cases
import meso_gpu as mg
from helpers import relerr

TOL = 1e-12


def _cudart():
    for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            return C.CDLL(name)
        except OSError:
            continue
    raise RuntimeError("libcudart not found")


class DeviceBuffers:
    """Test-side device memory (the entry point itself allocates none)."""

    def __init__(self):
        self.rt = _cudart()
        self.ptrs = []

    def put(self, a: np.ndarray) -> int:
        a = np.ascontiguousarray(a, np.float64)
        p = C.c_void_p()
        assert self.rt.cudaMalloc(C.byref(p), C.c_size_t(max(a.nbytes, 8))) == 0
        self.ptrs.append(p.value)
        assert self.rt.cudaMemcpy(C.c_void_p(p.value), a.ctypes.data_as(C.c_void_p), C.c_size_t(a.nbytes), 1) == 0
        return p.value

    def empty(self, n: int) -> int:
        return self.put(np.full(n, np.nan))

    def get(self, p: int, n: int) -> np.ndarray:
        out = np.zeros(n)
        assert self.rt.cudaMemcpy(out.ctypes.data_as(C.c_void_p), C.c_void_p(p), C.c_size_t(out.nbytes), 2) == 0
        return out

    def sync(self):
        assert self.rt.cudaDeviceSynchronize() == 0

    def close(self):
        for p in self.ptrs:
            self.rt.cudaFree(C.c_void_p(p))
        self.ptrs = []


def _equilibrium_state(case: mg.Case, seed: int):
    """Random 2-D macros and the mode-0 state of initial() (cdugks_shakhov.cpp:137-145)."""
    a = case.arrays()
    R, K = case.params.R, case.params.K
    n = case.ncell
    rng = np.random.default_rng(seed)
    rho = 1.0 + 0.2 * (rng.random(n) - 0.5)
    T = 1.0 + 0.3 * (rng.random(n) - 0.5)
    u = np.zeros((n, 3))
    u[:, :2] = 0.2 * (rng.random((n, 2)) - 0.5)
    xi, w = a["xi"], a["w"]
    c = xi[None, :, :2] - u[:, None, :2]
    cc = np.sum(c * c, axis=-1)
    over_RT2 = 0.5 / (R * T)
    g = rho[:, None] * over_RT2[:, None] / np.pi * np.exp(-cc * over_RT2[:, None])
    h = (K + 3.0 - 2.0) * (R * T)[:, None] * g
    q_scale = 0.5 * np.sum(np.abs(c) * (w[None, :, None] * np.abs(cc * g + h)[..., None]), axis=1)
    return rho, u, T, g, h, xi, w, R, K, q_scale


def _case(tmp_path, name):
    if name == "d2q9_10":
        return cases.shakhov_cavity(str(tmp_path / name), "quad", 10, "d2q9", 3, 0.1, 0.15, 5)
    if name == "hgh8_12":
        return cases.shakhov_cavity(str(tmp_path / name), "quad", 12, "hgh", 8, 0.1, 0.15, 5)
    return cases.shakhov_cavity(str(tmp_path / name), "jquad", 20, "nc", 21, 1.0, 0.15, 5)


@pytest.mark.gpu
def test_noalloc_moments_match_init_macros(gpu, tmp_path):
    lib = mg.lib()
    buf = DeviceBuffers()
    try:
        for k, name in enumerate(("hgh8_12", "nc21_20", "d2q9_10", "hgh8_12")):
            case = mg.Case(_case(tmp_path, name))
            n, nv = case.ncell, case.nv
            rho, u, T, g, h, xi, w, R, K, q_scale = _equilibrium_state(case, seed=k)
            s = mg.Solver(case=case, precision=mg.FP64)
            s.init_macros(rho, u, T, None, 0)
            ref = s.macros(n)
            s.close()

            args = [buf.put(g), buf.put(h), n, nv, 2, buf.put(xi), buf.put(w), buf.put(u), R, K]
            outs = [buf.empty(n), buf.empty(3 * n), buf.empty(n), buf.empty(3 * n)]
            rc = lib.meso_shakhov_moments_noalloc(*args, *outs, None)
            assert rc == mg.OK, lib.meso_last_error().decode()
            buf.sync()
            r, uu, t, q = (buf.get(outs[0], n), buf.get(outs[1], 3 * n).reshape(n, 3), buf.get(outs[2], n),
                           buf.get(outs[3], 3 * n).reshape(n, 3))
            errs = {"rho": relerr(r, ref[0]), "u": relerr(uu, ref[1]), "T": relerr(t, ref[2]),
                    "q/terms": float(np.max(np.abs(q - ref[3])) / np.max(q_scale))}
            print(name, n, nv, errs)
            for key, e in errs.items():
                assert e <= TOL, (name, key, e)
            buf.close()
    finally:
        buf.close()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    """Host-side checks, before any device work: no GPU needed."""
    lib = mg.lib()
    too_many = mg.NOALLOC_MAX_CELLS + 1
    rc = lib.meso_shakhov_moments_noalloc(None, None, too_many, 9, 2, None, None, None, 0.5, 0.0,
                                          None, None, None, None, None)
    assert rc == mg.ERR_CAPACITY
    assert "MESO_NOALLOC_MAX_CELLS" in lib.meso_last_error().decode()
    rc = lib.meso_shakhov_moments_noalloc(None, None, 0, 9, 2, None, None, None, 0.5, 0.0,
                                          None, None, None, None, None)
    assert rc == mg.ERR_INVALID
