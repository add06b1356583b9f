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


def _numpy_moments(g, h, xi, w, u0, R, K, dim):
    """The same sums in numpy (FP64): rho, u, T, q of a state, heat flux about u0."""
    rho = g @ w
    mom = (g * w[None, :]) @ xi[:, :dim]
    u = np.zeros((g.shape[0], 3))
    u[:, :dim] = mom / rho[:, None]
    kk = np.sum(xi[:, :dim] ** 2, axis=1)
    rhoE = 0.5 * ((g * kk[None, :] + h) @ w)
    Cv = (K + 3.0) * R * 0.5
    T = (rhoE / rho - 0.5 * np.sum(u * u, axis=1)) / Cv
    c = xi[None, :, :dim] - u0[:, None, :dim]
    s = np.sum(c * c, axis=-1) * g + h
    q = np.zeros((g.shape[0], 3))
    q[:, :dim] = 0.5 * np.einsum("cpd,cp,p->cd", c, s, w)
    qs = 0.5 * np.einsum("cpd,cp,p->d", np.abs(c), np.abs(s), w).max()
    return rho, u, T, q, qs


def _tensor_set(n: int, dim: int, lim: float):
    """A Newton-Cotes-like tensor velocity set on [-lim, lim]^dim (trapezoid weights)."""
    x = np.linspace(-lim, lim, n)
    wx = np.full(n, x[1] - x[0])
    wx[0] = wx[-1] = 0.5 * (x[1] - x[0])
    grids = np.meshgrid(*([x] * dim), indexing="ij")
    wg = np.meshgrid(*([wx] * dim), indexing="ij")
    xi = np.zeros((n ** dim, 3))
    for d in range(dim):
        xi[:, d] = grids[d].reshape(-1)
    w = np.prod(np.stack([a.reshape(-1) for a in wg]), axis=0)
    return xi, w


def _maxwell(rho, u, T, xi, R, K, dim):
    c = xi[None, :, :dim] - u[:, None, :dim]
    cc = np.sum(c * c, axis=-1)
    RT = R * T
    g = rho[:, None] / (2.0 * np.pi * RT[:, None]) ** (dim / 2.0) * np.exp(-cc / (2.0 * RT[:, None]))
    h = (K + 3.0 - dim) * RT[:, None] * g
    return g, h


@pytest.mark.gpu
@pytest.mark.parametrize("dim,ncell,nside,lim", [(3, 300, 13, 4.0), (2, 131072, 3, 1.7320508075688772)])
def test_noalloc_moments_match_numpy(gpu, dim, ncell, nside, lim):
    """3-D states, and the largest accepted cell count (one velocity group: the partials fill the
    scratch array), against the same sums evaluated in numpy, two calls in a row."""
    lib = mg.lib()
    R, K = 0.5, 1.0
    xi, w = _tensor_set(nside, dim, lim)
    nv = xi.shape[0]
    buf = DeviceBuffers()
    try:
        for call in range(2):
            rng = np.random.default_rng(10 * dim + call)
            rho = 1.0 + 0.2 * (rng.random(ncell) - 0.5)
            T = 1.0 + 0.3 * (rng.random(ncell) - 0.5)
            u = np.zeros((ncell, 3))
            u[:, :dim] = 0.2 * (rng.random((ncell, dim)) - 0.5)
            u0 = u + 0.05 * (rng.random((ncell, 3)) - 0.5)
            u0[:, dim:] = 0.0
            g, h = _maxwell(rho, u, T, xi, R, K, dim)
            g *= 1.0 + 0.01 * (rng.random(g.shape) - 0.5)  # off equilibrium: non-zero heat flux
            ref = _numpy_moments(g, h, xi, w, u0, R, K, dim)
            outs = [buf.empty(ncell), buf.empty(3 * ncell), buf.empty(ncell), buf.empty(3 * ncell)]
            rc = lib.meso_shakhov_moments_noalloc(buf.put(g), buf.put(h), ncell, nv, dim, buf.put(xi), buf.put(w),
                                                  buf.put(u0), R, K, *outs, None)
            assert rc == mg.OK, lib.meso_last_error().decode()
            buf.sync()
            got = (buf.get(outs[0], ncell), buf.get(outs[1], 3 * ncell).reshape(ncell, 3), buf.get(outs[2], ncell),
                   buf.get(outs[3], 3 * ncell).reshape(ncell, 3))
            errs = {"rho": relerr(got[0], ref[0]), "u": relerr(got[1], ref[1]), "T": relerr(got[2], ref[2]),
                    "q/terms": float(np.max(np.abs(got[3] - ref[3])) / ref[4])}
            print(dim, ncell, nv, call, errs)
            for key, e in errs.items():
                assert e <= TOL, (dim, ncell, call, key, e)
            buf.close()
    finally:
        buf.close()


@pytest.mark.gpu
def test_noalloc_moments_match_oracle(gpu, tmp_path):
    """The oracle's initial() moments of a mode-0 state (cdugks_shakhov.cpp:102-169) against the
    entry point on the same state, built in numpy."""
    import meso_oracle as mo

    lib = mg.lib()
    buf = DeviceBuffers()
    try:
        case = mg.Case(_case(tmp_path, "nc21_20"))
        n, nv = case.ncell, case.nv
        rho, u, T, g, h, xi, w, R, K, q_scale = _equilibrium_state(case, seed=7)
        o = mo.Oracle(case, 1)
        o.init(rho, u, T, None, 0)
        ref = o.macros()
        o.close()
        outs = [buf.empty(n), buf.empty(3 * n), buf.empty(n), buf.empty(3 * n)]
        rc = lib.meso_shakhov_moments_noalloc(buf.put(g), buf.put(h), n, nv, 2, buf.put(xi), buf.put(w), buf.put(u),
                                              R, K, *outs, None)
        assert rc == mg.OK, lib.meso_last_error().decode()
        buf.sync()
        got = (buf.get(outs[0], n), buf.get(outs[1], 3 * n).reshape(n, 3), buf.get(outs[2], n),
               buf.get(outs[3], 3 * n).reshape(n, 3))
        errs = {"rho": relerr(got[0], ref[0]), "u": relerr(got[1], ref[1]), "T": relerr(got[2], ref[2]),
                "q/terms": float(np.max(np.abs(got[3] - ref[3])) / np.max(q_scale))}
        print(errs)
        for key, e in errs.items():
            assert e <= TOL, (key, e)
    finally:
        buf.close()


def test_noalloc_rejects_host_memory():
    """A pageable host array is not device memory of the current GPU: MESO_ERR_INVALID, on a
    machine with or without a GPU."""
    lib = mg.lib()
    a = np.zeros(64)
    pa = a.ctypes.data
    rc = lib.meso_shakhov_moments_noalloc(pa, pa, 4, 9, 2, pa, pa, pa, 0.5, 0.0, pa, pa, pa, pa, None)
    assert rc == mg.ERR_INVALID, rc
    assert "device" in lib.meso_last_error().decode()


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
