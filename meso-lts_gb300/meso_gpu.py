"""ctypes binding of the C ABI in include/meso_gpu.h.

The product is the C-ABI library (lib/libmeso_gpu.so); this module only
declares its structs and entry points for Python callers (tests, bench,
the serving loop).  Every call goes through the library: there is no Python
or CPU implementation of the step here, and loading fails loudly when the
library has not been built.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libmeso_gpu.so")

OK, ERR_INVALID, ERR_CUDA, ERR_OOM, ERR_NAN, ERR_TIMEOUT, ERR_IO, ERR_UNSUPPORTED, ERR_CAPACITY = range(9)
SOLVER_DUGKS, SOLVER_CDUGKS, SOLVER_CDUGKS_SHAKHOV = 0, 1, 2
FP64, FP32 = 0, 1
NOALLOC_MAX_CELLS = 131072  # MESO_NOALLOC_MAX_CELLS
RES_RHO, RES_T, RES_U, RES_Q, RES_L2 = 1, 2, 4, 8, 16  # MESO_RES_*
BC = dict(fluid_interior=0, farfield_inlet=1, pressure_inlet=2, freestream_inlet=3, farfield_outlet=4,
          pressure_outlet=5, wall=6, slip_wall=7, symmetry=8)

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class MeshDesc(C.Structure):
    _fields_ = [("dim", C.c_int32), ("ncell", C.c_int32), ("nface", C.c_int32),
                ("cell_pos", _dp), ("cell_vol", _dp), ("cell_group", _ip),
                ("cell_face_ptr", _ip), ("cell_face", _ip), ("cell_nbr_ptr", _ip), ("cell_nbr", _ip),
                ("lsq_w", _dp), ("lsq_dr", _dp), ("lsq_c", _dp),
                ("face_cell", _ip), ("face_pos", _dp), ("face_area", _dp), ("face_normal", _dp),
                ("face_mark", _ip), ("min_cell_size", C.c_double), ("total_volume", C.c_double)]


class DvsDesc(C.Structure):
    _fields_ = [("nv", C.c_int32), ("xi", _dp), ("w", _dp), ("sym", _ip), ("tensor_n", C.c_int32),
                ("axis", _dp), ("max_magnitude", C.c_double)]


class MarkDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("temperature_type", C.c_int32), ("direction", C.c_int32),
                ("pad_", C.c_int32), ("density", C.c_double), ("temperature", C.c_double),
                ("pressure", C.c_double), ("velocity", C.c_double * 3), ("alpha_u", C.c_double),
                ("alpha_T", C.c_double)]


class Params(C.Structure):
    _fields_ = [("solver", C.c_int32), ("precision", C.c_int32), ("gradient_switch", C.c_int32),
                ("limiter_switch", C.c_int32), ("K", C.c_int32), ("residual_interval", C.c_int32),
                ("dt", C.c_double), ("R", C.c_double), ("T0", C.c_double), ("rho0", C.c_double),
                ("L0", C.c_double), ("mu0", C.c_double), ("vhs_index", C.c_double), ("Pr", C.c_double),
                ("Ma", C.c_double), ("Re", C.c_double), ("CFL", C.c_double), ("venkata_k", C.c_double),
                ("residual_limit", C.c_double), ("residual_fields", C.c_int32), ("tile_cells", C.c_int32),
                ("vpl", C.c_int32), ("ngroup", C.c_int32), ("pad_", C.c_int32)]


class Status(C.Structure):
    _fields_ = [("step", C.c_int32), ("run_state", C.c_int32), ("converged", C.c_int32),
                ("bad_cells", C.c_int32), ("first_bad_cell", C.c_int32), ("masked_repairs", C.c_int32),
                ("solution_time", C.c_double), ("residual", C.c_double * 8), ("nresidual", C.c_int32),
                ("pad_", C.c_int32)]


class MesoError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"meso error {code}: {msg}")
        self.code = code


_lib = None

# name -> (restype, argtypes)
_SIGS = {
    "meso_last_error": (C.c_char_p, []),
    "meso_version": (C.c_char_p, []),
    "meso_case_load": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
    "meso_case_free": (None, [C.c_void_p]),
    "meso_case_mesh": (C.c_int, [C.c_void_p, C.POINTER(MeshDesc)]),
    "meso_case_dvs": (C.c_int, [C.c_void_p, C.POINTER(DvsDesc)]),
    "meso_case_marks": (C.c_int, [C.c_void_p, C.POINTER(C.POINTER(MarkDesc)), C.POINTER(C.c_int32)]),
    "meso_case_params": (C.c_int, [C.c_void_p, C.POINTER(Params)]),
    "meso_case_initial_fields": (C.c_int, [C.c_void_p, _dp, _dp, _dp, C.POINTER(C.c_uint8)]),
    "meso_case_loop_settings": (C.c_int, [C.c_void_p, _ip, _ip, _ip, _ip, _ip]),
    "meso_ctx_create": (C.c_int, [C.POINTER(MeshDesc), C.POINTER(DvsDesc), C.POINTER(MarkDesc), C.c_int32,
                                  C.POINTER(Params), C.POINTER(C.c_uint8), C.POINTER(C.c_void_p)]),
    "meso_ctx_create_from_case": (C.c_int, [C.c_char_p, C.c_int32, C.POINTER(C.c_void_p)]),
    "meso_ctx_destroy": (None, [C.c_void_p]),
    "meso_init_macros": (C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp, C.c_int32]),
    "meso_initial": (C.c_int, [C.c_void_p]),
    "meso_step": (C.c_int, [C.c_void_p, C.c_int32, _ip]),
    "meso_fp32_refine": (C.c_int, [C.c_void_p, C.c_int32]),
    "meso_get_macros": (C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp]),
    "meso_get_flux_moments": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
    "meso_get_status": (C.c_int, [C.c_void_p, C.POINTER(Status)]),
    "meso_set_params": (C.c_int, [C.c_void_p, C.POINTER(Params)]),
    "meso_get_params": (C.c_int, [C.c_void_p, C.POINTER(Params)]),
    "meso_output": (C.c_int, [C.c_void_p]),
    "meso_snapshot_size": (C.c_size_t, [C.c_void_p]),
    "meso_snapshot": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "meso_restore": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "meso_ctx_device_bytes": (C.c_size_t, [C.c_void_p]),
    "meso_last_step_ms": (C.c_double, [C.c_void_p]),
    "meso_last_step_launches": (C.c_int64, [C.c_void_p]),
    "meso_phase_times": (C.c_int, [C.c_void_p, C.c_int32, _dp, C.c_int32, _ip]),
    "meso_phase_name": (C.c_char_p, [C.c_void_p, C.c_int32]),
    "meso_batch_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(C.c_void_p)]),
    "meso_batch_destroy": (None, [C.c_void_p]),
    "meso_batch_step": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]),
    "meso_batch_size": (C.c_int32, [C.c_void_p]),
    "meso_batch_last_step_ms": (C.c_double, [C.c_void_p]),
    "meso_batch_last_step_launches": (C.c_int64, [C.c_void_p]),
    "meso_batch_phase_times": (C.c_int, [C.c_void_p, C.c_int32, _dp, C.c_int32, _ip]),
    "meso_autotune": (C.c_int, [C.POINTER(MeshDesc), C.POINTER(DvsDesc), C.POINTER(MarkDesc), C.c_int32,
                                 C.POINTER(Params), C.c_int32, C.POINTER(Params), _dp]),
    "meso_autotune_case": (C.c_int, [C.c_char_p, C.c_int32, C.POINTER(Params), _dp]),
    "meso_autotune_forget": (None, []),
    "meso_server_create": (C.c_int, [C.c_int64, C.c_int32, C.POINTER(C.c_void_p)]),
    "meso_server_destroy": (None, [C.c_void_p]),
    "meso_server_submit": (C.c_int, [C.c_void_p, C.c_char_p, C.c_void_p, C.POINTER(C.c_int64)]),
    "meso_server_poll": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int64), C.c_int32, C.POINTER(C.c_int32)]),
    "meso_server_counts": (C.c_int, [C.c_void_p, _ip, _ip, _ip]),
    "meso_server_result": (C.c_int, [C.c_void_p, C.c_int64, _dp, _dp, _dp, _dp, C.c_void_p, _dp]),
    "meso_server_release": (C.c_int, [C.c_void_p, C.c_int64]),
    "meso_server_device_bytes": (C.c_int64, [C.c_void_p]),
    "meso_server_stats": (C.c_int, [C.c_void_p, _dp, _dp, C.POINTER(C.c_int64)]),
    "meso_case_output_grid": (C.c_int, [C.c_void_p, C.c_char_p]),
    # device pointers are passed as integers (c_void_p)
    "meso_shakhov_moments_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                                               C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_void_p,
                                               C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
}

EXPORTED = tuple(_SIGS)


def lib() -> C.CDLL:
    """Loads the library (raises if it is missing: the step has no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} not built; run `python meso-lts_gb300/build.py` first")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(rc: int) -> None:
    if rc != OK:
        raise MesoError(rc, lib().meso_last_error().decode())


def _ptr(a, t=C.c_double):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


class Case:
    """Host-only view of a case file (no GPU needed)."""

    def __init__(self, path: str):
        h = C.c_void_p()
        _check(lib().meso_case_load(os.fsencode(path), C.byref(h)))
        self._h = h
        m = MeshDesc()
        _check(lib().meso_case_mesh(h, C.byref(m)))
        self.mesh = m
        d = DvsDesc()
        _check(lib().meso_case_dvs(h, C.byref(d)))
        self.dvs = d
        mp = C.POINTER(MarkDesc)()
        n = C.c_int32()
        _check(lib().meso_case_marks(h, C.byref(mp), C.byref(n)))
        self.marks_ptr, self.nmarks = mp, n.value
        p = Params()
        _check(lib().meso_case_params(h, C.byref(p)))
        self.params = p

    @property
    def ncell(self) -> int:
        return self.mesh.ncell

    @property
    def nv(self) -> int:
        return self.dvs.nv

    def initial_fields(self):
        n = self.ncell
        rho, u, T = np.zeros(n), np.zeros(3 * n), np.zeros(n)
        mask = np.zeros(n, np.uint8)
        _check(lib().meso_case_initial_fields(self._h, _ptr(rho), _ptr(u), _ptr(T), _ptr(mask, C.c_uint8)))
        return rho, u.reshape(n, 3), T, mask

    def loop_settings(self) -> dict:
        v = [C.c_int32() for _ in range(5)]
        _check(lib().meso_case_loop_settings(self._h, *[C.byref(x) for x in v]))
        keys = ("max_step", "write_interval", "read_np_data", "output_latest", "output_np")
        return dict(zip(keys, (x.value for x in v)))

    def output_grid(self, path: str) -> None:
        """The mesh's Tecplot grid file (the grid.plt output() writes at step 0), on the host."""
        _check(lib().meso_case_output_grid(self._h, os.fsencode(path)))

    def arrays(self) -> dict:
        """Copies of the flattened tables as numpy arrays (original order)."""
        m, d = self.mesh, self.dvs
        C_, F = m.ncell, m.nface
        nf = m.cell_face_ptr[C_]
        nn = m.cell_nbr_ptr[C_]
        A = lambda p, n, dt=np.float64: np.ctypeslib.as_array(p, shape=(n,)).astype(dt).copy() if n else np.zeros(0, dt)
        out = dict(dim=m.dim, ncell=C_, nface=F, cell_pos=A(m.cell_pos, 3 * C_).reshape(C_, 3),
                   cell_vol=A(m.cell_vol, C_), cell_group=A(m.cell_group, C_, np.int32),
                   cell_face_ptr=A(m.cell_face_ptr, C_ + 1, np.int32), cell_face=A(m.cell_face, nf, np.int32),
                   cell_nbr_ptr=A(m.cell_nbr_ptr, C_ + 1, np.int32), cell_nbr=A(m.cell_nbr, nn, np.int32),
                   lsq_w=A(m.lsq_w, nn), lsq_dr=A(m.lsq_dr, 3 * nn).reshape(-1, 3), lsq_c=A(m.lsq_c, 9 * C_).reshape(C_, 9),
                   face_cell=A(m.face_cell, 2 * F, np.int32).reshape(F, 2), face_pos=A(m.face_pos, 3 * F).reshape(F, 3),
                   face_area=A(m.face_area, F), face_normal=A(m.face_normal, 3 * F).reshape(F, 3),
                   face_mark=A(m.face_mark, F, np.int32), min_cell_size=m.min_cell_size,
                   total_volume=m.total_volume, nv=d.nv, xi=A(d.xi, 3 * d.nv).reshape(-1, 3), w=A(d.w, d.nv),
                   sym=A(d.sym, 3 * d.nv, np.int32).reshape(-1, 3), tensor_n=d.tensor_n,
                   dvs_max_magnitude=d.max_magnitude)
        return out

    def close(self):
        if self._h:
            lib().meso_case_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Solver:
    """One solve on the current CUDA device (a meso_ctx)."""

    def __init__(self, case_path: str | None = None, precision: int = -1, *, case: Case | None = None,
                 params: Params | None = None, mask: np.ndarray | None = None):
        h = C.c_void_p()
        if case_path is not None:
            _check(lib().meso_ctx_create_from_case(os.fsencode(case_path), precision, C.byref(h)))
        else:
            p = Params.from_buffer_copy(params if params is not None else case.params)
            if precision in (FP64, FP32):
                p.precision = precision
            mk = None if mask is None else np.ascontiguousarray(mask, np.uint8)
            _check(lib().meso_ctx_create(C.byref(case.mesh), C.byref(case.dvs), case.marks_ptr, case.nmarks,
                                         C.byref(p), _ptr(mk, C.c_uint8), C.byref(h)))
        self._h = h
        p = Params()
        _check(lib().meso_get_params(h, C.byref(p)))
        self.params = p
        self.ncell = None

    def _n(self) -> int:
        if self.ncell is None:
            st = self.snapshot_size()  # cheap way to confirm the handle; ncell comes from macros below
        return self.ncell

    def initial(self):
        _check(lib().meso_initial(self._h))

    def init_macros(self, rho, u, T=None, q=None, mode: int = 0):
        rho = np.ascontiguousarray(rho, np.float64)
        self.ncell = rho.size
        u = np.ascontiguousarray(u, np.float64).reshape(-1)
        T = None if T is None else np.ascontiguousarray(T, np.float64)
        q = None if q is None else np.ascontiguousarray(q, np.float64).reshape(-1)
        _check(lib().meso_init_macros(self._h, _ptr(rho), _ptr(u), _ptr(T), _ptr(q), mode))

    def step(self, n: int = 1) -> int:
        done = C.c_int32()
        rc = lib().meso_step(self._h, n, C.byref(done))
        if rc != OK:
            raise MesoError(rc, lib().meso_last_error().decode())
        return done.value

    def refine(self, interval: int):
        """FP32 defect correction every `interval` steps (0: off); meso_fp32_refine."""
        _check(lib().meso_fp32_refine(self._h, interval))

    def macros(self, ncell: int):
        rho, u, T, q = np.zeros(ncell), np.zeros(3 * ncell), np.zeros(ncell), np.zeros(3 * ncell)
        _check(lib().meso_get_macros(self._h, _ptr(rho), _ptr(u), _ptr(T), _ptr(q)))
        return rho, u.reshape(ncell, 3), T, q.reshape(ncell, 3)

    def flux_moments(self, ncell: int):
        a, b, c = np.zeros(ncell), np.zeros(3 * ncell), np.zeros(ncell)
        _check(lib().meso_get_flux_moments(self._h, _ptr(a), _ptr(b), _ptr(c)))
        return a, b.reshape(ncell, 3), c

    def status(self) -> Status:
        s = Status()
        _check(lib().meso_get_status(self._h, C.byref(s)))
        return s

    def set_params(self, p: Params):
        _check(lib().meso_set_params(self._h, C.byref(p)))
        self.params = Params.from_buffer_copy(p)

    def output(self):
        _check(lib().meso_output(self._h))

    def snapshot_size(self) -> int:
        return lib().meso_snapshot_size(self._h)

    def snapshot(self) -> bytes:
        n = self.snapshot_size()
        buf = C.create_string_buffer(n)
        _check(lib().meso_snapshot(self._h, buf, n))
        return buf.raw

    def restore(self, data: bytes):
        buf = C.create_string_buffer(data, len(data))
        _check(lib().meso_restore(self._h, buf, len(data)))

    def device_bytes(self) -> int:
        return lib().meso_ctx_device_bytes(self._h)

    def last_step_ms(self) -> float:
        return lib().meso_last_step_ms(self._h)

    def last_step_launches(self) -> int:
        return lib().meso_last_step_launches(self._h)

    def phase_times(self, nsteps: int) -> dict:
        """Mean device ms per step of each kernel phase over nsteps real steps."""
        ms = np.zeros(16)
        n = C.c_int32()
        _check(lib().meso_phase_times(self._h, nsteps, _ptr(ms), 16, C.byref(n)))
        return {lib().meso_phase_name(self._h, i).decode(): float(ms[i]) for i in range(n.value)}

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            lib().meso_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """meso_batch: FP32 solvers stepped together (one set of launches per step)."""

    def __init__(self, solvers):
        self.solvers = list(solvers)
        arr = (C.c_void_p * len(self.solvers))(*[s.handle.value for s in self.solvers])
        h = C.c_void_p()
        _check(lib().meso_batch_create(arr, len(self.solvers), C.byref(h)))
        self._h = h

    def step(self, n: int = 1) -> int:
        """n steps of every running member; returns the number still running."""
        r = C.c_int32()
        _check(lib().meso_batch_step(self._h, n, C.byref(r)))
        return r.value

    def last_step_ms(self) -> float:
        return lib().meso_batch_last_step_ms(self._h)

    def last_step_launches(self) -> int:
        return lib().meso_batch_last_step_launches(self._h)

    def phase_times(self, nsteps: int = 3) -> dict:
        """Mean device ms per step of each phase, kernels launched one by one (steps the batch)."""
        ms = np.zeros(16)
        n = C.c_int32()
        _check(lib().meso_batch_phase_times(self._h, nsteps, _ptr(ms), 16, C.byref(n)))
        names = [lib().meso_phase_name(self.solvers[0].handle, i).decode() for i in range(n.value)]
        return dict(zip(names, ms[: n.value].tolist()))

    def close(self):
        if self._h:
            lib().meso_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """meso_server: served FP32 Shakhov solves with continuous batching."""

    def __init__(self, hbm_budget_bytes: int, max_members: int = 64):
        h = C.c_void_p()
        _check(lib().meso_server_create(int(hbm_budget_bytes), int(max_members), C.byref(h)))
        self._h = h
        self.ncell = {}

    def submit(self, case_path: str, params: Params | None = None) -> int:
        t = C.c_int64()
        _check(lib().meso_server_submit(self._h, os.fsencode(case_path),
                                        C.byref(params) if params is not None else None, C.byref(t)))
        c = Case(case_path)
        self.ncell[t.value] = c.ncell
        c.close()
        return t.value

    def poll(self, nsteps: int, max_done: int = 1024) -> list:
        tags = (C.c_int64 * max_done)()
        n = C.c_int32()
        _check(lib().meso_server_poll(self._h, nsteps, tags, max_done, C.byref(n)))
        return [tags[i] for i in range(n.value)]

    def stats(self) -> tuple:
        """(device ms of the batch steps, wall ms inside poll, batch steps issued) since creation."""
        g, w, n = C.c_double(), C.c_double(), C.c_int64()
        _check(lib().meso_server_stats(self._h, C.byref(g), C.byref(w), C.byref(n)))
        return g.value, w.value, n.value

    def counts(self) -> tuple:
        a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
        _check(lib().meso_server_counts(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def result(self, tag: int):
        n = self.ncell[tag]
        rho, u, T, q = np.zeros(n), np.zeros(3 * n), np.zeros(n), np.zeros(3 * n)
        st = Status()
        sec = np.zeros(2)
        _check(lib().meso_server_result(self._h, tag, _ptr(rho), _ptr(u), _ptr(T), _ptr(q), C.byref(st), _ptr(sec)))
        return (rho, u.reshape(n, 3), T, q.reshape(n, 3)), st, (float(sec[0]), float(sec[1]))

    def release(self, tag: int):
        _check(lib().meso_server_release(self._h, tag))
        self.ncell.pop(tag, None)

    def device_bytes(self) -> int:
        return lib().meso_server_device_bytes(self._h)

    def close(self):
        if self._h:
            lib().meso_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune(case_path: str, steps: int = 5) -> tuple:
    """FP32 kernel shape measured for a case file: (Params with tile_cells / vpl / ngroup, ms per step)."""
    best = Params()
    ms = np.zeros(1)
    _check(lib().meso_autotune_case(os.fsencode(case_path), steps, C.byref(best), _ptr(ms)))
    return best, float(ms[0])
