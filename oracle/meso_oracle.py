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
        L.mo_set_storage_rounding.argtypes = [vp, C.c_int32]
        L.mo_set_storage_rounding.restype = C.c_int
        L.mo_get_residual.argtypes = [vp, dp, C.POINTER(C.c_int32)]
        L.mo_get_residual.restype = C.c_int
        L.mo_set_params.argtypes = [vp, vp]
        L.mo_set_params.restype = C.c_int
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


# The C ABI's descriptor layouts (include/meso_gpu.h), so that the oracle can be fed without the
# product library: meso_mesh_desc, meso_dvs_desc, meso_mark_desc, meso_params.
_dp, _ip = C.POINTER(C.c_double), C.POINTER(C.c_int32)


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


_BC = {"fluid-interior": 0, "farfield-inlet": 1, "pressure-inlet": 2, "freestream-inlet": 3, "farfield-outlet": 4,
       "pressure-outlet": 5, "wall": 6, "slip-wall": 7, "symmetry": 8}  # config.cpp:5-15
_PATCH = {"zeroGradient": 0, "fixedValue": 1, "calculated": 2, "fromFile": 3, "switch": 4}


def _case_blocks(text: str):
    """[settings] key/value pairs and the [group] / [mark] blocks of a case file (config.cpp:30-108):
    each block a dict of key -> tokens."""
    settings, blocks, cur = {}, [], None
    for line in text.splitlines():
        t = line.split()
        if not t or t[0] == "#":
            continue
        if t[0] == "[settings]":
            cur = None
        elif t[0] in ("[group]", "[mark]"):
            cur = {"kind": t[0][1:-1]}
            blocks.append(cur)
        elif cur is None:
            settings[t[0]] = t[1] if len(t) > 1 else ""
        else:
            cur[t[0]] = t[1:]
    return settings, blocks


class Workload:
    """A Shakhov case from the reference's own mesh and velocity tables (tests/golden/
    workload_config2.npz, written by the reference's constructor) and its case file text: the
    descriptors the oracle takes, built without the product library.  Covers what the rarefied-cavity
    workload uses: fixedValue group patches and wall marks with fixedValue velocity / temperature."""

    def __init__(self, npz_path: str):
        z = np.load(npz_path)
        self._a = {k: (np.ascontiguousarray(z[k]) if z[k].ndim else z[k][()]) for k in z.files
                   if k not in ("case_text", "face_names")}
        a = self._a
        settings, blocks = _case_blocks(str(z["case_text"]))
        if settings.get("solver") != "cdugks@shakhov":
            raise NotImplementedError("Workload covers the Shakhov solver")
        m = MeshDesc()
        m.dim, m.ncell, m.nface = int(a["dim"]), int(a["ncell"]), int(a["nface"])
        for k in ("cell_pos", "cell_vol", "lsq_w", "lsq_dr", "lsq_c", "face_pos", "face_area", "face_normal"):
            setattr(m, k, a[k].ctypes.data_as(_dp))
        a["face_mark"] = a["face_group"]
        for k in ("cell_group", "cell_face_ptr", "cell_face", "cell_nbr_ptr", "cell_nbr", "face_cell", "face_mark"):
            setattr(m, k, a[k].ctypes.data_as(_ip))
        m.min_cell_size, m.total_volume = float(a["min_cell_size"]), float(a["total_volume"])
        self.mesh = m
        d = DvsDesc()
        d.nv = int(a["w"].size)
        d.xi, d.w, d.sym = a["xi"].ctypes.data_as(_dp), a["w"].ctypes.data_as(_dp), a["sym"].ctypes.data_as(_ip)
        d.tensor_n, d.axis, d.max_magnitude = 0, None, float(a["dvs_max_magnitude"])
        self.dvs = d
        marks = {b["name"][0]: b for b in blocks if b["kind"] == "mark"}
        names = [str(x) for x in z["face_names"]]
        self._marks = (MarkDesc * len(names))()
        for g, name in enumerate(names):
            md = self._marks[g]
            if name == "fluid-interior":
                continue
            b = marks[name]
            md.type = _BC[b["type"][0]]
            if md.type != _BC["wall"]:
                raise NotImplementedError("Workload covers wall marks")
            if "velocity" in b:
                for k in range(3):
                    md.velocity[k] = float(b["velocity"][2 + k])
            if "temperature" in b:
                md.temperature_type = _PATCH[b["temperature"][0]]
                md.temperature = float(b["temperature"][2])
        self.marks_ptr = C.cast(self._marks, C.POINTER(MarkDesc))
        self.nmarks = len(names)
        get = lambda k, dflt: float(settings.get(k, dflt))
        p = Params()
        p.solver, p.precision = 2, 0
        p.gradient_switch = 1 if settings.get("gradient-switch", "True") == "True" else 0
        p.limiter_switch = 1 if settings.get("limiter-switch", "False") == "True" else 0
        p.K, p.residual_interval = int(settings.get("gas-k", "0")), 100
        p.dt, p.R, p.T0 = get("timeStep", 1e-5), get("gas-constant", 0.5), get("ref-temperature", 1.0)
        p.rho0, p.L0, p.mu0 = get("ref-density", 1.0), get("ref-length", 1.0), get("ref-viscosity", 1.6e-5)
        p.vhs_index, p.Pr, p.residual_limit = get("vhs-index", 0.81), get("Pr", 0.67), get("residual-limit", 1e-6)
        self.params = p
        # initial fields from the one cell group (fixedValue density / temperature / velocity)
        groups = [b for b in blocks if b["kind"] == "group"]
        if len(groups) != 1:
            raise NotImplementedError("Workload covers one cell group")
        gb = groups[0]
        n = m.ncell
        val = lambda key: float(gb[key][2]) if key in gb else 0.0
        self.rho = np.full(n, val("density"))
        self.T = np.full(n, val("temperature"))
        self.u = np.zeros((n, 3))
        if "velocity" in gb:
            self.u[:] = [float(x) for x in gb["velocity"][2:5]]
        self.ncell, self.nv = n, d.nv


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

    def set_storage_rounding(self, on: bool, stochastic: bool = False) -> None:
        """Test hook: round the stored deviations from the reference Maxwellian to FP32 after every
        step (2-D Shakhov), the storage rounding of the FP32 form in isolation: to nearest, or
        stochastically (up with probability equal to the distance from the float below in units of
        the gap, the draw a hash of cell, velocity and step)."""
        if lib().mo_set_storage_rounding(self._h, (2 if stochastic else 1) if on else 0):
            raise RuntimeError("mo_set_storage_rounding: 2-D Shakhov only")

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
