"""Generates tests/golden/: small case inputs and the reference's own outputs on them.

Run here (where the reference sources and oracle/_ref/meso_ref exist):

    bash oracle/build_ref.sh && python tests/golden/make_golden.py

For every case below it writes the inputs (case.txt, mesh.neu, the .dvs file)
into tests/golden/cases/<name>/, runs the unmodified reference solver through
oracle/_ref/meso_ref for the listed number of steps, and stores its
macroscopic fields (rho, u, T, q), step count, run_state and solution time in
<name>.npz.  Two cases also store the mesh and DVS tables the reference built
(geometry_<name>.npz).  The inputs are committed so the fixtures do not depend
on the scipy / numpy versions that generated them.
"""
from __future__ import annotations

import os
import shutil
import struct
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "meso-lts_gb300"))
import cases  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "meso_ref")
CASE_DIR = os.path.join(HERE, "cases")

# name -> (builder(dir) -> case path, steps)
GOLDEN = {
    "cdugks_q8": (lambda d: cases.bgk_cavity(d, 8, 100), 100),
    "cdugks_q8_nograd": (lambda d: cases.bgk_cavity(d, 8, 60, gradient=False), 60),
    "dugks_q8": (lambda d: cases.bgk_cavity(d, 8, 100, solver="dugks@incompressible"), 100),
    "shakhov_q8_hgh8": (lambda d: cases.shakhov_cavity(d, "quad", 8, "hgh", 8, 0.1, 0.15, 40), 40),
    "shakhov_m10_nc21": (lambda d: cases.shakhov_cavity(d, "mixed", 10, "nc", 21, 1.0, 0.15, 100), 100),
    "shakhov_t8_nc21": (lambda d: cases.shakhov_cavity(d, "tri", 8, "nc", 21, 1.0, 0.15, 10), 10),
    "shakhov_t8_blowup": (lambda d: cases.shakhov_cavity(d, "tri", 8, "nc", 21, 1.0, 0.15, 40), 40),
    "shakhov_q8_d2q9": (lambda d: cases.shakhov_cavity(d, "quad", 8, "d2q9", 3, 0.05, 0.15, 60), 60),
    "shakhov_q8_limiter": (lambda d: cases.shakhov_cavity(d, "quad", 8, "hgh", 8, 0.1, 0.15, 30, limiter=True), 30),
    "shakhov_q8_nograd": (lambda d: cases.shakhov_cavity(d, "quad", 8, "hgh", 8, 0.1, 0.15, 30, gradient=False), 30),
    "channel_pressure": (lambda d: cases.shakhov_channel(d, "pressure", steps=60), 60),
    "channel_farfield": (lambda d: cases.shakhov_channel(d, "farfield", steps=60), 60),
}
GEOMETRY = ("shakhov_m10_nc21", "channel_pressure")


def read_macros(path: str) -> dict:
    b = open(path, "rb").read()
    magic, n, step, rs = struct.unpack("<4i", b[:16])
    assert magic == 0x4D45534F
    t, secs = struct.unpack("<2d", b[16:32])
    a = np.frombuffer(b[32:], dtype="<f8")
    return dict(rho=a[:n].copy(), u=a[n:4 * n].reshape(n, 3).copy(), T=a[4 * n:5 * n].copy(),
                q=a[5 * n:8 * n].reshape(n, 3).copy(), step=step, run_state=rs, time=t)


def read_mesh(path: str) -> dict:
    b = open(path, "rb").read()
    o = [0]

    def take(fmt):
        v = struct.unpack_from("<" + fmt, b, o[0])
        o[0] += struct.calcsize("<" + fmt)
        return v if len(v) > 1 else v[0]

    assert take("i") == 0x4D455348
    dim, C, F, N = take("4i")
    mcs, tv = take("2d")
    pos, vol, nbr, w, Cm = [], [], [], [], []
    for _ in range(C):
        take("2i")
        pos.append(take("3d"))
        vol.append(take("d"))
        nf = take("i")
        take(f"{nf}i") if nf > 1 else take("i")
        nn = take("i")
        for _ in range(nn):
            nbr.append(take("i"))
            w.append(take("d"))
            take("3d")
        Cm.append(take("9d"))
    fc, fpos, area, n0 = [], [], [], []
    for _ in range(F):
        fc.append(take("2i"))
        take("i")
        fpos.append(take("3d"))
        area.append(take("d"))
        n0.append(take("3d"))
        take("3d")
    nv = take("i")
    vmax = take("d")
    xi, wv, sym = [], [], []
    for _ in range(nv):
        xi.append(take("3d"))
        wv.append(take("d"))
        sym.append(take("3i"))
    return dict(dim=dim, ncell=C, nface=F, min_cell_size=mcs, total_volume=tv, cell_pos=np.array(pos),
                cell_vol=np.array(vol), cell_nbr=np.array(nbr, np.int32), lsq_w=np.array(w),
                lsq_c=np.array(Cm), face_cell=np.array(fc, np.int32), face_pos=np.array(fpos),
                face_area=np.array(area), face_normal=np.array(n0), xi=np.array(xi), w=np.array(wv),
                sym=np.array(sym, np.int32), dvs_max_magnitude=vmax)


def main() -> None:
    if not os.path.exists(REF):
        sys.exit("oracle/_ref/meso_ref missing: run oracle/build_ref.sh first")
    os.makedirs(CASE_DIR, exist_ok=True)
    for name, (build, steps) in GOLDEN.items():
        d = os.path.join(CASE_DIR, name)
        if os.path.isdir(d):
            shutil.rmtree(d)
        path = build(d)
        args = [REF, os.path.basename(path), str(steps), "out.bin"]
        if name in GEOMETRY:
            args += ["--mesh", "mesh.bin"]
        r = subprocess.run(args, cwd=d, capture_output=True, text=True)
        if r.returncode != 0:
            raise SystemExit(f"{name}: reference failed: {r.stderr}")
        m = read_macros(os.path.join(d, "out.bin"))
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), requested=steps, **m)
        if name in GEOMETRY:
            g = read_mesh(os.path.join(d, "mesh.bin"))
            np.savez_compressed(os.path.join(HERE, f"geometry_{name}.npz"), **g)
        for junk in ("out.bin", "mesh.bin"):
            if os.path.exists(os.path.join(d, junk)):
                os.remove(os.path.join(d, junk))
        for sub in os.listdir(d):  # the reference's output folder (case-name/)
            if os.path.isdir(os.path.join(d, sub)):
                shutil.rmtree(os.path.join(d, sub))
        print(f"{name}: step {m['step']} run_state {m['run_state']}")


if __name__ == "__main__":
    main()
