"""Generates tests/golden/: small case inputs and the reference's own outputs on them.

Run where the reference sources and oracle/_ref/meso_ref exist:

    MESO_REF_SRC=<meso-lts checkout> bash oracle/build_ref.sh
    MESO_REF_SRC=<meso-lts checkout> python tests/golden/make_golden.py [name ...]

(no names: every case).

For every case below it writes the inputs (case.txt, mesh.neu, the .dvs file)
into tests/golden/cases/<name>/, runs the unmodified reference solver through
oracle/_ref/meso_ref for the listed number of steps, and stores its
macroscopic fields (rho, u, T, q), step count, run_state and solution time in
<name>.npz.  Two cases also store the mesh and DVS tables the reference built
(geometry_<name>.npz).  The inputs are committed so the fixtures do not depend
on the scipy / numpy versions that generated them.

The rarefied-cavity workload's tables as the reference builds them go to
workload_config2.npz (make_workload).

Further cases:
  * ref_*: the reference's own shipped inputs (files/cavity.neu with
    case-re400.txt, case-re1000.txt and case-kn0.075.txt and their velocity
    sets; files/case-neumann.txt with its gambit physical and velocity
    meshes), copied verbatim from the checkout MESO_REF_SRC names as test
    inputs.
  * *_blowup cases store the step at which the reference stops with a NaN /
    T < 0 cell (run_state 0).
  * OUTPUT cases also keep the reference's output() files (grid.plt,
    step-N/data.plt or result-N, latest/*) under output/<name>/.
  * RESTART cases run twice: the first run writes latest/ through output(),
    the second starts from it with read-np-data True; the first run's latest/
    files are kept as inputs of the second, whose fields are the golden.
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


def _with_key(case_path: str, key: str, value: str) -> str:
    _set_key(case_path, key, value)
    return case_path


def _ref_file(rel: str) -> str:
    src = os.environ.get("MESO_REF_SRC")
    if not src:
        sys.exit("MESO_REF_SRC must name the reference checkout")
    return os.path.join(src, "files", rel)


def _ref_case(case_file: str, extra: list[str]):
    """Copies one of the reference's shipped cases (and the files it reads) into d."""

    def build(d):
        os.makedirs(d, exist_ok=True)
        for rel in [case_file] + extra:
            dst = os.path.join(d, rel)
            os.makedirs(os.path.dirname(dst), exist_ok=True)
            shutil.copyfile(_ref_file(rel), dst)
        return os.path.join(d, case_file)

    return build


GOLDEN.update({
    # the reference's own inputs
    "ref_re400": (_ref_case("case-re400.txt", ["cavity.neu", "gh-3.dvs"]), 300),
    "ref_re1000": (_ref_case("case-re1000.txt", ["cavity.neu", "hGH.dvs"]), 40),
    "ref_kn0075": (_ref_case("case-kn0.075.txt", ["cavity.neu", "nc.dvs"]), 5),
    "ref_neumann": (_ref_case("case-neumann.txt", ["neumann/neumann_phy.neu", "neumann/neumann_dvs.neu"]), 4),
    # where the reference scheme blows up: the transitional cavity (61x61 quads, hGH 28^2, Kn 0.075) at
    # CFL 0.8, and the Delaunay-triangle cavity of the rarefied workload (7938 triangles, corner
    # triangles flipped; NC 21^2 velocities, Kn 1, CFL 0.8)
    "config3_cfl08_blowup": (lambda d: cases.shakhov_cavity(d, "quad", 61, "hgh", 28, 0.075, 0.15, 400,
                                                            name="config3", cfl=0.8), 400),
    "tri64_nc21_blowup": (lambda d: cases.shakhov_cavity(d, "tri", 64, "nc", 21, 1.0, 0.15, 200, name="tri64",
                                                         cfl=0.8), 200),
    # output() files and the read-np-data restart
    "out_shakhov_q8": (lambda d: cases.shakhov_cavity(d, "quad", 8, "hgh", 8, 0.1, 0.15, 20, name="outs"), 20),
    "out_cdugks_q8": (lambda d: cases.bgk_cavity(d, 8, 30, name="outb"), 30),
    "restart_shakhov_q8": (lambda d: cases.shakhov_cavity(d, "quad", 8, "hgh", 8, 0.1, 0.15, 20, name="rs"), 20),
    "restart_cdugks_q8": (lambda d: cases.bgk_cavity(d, 8, 30, name="rb"), 30),
    # 3-D: bricks with the gradient, tetrahedra without (their corner cells have two neighbours);
    # Newton-Cotes 9^3 velocities on [-4, 4]^3, W and qz in the output
    "shakhov_brick4_nc9": (lambda d: cases.shakhov_cavity3d(d, "brick", 4, 9, 0.5, 0.15, 20), 20),
    "shakhov_tetra3_nc9": (lambda d: cases.shakhov_cavity3d(d, "tetra", 3, 9, 0.5, 0.15, 20, gradient=False), 20),
    # the residual check and the 10-check convergence counter: both stop with run_state 0 by convergence
    "cdugks_q8_converge": (lambda d: _with_key(cases.bgk_cavity(d, 8, 100000), "residual-limit", "1e-05"), 100000),
    "shakhov_q8_converge": (lambda d: cases.shakhov_cavity(d, "quad", 8, "hgh", 8, 0.1, 0.15, 100000), 100000),
})
OUTPUT = ("out_shakhov_q8", "out_cdugks_q8")
RESTART = ("restart_shakhov_q8", "restart_cdugks_q8")


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


def read_mesh_full(path: str) -> dict:
    """Every table the harness's --mesh dump holds, as flat arrays in the layout of the C ABI's
    mesh and velocity-set descriptors (cells and faces in the reference's order)."""
    b = open(path, "rb").read()
    o = [0]

    def take(fmt):
        v = struct.unpack_from("<" + fmt, b, o[0])
        o[0] += struct.calcsize("<" + fmt)
        return v if len(v) > 1 else v[0]

    assert take("i") == 0x4D455348
    dim, C, F, N = take("4i")
    mcs, tv = take("2d")
    pos, vol, grp, cf_ptr, cf, nb_ptr, nbr, w, dr, lsq_c = [], [], [], [0], [], [0], [], [], [], []
    for _ in range(C):
        _, g = take("2i")
        grp.append(g)
        pos.append(take("3d"))
        vol.append(take("d"))
        nf = take("i")
        ids = take(f"{nf}i")
        cf.extend(ids if nf > 1 else [ids])
        cf_ptr.append(len(cf))
        nn = take("i")
        for _ in range(nn):
            nbr.append(take("i"))
            w.append(take("d"))
            dr.append(take("3d"))
        nb_ptr.append(len(nbr))
        lsq_c.append(take("9d"))
    fc, fgrp, fpos, area, n0 = [], [], [], [], []
    for _ in range(F):
        fc.append(take("2i"))
        fgrp.append(take("i"))
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
    i32 = lambda a: np.asarray(a, np.int32)
    f64 = lambda a: np.asarray(a, np.float64)
    return dict(dim=dim, ncell=C, nface=F, nnode=N, min_cell_size=mcs, total_volume=tv,
                cell_pos=f64(pos).reshape(-1), cell_vol=f64(vol), cell_group=i32(grp), cell_face_ptr=i32(cf_ptr),
                cell_face=i32(cf), cell_nbr_ptr=i32(nb_ptr), cell_nbr=i32(nbr), lsq_w=f64(w),
                lsq_dr=f64(dr).reshape(-1), lsq_c=f64(lsq_c).reshape(-1), face_cell=i32(fc).reshape(-1),
                face_group=i32(fgrp), face_pos=f64(fpos).reshape(-1), face_area=f64(area),
                face_normal=f64(n0).reshape(-1), xi=f64(xi).reshape(-1), w=f64(wv), sym=i32(sym).reshape(-1),
                dvs_max_magnitude=vmax)


def make_workload() -> None:
    """tests/golden/workload_config2.npz: the rarefied-cavity workload's mesh and velocity tables as
    the reference itself builds them (its constructor, --mesh-only), with the case file text and the
    mesh's face-group names; the CPU reference arm of bench.py runs the oracle on them."""
    import tempfile

    with tempfile.TemporaryDirectory() as d:
        path = cases.config2(os.path.join(d, "c2"), 500, "fp64")
        cd = os.path.dirname(path)
        r = subprocess.run([REF, os.path.basename(path), "0", "out.bin", "--mesh", "mesh.bin", "--mesh-only", "1"],
                           cwd=cd, capture_output=True, text=True)
        if r.returncode != 0:
            raise SystemExit(f"workload: reference failed: {r.stderr}")
        m = read_mesh_full(os.path.join(cd, "mesh.bin"))
        names = ["fluid-interior"]
        lines = open(os.path.join(cd, "mesh.neu")).read().splitlines()
        for i, line in enumerate(lines):
            if line.split()[:2] == ["BOUNDARY", "CONDITIONS"]:
                names.append(lines[i + 1].split()[0])
        np.savez_compressed(os.path.join(HERE, "workload_config2.npz"), case_text=open(path).read(),
                            face_names=np.array(names), **m)
    print(f"workload_config2: {m['ncell']} cells, {m['nface']} faces, {len(m['w'])} velocities")


def _case_name(case_path: str) -> str:
    for line in open(case_path):
        t = line.split()
        if len(t) >= 2 and t[0] == "case-name":
            return t[1]
    return "unnamed"


def _set_key(case_path: str, key: str, value: str) -> None:
    lines = open(case_path).read().splitlines()
    out, done = [], False
    for line in lines:
        t = line.split()
        if t and t[0] == key:
            out.append(f"{key} {value}")
            done = True
        else:
            out.append(line)
            if not done and t and t[0] == "[settings]":
                out.append(f"{key} {value}")
                done = True
    open(case_path, "w").write("\n".join(out) + "\n")


def main() -> None:
    if not os.path.exists(REF):
        sys.exit("oracle/_ref/meso_ref missing: run oracle/build_ref.sh first")
    os.makedirs(CASE_DIR, exist_ok=True)
    only = set(sys.argv[1:])
    if not only or "workload_config2" in only:
        make_workload()
    for name, (build, steps) in GOLDEN.items():
        if only and name not in only:
            continue
        d = os.path.join(CASE_DIR, name)
        if os.path.isdir(d):
            shutil.rmtree(d)
        path = build(d)
        inputs = set(os.listdir(d))  # files and folders the case reads (not the reference's output)
        cname = _case_name(path)
        args = [REF, os.path.relpath(path, d), str(steps), "out.bin"]
        if name in GEOMETRY:
            args += ["--mesh", "mesh.bin"]
        if name in OUTPUT or name in RESTART:
            args += ["--output", "1"]
        r = subprocess.run(args, cwd=d, capture_output=True, text=True)
        if r.returncode != 0:
            raise SystemExit(f"{name}: reference failed: {r.stderr}")
        if name in OUTPUT:  # keep the reference's output() files
            dst = os.path.join(HERE, "output", name)
            if os.path.isdir(dst):
                shutil.rmtree(dst)
            shutil.copytree(os.path.join(d, cname), dst)
        if name in RESTART:  # second run from the first run's latest/ files
            _set_key(path, "read-np-data", "True")
            r = subprocess.run(args[:4], cwd=d, capture_output=True, text=True)
            if r.returncode != 0:
                raise SystemExit(f"{name}: reference restart failed: {r.stderr}")
            for sub in os.listdir(os.path.join(d, cname)):  # keep only the restart inputs
                if sub != "latest":
                    p = os.path.join(d, cname, sub)
                    shutil.rmtree(p) if os.path.isdir(p) else os.remove(p)
        m = read_macros(os.path.join(d, "out.bin"))
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), requested=steps, **m)
        if name in GEOMETRY:
            g = read_mesh(os.path.join(d, "mesh.bin"))
            np.savez_compressed(os.path.join(HERE, f"geometry_{name}.npz"), **g)
        for junk in ("out.bin", "mesh.bin"):
            if os.path.exists(os.path.join(d, junk)):
                os.remove(os.path.join(d, junk))
        for sub in os.listdir(d):  # the reference's output folder (case-name/), except restart inputs
            if sub not in inputs and os.path.isdir(os.path.join(d, sub)) and not (name in RESTART and sub == cname):
                shutil.rmtree(os.path.join(d, sub))
        print(f"{name}: step {m['step']} run_state {m['run_state']}")


if __name__ == "__main__":
    main()
