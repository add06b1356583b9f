#!/usr/bin/env python3
"""Benchmark of the Shakhov CDUGKS step on one GB300 (or N replicas).

Workload (the configuration the headline metric is quoted on): rarefied 2-D
lid-driven cavity, Shakhov CDUGKS, 7744-cell unstructured mesh (seeded
jittered quadrilaterals), Newton-Cotes 101x101 velocity set on [-5,5]^2
(10201 velocities), Kn = 1, Pr = 2/3, lid 0.15, diffuse walls, FP32 storage.  Synthetic inputs written by meso-lts_gb300/cases.py in the
reference's own formats.

Metric: cell-velocity updates per second (cells x velocities x steps / time).
  value        device time of K steps (CUDA events on the library's stream),
               state resident in HBM (1.3 GB, larger than L2)
  e2e          the same through the C ABI with pinned host buffers: initial
               fields copied host->device, K steps, the macroscopic fields read
               back device->host after every step
  fp64_*       the plain FP64 step on the same workload, and the FP32 form's
               error against it after the same number of steps
  roofline     the dominant kernel (the tile kernel with the larger share of
               the step): algorithmic bytes (16 B per cell-velocity: g, h read
               and written in FP32; each launch covers every cell-velocity) /
               its event-timed duration, against the measured HBM copy bandwidth
  cpu_baseline the oracle (CPU restatement of the reference step) on all host
               cores, on a bounded sample of the same workload, fed the
               workload's mesh and velocity tables as the reference itself
               builds them (tests/golden/workload_config2.npz), not through
               the product library

--impl reference times that CPU implementation alone (rank 0) on the same
workload and prints the same JSON line with "impl": "reference".

--profile WORKLOAD runs a few steps of one workload and prints the mean device
time per step (and, with --phases, of each kernel phase), for profiler
captures; no JSON line.  WORKLOAD: config1 (FP64 BGK cavity), config2 or
config3 (--precision fp32|fp64), served64 (the first 64 requests of the served
stream, stepped as one batch, one velocity group per tile as the server runs
them).  A capture that collects more than gpu__time_duration.sum names one
kernel, e.g.

    ncu --set full --clock-control none -k regex:k32_update -s 2 -c 1 \
        python bench.py --profile config2 --steps 3
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in ("meso-lts_gb300", "oracle"):
    sys.path.insert(0, os.path.join(ROOT, _p))

import numpy as np  # noqa: E402

METRIC = "cell-xi updates/s (FP32-storage Shakhov CDUGKS step)"
UNIT = "cell-xi/s"
WORKLOAD = ("rarefied 2-D cavity, Shakhov CDUGKS, 7744-cell unstructured mesh (seeded jittered quadrilaterals), "
            "Newton-Cotes 101x101 DVS on [-5,5]^2, Kn=1, Pr=2/3, lid 0.15, FP32 storage")


def _cudart():
    for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            return ctypes.CDLL(name)
        except OSError:
            continue
    raise RuntimeError("libcudart not found")


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    """Host-side barrier and max over ranks (the replicas exchange no data)."""

    def __init__(self, world: int):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as td

            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, v: float) -> float:
        if self.world == 1:
            return v
        import torch

        t = torch.tensor([v], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v: float) -> float:
        if self.world == 1:
            return v
        import torch

        t = torch.tensor([v], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int, interval_ms: int = 50):
        self.gpu = gpu
        self.interval_ms = interval_ms
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", str(self.interval_ms)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak_hbm() -> tuple[float, str]:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic(kernel: str) -> tuple[float | None, str | None]:
    """DRAM bytes per launch of a kernel from the committed ncu summary (profiles/), if present."""
    p = os.path.join(ROOT, "profiles", f"{kernel}_config2.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["dram_bytes_per_launch"]), d.get("traffic_note")
    except (OSError, KeyError, ValueError):
        return None, None


def build_workload(tmp: str, precision: str) -> str:
    import cases

    return cases.config2(os.path.join(tmp, f"config2_{precision}"), steps=500, precision=precision)


def relerr(a, b) -> float:
    s = float(np.max(np.abs(b)))
    return float(np.max(np.abs(a - b))) / s if s > 0 else float(np.max(np.abs(a)))


def pinned(n: int):
    """numpy view of page-locked host memory (cudaHostAlloc)."""
    rt = _cudart()
    p = ctypes.c_void_p()
    if rt.cudaHostAlloc(ctypes.byref(p), ctypes.c_size_t(n * 8), 0) != 0:
        return np.zeros(n)
    buf = (ctypes.c_double * n).from_address(p.value)
    return np.frombuffer(buf, dtype=np.float64)


WORKLOAD_TABLES = os.path.join(ROOT, "tests", "golden", "workload_config2.npz")


def _oracle_workload(threads: int):
    """The oracle on the workload's mesh and velocity tables as the reference builds them
    (tests/golden/workload_config2.npz): the CPU legs load no part of the product library."""
    import meso_oracle as mo

    w = mo.Workload(WORKLOAD_TABLES)
    o = mo.Oracle(w, threads)
    o.init(w.rho, w.u, w.T, None, 0)
    return w, o


def cpu_baseline(seconds: float, threads: int) -> dict:
    w, o = _oracle_workload(threads)
    # one step to size the sample, then about `seconds` of steps (at most 30)
    t0 = time.perf_counter()
    done, _ = o.step(1)
    first = time.perf_counter() - t0
    more = max(0, min(29, int(seconds / max(first, 1e-3)) - 1))
    t1 = time.perf_counter()
    d2, _ = o.step(more) if more else (0, 0)
    done += d2
    secs = first + (time.perf_counter() - t1)
    o.close()
    cx = w.ncell * w.nv
    return {"value": cx * done / secs, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{done} full step(s) of the workload ({w.ncell} cells x {w.nv} velocities, the reference's own "
                      f"mesh and velocity tables) on {threads} threads, velocity set split as the reference's MPI "
                      "ranks split it",
            "seconds": secs}


def run_reference(args, rank: int, dist: Dist) -> None:
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    # the same step count as the GPU arm, bounded: a step takes about 0.65 s on 16 Grace cores, so
    # at most 200 timed steps after 3 to 5 warm-up steps keep the run within a few minutes
    steps = max(1, min(args.steps, 200))
    warm = max(3, min(args.warmup, 5))
    w, o = _oracle_workload(threads)
    o.step(warm)
    t0 = time.perf_counter()
    done, _ = o.step(steps)
    secs = time.perf_counter() - t0
    o.close()
    cx = w.ncell * w.nv
    v = cx * done / secs
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": done, "warmup": warm, "ms_per_step": secs * 1e3 / done, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "cells": w.ncell, "velocities": w.nv,
                       "tables": "the reference's own mesh and velocity tables of the workload "
                                 "(tests/golden/workload_config2.npz)"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{done} timed steps (requested {args.steps}, at most 200) of the full "
                                       f"workload after {warm} warm-up step(s), {threads} threads"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_other_configs(tmp: str) -> dict:
    """Config 1 (incompressible BGK cavity, 64^2 quads, D2Q9, FP64, the full 2000 steps) against the
    oracle run alongside, and config 3 (61^2 quads, hGH 28^2, Kn 0.075) in FP32 against FP64."""
    import cases
    import meso_gpu as mg
    import meso_oracle as mo

    out = {}
    p1 = cases.config1(os.path.join(tmp, "c1"), 2000)
    c1 = mg.Case(p1)
    rho, u, T, mask = c1.initial_fields()
    s = mg.Solver(case=c1, precision=mg.FP64, mask=mask)
    s.init_macros(rho, u, T, None, 0)
    s.step(2000)
    ms = s.last_step_ms()
    a = s.macros(c1.ncell)
    s.close()
    o = mo.Oracle(c1, min(os.cpu_count() or 1, c1.nv), mask)
    o.init(rho, u, T, None, 0)
    t0 = time.perf_counter()
    o.step(2000)
    cpu_s = time.perf_counter() - t0
    b = o.macros()
    o.close()
    cx1 = c1.ncell * c1.nv * 2000
    out["config1_bgk_fp64"] = {"cells": c1.ncell, "velocities": c1.nv, "steps": 2000,
                               "value": cx1 / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms / 2000,
                               "cpu_port_value": cx1 / cpu_s, "cpu_cores": min(os.cpu_count() or 1, c1.nv),
                               "max_rel_err_vs_oracle": {"rho": relerr(a[0], b[0]), "u": relerr(a[1], b[1])},
                               "note": "4096 cells x 9 velocities fits in L2; launch- and latency-bound"}
    p3 = cases.config3(os.path.join(tmp, "c3"), 5000, "fp32")
    c3 = mg.Case(p3)
    rho, u, T, mask = c3.initial_fields()
    res = {}
    for prec in (mg.FP32, mg.FP64, "refined"):  # the workload's 5000 steps; 200 of them timed
        s = mg.Solver(case=c3, precision=mg.FP32 if prec == "refined" else prec, mask=mask)
        s.init_macros(rho, u, T, None, 0)
        if prec == "refined":  # FP32 with an FP64 defect correction every 20 steps
            s.refine(20)
        s.step(3)
        s.step(200)
        ms = s.last_step_ms() / 200
        s.step(4900 - 203)
        before = s.macros(c3.ncell)
        s.step(100)
        res[prec] = (ms, s.macros(c3.ncell), before, s.status().step)
        s.close()
    cx3 = c3.ncell * c3.nv
    comps = lambda a: {"rho": a[0], "T": a[2], "u": a[1][:, 0], "v": a[1][:, 1], "qx": a[3][:, 0], "qy": a[3][:, 1]}
    e32 = {k: relerr(comps(res[mg.FP32][1])[k], v) for k, v in comps(res[mg.FP64][1]).items()}
    drift = {k: relerr(comps(res[mg.FP64][2])[k], v) for k, v in comps(res[mg.FP64][1]).items()}
    out["config3_shakhov_fp32"] = {"cells": c3.ncell, "velocities": c3.nv, "steps": res[mg.FP32][3],
                                   "value": cx3 / (res[mg.FP32][0] * 1e-3), "unit": UNIT,
                                   "ms_per_step": res[mg.FP32][0], "fp64_ms_per_step": res[mg.FP64][0],
                                   "fp32_error_vs_fp64": e32, "fp64_change_steps_4900_5000": drift,
                                   "refined_every_20": {
                                       "ms_per_step": res["refined"][0],
                                       "error_vs_fp64": {k: relerr(comps(res["refined"][1])[k], v)
                                                         for k, v in comps(res[mg.FP64][1]).items()},
                                       "note": "meso_fp32_refine(20): one FP64 step and one FP32 step from the "
                                               "same state every 20 steps measure the FP32 step's error, which the "
                                               "FP32 steps between add back"},
                                   "note": "state 23 MB fits in L2; CFL 0.5 (at 0.8 the reference blows up at step "
                                           "140, tests/golden/config3_cfl08_blowup.npz)"}
    return out


def run_host_pipeline(tmp: str, repeats: int = 5) -> dict:
    """Admission cost of a solve on the host: case load (case file, Gambit mesh, faces, geometry,
    least squares, velocity set, flattening), context creation (renumbering, tile plan, device
    tables) and the initial state, for the rarefied workload and a 128^2 hGH 28^2 served-size
    cavity; medians of `repeats` runs, wall time."""
    import cases
    import meso_gpu as mg

    out = {}
    paths = {"config2_7744_nc101": cases.config2(os.path.join(tmp, "hp_c2"), 500, "fp32"),
             "quad128_hgh28": cases.shakhov_cavity(os.path.join(tmp, "hp_q128"), "quad", 128, "hgh", 28, 0.1, 0.15,
                                                   100, name="q128", precision="fp32")}
    rt = _cudart()
    for name, p in paths.items():
        t_load, t_ctx, t_init = [], [], []
        for _ in range(repeats):
            t0 = time.perf_counter()
            case = mg.Case(p)
            t1 = time.perf_counter()
            rho, u, T, mask = case.initial_fields()
            s = mg.Solver(case=case, precision=mg.FP32, mask=mask)
            rt.cudaDeviceSynchronize()
            t2 = time.perf_counter()
            s.init_macros(rho, u, T, None, 0)
            rt.cudaDeviceSynchronize()
            t3 = time.perf_counter()
            s.close()
            case.close()
            t_load.append((t1 - t0) * 1e3)
            t_ctx.append((t2 - t1) * 1e3)
            t_init.append((t3 - t2) * 1e3)
        out[name] = {"case_load_ms": statistics.median(t_load), "context_ms": statistics.median(t_ctx),
                     "initial_state_ms": statistics.median(t_init)}
    return out


def run_batched(tmp: str, steps: int = 20, warm: int = 3, autotune: bool = True) -> dict:
    """Config 4: 64 cavity instances (seeded draws of mesh side, Kn, velocity set, lid) in one batch."""
    import cases
    import meso_gpu as mg

    insts = cases.config4_instances()
    t0 = time.perf_counter()
    paths = [cases.config4_case(os.path.join(tmp, f"b{inst['index']}"), inst, steps=1000000) for inst in insts]
    # kernel shapes: the autotuner measures one instance of each (side, velocity set) class; the
    # other instances of the class are the same size and pick the remembered shape up
    tuned = {}
    if autotune:
        for inst, path in zip(insts, paths):
            key = (inst["side"], inst["dvs"])
            if key not in tuned:
                best, ms = mg.autotune(path, steps=3)
                tuned[key] = (best.tile_cells, best.vpl, best.ngroup, round(ms, 4))
    tune_s = time.perf_counter() - t0
    # the same instances stepped one at a time, each with its tuned shape (device time per step, summed)
    alone_ms = 0.0
    alone_by_dvs, cx_by_dvs = {}, {}
    for inst, path in zip(insts, paths):
        case = mg.Case(path)
        rho, u, T, mask = case.initial_fields()
        s = mg.Solver(case=case, precision=mg.FP32, mask=mask)
        s.init_macros(rho, u, T, None, 0)
        s.step(1)
        s.step(3)
        ms1 = s.last_step_ms() / 3
        alone_ms += ms1
        alone_by_dvs[inst["dvs"]] = alone_by_dvs.get(inst["dvs"], 0.0) + ms1
        cx_by_dvs[inst["dvs"]] = cx_by_dvs.get(inst["dvs"], 0) + case.ncell * case.nv
        s.close()
        case.close()
    # batch members: the tuned tile size and velocities per lane, one velocity group per tile (the
    # batch supplies the parallelism that the groups give a solve alone)
    members = []
    for inst, path in zip(insts, paths):
        case = mg.Case(path)
        rho, u, T, mask = case.initial_fields()
        prm = case.params
        prm.precision = mg.FP32
        key = (inst["side"], inst["dvs"])
        if key in tuned:
            prm.tile_cells, prm.vpl = tuned[key][0], tuned[key][1]
        prm.ngroup = 1
        s = mg.Solver(case=case, precision=mg.FP32, mask=mask, params=prm)
        s.init_macros(rho, u, T, None, 0)
        members.append((case, s))
    setup_s = time.perf_counter() - t0
    dev_bytes = sum(s.device_bytes() for _, s in members)
    b = mg.Batch([s for _, s in members])
    b.step(warm)
    before = [s.status().step for _, s in members]
    b.step(steps)
    ms = b.last_step_ms()
    launches = b.last_step_launches()
    after = [s.status().step for _, s in members]
    cx = sum(c.ncell * c.nv * (a - b0) for (c, _), a, b0 in zip(members, after, before))
    stopped = sum(1 for _, s in members if s.status().run_state == 0)
    cx_step = sum(c.ncell * c.nv for c, _ in members)
    b.close()
    for _, s in members:
        s.close()
    mg.lib().meso_autotune_forget()
    return {"workload": "64 Shakhov cavity instances, sides {32,48,64,96,128} quads, log10 Kn ~ U(-2,0), "
                        "DVS {D2Q9, hGH 28x28, NC 101x101}, lid ~ U(0.05,0.15), seed 1, FP32 storage",
            "value": cx / (ms * 1e-3), "unit": UNIT, "steps": steps, "ms_per_step": ms / steps,
            "cell_xi_per_step": cx_step, "device_bytes": dev_bytes, "graph_launches_per_step": launches / steps,
            "alone_ms_per_step_sum": alone_ms, "batch_over_alone": alone_ms / (ms / steps),
            "alone_by_dvs": {d: {"members": sum(1 for i in insts if i["dvs"] == d), "ms_per_step_sum": alone_by_dvs[d],
                                 "cell_xi_per_step": cx_by_dvs[d],
                                 "cell_xi_per_s": cx_by_dvs[d] / (alone_by_dvs[d] * 1e-3)} for d in alone_by_dvs},
            "batch_hbm_frac": 16.0 * cx / (ms * 1e-3) / 1e9 / measured_peak_hbm()[0],
            "members_stopped": stopped, "setup_seconds": setup_s, "autotune_seconds": tune_s,
            "tuned_shapes": {f"{k[0]}^2 {k[1]}": v for k, v in tuned.items()}}


def _serve(reqs, paths, params, members: int, poll_steps: int) -> tuple[list[dict], float, tuple]:
    """Submits each request at its arrival time to a server with continuous batching and polls until
    every solve has retired; per request (in submission order): steps, converged, NaN cells, seconds
    from submission to retirement."""
    import meso_gpu as mg

    rt = _cudart()
    free_b, total_b = ctypes.c_size_t(), ctypes.c_size_t()
    rt.cudaMemGetInfo(ctypes.byref(free_b), ctypes.byref(total_b))
    srv = mg.Server(hbm_budget_bytes=int(free_b.value * 0.8), max_members=members)
    done, i, count = {}, 0, len(reqs)
    t0 = time.perf_counter()
    while len(done) < count:
        now = time.perf_counter() - t0
        while i < count and reqs[i]["arrival"] <= now:
            srv.submit(paths[i], params[i])
            i += 1
        pend, run, _ = srv.counts()
        if pend + run == 0:
            time.sleep(max(0.0, min(0.01, reqs[i]["arrival"] - now)) if i < count else 0.0)
            continue
        for t in srv.poll(poll_steps):
            _, st, sec = srv.result(t)
            done[t] = dict(step=st.step, converged=st.converged, bad=st.bad_cells, latency=sec[0])
            srv.release(t)
    wall = time.perf_counter() - t0
    stats = srv.stats()
    srv.close()
    return [done[k] for k in sorted(done)], wall, stats  # tags follow submission order


def _serial_fp64(reqs, paths, params, res, sample: list[int], max_step: int, poll_steps: int,
                 budget_s: float) -> list[dict]:
    """The sampled requests run one at a time in plain FP64 with the same stopping rule, timed on the
    host (wall time of the steps), each within a wall-time budget."""
    import meso_gpu as mg

    out = []
    for k in sample:
        case = mg.Case(paths[k])
        rho, u, T, mask = case.initial_fields()
        prm = params[k]
        prm.precision = mg.FP64
        s = mg.Solver(case=case, precision=mg.FP64, mask=mask, params=prm)
        s.init_macros(rho, u, T, None, 0)
        t1 = time.perf_counter()
        n, within = 0, True
        try:
            while n < max_step:
                if time.perf_counter() - t1 > budget_s:
                    within = False
                    break
                got = s.step(min(poll_steps, max_step - n))
                n += got
                if got == 0 or s.status().run_state == 0:
                    break
        except mg.MesoError:
            pass
        secs = time.perf_counter() - t1
        st = s.status()
        s.close()
        case.close()
        out.append({"request": k, "cells": reqs[k]["side"] ** 2, "dvs": reqs[k]["dvs"], "steps": st.step,
                    "converged": st.converged, "finished_within_budget": within, "seconds": secs,
                    "served_seconds": res[k]["latency"], "served_steps": res[k]["step"]})
    return out


def _served_summary(reqs, res, wall: float, stats: tuple, fp64: list[dict]) -> dict:
    conv = [r for r in res if r["converged"]]
    lat = sorted(r["latency"] for r in conv)
    q = lambda f: lat[min(len(lat) - 1, int(f * len(lat)))] if lat else None
    gpu_ms, poll_ms, batch_steps = stats
    fin = [x for x in fp64 if x["finished_within_budget"]]
    return {"solves_per_s": len(res) / wall, "wall_seconds": wall, "batch_steps": batch_steps,
            "gpu_seconds": gpu_ms * 1e-3, "poll_host_seconds": (poll_ms - gpu_ms) * 1e-3,
            "converged": len(conv), "capped": sum(1 for r in res if not r["converged"] and r["bad"] == 0),
            "failed_nan": sum(1 for r in res if not r["converged"] and r["bad"] > 0),
            "p50_s_converged": q(0.50), "p99_s_converged": q(0.99),
            "mean_steps_converged": float(np.mean([r["step"] for r in conv])) if conv else None,
            "by_dvs": {d: {"requests": sum(1 for r in reqs if r["dvs"] == d),
                           "converged": sum(1 for r, x in zip(reqs, res) if r["dvs"] == d and x["converged"])}
                       for d in sorted({r["dvs"] for r in reqs})},
            "serial_fp64_sample": fp64,
            "serial_fp64_solves_per_s_sample": (len(fin) / sum(x["seconds"] for x in fin)) if fin else None,
            "served_solves_per_s_same_sample": (len(fin) / sum(x["served_seconds"] for x in fin)) if fin else None,
            "serial_fp64_note": "measured: the sampled requests run one at a time in plain FP64, same stopping rule"}


def _requests(tmp, tag, reqs, max_step, nc_points):
    import cases
    import meso_gpu as mg

    paths, params = [], []
    for r in reqs:
        p = cases.config5_case(os.path.join(tmp, f"{tag}{r['index']}"), r, max_step, nc_points=nc_points)
        prm = mg.Case(p).params
        prm.residual_interval = 100
        prm.residual_limit = 1e-6
        prm.residual_fields = mg.RES_U | mg.RES_L2
        paths.append(p)
        params.append(prm)
    return paths, params


def run_served(tmp: str, count: int = 200, rate: float = 20.0, max_step: int = 8000, poll_steps: int = 100,
               members: int = 64, fp64_sample: int = 6, fp64_budget_s: float = 20.0) -> dict:
    """Config 5 scaled to a bench run: a seeded Poisson stream of small cavity solves, each run to
    convergence on U, served with continuous batching; time-to-converged per request (submission to
    retirement) over the solves that converged, capped and failed solves counted apart; serial plain
    FP64 measured on a seeded sample of the requests."""
    import cases

    reqs = cases.config5_requests(count=count, rate=rate)
    paths, params = _requests(tmp, "s", reqs, max_step, 21)
    res, wall, stats = _serve(reqs, paths, params, members, poll_steps)
    sample = sorted(int(x) for x in np.random.default_rng(5).choice(count, size=min(fp64_sample, count), replace=False))
    fp64 = _serial_fp64(reqs, paths, params, res, sample, max_step, poll_steps, fp64_budget_s)
    return {"workload": f"{count} cavity solves, Poisson arrivals {rate}/s (seed 2), sides {{16,24,32}} quads, "
                        "log10 Kn ~ U(-2,0), DVS {hGH 28x28, NC 21x21}, lid ~ U(0.05,0.15), FP32 storage, "
                        f"run to L2-relative residual 1e-6 on U per 100 steps (max-step {max_step})",
            "max_members": members, **_served_summary(reqs, res, wall, stats, fp64)}


def run_profile(args) -> int:
    """A few steps of one workload for a profiler capture (no JSON line)."""
    import cases
    import meso_gpu as mg

    with tempfile.TemporaryDirectory() as d:
        if args.profile == "served64":
            solvers, kases, work = [], [], 0
            for r in cases.config5_requests(count=64):
                case = mg.Case(cases.config5_case(os.path.join(d, f"s{r['index']}"), r, 8000))
                rho, u, T, mask = case.initial_fields()
                prm = case.params
                prm.precision = mg.FP32
                prm.ngroup = 1  # as the server runs requests that set no kernel shape
                s = mg.Solver(case=case, precision=mg.FP32, mask=mask, params=prm)
                s.init_macros(rho, u, T, None, 0)
                solvers.append(s)
                kases.append(case)
                work += case.ncell * case.nv
            b = mg.Batch(solvers)
            b.step(args.steps)
            ms = b.last_step_ms() / args.steps
            print(f"served64: 64 solves, {work} cell-velocities, {ms:.3f} ms/step, "
                  f"{work / ms * 1e3 / 1e9:.2f} G cell-xi/s")
            if args.phases:
                for k, v in b.phase_times(5).items():
                    print(f"  {k}: {v:.4f} ms")
            b.close()
            for s in solvers:
                s.close()
            for case in kases:
                case.close()
            return 0
        build = {"config1": lambda p: cases.config1(p, 10),
                 "config2": lambda p: cases.config2(p, 10, args.precision, nv1d=args.nv1d or 101),
                 "config3": lambda p: cases.config3(p, 10, args.precision)}[args.profile]
        case = mg.Case(build(os.path.join(d, args.profile)))
        rho, u, T, mask = case.initial_fields()
        prec = mg.FP32 if args.precision == "fp32" and args.profile != "config1" else mg.FP64
        s = mg.Solver(case=case, precision=prec, mask=mask)
        s.init_macros(rho, u, T, None, 0)
        s.step(args.steps)
        print(f"{args.profile} {'fp32' if prec == mg.FP32 else 'fp64'}: {case.ncell} cells x {case.nv} velocities, "
              f"{s.last_step_ms() / args.steps:.3f} ms/step, {s.last_step_launches()} launches")
        if args.phases:
            for k, v in s.phase_times(5).items():
                print(f"  {k}: {v:.4f} ms")
        s.close()
    return 0


def run_served_config5(tmp: str, count: int = 40, rate: float = 20.0, max_step: int = 3000, poll_steps: int = 100,
                       members: int = 64, fp64_sample: int = 3, fp64_budget_s: float = 20.0) -> dict:
    """The served stream drawn from the batch workload's distribution (sides {32,48,64,96,128} quads,
    DVS {D2Q9, hGH 28^2, NC 101^2}, log10 Kn ~ U(-2,0), lid ~ U(.05,.15)), Poisson arrivals at 20/s
    (seed 2), bounded to `count` requests and `max_step` steps each, reported like run_served."""
    import cases

    reqs = cases.config5_requests(count=count, rate=rate, sides=(32, 48, 64, 96, 128), dvs_kinds=("d2q9", "hgh", "nc"))
    paths, params = _requests(tmp, "c5_", reqs, max_step, 101)
    res, wall, stats = _serve(reqs, paths, params, members, poll_steps)
    sample = sorted(int(x) for x in np.random.default_rng(5).choice(count, size=min(fp64_sample, count), replace=False))
    fp64 = _serial_fp64(reqs, paths, params, res, sample, max_step, poll_steps, fp64_budget_s)
    return {"workload": f"{count} cavity solves drawn like the batch workload: sides {{32,48,64,96,128}} quads, "
                        "log10 Kn ~ U(-2,0), DVS {D2Q9, hGH 28x28, NC 101x101}, lid ~ U(0.05,0.15), Poisson arrivals "
                        f"{rate}/s (seed 2), FP32 storage, run to L2-relative residual 1e-6 on U per 100 steps, "
                        f"at most {max_step} steps",
            "max_members": members, **_served_summary(reqs, res, wall, stats, fp64)}


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--served-count", type=int, default=200)
    ap.add_argument("--served-members", type=int, default=64, help="solves stepped together at most")
    ap.add_argument("--served5-count", type=int, default=40,
                    help="requests of the served stream drawn from the batch workload's distribution")
    ap.add_argument("--profile", choices=["config1", "config2", "config3", "served64"],
                    help="run a few steps of one workload for a profiler capture and exit")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"], help="with --profile")
    ap.add_argument("--phases", action="store_true", help="with --profile: per-phase device times")
    ap.add_argument("--nv1d", type=int, default=0,
                    help="with --profile config2: Newton-Cotes points per axis (a smaller case for ncu captures)")
    args = ap.parse_args()
    if args.profile:
        _cudart().cudaSetDevice(dist_env()[2])
        return run_profile(args)
    args.warmup = max(args.warmup, 3)
    rank, world, local = dist_env()
    dist = Dist(world)
    if args.impl == "reference":
        run_reference(args, rank, dist)
        dist.close()
        return 0

    rt = _cudart()
    rt.cudaSetDevice(local)
    import meso_gpu as mg

    with tempfile.TemporaryDirectory() as tmp:
        path = build_workload(tmp, "fp32")
        case = mg.Case(path)
        rho, u, T, mask = case.initial_fields()
        C, NV = case.ncell, case.nv
        cx = C * NV
        K, W = args.steps, args.warmup

        # ---- device-timed FP32 step, state resident.  Blocks of exactly K steps, each bracketed by a
        # barrier and synchronisations and timed with CUDA events on the library's stream, repeated
        # until about a second has passed so that the clock record covers the timed region; the
        # median block is reported (all ranks run the same number of blocks)
        s = mg.Solver(case=case, precision=mg.FP32, mask=mask)
        s.init_macros(rho, u, T, None, 0)
        s.step(W)
        block_ms, ok = [], True
        with ClockSampler(local) as clk:
            reps = 1
            while len(block_ms) < reps:
                dist.barrier()
                rt.cudaDeviceSynchronize()
                done = s.step(K)
                rt.cudaDeviceSynchronize()
                block_ms.append(s.last_step_ms())
                ok = ok and done == K
                if len(block_ms) == 1:
                    reps = int(dist.max(float(min(200, max(1, math.ceil(1000.0 / max(block_ms[0], 1e-3)))))))
        ms = statistics.median(block_ms)
        launches = s.last_step_launches()
        st = s.status()
        ok = ok and st.run_state == 1
        ms_max = dist.max(ms)
        total_cx = dist.sum(float(cx * K))
        value = total_cx / (ms_max * 1e-3)
        # phase times (events on the library's stream) for the roofline of the dominant kernel
        phases = s.phase_times(5)
        fp32_macros = None
        s.close()

        # ---- plain FP64 step on the same workload, run for the workload's 500 steps (K64 of them
        # timed), and the FP32 form's error against it there; the FP64 fields' own change over the
        # last 100 steps shows how far from steady state step 500 is
        # (under torchrun, N > 1, only the timed FP64 steps: the rest holds every GPU for a minute)
        extras = world == 1
        K64 = max(3, min(K, 50))
        nerr = 500
        s64 = mg.Solver(case=case, precision=mg.FP64, mask=mask)
        s64.init_macros(rho, u, T, None, 0)
        s64.step(1)
        s64.step(K64)
        ms64 = s64.last_step_ms()
        fp64_value = cx * K64 / (ms64 * 1e-3)
        err = None
        if extras:
            s64.step(nerr - 100 - 1 - K64)
            b400 = s64.macros(C)
            s64.step(100)
            b = s64.macros(C)
            s32 = mg.Solver(case=case, precision=mg.FP32, mask=mask)
            s32.init_macros(rho, u, T, None, 0)
            s32.step(nerr)
            a = s32.macros(C)
            s32.close()
            err = {k: relerr(x, y) for k, x, y in zip(("rho", "u", "T", "q"), a, b)}
            err["fp64_change_steps_400_500"] = {k: relerr(x, y) for k, x, y in zip(("rho", "u", "T", "q"), b400, b)}
        s64.close()

        # ---- e2e through the C ABI with pinned host buffers
        hr, hu, hT = pinned(C), pinned(3 * C), pinned(C)
        hr[:] = rho
        hu[:] = u.reshape(-1)
        hT[:] = T
        orho, ou, oT, oq = pinned(C), pinned(3 * C), pinned(C), pinned(3 * C)
        e = mg.Solver(case=case, precision=mg.FP32, mask=mask)
        L = mg.lib()
        P = lambda x: x.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        L.meso_init_macros(e.handle, P(hr), P(hu), P(hT), None, 0)
        e.step(W)
        dist.barrier()
        rt.cudaDeviceSynchronize()
        t0 = time.perf_counter()
        L.meso_init_macros(e.handle, P(hr), P(hu), P(hT), None, 0)
        for _ in range(K):
            e.step(1)
            L.meso_get_macros(e.handle, P(orho), P(ou), P(oT), P(oq))
        rt.cudaDeviceSynchronize()
        e2e_secs = dist.max(time.perf_counter() - t0)
        e.close()
        e2e_value = total_cx / e2e_secs
        h2d = (C + 3 * C + C) * 8 / K
        d2h = (C + 3 * C + C + 3 * C) * 8

        peak, peak_kind = measured_peak_hbm()
        # the dominant kernel: the tile kernel with the larger share of the step; each launch of either
        # processes every cell-velocity of the step
        dom = max(("k32_reconstruct", "k32_update"), key=lambda k: phases.get(k, 0.0))
        dom_ms = phases.get(dom, None)
        alg_bytes = 16.0 * cx
        achieved = alg_bytes / (dom_ms * 1e-3) / 1e9 if dom_ms else None
        traffic, traffic_note = ncu_traffic(dom)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": ms_max / K, "timed_blocks": len(block_ms), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32 (FP64 moments and equilibria)", "data": "synthetic",
            "config": {"workload": WORKLOAD, "cells": C, "velocities": NV, "state_bytes": 16 * cx,
                       "l2": "state (1.3 GB, two buffers) larger than L2; no flush needed",
                       "timing": f"median of {len(block_ms)} blocks of {K} steps (CUDA events per block)",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "run_ok": ok,
            "fp64_value": fp64_value, "fp64_ms_per_step": ms64 / K64, "fp32_over_fp64": value / world / fp64_value,
            "fp32_error_vs_fp64": {"steps": nerr, **err} if err else None,
            "phases_ms": phases,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak if achieved else None,
                         "traffic": traffic, "alg_bytes_per_launch": alg_bytes, "traffic_note": traffic_note,
                         "step_achieved": alg_bytes / (ms_max / K * 1e-3) / 1e9,
                         "step_note": "whole step: state bytes (16 B per cell-velocity) over the step time"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "note": "initial fields host->device once per K steps; macros device->host every step"},
            "clocks": clk.summary(),
            "gpu_launches": launches,
        }
        if rank == 0 and world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(12.0, os.cpu_count() or 1)
        # the other configurations, the batch and the served streams: one GPU only (with N > 1 the
        # replicas would repeat them and hold every GPU for minutes)
        if not args.no_batched and extras:
            line["host_pipeline"] = run_host_pipeline(tmp)
            line["other_configs"] = run_other_configs(tmp)
            line["batched"] = run_batched(tmp)
        if not args.no_served and extras:
            line["served"] = run_served(tmp, count=args.served_count, members=args.served_members)
            line["served_config5"] = run_served_config5(tmp, count=args.served5_count, members=args.served_members)
        if rank == 0:
            print(json.dumps(line), flush=True)
    dist.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
