"""Benchmark of the fused D3Q19 MRT step on GB300.

Workload (single GPU): single-phase porous flow on a 256^3 seeded sphere pack
(radii U[4,10], porosity 0.35, percolating cluster only), fixed pressure
rho = 1.0005 / 1.0 on the x faces, periodic y/z, niu = 0.1, FP32 populations.
A "step" is one lattice time step over that lattice (one kernel launch).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line.  ``value`` = fluid-node MLUPS with the state resident in
HBM, timed with CUDA events on the library's stream; ``e2e`` = the same metric
through the public solver class with host buffers (geometry upload, init, K
steps, rho/v download inside the timed region); ``roofline`` = algorithmic
bytes (152 B per fluid node per step) / launch time against the measured HBM
copy bandwidth; ``cpu_baseline`` = the CPU oracle (the reference's four-sweep
algorithm in C/OpenMP) on a bounded sample of the same workload;
``time_to_converged_k`` = the metric's second half: the same lattice run to a
steady permeability (|dk/k| <= 1e-6 over 500 steps) by the plain FP32 kernel and
by the chosen FP16 deviation storage, wall time and k error against an FP64 run
of the same solver (skip with ``--no-convergence``).
``--impl reference`` times that CPU implementation alone on all host threads.
Under torchrun (N > 1) every rank runs its own replica (the path is replicated,
not sharded: there is no exchange step).
"""
import argparse
import importlib.util
import json
import os
import re
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SHAPE = (256, 256, 256)
PACK = dict(rmin=4.0, rmax=10.0, porosity=0.35, seed=2)
RHO_IN, RHO_OUT, NIU = 1.0005, 1.0, 0.1
BYTES_PER_NODE = {"f32": 152, "f32dev": 152, "f16": 76, "bf16": 76, "f64": 304}
METRIC = "MLUPS"
UNIT = "MLUPS (1e6 fluid-node updates per second)"
PROFILE_MD = os.path.join(ROOT, "profiles", "sp_step_kernel_f32_porous256.md")


def workload_config(storage="f32"):
    return {"workload": "single-phase D3Q19 MRT step, 256^3 sphere pack (r U[4,10], phi 0.35, seed 2, "
                        "percolating), pressure x 1.0005/1.0, periodic y/z, niu 0.1",
            "lattice": list(SHAPE), "storage": storage, "steps_per_launch": 1,
            "l2": "inputs larger than L2 (populations ~0.9 GB per step vs 129 MB L2), no flush",
            "parallelism": "replicas"}


def geometry():
    from taichi_lbm3d_gb300.geometry import sphere_pack
    return sphere_pack(SHAPE, PACK["rmin"], PACK["rmax"], PACK["porosity"], PACK["seed"])


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic_per_node():
    """dram bytes per fluid node per launch from the committed ncu summary."""
    try:
        txt = open(PROFILE_MD).read()
        m = re.search(r"dram_bytes_per_fluid_node:\s*([0-9.]+)", txt)
        return float(m.group(1)) if m else None
    except OSError:
        return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms."""
    Q = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.samples = []
        self.proc = None
        self.index = index

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append((time.time(), line.strip()))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self, t0, t1):
        rows = [s for t, s in self.samples if t0 <= t <= t1] or [s for _, s in self.samples[-3:]]
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            f = [x.strip() for x in r.split(",")]
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(secs, device="cpu"):
    """Slowest rank's time: every replica does the same work, the job ends with the last."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(secs)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def time_device(lat, steps, warmup):
    """Warm up, then time `steps` launches with CUDA events on the library stream."""
    import torch
    stream = torch.cuda.ExternalStream(lat.stream())
    lat.step_async(warmup)
    lat.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    lat.step_async(steps)
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / 1e3


def run_variant(solid, storage, steps, warmup):
    from taichi_lbm3d_gb300 import _native
    p = _native.make_params(SHAPE, niu=NIU, bc=(1, 1, 0, 0, 0, 0), rho_bc=(RHO_IN, RHO_OUT, 1, 1, 1, 1),
                            storage=storage)
    lat = _native.Lattice(p)
    lat.set_geometry(solid)
    lat.init()
    secs = time_device(lat, steps, warmup)
    nf = lat.info().n_fluid
    lat.close()
    return nf, secs


def e2e_run(solid, steps):
    """Same metric through the public class, host buffers in and out.  Returns
    the MLUPS over the whole sequence and the seconds of its three phases:
    setup (class construction, mask upload, device index build, init), steps
    (run(K), synchronous) and readback (dense rho and v as fresh numpy arrays)."""
    from taichi_lbm3d_gb300 import LB3D_Solver_Single_Phase
    t0 = time.perf_counter()
    lb = LB3D_Solver_Single_Phase(*SHAPE)
    lb.solid.from_numpy(solid)
    lb.set_viscosity(NIU)
    lb.set_bc_rho_x0(RHO_IN)
    lb.set_bc_rho_x1(RHO_OUT)
    lb.init_simulation()
    t1 = time.perf_counter()
    lb.run(steps)
    t2 = time.perf_counter()
    rho = lb.rho.to_numpy()
    v = lb.v.to_numpy()
    t3 = time.perf_counter()
    nf = lb.n_fluid
    lb.close()
    h2d = solid.size * 1                                         # the int8 mask (index built on the device)
    d2h = 16 * solid.size                                        # dense rho + v (scattered on the device)
    assert np.isfinite(rho).all() and np.isfinite(v).all()
    phases = {"setup_s": t1 - t0, "steps_s": t2 - t1, "readback_s": t3 - t2,
              "steps_only_mlups": nf * steps / (t2 - t1) / 1e6}
    return nf * steps / (t3 - t0) / 1e6, h2d / steps, d2h / steps, phases


def cpu_baseline(solid, max_seconds=20.0):
    """The CPU oracle (reference algorithm: 4 sweeps, AoS, OpenMP) on this
    workload for a bounded number of steps."""
    from oracle.oracle import Oracle, make_params
    cores = len(os.sched_getaffinity(0))
    p = make_params(SHAPE, niu=NIU, bc=(1, 1, 0, 0, 0, 0), rho_bc=(RHO_IN, RHO_OUT, 1, 1, 1, 1))
    o = Oracle(p, solid)
    o.step(1)                       # warm-up (page-in)
    nf = int((solid == 0).sum())
    n, t = 0, 0.0
    while t < max_seconds and n < 200:
        t0 = time.perf_counter()
        o.step(1)
        t += time.perf_counter() - t0
        n += 1
    o.close()
    return {"value": nf * n / t / 1e6, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%d steps of the full 256^3 workload (%.1f s)" % (n, t)}


def convergence(storages=("f64", "f32", "f32dev", "f16", "bf16"), tol=1e-6, check_every=500, max_steps=200_000,
                shape=SHAPE, visc="standard", solid=None):
    """The 256^3 pack run to steady state: |dk/k| <= tol over check_every steps.
    Each storage variant reports steps, wall time and its permeability error
    against the FP64 run of the same solver."""
    from taichi_lbm3d_gb300 import LB3D_Solver_Single_Phase
    if solid is None and shape == SHAPE:
        solid = geometry()
    if solid is None:
        from taichi_lbm3d_gb300.geometry import sphere_pack
        solid = sphere_pack(shape, PACK["rmin"], PACK["rmax"], PACK["porosity"], PACK["seed"])
    out = {}
    for sto in storages:
        lb = LB3D_Solver_Single_Phase(*shape, storage=sto, viscosity_convention=visc, guo_convention="standard")
        lb.solid.from_numpy(solid)
        lb.set_viscosity(NIU)
        lb.set_bc_rho_x0(RHO_IN)
        lb.set_bc_rho_x1(RHO_OUT)
        lb.init_simulation()
        t0 = time.perf_counter()
        r = lb.run_to_convergence(tol=tol, check_every=check_every, max_steps=max_steps)
        secs = time.perf_counter() - t0
        r.update(seconds=secs, mlups=lb.n_fluid * r["steps"] / secs / 1e6)
        lb.close()
        out[sto] = r
    if "f64" in out:
        k64 = out["f64"]["k"]
        for sto, r in out.items():
            r["k_rel_err_vs_f64"] = abs(r["k"] - k64) / abs(k64)
    return out


CHOSEN_STORAGE = "f16"      # the mixed-precision storage the method uses (FP16 deviations, FP32 collide)


def converged_k_summary(res, tol=1e-6, check_every=500):
    """The metric's second half: wall time to the converged permeability of
    the plain FP32 kernel (reference arithmetic) and of the chosen storage, each
    with its k error against the FP64 run of the same solver."""
    def one(r):
        return {"steps": int(r["steps"]), "seconds": r["seconds"], "mlups": r["mlups"], "k": r["k"],
                "converged": bool(r["converged"]), "k_rel_err_vs_f64": r.get("k_rel_err_vs_f64")}
    out = {"criterion": "|dk/k| <= %g over %d steps" % (tol, check_every),
           "conventions": "standard (tau = 3 niu + 1/2, Guo 3/9), same lattice, faces and niu as the step",
           "accuracy_bar": 1e-3, "f64": one(res["f64"]), "plain_f32": one(res["f32"]),
           "chosen": dict(one(res[CHOSEN_STORAGE]), storage=CHOSEN_STORAGE)}
    out["others"] = {k: one(v) for k, v in res.items() if k not in ("f64", "f32", CHOSEN_STORAGE)}
    out["chosen_speedup_wall"] = res["f32"]["seconds"] / res[CHOSEN_STORAGE]["seconds"]
    out["plain_within_bar"] = res["f32"]["k_rel_err_vs_f64"] <= 1e-3
    out["chosen_within_bar"] = res[CHOSEN_STORAGE]["k_rel_err_vs_f64"] <= 1e-3
    return out


def batched(n_sub=256, seeds0=4000, fp64_subset=16, storage="f16", tol=1e-6, check_every=500,
            max_steps=100_000, log=lambda m: print(m, file=sys.stderr, flush=True)):
    """Batched permeability: n_sub seeded subvolumes (edges {48..160}, r U[3,8], phi
    U[0.25,0.5]), fx = 1e-6, periodic, niu 0.1, each to steady state:
    one persistent graph-captured batch (autotuned) against a serial loop of the
    plain FP32 kernel; per-sample k error against FP64 on a subset."""
    from taichi_lbm3d_gb300 import autotune
    from taichi_lbm3d_gb300.batch import Batch, subvolume_solids
    t0 = time.perf_counter()
    solids = subvolume_solids(range(seeds0, seeds0 + n_sub))          # spawned pool, before CUDA
    log("generated %d subvolumes in %.1f s" % (n_sub, time.perf_counter() - t0))
    edges = [s.shape[0] for s in solids]
    by_edge = {}
    for s in solids:
        by_edge.setdefault(s.shape[0], [])
        if len(by_edge[s.shape[0]]) < 4:
            by_edge[s.shape[0]].append(s)
    tuned = autotune.tune(by_edge, storage=storage, log=log)
    tiles, block = autotune.plan(edges, tuned)
    force = (1e-6, 0.0, 0.0)

    def run_batch(subset, sto, tl, blk):
        b = Batch([solids[q] for q in subset], niu=NIU, force=force, storage=sto)
        b.configure([tl[q] for q in subset], blk)
        b.init()
        t = time.perf_counter()
        d, st, cv = b.run_to_convergence(tol=tol, check_every=check_every, max_steps=max_steps)
        secs = time.perf_counter() - t
        k = b.permeability(d)
        nf = b.info()["n_fluid"]
        b.close()
        return k, st, cv, secs, nf

    allq = list(range(n_sub))
    k_b, st_b, cv_b, secs_b, nf_all = run_batch(allq, storage, tiles, block)
    log("batched %s: %.1f s, %d/%d converged" % (storage, secs_b, cv_b.sum(), n_sub))
    # serial loop of the plain FP32 kernel, one lattice at a time
    from taichi_lbm3d_gb300 import LB3D_Solver_Single_Phase
    t = time.perf_counter()
    k_s, st_s = [], []
    for q in allq:
        lb = LB3D_Solver_Single_Phase(*solids[q].shape, storage="f32", viscosity_convention="standard",
                                      guo_convention="standard")
        lb.solid.from_numpy(solids[q])
        lb.set_viscosity(NIU)
        lb.set_force(force)
        lb.init_simulation()
        r = lb.run_to_convergence(tol=tol, check_every=check_every, max_steps=max_steps)
        lb.close()
        k_s.append(r["k"])
        st_s.append(r["steps"])
    secs_s = time.perf_counter() - t
    log("serial f32: %.1f s" % secs_s)
    sub = allq[:fp64_subset]
    k64, _, cv64, secs64, _ = run_batch(sub, "f64", [256] * n_sub, 128)
    err_b = np.abs(k_b[sub] - k64) / np.abs(k64)
    err_s = np.abs(np.array(k_s)[sub] - k64) / np.abs(k64)
    total_updates = float(np.sum([int((s == 0).sum()) * n for s, n in zip(solids, st_b)]))
    return {"n_sub": n_sub, "edges": {str(e): edges.count(e) for e in sorted(set(edges))},
            "n_fluid_total": int(nf_all), "storage": storage, "block": block,
            "tiles": {str(e): int(tuned[e]["tile"]) for e in sorted(tuned)},
            "batched_seconds": secs_b, "batched_mlups": total_updates / secs_b / 1e6,
            "batched_converged": int(cv_b.sum()), "serial_f32_seconds": secs_s,
            "wall_time_ratio_serial_over_batched": secs_s / secs_b,
            "steps_batched_mean": float(np.mean(st_b)), "steps_serial_mean": float(np.mean(st_s)),
            "fp64_subset": len(sub), "fp64_seconds": secs64, "fp64_converged": int(cv64.sum()),
            "k_rel_err_batched_vs_f64_max": float(err_b.max()), "k_rel_err_batched_vs_f64_median": float(np.median(err_b)),
            "k_rel_err_serial_f32_vs_f64_max": float(err_s.max()),
            "k_rel_err_serial_f32_vs_f64_median": float(np.median(err_s))}


def two_phase(steps=20000, every=500, shape=(131, 131, 131), storages=("f64", "f32", "f16"), cpu=True,
              cpu_seconds=20.0, log=lambda m: print(m, file=sys.stderr, flush=True)):
    """Two-phase colour-gradient drainage on a 131^3 pack (seed 3, r U[3,8],
    phi 0.40), psi = -1 with a 5-node psi = +1 slab at x-left, constant psi +1 /
    -1 and pressure 1.001 / 1.0 on the x faces, periodic y/z, CapA 0.005,
    psi_solid 0.7, niu_l 0.05, niu_g 0.2.  Saturation and interface position
    every `every` steps for each storage, compared with FP64; MLUPS timed with
    CUDA events on a separate 2000-step run."""
    import torch
    from taichi_lbm3d_gb300 import LB3D_Solver_Two_Phase
    from taichi_lbm3d_gb300.geometry import sphere_pack
    solid = sphere_pack(shape, 3.0, 8.0, 0.40, seed=3)
    psi0 = -np.ones(shape, np.float32)
    psi0[:5] = 1.0

    def make(sto):
        s = LB3D_Solver_Two_Phase(*shape, storage=sto)
        s.fx = 0.0
        s.niu_l, s.niu_g, s.psi_solid, s.CapA = 0.05, 0.2, 0.7, 0.005
        s.bc_x_left, s.rho_bcxl, s.bc_x_right, s.rho_bcxr = 1, 1.001, 1, 1.0
        s.bc_psi_x_left, s.psi_x_left, s.bc_psi_x_right, s.psi_x_right = 1, 1.0, 1, -1.0
        s.solid.from_numpy(solid)
        s.psi.from_numpy(psi0)
        s.init_simulation()
        return s

    every = min(every, steps)
    out = {"n_fluid": int((solid == 0).sum()), "steps": steps, "every": every}
    curves = {}
    for sto in storages:
        s = make(sto)
        sat, pos = [], []
        t = time.perf_counter()
        for _ in range(steps // every):
            s.run(every)
            sat.append(s.saturation())
            pos.append(s.interface_position())
        curves[sto] = (np.array(sat), np.array(pos))
        log("two-phase %s: %d steps in %.1f s, final S %.4f" % (sto, steps, time.perf_counter() - t, sat[-1]))
        s.close()
        if sto != "f64":
            s = make(sto)
            lat = s._lat
            nsteps = min(2000, steps)
            stream = torch.cuda.ExternalStream(lat.stream())
            lat.step_async(20)
            lat.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            lat.step_async(nsteps)
            e1.record(stream)
            e1.synchronize()
            secs = e0.elapsed_time(e1) / 1e3
            out["mlups_" + sto] = out["n_fluid"] * nsteps / secs / 1e6
            out["gbs_algorithmic_" + sto] = {"f32": 176, "f16": 100}[sto] * out["n_fluid"] * nsteps / secs / 1e9
            s.close()
    s64, p64 = curves["f64"]
    for sto in storages:
        if sto == "f64":
            continue
        sa, pa = curves[sto]
        out["saturation_max_abs_err_" + sto] = float(np.abs(sa - s64).max())
        out["interface_max_abs_err_" + sto] = float(np.nanmax(np.abs(pa - p64)))
    out["saturation_f64"] = [float(x) for x in s64]
    out["interface_f64"] = [float(x) for x in p64]
    if cpu:
        # the C oracle's two-phase step (reference algorithm) on a bounded sample of the same lattice
        from oracle.oracle import Oracle, make_params
        p = make_params(shape, bc=(1, 1, 0, 0, 0, 0), rho_bc=(1.001, 1.0, 1, 1, 1, 1), visc_convention=1,
                        guo_convention=1, bc_form=1, two_phase=True, niu_l=0.05, niu_g=0.2, psi_solid=0.7,
                        cap_a=0.005, psi_bc=(1, 1, 0, 0, 0, 0), psi_val=(1.0, -1.0, 1, 1, 1, 1))
        o = Oracle(p, solid, psi0)
        o.step(1)
        n, t = 0, 0.0
        while t < cpu_seconds and n < 100:
            t0 = time.perf_counter()
            o.step(1)
            t += time.perf_counter() - t0
            n += 1
        o.close()
        out["cpu_baseline"] = {"value": out["n_fluid"] * n / t / 1e6, "unit": UNIT,
                               "cores": len(os.sched_getaffinity(0)), "kind": "port",
                               "sample": "%d two-phase steps of the full %d^3 lattice (%.1f s)" % (n, shape[0], t)}
    return out


def cavity(steps=1000, log=lambda m: print(m, file=sys.stderr, flush=True)):
    """64^3 lid-driven cavity (one-node solid shell on five faces,
    top z face fixed velocity (0.1, 0, 0), niu 0.1, FP32 reference
    arithmetic, class conventions): GPU MLUPS over `steps` steps with CUDA
    events, the CPU oracle over the same steps on all host cores, and the
    largest rho/v difference between the two after `steps` steps."""
    import torch
    from oracle.oracle import Oracle, make_params as oracle_params
    from taichi_lbm3d_gb300 import _native
    from taichi_lbm3d_gb300.geometry import cavity_shell
    solid = cavity_shell(64)
    vel = [[0.0, 0.0, 0.0]] * 5 + [[0.1, 0.0, 0.0]]
    op = oracle_params((64, 64, 64), niu=0.1, bc=(0, 0, 0, 0, 0, 2), vel_bc=vel)
    p = _native.make_params((64, 64, 64), niu=0.1, bc=(0, 0, 0, 0, 0, 2), vel_bc=vel)
    lat = _native.Lattice(p)
    lat.set_geometry(solid)
    lat.init()
    nf = lat.info().n_fluid
    stream = torch.cuda.ExternalStream(lat.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    lat.step_async(steps)
    e1.record(stream)
    e1.synchronize()
    gpu_s = e0.elapsed_time(e1) / 1e3
    rho, v = lat.macros()
    o = Oracle(op, solid)
    t = time.perf_counter()
    o.step(steps)
    cpu_s = time.perf_counter() - t
    fl = solid == 0
    d_rho = float(np.abs(rho[fl] - o.field("rho").astype(np.float32)[fl]).max())
    d_v = float(np.abs(v[fl] - o.field("v").astype(np.float32)[fl]).max())
    log("cavity: GPU %.0f MLUPS, CPU oracle %.1f MLUPS, max |drho| %g |dv| %g" % (
        nf * steps / gpu_s / 1e6, nf * steps / cpu_s / 1e6, d_rho, d_v))
    return {"workload": "64^3 lid-driven cavity, top face v = (0.1, 0, 0), niu 0.1, FP32, %d steps from rest" % steps,
            "n_fluid": nf, "gpu_mlups": nf * steps / gpu_s / 1e6, "gpu_seconds": gpu_s,
            "cpu_oracle_mlups": nf * steps / cpu_s / 1e6, "cpu_cores": len(os.sched_getaffinity(0)),
            "max_abs_diff_rho_vs_oracle": d_rho, "max_abs_diff_v_vs_oracle": d_v,
            "note": "first launches included (no warm-up): the lattice is L2-resident"}


def unet_step(steps=10, warmup=3, n=2, edge=96, activation="relu"):
    """Warm-start U-Net training step (forward, masked MSE, backward, Adam) on
    n seeded random samples of edge^3 with 16 input channels: ms per step from
    CUDA events, and the convolution work per step (forward, backward-data and
    weight gradient: 3 x 2 x voxels x 27 x cin x cout per layer) in TFLOP/s."""
    import torch
    from taichi_lbm3d_gb300.unet import LAYERS, UNet3D
    torch.manual_seed(0)
    m = UNet3D(seed=0, activation=activation)
    x = torch.randn((n, edge, edge, edge, 16), device="cuda").to(torch.bfloat16)
    t = torch.randn((n, edge, edge, edge, 4), device="cuda")
    mk = torch.ones((n, edge, edge, edge), device="cuda", dtype=torch.uint8)

    def one():
        y = m.forward(x)
        loss, gy = m.loss(y, t, mk, float(mk.numel()) * 4)
        m.backward(gy)
        m.adam_step(lr=1e-4)
        return loss

    for _ in range(warmup):
        one()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        loss = one()
    e1.record()
    e1.synchronize()
    ms = e0.elapsed_time(e1) / steps
    flop = 0.0
    for _, cin, cout, lv in LAYERS:
        vox = n * (edge >> lv) ** 3
        flop += 3 * 2.0 * vox * 27 * cin * cout
    return {"workload": "U-Net training step, %d x %d^3, 16 input channels, random data" % (n, edge),
            "activation": activation,
            "steps": steps, "ms_per_step": ms, "conv_tflops": flop / (ms * 1e-3) / 1e12,
            "loss_finite": bool(torch.isfinite(loss).all().item())}


# (cin, cout, level) of the warm-start network's convolutions; level l runs on edge >> l
UNET_LAYER_SHAPES = [(16, 16, 0), (16, 32, 1), (32, 32, 1), (32, 64, 2), (64, 64, 2), (96, 32, 1), (48, 16, 0)]


# wider convolutions than the network's, for the kernels' ceiling: (cin, cout) on n x edge^3
UNET_WIDE_SHAPES = [(64, 64), (96, 96), (128, 96), (64, 96), (96, 64), (128, 64)]


def unet_wide(n=2, edge=96, iters=10):
    """Forward 3x3x3 convolutions (ReLU epilogue) wider than the network's layers, each timed
    alone with CUDA events: TFLOP/s of 2 x voxels x 27 x cin x cout, against the measured
    bf16 peak."""
    import ctypes
    import torch
    from taichi_lbm3d_gb300 import unet
    L = unet._lib()
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    peak = None
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")) as f:
            peak = float(json.load(f)["bf16_tflops"])
    except (OSError, KeyError, ValueError):
        pass
    rows = []
    torch.manual_seed(0)
    for cin, cout in UNET_WIDE_SHAPES:
        x = torch.randn((n, edge, edge, edge, cin), device="cuda").to(torch.bfloat16)
        w = (torch.randn((cout, 27, cin), device="cuda") / (27 * cin) ** 0.5).to(torch.bfloat16)
        b = torch.randn(cout, device="cuda")
        y = torch.empty((n, edge, edge, edge, cout), device="cuda", dtype=torch.bfloat16)
        f = lambda: L.lbm_nn_conv3d_act(p(x), p(w), p(b), None, p(y), None, n, edge, edge, edge, cin, cout, 0, s)
        for _ in range(3):
            assert f() == 0
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(iters):
            f()
        e1.record()
        e1.synchronize()
        us = e0.elapsed_time(e1) / iters * 1e3
        tf = 2.0 * n * edge ** 3 * 27 * cin * cout / us / 1e6
        rows.append({"cin": cin, "cout": cout, "us": us, "tflops": tf,
                     "frac_of_bf16_peak": tf / peak if peak else None})
        del x, w, b, y
    return {"workload": "forward 3x3x3 convolutions, %d x %d^3, random data" % (n, edge), "layers": rows}


def unet_layers(n=2, edge=96, iters=20):
    """Per-layer 3x3x3 convolution kernels of the warm-start network on n x edge^3:
    forward (ReLU epilogue), backward-data (the transposed shape, masked
    epilogue) and weight gradient, each timed alone with CUDA events over
    `iters` launches after 3 warm-up launches; TFLOP/s = 2 x voxels x 27 x
    cin x cout per launch."""
    import ctypes
    import torch
    from taichi_lbm3d_gb300 import unet
    L = unet._lib()
    p = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def timed(f):
        for _ in range(3):
            assert f() == 0
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(iters):
            f()
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1) / iters * 1e3

    rows = []
    torch.manual_seed(0)
    for cin, cout, lv in UNET_LAYER_SHAPES:
        e = edge >> lv
        fl = 2.0 * n * e ** 3 * 27 * cin * cout
        x = torch.randn((n, e, e, e, cin), device="cuda").to(torch.bfloat16)
        g = torch.randn((n, e, e, e, cout), device="cuda").to(torch.bfloat16)
        w = (torch.randn((cout, 27, cin), device="cuda") / (27 * cin) ** 0.5).to(torch.bfloat16)
        wt = (torch.randn((cin, 27, cout), device="cuda") / (27 * cout) ** 0.5).to(torch.bfloat16)
        b = torch.randn(cout, device="cuda")
        y = torch.empty((n, e, e, e, cout), device="cuda", dtype=torch.bfloat16)
        gx = torch.empty((n, e, e, e, cin), device="cuda", dtype=torch.bfloat16)
        dw = torch.zeros((cout, 27, cin), device="cuda")
        db = torch.zeros(cout, device="cuda")
        scr = torch.empty(int(L.lbm_nn_wgrad_scratch_floats(n, e, e, e, cin, cout)), device="cuda")
        us_f = timed(lambda: L.lbm_nn_conv3d_act(p(x), p(w), p(b), None, p(y), None, n, e, e, e, cin, cout, 0, s))
        us_d = timed(lambda: L.lbm_nn_conv3d_act(p(g), p(wt), None, p(x), p(gx), None, n, e, e, e, cout, cin, 1, s))
        us_w = timed(lambda: L.lbm_nn_conv3d_wgrad(p(x), p(g), p(dw), p(db), p(scr), scr.numel(), n, e, e, e, cin,
                                                   cout, s))
        flag = ctypes.c_int32(0)
        assert L.lbm_nn_tc_status(ctypes.byref(flag)) == 0 and flag.value == 0
        rows.append({"cin": cin, "cout": cout, "edge": e,
                     "fwd_us": us_f, "fwd_tflops": fl / us_f / 1e6,
                     "bwd_data_us": us_d, "bwd_data_tflops": fl / us_d / 1e6,
                     "wgrad_us": us_w, "wgrad_tflops": fl / us_w / 1e6})
    return {"workload": "warm-start U-Net convolution layers, %d x %d^3 at level 0, random data" % (n, edge),
            "paths": {k: os.environ.get(k, "default") for k in ("LBM_NN_HALO", "LBM_NN_TMA", "LBM_NN_HALO_TD")},
            "layers": rows}


def grey_field(shape=SHAPE):
    """Grey-scale workload: the 256^3 pack of the default bench with ns = 1 in
    the spheres and a grey layer ns = 0.25 on pore cells within 1.5 cells of a
    sphere (unresolved roughness), ns = 0 elsewhere."""
    from taichi_lbm3d_gb300.geometry import distance_to_solid
    if solid is None and shape == SHAPE:
        solid = geometry()
    if solid is None:
        from taichi_lbm3d_gb300.geometry import sphere_pack
        solid = sphere_pack(shape, PACK["rmin"], PACK["rmax"], PACK["porosity"], PACK["seed"])
    ns = np.where(solid > 0, 1.0, 0.0)
    ns[(solid == 0) & (distance_to_solid(solid) <= 1.5)] = 0.25
    return ns


def grey(steps=1000, cpu=True, cpu_seconds=20.0, log=lambda m: print(m, file=sys.stderr, flush=True)):
    """Grey-scale (partial bounce-back) step on the grey 256^3 field: body
    force fx = 1e-6, periodic, niu 0.1 (script conventions).  MLUPS with CUDA
    events on the library's stream for FP32 reference arithmetic, FP32
    deviation form and FP16; the CPU oracle's grey sweeps on a bounded sample
    of the same lattice."""
    import torch
    from taichi_lbm3d_gb300 import LB3D_Solver_Grey_Scale
    ns = grey_field()
    nf = int((ns < 1.0).sum())
    out = {"workload": "grey-scale step, 256^3 pack (seed 2) with ns = 1 spheres and an ns = 0.25 layer "
                       "within 1.5 cells of them, fx 1e-6, periodic, niu 0.1",
           "n_fluid": nf, "n_grey": int(((ns > 0) & (ns < 1)).sum()), "steps": steps}
    peak, kind = measured_peak()
    for sto in ("f32", "f32dev", "f16"):
        lb = LB3D_Solver_Grey_Scale(*SHAPE, storage=sto)
        lb.fx = 1e-6
        lb.ns.from_numpy(ns)
        lb.solid.from_numpy(ns.astype(int))
        lb.init_simulation()
        lat = lb._lat
        stream = torch.cuda.ExternalStream(lat.stream())
        lat.step_async(20)
        lat.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        lat.step_async(steps)
        e1.record(stream)
        e1.synchronize()
        secs = e0.elapsed_time(e1) / 1e3
        mlups = nf * steps / secs / 1e6
        # algorithmic bytes per node: populations in + out, plus the node's ns
        bpn = {"f32": 156, "f32dev": 156, "f16": 80}[sto]
        out["mlups_" + sto] = mlups
        out["gbs_algorithmic_" + sto] = bpn * mlups / 1e3
        out["roofline_frac_" + sto] = bpn * mlups / 1e3 / peak
        st = lb.stats()
        out["max_v_" + sto] = st.max_v
        log("grey %s: %.0f MLUPS (%.0f GB/s algorithmic, %.1f%% of %s HBM copy)" % (
            sto, mlups, bpn * mlups / 1e3, 100 * bpn * mlups / 1e3 / peak, kind))
        lb.close()
    out["peak_gbs"] = peak
    out["peak_kind"] = kind
    if not cpu:
        return out
    from oracle.oracle import Oracle, make_params
    p = make_params(SHAPE, niu=0.1, force=(1e-6, 0, 0), visc_convention=1, guo_convention=1, bc_form=1, grey=True)
    o = Oracle(p, (ns.astype(int) != 0).astype(np.int8))
    o.set_field("ns", ns)
    o.step(1)
    n, t = 0, 0.0
    while t < cpu_seconds and n < 50:
        t0 = time.perf_counter()
        o.step(1)
        t += time.perf_counter() - t0
        n += 1
    o.close()
    out["cpu_baseline"] = {"value": nf * n / t / 1e6, "unit": UNIT, "cores": len(os.sched_getaffinity(0)),
                           "kind": "port", "sample": "%d grey steps of the full 256^3 lattice (%.1f s)" % (n, t)}
    return out


def voxelize_bench(log=lambda m: print(m, file=sys.stderr, flush=True)):
    """STL voxeliser: NACA 0012 wing (chord 40, span 20, 80 stations) in the
    reference tool's box (-10..50, -5..5, -15..15) at dx 0.5 (its setting) and
    0.1; GPU wall time per call (upload, kernel, download) and the FP64 CPU
    oracle on the dx 0.5 grid."""
    from taichi_lbm3d_gb300 import voxelize as vx
    from oracle import oracle
    tris = vx.naca4_wing("0012")
    out = {"triangles": int(len(tris))}
    vx.voxelize(tris, vx.REF_LO, vx.REF_HI, 1.0)           # context + module load
    for dx in (0.5, 0.1):
        dims = vx.grid_dims(vx.REF_LO, vx.REF_HI, dx)
        best = float("inf")
        for _ in range(3):
            t0 = time.perf_counter()
            solid = vx.voxelize(tris, vx.REF_LO, vx.REF_HI, dx)
            best = min(best, time.perf_counter() - t0)
        npts = int(np.prod(dims))
        out["dx_%g" % dx] = {"dims": list(dims), "seconds": best, "solid_fraction": float(solid.mean()),
                             "gpairs_per_s": npts * len(tris) / best / 1e9}
        log("voxelise dx %g: %s points in %.3f s" % (dx, dims, best))
    dims = vx.grid_dims(vx.REF_LO, vx.REF_HI, 0.5)
    t0 = time.perf_counter()
    o_solid, _ = oracle.voxelize(tris, vx.REF_LO, 0.5, dims)
    secs = time.perf_counter() - t0
    g_solid = vx.voxelize(tris, vx.REF_LO, vx.REF_HI, 0.5)
    out["cpu_oracle_dx_0.5"] = {"seconds": secs, "cores": len(os.sched_getaffinity(0)),
                                "flags_equal_gpu": bool(np.array_equal(o_solid, g_solid))}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 2000; the --grey/--two-phase/--unet modes have their own defaults)")
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--no-convergence", action="store_true",
                    help="skip the time-to-converged-k legs (FP64, FP32, FP16, ...) of the default line")
    ap.add_argument("--convergence", action="store_true",
                    help="run the 256^3 pack to steady state in FP64/FP32/FP16/BF16 and print k errors")
    ap.add_argument("--batched", action="store_true",
                    help="256 subvolumes to steady state: batched persistent launch vs serial plain kernel, k error vs FP64")
    ap.add_argument("--n-sub", type=int, default=256)
    ap.add_argument("--two-phase", action="store_true", help="131^3 two-phase drainage vs FP64")
    ap.add_argument("--grey", action="store_true", help="grey-scale (partial bounce-back) step on a 256^3 grey field")
    ap.add_argument("--voxelize", action="store_true", help="STL voxeliser on a NACA wing in the reference box")
    ap.add_argument("--unet", action="store_true", help="warm-start U-Net training step on 2 x 96^3")
    ap.add_argument("--unet-layers", action="store_true",
                    help="each U-Net convolution kernel (forward, backward-data, weight gradient) timed alone")
    ap.add_argument("--unet-wide", action="store_true",
                    help="forward convolutions wider than the network's (64-128 channels) timed alone")
    ap.add_argument("--cavity", action="store_true", help="64^3 lid-driven cavity, GPU vs CPU oracle")
    a = ap.parse_args()
    if a.cavity:
        print(json.dumps({"cavity": cavity(steps=a.steps or 1000)}))
        return 0
    if a.voxelize:
        print(json.dumps({"voxelize": voxelize_bench()}))
        return 0
    if a.unet_layers:
        print(json.dumps({"unet_layers": unet_layers(iters=a.steps or 20)}))
        return 0
    if a.unet_wide:
        print(json.dumps({"unet_wide": unet_wide(iters=a.steps or 10)}))
        return 0
    if a.unet:
        print(json.dumps({"unet": unet_step(steps=a.steps or 10),
                          "unet_gelu": unet_step(steps=a.steps or 10, activation="gelu")}))
        return 0
    if a.grey:
        print(json.dumps({"grey": grey(steps=a.steps or 1000, cpu=not a.no_cpu_baseline)}))
        return 0
    if a.two_phase:
        print(json.dumps({"two_phase": two_phase(steps=a.steps or 20000, cpu=not a.no_cpu_baseline)}))
        return 0
    if a.steps is None:
        a.steps = 2000
    if a.batched:
        res = batched(n_sub=a.n_sub)
        print(json.dumps({"batched": res}))
        return 0
    if a.convergence:
        res = convergence()
        print(json.dumps({"convergence": res, "config": workload_config(), "tol": 1e-6, "check_every": 500,
                          "viscosity_convention": "standard (tau = 3 niu + 1/2)"}))
        return 0
    warmup = max(3, a.warmup)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if a.impl == "reference":
        if rank != 0:
            return 0
        solid = geometry()
        nf = int((solid == 0).sum())
        cb = cpu_baseline(solid, max_seconds=min(120.0, 3.0 * max(1, a.steps)))
        line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": a.gpus,
                "steps": int(re.match(r"(\d+)", cb["sample"]).group(1)), "warmup": 1,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded sphere pack, numpy default_rng seed 2)",
                "config": dict(workload_config(), n_fluid=nf, porosity_after_percolation=float(nf) / solid.size),
                "cpu_baseline": cb,
                "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "note": "the reference's Taichi ti.cpu path is not installable offline; this is the C oracle "
                        "restating its four-sweep algorithm",
                "taichi_importable": importlib.util.find_spec("taichi") is not None}
        print(json.dumps(line))
        return 0

    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)

    solid = geometry()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)

    from taichi_lbm3d_gb300 import _native
    p = _native.make_params(SHAPE, niu=NIU, bc=(1, 1, 0, 0, 0, 0), rho_bc=(RHO_IN, RHO_OUT, 1, 1, 1, 1),
                            storage="f32", device=local)
    lat = _native.Lattice(p)
    lat.set_geometry(solid)
    lat.init()
    nf = lat.info().n_fluid
    stream = torch.cuda.ExternalStream(lat.stream())
    lat.step_async(warmup)
    lat.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    t_wall0 = time.time()
    e0.record(stream)
    lat.step_async(a.steps)
    e1.record(stream)
    e1.synchronize()
    t_wall1 = time.time()
    torch.cuda.synchronize()
    secs = e0.elapsed_time(e1) / 1e3
    st = lat.stats()
    lat.close()
    if world > 1:
        secs = max_over_ranks(secs, "cuda")
        torch.distributed.barrier()
    clocks.stop()
    clk = clocks.summary(t_wall0, t_wall1)

    mlups = nf * a.steps * world / secs / 1e6
    per_launch = secs / a.steps
    peak, peak_kind = measured_peak()
    achieved = BYTES_PER_NODE["f32"] * nf / per_launch / 1e9
    tpn = profiled_traffic_per_node()
    line = {
        "metric": METRIC, "value": mlups, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": warmup,
        "ms_per_step": per_launch * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded sphere pack, numpy default_rng seed 2)",
        "config": dict(workload_config(), n_fluid=nf, porosity_after_percolation=float(nf) / solid.size),
        "clocks": clk, "gpu_launches": a.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": (tpn * nf) if tpn else None,
                     "algorithmic_bytes_per_node": BYTES_PER_NODE["f32"]},
        "checks": {"mass": st.mass, "n_nonfinite": st.n_nonfinite},
        # all lattice cells (solid included) per second: the unit of the
        # reference's own MLUPS figures, which count every cell of the box
        "total_cell_mlups": mlups * float(solid.size) / nf,
    }
    if rank == 0:
        if not a.no_variants:
            var = {}
            for sto in ("f32dev", "f16", "bf16"):
                nfv, sv = run_variant(solid, sto, min(a.steps, 1000), warmup)
                var[sto] = {"value": nfv * min(a.steps, 1000) / sv / 1e6, "unit": UNIT,
                            "gbs_algorithmic": BYTES_PER_NODE[sto] * nfv * min(a.steps, 1000) / sv / 1e9}
            line["variants"] = var
        e2e, h2d, d2h, phases = e2e_run(solid, a.steps)
        line["e2e"] = {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                       "path": "LB3D_Solver_Single_Phase: solid.from_numpy, init_simulation, run(K), "
                               "rho/v to_numpy, host wall clock", "phases": phases}
        if not a.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(solid)
        if not a.no_convergence:
            line["time_to_converged_k"] = converged_k_summary(convergence(solid=solid))
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
