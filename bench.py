#!/usr/bin/env python3
"""Benchmark of the D3Q27 entropic LB level step on GB300.

Workload (one GPU): the learned-alpha boundary-layer case, D3Q27, FP32
deviation storage, 512x256x256 nodes, inlet u = 0.06, nu = 2e-5, seeded
+-5e-3 velocity noise; flat-plate faces (inlet x=0, outlet x=511, no-slip
bounce-back wall z=0, freestream z=255, inviscid walls y=0 and y=255).
A "step" is one fused level step (stream + boundaries + moments + alpha +
collision) over all 33.5 M nodes: the step kernel, then a second kernel that
finishes the ~1.5% of nodes whose populations are far from equilibrium (the
step kernel lists them).  The populations (7.2 GB) exceed L2 (129 MB), so
every step streams from HBM without an explicit flush.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU restatement of the step (the reference solver
is Fortran/AMReX and cannot be built here) on a bounded sample of the same
workload, with all host threads.
"""
from __future__ import annotations

import argparse
import json
import os
import pathlib
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "D3Q27 ELBM MLUPS: learned-α vs Newton-α at |ΔH|≤1e-10; % of HBM roofline"
UNIT = "MLUPS"
NX, NY, NZ = 512, 256, 256
U_IN = (0.06, 0.0, 0.0)
NU = 2e-5
NOISE = 5e-3
SEED = 1234 + 5
BYTES_PER_NODE_FP32 = 216  # 27 x 4 B read + 27 x 4 B written
# DRAM bytes (read + written) per node of the step kernel, from an ncu capture of a
# 256x128x128 launch of the same workload (traffic grows in proportion to the nodes)
DRAM_BYTES_PER_NODE_NCU = 203  # the bulk-node step kernel, per node of the level (ncu, 256x128x128 launch)
KERNELS_PER_STEP = 3  # the bulk-node step kernel, the boundary-node kernel and the listed-node kernel
BYTES_PER_NODE_FP64 = 432
BYTES_PER_NODE_D3Q39 = 1456  # f, g: 39 x 8 B read + written each; 13 multipliers x 8 B read + written
NU_WEDGE = 2e-4  # lattice kinematic viscosity of the D3Q39 wedge case
BYTES_PER_NODE_D3Q39_FP32 = 832  # f, g: 39 x 4 B read + written each; 13 multipliers x 8 B read + written


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return 6800.0, "fallback"


def build_workload(pkg):
    geo = pkg.geometry
    state = geo.box_state27(NX, NY, NZ, geo.flat_plate_faces())
    f0 = geo.perturbed_equilibrium(NX, NY, NZ, U_IN, NOISE, seed=SEED)
    bp = geo.d3q27_boundary_params(U_IN, NU)
    return state, f0, bp


def run_reference(args):
    """CPU restatement of the step (oracle port) on a bounded sample of the workload."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import __graft_entry__ as ge

    pkg = ge.load_package()
    from oracle import oracle as orc

    geo = pkg.geometry
    sx, sy, sz = 128, 64, 64  # sample: a 128x64x64 box of the same boundary-layer case
    state = geo.box_state27(sx, sy, sz, geo.flat_plate_faces())
    f = geo.perturbed_equilibrium(sx, sy, sz, U_IN, NOISE, seed=SEED)
    bp = geo.d3q27_boundary_params(U_IN, NU)
    p = orc.params(bp["nu"], bp["fs_feq"], bp["inl_feq"], bp["outl_feq"], bp["outlet_type"])
    for _ in range(args.warmup):
        f, _, _, _ = orc.step27(state, f, p)
    t0 = time.perf_counter()
    nodes = 0
    for _ in range(args.steps):
        f, _, _, s = orc.step27(state, f, p)
        nodes += s["fluid_nodes"]
    dt = time.perf_counter() - t0
    mlups = nodes / dt / 1e6
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    line = {
        "impl": "reference", "metric": METRIC, "value": mlups, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"D3Q27 boundary layer {NX}x{NY}x{NZ} (sampled {sx}x{sy}x{sz})", "alpha": "newton",
                   "storage": "fp64",
                   "arm": "the reference has no D3Q27 step to run: this arm times the FP64 CPU restatement of "
                          "the method (the oracle port) on the host cores, a stated baseline"},
        "cpu_baseline": {"value": mlups, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{sx}x{sy}x{sz} sub-box of the workload, {args.steps} steps, OpenMP"},
        "e2e": {"value": mlups, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def cpu_baseline_sample(pkg, budget_s=15.0):
    """The oracle port timed on the host cores on a bounded sample (rank 0, N = 1)."""
    from oracle import oracle as orc

    geo = pkg.geometry
    sx, sy, sz = 128, 64, 64
    state = geo.box_state27(sx, sy, sz, geo.flat_plate_faces())
    f = geo.perturbed_equilibrium(sx, sy, sz, U_IN, NOISE, seed=SEED)
    bp = geo.d3q27_boundary_params(U_IN, NU)
    p = orc.params(bp["nu"], bp["fs_feq"], bp["inl_feq"], bp["outl_feq"], bp["outlet_type"])
    f, _, _, _ = orc.step27(state, f, p)  # warm-up
    t0 = time.perf_counter()
    steps = nodes = 0
    while time.perf_counter() - t0 < budget_s and steps < 50:
        f, _, _, s = orc.step27(state, f, p)
        nodes += s["fluid_nodes"]
        steps += 1
    dt = time.perf_counter() - t0
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": nodes / dt / 1e6, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{sx}x{sy}x{sz} sub-box of the workload, {steps} FP64 Newton-alpha steps, {dt:.1f} s"}


def d3q27_config_legs(pkg, local_rank, cpu=True, budget_s=10.0):
    """The two smaller D3Q27 configurations on one GPU: the 64^3 flat-plate
    boundary layer (FP64, Newton alpha, nu = 1e-3, u = 0.05, +-1e-3 noise, 200
    steps; the reference's own CPU-runnable case, with the oracle timed on the
    same box's host cores for a bounded number of its steps) and the
    256x128x128 sphere (5,120 triangles, r = 16, u = 0.08, nu = 5e-4) in FP64 and
    in FP32 deviation storage, 20 steps each after one untimed step."""
    geo, cap = pkg.geometry, pkg.capi
    out = {}
    n = 64
    st = geo.box_state27(n, n, n, geo.flat_plate_faces())
    f0 = geo.perturbed_equilibrium(n, n, n, (0.05, 0.0, 0.0), 1e-3, seed=SEED)
    bp = geo.d3q27_boundary_params((0.05, 0.0, 0.0), 1e-3)
    ctx = cap.Context(local_rank)
    ctx.level_register(0, cap.ELBM_D3Q27, cap.ELBM_STORE_FP64, [[0, 0, 0, n - 1, n - 1, n - 1]])
    ctx.set_d3q27_params(0, cap.make_d3q27_params(**bp))
    ctx.set_links(0, 0, st)
    ctx.upload(0, 0, f0)
    s = ctx.step(0, 200)
    ctx.close()
    leg = {"workload": "D3Q27 flat plate 64^3, FP64, Newton alpha, 200 steps",
           "mlups": s["node_updates"] / (s["kernel_ms"] / 1e3) / 1e6, "fallbacks": s["fallbacks"],
           "status": s["status"], "bytes_per_node": 432}
    if cpu:
        from oracle import oracle as orc

        p = orc.params(bp["nu"], bp["fs_feq"], bp["inl_feq"], bp["outl_feq"], bp["outlet_type"])
        f = f0.copy()
        t0 = time.perf_counter()
        steps = nodes = 0
        while steps < 2 or (time.perf_counter() - t0 < budget_s and steps < 200):
            f, _, _, so = orc.step27(st, f, p)
            nodes += so["fluid_nodes"]
            steps += 1
        dt = time.perf_counter() - t0
        leg["cpu_baseline"] = {"value": nodes / dt / 1e6, "unit": UNIT,
                               "cores": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1)), "kind": "port",
                               "sample": f"the same 64^3 case, {steps} FP64 Newton-alpha steps, {dt:.1f} s"}
    out["flat_plate_64"] = leg
    nx, ny, nz = 256, 128, 128
    st = geo.box_state27(nx, ny, nz, geo.sphere_faces())
    cap.mark_triangles(st, (0.0, 0.0, 0.0), 1.0, geo.icosphere(4, 16.0, (64.0, 64.0, 64.0)))
    f0 = geo.perturbed_equilibrium(nx, ny, nz, (0.08, 0.0, 0.0), 1e-3, seed=SEED)
    f0[:, st[0] == -1001] = pkg.lattice.W[:, None]
    bp = geo.d3q27_boundary_params((0.08, 0.0, 0.0), 5e-4)
    for name, storage, bpn in (("fp64", cap.ELBM_STORE_FP64, 432), ("fp32", cap.ELBM_STORE_FP32_DEV, 216)):
        ctx = cap.Context(local_rank)
        ctx.level_register(0, cap.ELBM_D3Q27, storage, [[0, 0, 0, nx - 1, ny - 1, nz - 1]])
        ctx.set_d3q27_params(0, cap.make_d3q27_params(**bp))
        ctx.set_links(0, 0, st)
        ctx.upload(0, 0, f0)
        if storage == cap.ELBM_STORE_FP32_DEV:
            ctx.autotune(0)
        ctx.step(0, 1, want_stats=False)
        s = ctx.step(0, 20)
        ctx.close()
        out["sphere_" + name] = {"workload": f"D3Q27 sphere 256x128x128, {name.upper()}, Newton alpha",
                                 "mlups": s["node_updates"] / (s["kernel_ms"] / 1e3) / 1e6,
                                 "fallbacks": s["fallbacks"], "status": s["status"], "bytes_per_node": bpn}
    return out


def d3q39_wedge_leg(pkg, local_rank, fp32=False, steps=3, size=(384, 48, 192)):
    """The compressible D3Q39 wedge case at its full size (384x48x192: 48-node span
    between inviscid side walls, 192 high; Mach 1.5, shifted lattice, 10-degree
    wedge with interpolated wall links; FP64 populations, or FP32
    deviation storage of f and g with FP64 multipliers and arithmetic), each step
    followed by the negative-population repair as the reference's loop runs it
    (damp_it): MLUPS of the step and repair kernels from CUDA events, after one
    untimed step.  `size` scales the box (the
    wedge spans x from nx/4 to 25nx/32 at any size) for small profiling runs."""
    s39, cap = pkg.d3q39_setup, pkg.capi
    c = s39.wedge_case_consts(nu_lattice=NU_WEDGE)
    (nx, ny, nz), periodic = size, 0
    t0 = time.perf_counter()
    ctx = cap.Context(local_rank)
    params = cap.make_d3q39_params(c, timestep=0, periodic=periodic, damp=1)
    lm0 = s39.freestream_start_lm(c)
    _, f, g = ctx.d3q39_equilibrium(params, 1.0, c.mach, 0.0, 0.0, c.temperature, lm0)  # freestream equilibria
    st = s39.wedge_case_state(nx, ny, nz)
    shape = (nz, ny, nx)
    bc = cap.make_d3q39_bc([1] * 8, [6] + [1] * 7, f, g, [f] * 8, [g] * 8, [f] * 8, [g] * 8,
                           (c.mach, 0.0, 0.0, c.temperature))
    storage = cap.ELBM_STORE_FP32_DEV if fp32 else cap.ELBM_STORE_FP64
    ctx.level_register(0, cap.ELBM_D3Q39, storage, [[0, 0, 0, nx - 1, ny - 1, nz - 1]])
    ctx.set_d3q39_params(0, params)
    ctx.set_links39(0, 0, st, bc)
    setup_s = time.perf_counter() - t0
    # every node starts at the freestream (multilevel_initialization.f90), solved on the device
    ctx.init_level39(0, 0, np.stack([np.full(shape, 1.0), np.full(shape, c.mach), np.zeros(shape),
                                     np.zeros(shape), np.full(shape, c.temperature)]), lm0)
    ctx.step(0, 1, want_stats=False)
    s = ctx.step(0, steps)
    ctx.close()
    walls = int(((st[0] >= 0) & (st[1:] <= -1001).any(axis=0)).sum())
    name = "FP32 deviation storage, FP64 arithmetic" if fp32 else "FP64"
    return {"workload": f"D3Q39 Mach 1.5 wedge {nx}x{ny}x{nz}, {name}, shifted lattice", "steps": steps,
            "mlups": s["node_updates"] / (s["kernel_ms"] / 1e3) / 1e6, "ms_per_step": s["kernel_ms"] / steps,
            "wall_nodes": walls, "fallbacks": s["fallbacks"], "status": s["status"],
            "lm_iters_per_node": s["newton_iters"] / max(1, s["node_updates"]), "setup_s": setup_s,
            "algorithmic_bytes_per_node": BYTES_PER_NODE_D3Q39_FP32 if fp32 else BYTES_PER_NODE_D3Q39}


def d3q39_cpu_sample(pkg, seconds=10.0):
    """The oracle's D3Q39 link step with the negative-population repair on a
    96x12x48 wedge of the same shape (inlet, outlet, floor, freestream top,
    inviscid side walls, a 10-degree wedge with interpolated wall links), every
    node starting at the Mach 1.5 freestream:
    steps until about `seconds` have passed (at least two)."""
    from oracle import oracle39 as o39

    s39 = pkg.d3q39_setup
    c = s39.wedge_case_consts(nu_lattice=NU_WEDGE)
    k = o39.consts(c)
    nx, ny, nz = 96, 12, 48
    st = s39.wedge_case_state(nx, ny, nz)
    lm, f, g, _ = o39.init_node(k, 1.0, c.mach, 0.0, 0.0, c.temperature, s39.freestream_start_lm(c))
    lev = o39.Level39(nx, ny, nz)
    lev.fout[...] = np.asarray(f)[:, None, None, None]
    lev.gout[...] = np.asarray(g)[:, None, None, None]
    lev.lm[...] = np.asarray(lm)[:, None, None, None]
    lev.rho[...], lev.u[...], lev.temp[...] = 1.0, c.mach, c.temperature
    b = o39.bc([1] * 8, [6] + [1] * 7, f, g, [f] * 8, [g] * 8, [f] * 8, [g] * 8, (c.mach, 0.0, 0.0, c.temperature))
    pf, pg = lev.fout.copy(), lev.gout.copy()
    nodes, steps = 0, 0
    t0 = time.perf_counter()
    while steps < 2 or time.perf_counter() - t0 < seconds:
        nodes += o39.step_links_damp(k, lev, steps, st, 0, b, pf, pg, (0, 0, 0), (nx - 1, ny - 1, nz - 1))["nodes"]
        steps += 1
    dt = time.perf_counter() - t0
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": nodes / dt / 1e6, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{nx}x{ny}x{nz} wedge, {steps} FP64 link steps of the oracle (collision on OpenMP "
                      f"threads, streaming and wall targets on one), {dt:.1f} s"}


def amr_sphere_leg(pkg, local_rank, coarse_steps=500):
    """The 3-level AMR case around the sphere (geometry.amr_sphere_hierarchy:
    128x64x64 level 0, 24 and 96 boxes on levels 1 and 2, FP32 deviation
    storage), each level on the variant its autotuner picked, coarse_steps
    coarse steps through elbm_amr_run (the graph captured by one untimed
    two-cycle run first): node updates of all levels over the graph replays'
    device time, then each level stepped alone for its own MLUPS."""
    geo, cap = pkg.geometry, pkg.capi
    t0 = time.perf_counter()
    H = geo.amr_sphere_hierarchy()
    ctx = cap.Context(local_rank)
    geo.register_amr_hierarchy(ctx, H, cap.ELBM_STORE_FP32_DEV)
    variants = [ctx.autotune(l)[0] for l in range(len(H))]
    setup_s = time.perf_counter() - t0
    ctx.amr_run(len(H), 2)
    s = ctx.amr_run(len(H), coarse_steps)
    levels = []
    for l, L in enumerate(H):
        sl = ctx.step(l, 4)
        valid = int(((L["state"][0] >= 0) & (L["state"][0] != geo.AMR_GHOST)).sum())
        levels.append({"level": l, "boxes": L["nvalid"], "ghost_slab_boxes": len(L["boxes"]) - L["nvalid"],
                       "valid_fluid_nodes": valid, "variant": int(variants[l]),
                       "mlups_alone": sl["node_updates"] / (sl["kernel_ms"] / 1e3) / 1e6})
    ctx.close()
    return {"workload": "D3Q27 3-level AMR around the sphere, 24 + 96 fine boxes, FP32 deviation storage",
            "coarse_steps": coarse_steps, "node_updates": s["node_updates"],
            "mlups": s["node_updates"] / (s["kernel_ms"] / 1e3) / 1e6,
            "graph_ms_per_coarse_step": s["kernel_ms"] / coarse_steps, "fallbacks": s["fallbacks"],
            "status": s["status"], "levels": levels, "setup_s": setup_s}


def learned_alpha_leg(pkg, ctx, args, bp, local_rank):
    """Harvest, train, and time the learned-alpha path; returns a summary dict."""

    cap, geo = pkg.capi, pkg.geometry
    recs = []
    for kind in ("plate", "sphere"):
        h = cap.Context(local_rank)
        if kind == "plate":
            n = (128, 64, 64)
            st = geo.box_state27(*n, geo.flat_plate_faces())
            f0 = geo.perturbed_equilibrium(*n, U_IN, NOISE, seed=SEED + 1)
            hb = geo.d3q27_boundary_params(U_IN, NU)
        else:
            n = (128, 64, 64)
            st = geo.box_state27(*n, geo.sphere_faces())
            cap.mark_triangles(st, (0.0, 0.0, 0.0), 1.0, geo.icosphere(4, 8.0, (32.0, 32.0, 32.0)))
            f0 = geo.perturbed_equilibrium(*n, (0.08, 0, 0), 1e-3, seed=SEED + 2)
            f0[:, st[0] == -1001] = pkg.lattice.W[:, None]
            hb = geo.d3q27_boundary_params((0.08, 0, 0), 5e-4)
        h.level_register(0, cap.ELBM_D3Q27, cap.ELBM_STORE_FP32_DEV, [[0, 0, 0, n[0] - 1, n[1] - 1, n[2] - 1]])
        h.set_d3q27_params(0, cap.make_d3q27_params(**hb))
        h.set_links(0, 0, st)
        h.upload(0, 0, f0)
        recs.append(h.alpha_harvest(0, nsteps=40, stride=4, capacity=1 << 21))
        h.close()
    rec = np.concatenate(recs)
    t0 = time.perf_counter()
    w, hist = ctx.alpha_mlp_train(rec, cap.mlp_init_weights(0), epochs=4, batch=8192, lr=2e-3, seed=1)
    train_s = time.perf_counter() - t0
    ctx.set_alpha_mlp(0, w)
    lp = cap.make_d3q27_params(**dict(bp, alpha_mode=cap.ELBM_ALPHA_LEARNED))
    ctx.set_d3q27_params(0, lp)
    ctx.step(0, 2, want_stats=False)
    st = ctx.step(0, args.steps)
    mlups = st["node_updates"] / (st["kernel_ms"] / 1e3) / 1e6
    chk = cap.make_d3q27_params(**dict(bp, alpha_mode=cap.ELBM_ALPHA_LEARNED, check_dH=1))
    ctx.set_d3q27_params(0, chk)
    v = ctx.step(0, 3)
    ctx.set_d3q27_params(0, cap.make_d3q27_params(**bp))
    return {"mlups": mlups, "records": int(rec.shape[0]), "train_s": train_s, "loss": [float(x) for x in hist],
            "newton_iters_per_node": st["newton_iters"] / max(1, st["node_updates"]),
            "guess_misses_per_node": st["guess_misses"] / max(1, st["node_updates"]),
            "max_abs_dH": v["max_abs_dH"], "dh_over_tol": v["dh_over_tol"], "fallbacks": v["fallbacks"]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-d3q39", action="store_true", help="skip the D3Q39 wedge leg")
    ap.add_argument("--no-amr", action="store_true", help="skip the 3-level AMR leg")
    ap.add_argument("--amr-only", type=int, default=None, metavar="COARSE_STEPS",
                    help="run only the 3-level AMR leg for this many coarse steps and print it")
    ap.add_argument("--size", default=None, help="NXxNYxNZ override (profiling runs on a smaller box)")
    ap.add_argument("--alpha", default="newton", choices=["newton", "fixed2"],
                    help="alpha of the timed path (fixed2 = LBGK limit, to separate the alpha solve's cost)")
    ap.add_argument("--variant", type=int, default=None, choices=list(range(10)),
                    help="step-kernel variant instead of the autotuner's choice")
    ap.add_argument("--d3q39-only", default=None, metavar="NXxNYxNZ",
                    help="run only the D3Q39 wedge legs (FP64 and FP32 storage) at this size and print them")
    ap.add_argument("--profile", action="store_true",
                    help="timed steps only: no validation, end-to-end, FP64 or CPU legs (for ncu captures)")
    args = ap.parse_args()
    if args.size:
        global NX, NY, NZ
        NX, NY, NZ = (int(v) for v in args.size.lower().split("x"))
    if args.profile:
        args.no_cpu_baseline = args.no_fp64 = args.no_d3q39 = args.no_amr = True
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
        return

    rank, world, local_rank = dist_env()
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
        pg = dist
    import __graft_entry__ as ge

    ge.build() if rank == 0 or world == 1 else None
    if args.amr_only:
        leg = amr_sphere_leg(ge.load_package(), local_rank, coarse_steps=args.amr_only)
        if rank == 0:
            print(json.dumps({"amr_sphere": leg}), flush=True)
        return
    if args.d3q39_only:
        pkg = ge.load_package()
        size = tuple(int(v) for v in args.d3q39_only.lower().split("x"))
        legs = [d3q39_wedge_leg(pkg, local_rank, fp32=f, steps=args.steps, size=size) for f in (False, True)]
        if rank == 0:
            print(json.dumps({"d3q39_wedge": legs[0], "d3q39_wedge_fp32": legs[1]}), flush=True)
        return
    if pg:
        pg.barrier()
    pkg = ge.load_package()
    cap = pkg.capi
    state, f0, bp = build_workload(pkg)
    if args.alpha == "fixed2":
        bp["alpha_mode"] = cap.ELBM_ALPHA_FIXED2

    ctx = cap.Context(local_rank)
    box = [[0, 0, 0, NX - 1, NY - 1, NZ - 1]]
    ctx.level_register(0, cap.ELBM_D3Q27, cap.ELBM_STORE_FP32_DEV, box)
    ctx.set_d3q27_params(0, cap.make_d3q27_params(**bp))
    ctx.set_links(0, 0, state)
    ctx.upload(0, 0, f0)

    # warm-up, autotune the step-kernel variant, then the timed region: K fused steps,
    # CUDA events on the library's stream
    ctx.step(0, args.warmup, want_stats=False)
    if args.variant is None:
        variant, variant_ms = ctx.autotune(0, reps=3)
    else:
        variant, variant_ms = args.variant, np.full(cap.ELBM_KERNEL_VARIANTS, np.nan)
        ctx.set_kernel_variant(0, variant)
    ctx.sync()
    if pg:
        pg.barrier()
    clocks = ClockSampler(local_rank)
    clocks.start()
    t0 = time.perf_counter()
    st = ctx.step(0, args.steps)  # synchronises; kernel_ms from CUDA events around the K launches
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    kernel_s = st["kernel_ms"] / 1e3
    if pg:
        import torch

        t = torch.tensor([kernel_s], dtype=torch.float64)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        kernel_s = float(t[0])
    nodes_per_step = st["node_updates"] / args.steps
    value = nodes_per_step * args.steps * world / kernel_s / 1e6
    per_launch_s = kernel_s / args.steps
    peak, peak_kind = measured_peak_hbm()
    achieved = BYTES_PER_NODE_FP32 * nodes_per_step / per_launch_s / 1e9

    if args.profile:
        if rank == 0:
            print(json.dumps({"profile_run": True, "size": [NX, NY, NZ], "alpha": args.alpha, "variant": variant,
                              "variant_ms": [float(x) if np.isfinite(x) else None for x in variant_ms], "mlups": value,
                              "ms_per_step": per_launch_s * 1e3, "achieved_gbs": achieved}), flush=True)
        ctx.close()
        return
    # entropy condition and fallbacks over a validation window (check mode, not timed)
    chk = cap.make_d3q27_params(**bp)
    chk.check_dH = 1
    ctx.set_d3q27_params(0, chk)
    vst = ctx.step(0, 3)
    ctx.set_d3q27_params(0, cap.make_d3q27_params(**bp))

    # learned alpha: harvest (populations, alpha) records from Newton solves of smaller
    # boxes of the boundary layer and of the sphere case, train the network on the GPU,
    # then time the learned guess + at most two Newton steps on the same workload
    learned = learned_alpha_leg(pkg, ctx, args, bp, local_rank)

    # end to end through the C ABI with host buffers: upload, K steps, download
    import torch

    host_in = torch.from_numpy(f0).pin_memory()
    host_out = torch.empty_like(host_in).pin_memory()
    # one untimed round trip through the same pinned buffers: the first DMA use of freshly
    # pinned pages costs ~0.8 s once per buffer on this host (warm-up, like the warm-up steps)
    ctx.upload(0, 0, host_in.numpy())
    ctx.download(0, 0, host_out.numpy())
    ctx.sync()
    te = time.perf_counter()
    ctx.upload(0, 0, host_in.numpy())
    ctx.sync()
    t_up = time.perf_counter() - te
    ctx.step(0, args.steps, want_stats=False)
    ctx.sync()
    t_steps = time.perf_counter() - te - t_up
    ctx.download(0, 0, host_out.numpy())
    e2e_s = time.perf_counter() - te
    e2e_phases_ms = {"upload": t_up * 1e3, "steps": t_steps * 1e3, "download": (e2e_s - t_up - t_steps) * 1e3}
    e2e = nodes_per_step * args.steps * world / e2e_s / 1e6
    h2d = f0.nbytes / args.steps
    d2h = f0.nbytes / args.steps
    ctx.close()

    # plain FP64 Newton-alpha path on the same workload (short window; FP64 is 1/60 of FP32 on GB300)
    fp64 = None
    if not args.no_fp64:
        c64 = cap.Context(local_rank)
        c64.level_register(0, cap.ELBM_D3Q27, cap.ELBM_STORE_FP64, box)
        c64.set_d3q27_params(0, cap.make_d3q27_params(**bp))
        c64.set_links(0, 0, state)
        c64.upload(0, 0, f0)
        c64.step(0, 1, want_stats=False)
        s64 = c64.step(0, 2)
        fp64 = s64["node_updates"] / (s64["kernel_ms"] / 1e3) / 1e6
        c64.close()

    wedge = wedge32 = None
    if not args.no_d3q39:
        wedge = d3q39_wedge_leg(pkg, local_rank)
        wedge32 = d3q39_wedge_leg(pkg, local_rank, fp32=True)
        if rank == 0 and world == 1 and not args.no_cpu_baseline:
            wedge["cpu_baseline"] = d3q39_cpu_sample(pkg)

    amr = None
    if not args.no_amr:
        amr = amr_sphere_leg(pkg, local_rank)

    small = None
    if not args.no_fp64:
        small = d3q27_config_legs(pkg, local_rank, cpu=(rank == 0 and world == 1 and not args.no_cpu_baseline))

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_sample(pkg)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": per_launch_s * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"D3Q27 boundary layer {NX}x{NY}x{NZ}, FP32 deviation storage, Newton alpha",
                       "alpha": "newton", "storage": "fp32_dev", "nu": NU, "u_in": U_IN[0], "noise": NOISE,
                       "l2": "inputs (7.2 GB) larger than L2, no flush", "parallelism": f"replicas x{world}",
                       "kernel_variant": variant,
                       "variant_ms": [float(x) if np.isfinite(x) else None for x in variant_ms]},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": DRAM_BYTES_PER_NODE_NCU * nodes_per_step,
                         "traffic_note": "bytes per launch of the step kernel: ncu DRAM bytes per node of a "
                                         "256x128x128 launch x nodes",
                         "achieved_note": "algorithmic bytes of a step over the step's device time (the step kernel "
                                          "and the listed-node kernel, CUDA events on the library's stream)",
                         "peak_kind": peak_kind,
                         "bytes_per_node": BYTES_PER_NODE_FP32},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "note": "upload + K steps + download through the C ABI, pinned host FP64 FAB "
                            "(after one untimed round trip of the same buffers)",
                    "phases_ms": e2e_phases_ms},
            "gpu_launches": KERNELS_PER_STEP * args.steps,
            "clocks": clk,
            "wall_ms_per_step": wall / args.steps * 1e3,
            "validation": {"max_abs_dH": vst["max_abs_dH"], "dh_over_tol": vst["dh_over_tol"],
                           "fallbacks": vst["fallbacks"],
                           "exact_path_nodes": vst["exact_path_nodes"], "status": vst["status"],
                           "newton_iters_per_node": vst["newton_iters"] / max(1, vst["node_updates"])},
            "plain_fp64_newton_mlups": fp64,
            "d3q39_wedge": wedge,
            "d3q39_wedge_fp32": wedge32,
            "amr_sphere": amr,
            "d3q27_configs": small,
            "learned_alpha": learned,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    if pg:
        pg.barrier()
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
