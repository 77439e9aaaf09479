#!/usr/bin/env python
"""Benchmark of the GB300 pressure projection (one JSON line on rank 0).

A step is one full projection of the 256^3 dam-break scene: cell classification
from the level set and the solid primitives, masked divergence, MGPCG to
relative residual 1e-6 (rel_tol 1e-12 on squared norms, abs_tol 0, at most 200
iterations, smoother "phases", 6 levels down to 8^3) and the pressure-gradient
velocity update.  Each step first restores the input velocity (a 200 MB
device-to-device copy) because the projection updates it in place.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU restatement of the same path (oracle/, the
reference's Warp kernels cannot run here) on all host cores, on rank 0 only.
With N > 1 (torchrun) every rank projects its own seeded scene (replicas, no
collective on the data path): value = max elapsed over ranks / (K * N).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ms per 256³ pressure solve to 1e-6 rel. residual: learned+mixed vs plain MGPCG"
UNIT = "ms"
# canonical algorithmic bytes per cell of the level a kernel runs on
SMOOTH_HALF_SWEEP_BYTES_PER_CELL = 6.5  # red + black iteration: R z, r, tag; W z = 13 B/cell
VARIANTS = {
    "plain": "plain FP32 MGPCG (reference V-cycle, FP64 inner products)",
    "mixed": "mixed-precision MGPCG (FP16 V-cycle levels, FP32 arithmetic, flexible CG, FP64 inner products)",
    "learned+mixed": "mixed-precision MGPCG started from the U-Net warm start (network on the 64^3 level of the "
                     "hierarchy, trilinear prolongation, energy-optimal scale), same tolerance",
    "plain-v22": "FP32 MGPCG with the light V-cycle: 2+2 red-black iterations per level, 4+4 at the bottom, "
                 "restriction scaled by 1/2 (flub_mg_set_schedule), same tolerance",
    "mixed-v22": "mixed-precision MGPCG (FP16 V-cycle levels) with the light V-cycle, same tolerance",
    "learned+mixed-v22": "mixed-precision MGPCG with the light V-cycle, started from the U-Net warm start, "
                         "same tolerance",
}
# variant -> (precision, schedule, warm start)
VARIANT_SETUP = {
    "plain": ("fp32", "reference", False),
    "mixed": ("mixed", "reference", False),
    "learned+mixed": ("mixed", "reference", True),
    "plain-v22": ("fp32", "v22", False),
    "mixed-v22": ("mixed", "v22", False),
    "learned+mixed-v22": ("mixed", "v22", True),
}


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", default="dam256")
    ap.add_argument("--variant", choices=sorted(VARIANTS), default="learned+mixed-v22",
                    help="the variant the headline value is measured on (the others are timed beside it)")
    ap.add_argument("--cpu-baseline-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-oracle-check", action="store_true",
                    help="skip the FP64 host projection that checks each variant's pressure")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-scale512", action="store_true", help="skip the 512^3 dam-break timings")
    ap.add_argument("--no-oracle512", action="store_true",
                    help="skip the FP64 host projection of the 512^3 scene (about a minute on 16 cores)")
    ap.add_argument("--no-sphere128", action="store_true", help="skip the 128^3 flow-past-a-sphere block")
    ap.add_argument("--profile-kernel",
                    choices=["smooth", "restrict", "matvec", "solve", "project", "advect", "warmstart"],
                    default=None,
                    help="set up the 256^3 solver state and launch only this kernel 3 times (for ncu)")
    return ap.parse_args()


def run_profile_kernel(args):
    """Small, bounded process for an ncu capture: the solver state of the
    benchmark scene on the device (about 0.6 GB) and three launches of one kernel."""
    import torch
    from flub_gb300 import MGPCG, Projection, learned, scenes
    from flub_gb300 import kernels as K
    from flub_gb300.fields import Field, MACGrid
    from flub_gb300.unet import UNet3D

    scene = scenes.CONFIGS[args.config]()
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    if args.profile_kernel == "project":
        # one whole projection of the chosen variant (every kernel launch of one step)
        prec, sched, use_net = VARIANT_SETUP[args.variant]
        proj = Projection(scene.shape, scene.levels, precision=prec, schedule=sched)
        ws = learned.WarmStart(UNet3D.load(learned.WEIGHTS)) if use_net else None
        velr = MACGrid(*(Field(dev(a), d=d + 1) for d, a in enumerate((scene.ur, scene.vr, scene.wr))))
        # a first projection pays the one-time work (network load, graph
        # captures); the second, inside the NVTX range "projection" (ncu
        # --nvtx --nvtx-include "projection/"), is one steady-state step
        for rep in range(2):
            vel = MACGrid(*(Field(dev(a), d=d + 1) for d, a in enumerate((scene.u, scene.v, scene.w))))
            phi_d = dev(scene.phi)
            torch.cuda.synchronize()
            if rep:
                torch.cuda.nvtx.range_push("projection")
            info = proj.project(vel, velr, phi_d, scene.prims, max_iters=200, eps=1e-12, abs_tol=0.0,
                                rel_tol=1e-12, smoother="phases", warm_start=ws)
            torch.cuda.synchronize()
            if rep:
                torch.cuda.nvtx.range_pop()
        print(json.dumps({"profile_kernel": "project", "variant": args.variant, "iterations": info["iterations"],
                          "ok": bool(info["converged"])}))
        return 0
    if args.profile_kernel == "advect":
        # the step's advection (water_3d.py:34-37) on the scene's velocity:
        # advect_phi once, then advect_uv_mc (three k_advect_mc<0> launches) twice
        vel = MACGrid(*(Field(dev(a), d=d + 1) for d, a in enumerate((scene.u, scene.v, scene.w))))
        new_vel = MACGrid(*(Field(torch.empty_like(a.f), d=d + 1) for d, a in enumerate((vel.u, vel.v, vel.w))))
        phi = Field(dev(scene.phi))
        new_phi = Field(torch.empty_like(phi.f))
        K.advect_phi_field(vel, phi, new_phi)
        for _ in range(2):
            K.advect_uv_mc(vel, new_vel)
        torch.cuda.synchronize()
        print(json.dumps({"profile_kernel": "advect", "config": args.config, "ok": True}))
        return 0
    tag = K.classify(dev(scene.phi), scene.prims, scene.h, scene.h0)
    vel = MACGrid(*(Field(dev(a), d=d + 1) for d, a in enumerate((scene.u, scene.v, scene.w))))
    velr = MACGrid(*(Field(dev(a), d=d + 1) for d, a in enumerate((scene.ur, scene.vr, scene.wr))))
    div = K.divergence(vel, velr, tag, scale=-1.0 / scene.h)
    del vel, velr
    mg = MGPCG(3, scene.shape, scene.levels)
    mg.set_tags(tag)
    mg.init(div, -scene.h0)
    mg.mask_interior()
    del div
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    if args.profile_kernel == "smooth":
        # one V-cycle of a seeded uniform residual on the fluid cells gives the
        # level-0 buffers generic values, as the benchmark's timing does (its
        # level-0 smoothing: launches 0-7 of k_smooth_split); then three level-0
        # red-black iterations, launches 8-13 (ncu -k regex:k_smooth_split -s 8)
        gen = torch.Generator(device="cuda")
        gen.manual_seed(7)
        mg.apply_preconditioner(r=torch.rand(scene.shape, generator=gen, device="cuda") * (tag == 1))
        for q in range(3):
            mg.smooth_iteration(0, q & 1)
    elif args.profile_kernel == "matvec":
        for _ in range(3):
            mg.matvec(mg.r0)
    elif args.profile_kernel == "solve":
        # two CG iterations (with FLUB_SOLVE_HOST_LOOP=1 every kernel is a separate launch)
        mg.solve(2, 1e-12, 0.0, 1e-12, smoother="phases")
    elif args.profile_kernel == "warmstart":
        # the network's guess for this right-hand side, twice, eagerly (each
        # pass: restriction to 64^3, ten convolutions, prolongation to 256^3)
        ws = learned.WarmStart(UNet3D.load(learned.WEIGHTS))
        for _ in range(2):
            ws.guess(mg)
    else:
        for _ in range(3):
            mg.apply_preconditioner()
    torch.cuda.synchronize()
    print(json.dumps({"profile_kernel": args.profile_kernel, "config": args.config, "ok": True}))
    return 0


SEED_BASE = {"dam256": 2, "dam512": 2, "sphere128": 1, "box64": 0}


def replica_seed(config, rank):
    """Each replica projects its own seeded scene (no data-path collective)."""
    return SEED_BASE.get(config, 0) + rank


def max_over_ranks(ms, world, device):
    """The job's time: the slowest rank's (all_reduce MAX; any backend)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_ms_per_projection(elapsed_ms, steps, world):
    """Whole-job ms per projection: steps x world projections in elapsed_ms."""
    return elapsed_ms / (steps * world)


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic(kernel):
    path = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        entry = json.load(f).get(kernel)
    return entry.get("bytes_per_launch") if isinstance(entry, dict) else entry


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, local_rank):
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
        ids = [v.strip() for v in vis.split(",") if v.strip()]
        self.gpu = ids[local_rank] if local_rank < len(ids) else str(local_rank)
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", self.gpu, f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) == 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[q] for r in rows for q in range(4) if r[5 + q].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def time_cpu_projection(scene, steps):
    """The oracle's full projection on all host threads; returns ms per step."""
    import oracle as O
    O.project(scene, max_iters=200, rel_tol=1e-12, abs_tol=0.0)  # warm (pages, thread pool)
    t0 = time.perf_counter()
    for _ in range(steps):
        res = O.project(scene, max_iters=200, rel_tol=1e-12, abs_tol=0.0)
    dt = (time.perf_counter() - t0) * 1000.0 / steps
    return dt, res, O.num_threads()


# ---------------------------------------------------------------------------- reference arm

def run_reference(args):
    rank, _, world = dist_env()
    if rank != 0:
        return 0
    from flub_gb300 import scenes
    scene = scenes.CONFIGS[args.config]()
    import oracle as O
    for _ in range(args.warmup):
        O.project(scene, max_iters=200, rel_tol=1e-12, abs_tol=0.0)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        res = O.project(scene, max_iters=200, rel_tol=1e-12, abs_tol=0.0)
    ms = (time.perf_counter() - t0) * 1000.0 / args.steps
    cores = O.num_threads()
    out = {
        "impl": "reference", "metric": METRIC, "value": ms, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded dam-break scene, Fourier velocity field)",
        "config": {"workload": f"{args.config}: 256^3 dam-break projection to rel. residual 1e-6",
                   "iterations": res["iters"], "converged": res["converged"],
                   "implementation": "CPU restatement of the reference path (Warp unavailable), OpenMP"},
        "cpu_baseline": {"value": ms, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{args.steps} full {args.config} projections"},
        "e2e": {"value": ms, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)
    return 0


# ---------------------------------------------------------------------------- our arm

def run_ours(args):
    import torch
    import torch.distributed as dist

    rank, local_rank, world = dist_env()
    torch.cuda.set_device(local_rank)
    if world > 1:
        dist.init_process_group(backend="nccl", device_id=torch.device("cuda", local_rank))

    from flub_gb300 import Projection, _lib, learned, scenes
    from flub_gb300.fields import Field, MACGrid
    from flub_gb300.unet import UNet3D

    lib = _lib.load()
    scene = scenes.CONFIGS[args.config](seed=replica_seed(args.config, rank))
    n = scene.n_cells

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(a)).cuda()

    phi = dev(scene.phi)
    vel0 = [dev(a) for a in (scene.u, scene.v, scene.w)]
    vel = MACGrid(*(Field(a.clone(), d=d + 1) for d, a in enumerate(vel0)))
    velr = MACGrid(*(Field(dev(a), d=d + 1) for d, a in enumerate((scene.ur, scene.vr, scene.wr))))
    solve_kw = dict(max_iters=200, eps=1e-12, abs_tol=0.0, rel_tol=1e-12, smoother="phases")
    stream = torch.cuda.current_stream()

    warm = {}

    def make_step(proj):
        ws = warm.get(id(proj))

        def step():
            for a, b in zip((vel.u.f, vel.v.f, vel.w.f), vel0):
                a.copy_(b)
            proj.project(vel, velr, phi, scene.prims, sync=False, warm_start=ws, **solve_kw)
        return step

    def time_variant(proj, sample_clocks):
        """W warm-up steps, then exactly K timed steps between barriers and
        synchronisations; returns (ms over K steps, max over ranks), info, launches, clocks."""
        step = make_step(proj)
        for _ in range(max(args.warmup, 1)):
            step()
        torch.cuda.synchronize()
        info = proj.mg.info()
        if not info["converged"]:
            raise RuntimeError(f"warm-up solve did not converge: {info}")
        sampler = ClockSampler(local_rank) if sample_clocks else None
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        host_l0, dev_l0 = lib.flub_launch_count(), proj.mg.kernels_executed()
        if sampler:
            sampler.start()
            time.sleep(0.3)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        torch.cuda.synchronize()
        clocks = sampler.stop() if sampler else None
        if world > 1:
            dist.barrier()
        elapsed = max_over_ranks(ev0.elapsed_time(ev1), world, "cuda")
        launches = (lib.flub_launch_count() - host_l0) + (proj.mg.kernels_executed() - dev_l0)
        return elapsed, proj.mg.info(), launches, clocks

    head = args.variant
    have_net = os.path.exists(learned.WEIGHTS)
    net = UNet3D.load(learned.WEIGHTS) if have_net else None
    variants = {}
    learned_info = None
    for name, (prec, sched, use_net) in VARIANT_SETUP.items():
        if use_net and not have_net:
            continue
        pj = Projection(scene.shape, scene.levels, precision=prec, schedule=sched)
        variants[name] = pj
        if use_net:
            warm[id(pj)] = learned.WarmStart(net)
            learned_info = {"weights": os.path.relpath(learned.WEIGHTS, ROOT), "parameters": net.num_parameters(),
                            "network_level": warm[id(pj)].choose_level(pj.mg)}
    if head not in variants:
        head = head.replace("learned+", "")  # no trained weights in the tree
    results = {}
    pressures = {}
    for name, pj in variants.items():
        if name != head:
            el, inf, _, _ = time_variant(pj, False)
            results[name] = {"ms_per_solve": el / args.steps, "iterations": inf["iterations"],
                             "x0_scale": inf["x0_scale"]}
            pressures[name] = pj.p.f.detach().clone()
    proj = variants[head]
    elapsed, info, launches, clocks = time_variant(proj, True)
    results[head] = {"ms_per_solve": elapsed / args.steps, "iterations": info["iterations"],
                     "x0_scale": info["x0_scale"]}
    pressures[head] = proj.p.f.detach().clone()
    div_after = proj.max_abs_div(vel, velr)
    ms_per_step = elapsed / args.steps
    value = job_ms_per_projection(elapsed, args.steps, world)

    # ---- end to end through the public API with host buffers.  Every step
    # copies its inputs from pinned host memory and reads its results back; the
    # steps are pipelined over two device input sets: step n+1's inputs go up
    # on a copy stream while step n solves, step n's velocity comes back on a
    # second copy stream while step n+1 solves, and the pressure comes back on
    # the compute stream right after its solve (the handle reuses that buffer).
    e2e = None
    if not args.no_e2e:
        pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        h_in = [pin(scene.phi)] + [pin(a) for a in (scene.u, scene.v, scene.w, scene.ur, scene.vr, scene.wr)]
        sets = [[phi, vel.u.f, vel.v.f, vel.w.f, velr.u.f, velr.v.f, velr.w.f],
                [torch.empty_like(t) for t in (phi, vel.u.f, vel.v.f, vel.w.f, velr.u.f, velr.v.f, velr.w.f)]]
        h_out = [[torch.empty(t.shape).pin_memory() for t in sets[0][1:4]] + [torch.empty(scene.shape).pin_memory()]
                 for _ in range(2)]
        s_up, s_down = torch.cuda.Stream(), torch.cuda.Stream()
        up_done = [torch.cuda.Event(), torch.cuda.Event()]
        set_free = [torch.cuda.Event(), torch.cuda.Event()]
        solved = torch.cuda.Event()
        for ev in set_free:
            ev.record(stream)

        def upload(n):
            b = n % 2
            with torch.cuda.stream(s_up):
                s_up.wait_event(set_free[b])
                for h, d in zip(h_in, sets[b]):
                    d.copy_(h, non_blocking=True)
                up_done[b].record(s_up)

        def solve_and_download(n):
            b = n % 2
            d = sets[b]
            stream.wait_event(up_done[b])
            v_b = MACGrid(*(Field(t, d=k + 1) for k, t in enumerate(d[1:4])))
            vr_b = MACGrid(*(Field(t, d=k + 1) for k, t in enumerate(d[4:7])))
            proj.project(v_b, vr_b, d[0], scene.prims, sync=False, warm_start=warm.get(id(proj)), **solve_kw)
            h_out[b][3].copy_(proj.p.f, non_blocking=True)
            solved.record(stream)
            with torch.cuda.stream(s_down):
                s_down.wait_event(solved)
                for h, t in zip(h_out[b][:3], d[1:4]):
                    h.copy_(t, non_blocking=True)
                set_free[b].record(s_down)

        def run_e2e(k, start_event=None):
            if start_event is not None:
                s_up.wait_event(start_event)
            upload(0)
            for n in range(k):
                if n + 1 < k:
                    upload(n + 1)
                solve_and_download(n)
            stream.wait_stream(s_down)

        run_e2e(max(args.warmup, 1))
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        run_e2e(args.steps, e0)
        e1.record(stream)
        torch.cuda.synchronize()
        et = max_over_ranks(e0.elapsed_time(e1), world, "cuda")
        e2e = {"value": job_ms_per_projection(et, args.steps, world), "unit": UNIT,
               "h2d_bytes_per_step": int(sum(t.numel() * t.element_size() for t in h_in)),
               "d2h_bytes_per_step": int(sum(t.numel() * t.element_size() for t in h_out[0])),
               "pipelining": "two device input sets; uploads of step n+1 and the velocity read-back of step n "
                             "overlap the solves on two copy streams; the first upload and the last read-back "
                             "are inside the timed region"}

    # ---- roofline of the dominant kernel of the plain path: the level-0
    # red-black half-sweep (flub_mg_smooth_iteration: the colour-split row
    # kernel, or with FLUB_TILE=1 the TMA-tiled one, two half-sweeps per
    # launch), timed on the plain handle's level-0 buffers
    peak, peak_kind = load_peaks()
    reps = 24
    plain_mg = variants["plain"].mg
    fluid = (variants["plain"].tag.f == 1)
    # the operands of the timed sweeps: the level-0 buffers of one V-cycle of a
    # seeded uniform residual on the fluid cells (generic values; what a
    # converged solve leaves behind holds exact zeros, which some updates
    # shortcut)
    gen = torch.Generator(device=fluid.device)
    gen.manual_seed(7)
    plain_mg.apply_preconditioner(r=torch.rand(fluid.shape, generator=gen, device=fluid.device) * fluid)
    smoother = plain_mg.smooth_iteration(0, 0)  # 0 natural-order rows, 1 TMA tiles, 2 colour-split rows
    tiled = smoother == 1
    plain_mg.smooth_iteration(0, 0)
    torch.cuda.synchronize()
    k0, k1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    k0.record(stream)
    for q in range(reps):
        plain_mg.smooth_iteration(0, q & 1)
    k1.record(stream)
    torch.cuda.synchronize()
    launch_ms = k0.elapsed_time(k1) / reps / (1 if tiled else 2)
    nx_, ny_, nz_ = scene.shape
    if tiled:
        # a CTA stages and updates the whole of every tile (8 x 8 x 32 cells)
        # that holds a fluid cell: the canonical 13 B per cell per iteration
        # (R z, r, tag; W z) for those cells, plus the 4-byte tile-list entry;
        # the fluid-free tiles are never read
        tiles = fluid.view(nx_ // 8, 8, ny_ // 8, 8, nz_ // 32, 32).any(dim=5).any(dim=3).any(dim=1)
        n_units = int(tiles.sum().item())
        alg_bytes = 2 * SMOOTH_HALF_SWEEP_BYTES_PER_CELL * 8 * 8 * 32 * n_units + 4.0 * n_units
        kname = "k_smooth_tile<0> (level-0 red-black iteration, TMA-staged 8x8x32 tiles, two half-sweeps per launch)"
        unit_frac = n_units / tiles.numel()
        traffic = load_traffic("k_smooth_tile")
    else:
        groups = fluid.view(nx_, ny_, nz_ // 8, 8).any(dim=-1)
        n_units = int(groups.sum().item())
        alg_bytes = SMOOTH_HALF_SWEEP_BYTES_PER_CELL * 8 * n_units + 4.0 * n_units
        if smoother == 2:
            kname = ("k_smooth_split<kInPlace> (level-0 red-black half-sweep on colour-split storage, "
                     "over the active list)")
            traffic = load_traffic("k_smooth_split")
        else:
            kname = "k_smooth8<false,false> (level-0 red-black half-sweep over the active list)"
            traffic = load_traffic("k_smooth8")
        unit_frac = n_units / groups.numel()
    achieved = alg_bytes / (launch_ms * 1e-3) / 1e9
    roofline = {"bound": "hbm", "kernel": kname,
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": f"{peak_kind} hbm_gbs", "traffic": traffic,
                "alg_bytes_per_launch": alg_bytes, "launch_ms": launch_ms,
                "active_unit_fraction": unit_frac}

    # ---- the TMA-tiled smoother (opt-in, FLUB_TILE=1) against the row kernel:
    # one level-0 red-black iteration each, on a handle of the same scene
    from flub_gb300 import MGPCG as _MG
    os.environ["FLUB_TILE"] = "1"
    try:
        tmg = _MG(3, scene.shape, scene.levels)
    finally:
        os.environ.pop("FLUB_TILE", None)
    tmg.set_tags(proj.tag.f)
    tmg.init(plain_mg.r0, 1.0)
    tmg.mask_interior()
    tiled_ok = tmg.smooth_iteration(0, 0)
    tmg.smooth_iteration(0, 1)
    torch.cuda.synchronize()
    k0.record(stream)
    for q in range(reps):
        tmg.smooth_iteration(0, q & 1)
    k1.record(stream)
    torch.cuda.synchronize()
    tile_smoother = {"level0_iteration_ms_tiles": k0.elapsed_time(k1) / reps if tiled_ok else None,
                     "level0_iteration_ms_rows": launch_ms * (1 if tiled else 2),
                     "note": "k_smooth_tile (TMA-staged 8x8x32 tiles, both half-sweeps in one launch, bit-identical) "
                             "is off by default: slower than the row kernel at this size"}
    del tmg

    # ---- velocity extrapolation after the projection (water_3d.py:70-73, the
    # step after project()): one pass over the three face arrays, timed warm
    from flub_gb300 import kernels as K
    from flub_gb300.fields import IntField, MACGridInt
    tags = MACGridInt(*(IntField(torch.zeros_like(a, dtype=torch.int32), d=d + 1)
                        for d, a in enumerate((vel.u.f, vel.v.f, vel.w.f))))
    K.set_unknown(phi, tags)
    K.extrapolate(vel, tags, None, 1)
    torch.cuda.synchronize()
    x0e, x1e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    x0e.record(stream)
    for _ in range(10):
        K.extrapolate(vel, tags, None, 1)
    x1e.record(stream)
    torch.cuda.synchronize()
    ext_ms = x0e.elapsed_time(x1e) / 10
    n_faces = sum(a.numel() for a in (vel.u.f, vel.v.f, vel.w.f))
    extrapolation = {"ms_per_pass": ext_ms, "passes_per_step_in_reference": 16 * scene.shape[0] // 128,
                     "faces": n_faces, "alg_bytes_per_pass": 12 * n_faces,
                     "achieved_GBps": 12 * n_faces / (ext_ms * 1e-3) / 1e9,
                     "note": "algorithmic bytes: read value and flag, write value, 12 B per face"}

    # ---- advection at the start of the reference's step (water_3d.py:34-37:
    # advect_phi, then advect_uv_mc on the three face arrays), timed warm
    from flub_gb300.fields import Field, MACGrid
    new_phi = torch.empty_like(phi)
    new_vel = MACGrid(*(Field(torch.empty_like(a), stagger=a_f.stagger, d=a_f.d)
                        for a_f, a in ((vel.u, vel.u.f), (vel.v, vel.v.f), (vel.w, vel.w.f))))

    def time_ms(fn, reps=10):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    uv_ms = time_ms(lambda: K.advect_uv_mc(vel, new_vel))
    phi_ms = time_ms(lambda: K.advect_phi_field(vel, Field(phi), Field(new_phi)))
    n_cells = phi.numel()
    advection = {"ms_advect_uv_mc": uv_ms, "ms_advect_phi": phi_ms, "faces": n_faces, "cells": n_cells,
                 "faces_per_s": n_faces / (uv_ms * 1e-3), "cells_per_s": n_cells / (phi_ms * 1e-3),
                 "alg_hbm_bytes": {"advect_uv_mc": 20 * n_faces, "advect_phi": 20 * n_cells},
                 "achieved_GBps_uv_mc": 20 * n_faces / (uv_ms * 1e-3) / 1e9,
                 "note": "algorithmic HBM bytes: the field read and written plus the three velocity components "
                         "once, 20 B per element; the kernels gather about 280 (MacCormack) or 136 (phi) values "
                         "per element through L1, which bounds them"}

    # ---- level-set redistance (redistance.py:125-136, as particles.py:267-270
    # calls it: set_boundary = 0): _init_distance + 2 x 8 sweeps of 2 halves
    rd_phi = torch.empty_like(phi)
    rd_ms = time_ms(lambda: (rd_phi.copy_(phi), K.redistance(rd_phi, None, 0)))
    copy_ms = time_ms(lambda: rd_phi.copy_(phi))
    redistance_info = {"ms": rd_ms - copy_ms, "cells": n_cells, "launches": 33,
                       "ms_per_half_sweep_estimate": (rd_ms - copy_ms) / 33,
                       "note": "in place through the Python call: the init kernel writes a temporary, the 32 "
                               "half-sweeps update it, one device copy brings it back; 256^3 FP32 phi (67 MB) "
                               "stays in L2"}

    # ---- U-Net training throughput: forward + backward + Adam on a batch of 4
    # random 64^3 scenes (the shape the warm start runs at), its conv FLOPs
    # counted as 2 * 27 * (cin0 + cin1) * cout per output voxel per layer, x3
    # for forward + the two backward convolutions
    unet_training = None
    if net is not None:
        from flub_gb300.unet import LAYERS, UNet3D as _U
        tnet = _U(seed=1)
        gen = torch.Generator(device="cuda").manual_seed(5)
        B, G = 4, 64
        div_b = torch.randn((B, G, G, G), generator=gen, device="cuda")
        tag_b = torch.ones((B, G, G, G), dtype=torch.int32, device="cuda")
        tag_b[:, :, G // 2:, :] = 0
        x_b = torch.randn((B, G, G, G), generator=gen, device="cuda")
        for _ in range(3):
            tnet.zero_grad()
            tnet.loss_and_grad(div_b, tag_b, x_b)
            tnet.adam_step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        n_it = 10
        for _ in range(n_it):
            tnet.zero_grad()
            tnet.loss_and_grad(div_b, tag_b, x_b)
            tnet.adam_step()
        e1.record(stream)
        torch.cuda.synchronize()
        t_ms = e0.elapsed_time(e1) / n_it
        flops_voxel = sum(2 * 27 * (c0 + c1) * co / 8 ** lv for _, c0, c1, co, lv in LAYERS)
        flops = 3 * flops_voxel * G ** 3 * B
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
            os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
        sustained = peaks.get("bf16_tflops_sustained", 1700.0)
        unet_training = {"batch": B, "grid": G, "ms_per_step": t_ms, "samples_per_s": B / (t_ms * 1e-3),
                         "conv_flops_per_step": flops, "achieved_tflops": flops / (t_ms * 1e-3) / 1e12,
                         "frac_of_sustained_bf16": flops / (t_ms * 1e-3) / 1e12 / sustained,
                         "note": "conv FLOPs only; the 16-64-channel convolutions are skinny GEMMs "
                                 "(N = 16..64) whose per-tap operand loads bound them, far from the tensor peak"}
        del tnet, div_b, tag_b, x_b

    # ---- config 1: 128^3 flow past a sphere, plain vs mixed precision, both
    # schedules, each against the FP64 oracle's projection of the same scene
    sphere128 = None
    if rank == 0 and not args.no_sphere128:
        import oracle as O
        s1 = scenes.CONFIGS["sphere128"]()
        ref1 = O.project(s1, max_iters=200, rel_tol=1e-12, abs_tol=0.0, dtype=np.float64)
        p1 = torch.from_numpy(ref1["p"].astype(np.float64)).cuda()
        dv = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        v1_0 = [dv(a) for a in (s1.u, s1.v, s1.w)]
        v1 = MACGrid(*(Field(a.clone(), d=d + 1) for d, a in enumerate(v1_0)))
        vr1 = MACGrid(*(Field(dv(a), d=d + 1) for d, a in enumerate((s1.ur, s1.vr, s1.wr))))
        phi1 = dv(s1.phi)
        sphere128 = {"scene": "sphere128: 128^3, solid sphere r = 0.15 at the centre, solid inflow layer (u = 1), "
                              "air outflow layer", "levels": s1.levels, "fp64_oracle_iterations": int(ref1["iters"])}
        for name in ("plain", "mixed", "plain-v22", "mixed-v22"):
            prec, sched, _ = VARIANT_SETUP[name]
            pj = Projection(s1.shape, s1.levels, precision=prec, schedule=sched)
            times = []
            for rep in range(6):
                for a, b in zip((v1.u.f, v1.v.f, v1.w.f), v1_0):
                    a.copy_(b)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                pj.project(v1, vr1, phi1, s1.prims, sync=False, **solve_kw)
                e1.record(stream)
                torch.cuda.synchronize()
                if rep >= 2:
                    times.append(e0.elapsed_time(e1))
            inf = pj.mg.info()
            sphere128[name] = {"ms_per_solve": statistics.median(times), "iterations": inf["iterations"],
                               "converged": bool(inf["converged"]),
                               "pressure_rel_l2_vs_fp64_oracle": float((pj.p.f.double() - p1).norm() / p1.norm()),
                               "max_abs_div_after": pj.max_abs_div(v1, vr1)}
            del pj
        del v1, vr1, v1_0, phi1, p1
        torch.cuda.empty_cache()

    # ---- the 512^3 dam break (the 256^3 scene scaled up, generated on the
    # device): ms per solve of plain FP32 (reference schedule), plain-v22 and
    # learned+mixed-v22, each to relative residual 1e-6; the pressures of the
    # light variants against the plain one, and of all three against the FP64
    # oracle's solve of the same scene on the host cores (--no-oracle512 skips it)
    scale512 = None
    if rank == 0 and not args.no_scale512:
        del variants
        torch.cuda.empty_cache()
        s5 = scenes.dam_device(512, 2, "cuda")
        v5_0 = [a.clone() for a in (s5.u, s5.v, s5.w)]
        v5 = MACGrid(*(Field(a, d=d + 1) for d, a in enumerate((s5.u, s5.v, s5.w))))
        vr5 = MACGrid(*(Field(a, d=d + 1) for d, a in enumerate((s5.ur, s5.vr, s5.wr))))
        scale512 = {"scene": "dam512 (device-generated, same layout as dam256)", "cells": s5.n_cells,
                    "levels": s5.levels}
        p_plain = None
        p5 = {}
        for name in ("plain", "plain-v22", "learned+mixed-v22"):
            prec, sched, use_net = VARIANT_SETUP[name]
            if use_net and net is None:
                continue
            pj = Projection(s5.shape, s5.levels, precision=prec, schedule=sched)
            ws5 = learned.WarmStart(net) if use_net else None
            times = []
            for rep in range(4):
                for a, b in zip((v5.u.f, v5.v.f, v5.w.f), v5_0):
                    a.copy_(b)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                pj.project(v5, vr5, s5.phi, s5.prims, sync=False, warm_start=ws5, **solve_kw)
                e1.record(stream)
                torch.cuda.synchronize()
                if rep:
                    times.append(e0.elapsed_time(e1))
            inf = pj.mg.info()
            entry = {"ms_per_solve": statistics.median(times), "iterations": inf["iterations"],
                     "converged": bool(inf["converged"]), "max_abs_div_after": pj.max_abs_div(v5, vr5)}
            if p_plain is None:
                p_plain = pj.p.f.detach().double().clone()
                # the level-0 half-sweep at 512^3 (8x the groups of the 256^3 launch),
                # the kernel the V-cycle runs there (two half-sweeps per call), on
                # the buffers of one V-cycle of a seeded residual as at 256^3
                g5 = torch.Generator(device=v5.u.f.device)
                g5.manual_seed(7)
                fl5 = pj.tag.f == 1
                pj.mg.apply_preconditioner(r=torch.rand(fl5.shape, generator=g5, device=fl5.device) * fl5)
                del fl5
                kind = pj.mg.smooth_iteration(0, 0)
                torch.cuda.synchronize()
                e0.record(stream)
                for q in range(12):
                    pj.mg.smooth_iteration(0, q & 1)
                e1.record(stream)
                torch.cuda.synchronize()
                sweep_ms = e0.elapsed_time(e1) / 12 / (1 if kind == 1 else 2)
                f5 = (pj.tag.f == 1).view(512, 512, 64, 8).any(dim=-1)
                na = int(f5.sum().item())
                ab = SMOOTH_HALF_SWEEP_BYTES_PER_CELL * 8 * na + 4.0 * na
                scale512["level0_half_sweep"] = {
                    "kernel": "k_smooth_split<kInPlace>" if kind == 2 else "k_smooth8<false,false>",
                    "launch_ms": sweep_ms, "active_groups": na, "alg_bytes": ab,
                    "achieved_GBps": ab / (sweep_ms * 1e-3) / 1e9,
                    "frac_of_measured_peak": ab / (sweep_ms * 1e-3) / 1e9 / peak}
            else:
                entry["pressure_rel_l2_vs_plain"] = float((pj.p.f.double() - p_plain).norm() / p_plain.norm())
            p5[name] = pj.p.f.detach().clone()
            scale512[name] = entry
            del pj, ws5
            torch.cuda.empty_cache()
        if not args.no_oracle512:
            # the FP64 oracle's projection of the same scene on the host cores
            import oracle as O
            t_o = time.time()
            host = scenes.Scene("dam512", s5.shape, s5.levels, s5.phi.cpu().numpy(), s5.prims,
                                *(a.cpu().numpy() for a in v5_0), *(a.f.cpu().numpy() for a in (vr5.u, vr5.v, vr5.w)))
            ref5 = O.project(host, max_iters=200, rel_tol=1e-12, abs_tol=0.0, dtype=np.float64)
            p64 = torch.from_numpy(ref5["p"].astype(np.float64)).cuda()
            for name, pv in p5.items():
                scale512[name]["pressure_rel_l2_vs_fp64_oracle"] = float((pv.double() - p64).norm() / p64.norm())
            scale512["fp64_oracle"] = {"iterations": int(ref5["iters"]), "host_s": time.time() - t_o,
                                       "threads": O.num_threads()}
            del host, ref5, p64
        del s5, v5, vr5, v5_0, p_plain, p5
        torch.cuda.empty_cache()

    # ---- CPU baseline: the oracle on the host cores (rank 0, N = 1 only)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline and args.cpu_baseline_steps > 0:
        cpu_ms, cpu_res, cores = time_cpu_projection(scene, args.cpu_baseline_steps)
        cpu = {"value": cpu_ms, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{args.cpu_baseline_steps} full {args.config} projections "
                         f"({cpu_res['iters']} CG iterations each), FP32 C restatement with OpenMP"}
        if not args.no_oracle_check:
            # the same projection in FP64 on the host checks every variant's pressure
            import oracle as O
            ref = O.project(scene, max_iters=200, rel_tol=1e-12, abs_tol=0.0, dtype=np.float64)
            p64 = torch.from_numpy(ref["p"].astype(np.float64))
            for name, pg in pressures.items():
                pv = pg.double().cpu()
                results[name]["pressure_rel_l2_vs_fp64_oracle"] = float((pv - p64).norm() / p64.norm())
            cpu["fp64_oracle_iterations"] = int(ref["iters"])

    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded dam-break scene and Fourier velocity field, generated on the host)",
            "config": {"workload": f"{args.config}: {scene.shape[0]}^3 dam-break projection (classify + divergence "
                                   f"+ MGPCG to rel. residual 1e-6 + gradient update)",
                       "variant": head, "variant_desc": VARIANTS[head], "variants_ms_per_solve": results,
                       "learned": learned_info, "levels": scene.levels,
                       "iterations": info["iterations"], "converged": bool(info["converged"]),
                       "fluid_cells": int((proj.tag.f == 1).sum().item()), "cells": n,
                       "cell_iterations_per_s": n * info["iterations"] / (ms_per_step * 1e-3),
                       "max_abs_div_after": div_after, "l2_flush": "inputs larger than L2 (~1.3 GB working set)",
                       "parallelism": f"replicas x{world}"},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches),
            "extrapolation": extrapolation, "advection": advection, "redistance": redistance_info,
            "tile_smoother": tile_smoother, "sphere128": sphere128, "dam512": scale512,
            "unet_training": unet_training,
            "clocks": clocks,
        }
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def main():
    args = parse_args()
    if args.profile_kernel:
        return run_profile_kernel(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
