"""Learned warm start: training data from the plain MGPCG solver, training of
the U-Net (flub_gb300/unet.py) with the library's own forward, backward and
Adam kernels, and the evaluation that counts the CG iterations it saves.

No reference counterpart: flub's solver always starts from x = 0.  The solve
the network feeds is unchanged -- it still stops at the same squared-residual
tolerance relative to the right-hand side (rTr < rel_tol * |b|^2, computed
before the initial guess is applied) -- so the network can only change the
iteration count.

The guess is scaled before use: with d = the network's guess and L the
solver's operator, x0 = gamma d with gamma = (d . b) / (d . L d) minimises the
energy-norm error along d, so a warm start is never worse than x = 0 in that
norm.  On grids larger than the training grid the network runs on a coarse
level of the solver's hierarchy and its output is interpolated (WarmStart).

Command line (on a GPU):
    python -m flub_gb300.learned --train 2000 --eval 200 --n 128 --epochs 4 \
        --out flub_gb300/weights/unet_warmstart.npz
"""
import argparse
import json
import math
import os
import time

import numpy as np
import torch

from . import kernels as K
from . import scenes
from .fields import Field, MACGrid
from .mgpcg import MGPCG
from .unet import UNet3D, conv_error

WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "unet_warmstart.npz")


class SolveSet:
    """Device-resident (rhs, tag, x) triples: rhs is the solver's right-hand
    side after masking (r0 of mgpcg.py:276-284 with k = -h0), x the converged
    plain-FP32 solution, tag the reference's cell tags."""

    def __init__(self, n_scenes, shape, device):
        self.shape = tuple(shape)
        self.rhs = torch.empty((n_scenes,) + self.shape, dtype=torch.float32, device=device)
        self.x = torch.empty_like(self.rhs)
        self.tag = torch.empty((n_scenes,) + self.shape, dtype=torch.int32, device=device)
        self.iters = np.zeros(n_scenes, np.int64)
        self.seeds = np.zeros(n_scenes, np.int64)

    def __len__(self):
        return self.rhs.shape[0]


def scene_rhs(scene, mg, tag_out=None):
    """Classify, divergence, r0 = -h0 * div on fluid (the first half of
    Projection.project); leaves the right-hand side in mg.r0."""
    phi = scene.phi if isinstance(scene.phi, torch.Tensor) else torch.as_tensor(scene.phi).to(mg.device)
    dev = lambda a: a if isinstance(a, torch.Tensor) else torch.as_tensor(a).to(mg.device)
    tag = K.classify(phi, scene.prims, scene.h, scene.h0, tag=tag_out)
    vel = MACGrid(*(Field(dev(a), d=d + 1) for d, a in enumerate((scene.u, scene.v, scene.w))))
    velr = MACGrid(*(Field(dev(a), d=d + 1) for d, a in enumerate((scene.ur, scene.vr, scene.wr))))
    div = K.divergence(vel, velr, tag, scale=-1.0 / scene.h)
    mg.set_tags(tag)
    mg.init(div, -scene.h0)
    mg.mask_interior()
    return tag


def generate(n_scenes, n=128, seed0=0, device="cuda", rel_tol=1e-12, max_iters=200, log=None):
    """Seeded random scenes (scenes.random_scene_device) labelled by the plain
    FP32 MGPCG solution at relative residual sqrt(rel_tol)."""
    shape = (n, n, n)
    data = SolveSet(n_scenes, shape, device)
    mg = MGPCG(3, shape, scenes._default_levels(n), float, precision="fp32", device=device)
    t0 = time.time()
    for s in range(n_scenes):
        seed = seed0 + s
        sc = scenes.random_scene_device(n, seed, device)
        tag = scene_rhs(sc, mg)
        data.tag[s].copy_(tag.f if hasattr(tag, "f") else tag)
        data.rhs[s].copy_(mg.r0.view(shape))
        info = mg.solve(max_iters, 1e-12, 0.0, rel_tol, smoother="phases")
        data.x[s].copy_(mg.x.view(shape))
        data.iters[s] = info["iterations"]
        data.seeds[s] = seed
        if log and (s + 1) % 100 == 0:
            log(f"generated {s + 1}/{n_scenes} scenes ({time.time() - t0:.1f} s)")
    torch.cuda.synchronize()
    return data


def train(net, data, epochs=1, batch=4, lr=1e-3, seed=0, log=None, max_steps=None):
    """Adam on the masked MSE of the normalised pressure; returns per-step losses."""
    rng = np.random.default_rng(seed)
    losses = []
    steps = 0
    t0 = time.time()
    for ep in range(epochs):
        order = rng.permutation(len(data))
        for b0 in range(0, len(order) - batch + 1, batch):
            idx = torch.as_tensor(np.sort(order[b0:b0 + batch]), device=data.rhs.device)
            net.zero_grad()
            loss = net.loss_and_grad(data.rhs.index_select(0, idx), data.tag.index_select(0, idx),
                                     data.x.index_select(0, idx))
            net.adam_step(lr=lr)
            losses.append(loss)
            steps += 1
            if log and steps % 50 == 0:
                recent = float(torch.stack(losses[-50:]).mean())
                log(f"epoch {ep} step {steps} loss {recent:.4f} ({time.time() - t0:.1f} s)")
            if max_steps and steps >= max_steps:
                break
        if max_steps and steps >= max_steps:
            break
    torch.cuda.synchronize()
    if conv_error():
        raise RuntimeError("a convolution kernel timed out during training")
    return [float(l) for l in losses]


class WarmStart:
    """The network's guess as CG's initial guess.  The network runs on level
    ``level`` of the solver's hierarchy (the right-hand side restricted by
    child sums, the hierarchy's own tags there); its output is prolonged to
    the grid by cell-centred trilinear interpolation and scaled on the device
    by gamma = (d . b) / (d . L d) (MGPCG.set_initial_guess_scaled).  With
    level=None the finest level whose extent is at most ``max_extent`` and
    whose shape the network accepts is used (64: level 1 at 128^3, level 2 at
    256^3, level 3 at 512^3), which keeps the network's cost a small fraction
    of a solve."""

    def __init__(self, net, level=None, max_extent=64, graph=True):
        self.net = net
        self.level = level
        self.max_extent = max_extent
        self.graph = graph
        self._graphs = {}  # id(mg) -> (mg, level, CUDA graph, its output d)

    def choose_level(self, mg):
        if self.level is not None:
            return self.level
        ok = [l for l in range(mg.n_mg_levels) if UNet3D.check_shape(mg.level_shape(l))]
        if not ok:
            raise ValueError(f"no level of a {mg.shape} hierarchy fits the network's shape rules")
        small = [l for l in ok if max(mg.level_shape(l)) <= self.max_extent]
        return small[0] if small else ok[-1]

    def guess(self, mg, level=None):
        """Unscaled guess d on the grid (0 off fluid)."""
        L = self.choose_level(mg) if level is None else level
        b = mg.r0.view(mg.shape)
        for l in range(1, L + 1):
            b = mg.restrict_vector(l, b)
        tag = mg.level_tags(L)
        d = self.net.predict(b, tag)[0]
        for l in range(L, 0, -1):
            d = mg.prolong_vector(l, d)
        return d

    def _captured(self, mg, level):
        """The guess of this handle as a CUDA graph (captured on first use after
        one eager run that initialises the kernels), replayed per solve: one
        launch instead of ~30 host calls.  Reads mg.r0 and the handle's level
        tags, both at fixed addresses."""
        L = self.choose_level(mg) if level is None else level
        key = id(mg)
        ent = self._graphs.get(key)
        if ent is None or ent[0] is not mg or ent[1] != L:
            side = torch.cuda.Stream()
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(side):
                self.guess(mg, L)  # warm-up: tensor maps, kernel attributes
            torch.cuda.current_stream().wait_stream(side)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                d = self.guess(mg, L)
            ent = (mg, L, g, d)
            self._graphs[key] = ent
        return ent

    def apply(self, mg, level=None):
        """Set the scaled guess for the next solve (after init/mask_interior)."""
        if self.graph:
            _, _, g, d = self._captured(mg, level)
            g.replay()
        else:
            d = self.guess(mg, level)
        mg.set_initial_guess_scaled(d)
        return d


def evaluate(net, data, precision="fp32", rel_tol=1e-12, max_iters=200, log=None, schedule="reference", level=0):
    """Solve every scene cold (x0 = 0) and warm (x0 = scaled network guess)
    to the same tolerance, with the V-cycle ``schedule`` and the network on
    hierarchy ``level``.  Returns per-scene iteration counts and the network's
    relative L2 error against the converged solution on fluid; the summary
    also times the guess and a cold solve (CUDA events, warm) and gives the
    break-even: the iterations a guess must save to pay for itself."""
    shape = data.shape
    n = shape[0]
    mg = MGPCG(3, shape, scenes._default_levels(n), float, precision=precision, device=data.rhs.device,
               schedule=schedule)
    ws = WarmStart(net, level=level)
    rows = []
    for s in range(len(data)):
        tag = data.tag[s]
        mg.set_tags(tag)
        mg.init(data.rhs[s], 1.0)
        mg.mask_interior()
        cold = mg.solve(max_iters, 1e-12, 0.0, rel_tol, smoother="phases")
        x_cold = mg.x.view(shape).clone()
        mg.init(data.rhs[s], 1.0)
        mg.mask_interior()
        d = ws.apply(mg)
        warm = mg.solve(max_iters, 1e-12, 0.0, rel_tol, smoother="phases")
        gamma = warm["x0_scale"]
        fl = tag == 1
        xs = data.x[s][fl].double()
        err_net = float((gamma * d[fl].double() - xs).norm() / xs.norm())
        err_warm = float((mg.x.view(shape)[fl].double() - xs).norm() / xs.norm())
        err_cold = float((x_cold[fl].double() - xs).norm() / xs.norm())
        rows.append(dict(seed=int(data.seeds[s]), cold=cold["iterations"], warm=warm["iterations"],
                         rtr0=cold["rtr0"], gamma=gamma,
                         err_net=err_net, err_warm=err_warm, err_cold=err_cold,
                         converged=bool(cold["converged"] and warm["converged"])))
        if log and (s + 1) % 50 == 0:
            log(f"evaluated {s + 1}/{len(data)}")
    cold = np.array([r["cold"] for r in rows])
    warm = np.array([r["warm"] for r in rows])
    # cost of a guess and of one CG iteration, on the last scene
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    reps = 10
    ws.apply(mg)
    torch.cuda.synchronize()
    ev[0].record()
    for _ in range(reps):
        ws.apply(mg)
    ev[1].record()
    for _ in range(reps):
        mg.init(data.rhs[len(data) - 1], 1.0)
        mg.mask_interior()
        info = mg.solve(max_iters, 1e-12, 0.0, rel_tol, smoother="phases", sync=False)
    ev[2].record()
    torch.cuda.synchronize()
    guess_ms = ev[0].elapsed_time(ev[1]) / reps
    solve_ms = ev[1].elapsed_time(ev[2]) / reps
    iters_last = mg.info()["iterations"]
    ms_per_iter = solve_ms / max(iters_last, 1)
    saved = cold - warm
    summary = dict(scenes=len(rows), precision=precision, schedule=schedule, network_level=level,
                   network_grid=list(mg.level_shape(level)), cold_mean=float(cold.mean()),
                   warm_mean=float(warm.mean()), saved_mean=float(saved.mean()), saved_min=int(saved.min()),
                   saved_max=int(saved.max()),
                   saved_histogram={str(int(k)): int(v) for k, v in zip(*np.unique(saved, return_counts=True))},
                   err_net_mean=float(np.mean([r["err_net"] for r in rows])),
                   gamma_mean=float(np.mean([r["gamma"] for r in rows])),
                   all_converged=all(r["converged"] for r in rows), guess_ms=guess_ms, cold_solve_ms=solve_ms,
                   ms_per_iteration=ms_per_iter, break_even_iterations=guess_ms / ms_per_iter,
                   net_gain_ms_mean=float(saved.mean()) * ms_per_iter - guess_ms)
    return summary, rows


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--train", type=int, default=2000)
    ap.add_argument("--eval", type=int, default=200)
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--epochs", type=float, default=4)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--report", default=None, help="JSON report path")
    ap.add_argument("--init", default=None, help="start from these weights")
    ap.add_argument("--eval-only", action="store_true",
                    help="evaluate the weights at --out on the held-out scenes under every schedule of "
                         "--schedules and network level of --levels, fp32 and mixed, and add the results to "
                         "--report (an existing report is updated)")
    ap.add_argument("--schedules", default="reference,v22")
    ap.add_argument("--levels", default="0,1")
    args = ap.parse_args(argv)
    dev = torch.device("cuda", 0)
    log = lambda m: print(m, flush=True)
    if args.eval_only:
        return _eval_only(args, dev, log)
    t0 = time.time()
    train_set = generate(args.train, args.n, seed0=100000 + args.seed * 1000003, device=dev, log=log)
    eval_set = generate(args.eval, args.n, seed0=900000 + args.seed * 1000003, device=dev, log=log)
    t_gen = time.time() - t0
    log(f"data: {args.train} + {args.eval} scenes at {args.n}^3 in {t_gen:.1f} s; "
        f"plain MGPCG iterations mean {train_set.iters.mean():.2f}")
    net = UNet3D.load(args.init, device=dev) if args.init else UNet3D(device=dev, seed=args.seed)
    steps_per_epoch = args.train // args.batch
    max_steps = int(round(args.epochs * steps_per_epoch))
    t1 = time.time()
    losses = train(net, train_set, epochs=int(math.ceil(args.epochs)), batch=args.batch, lr=args.lr,
                   seed=args.seed, log=log, max_steps=max_steps)
    t_train = time.time() - t1
    samples = len(losses) * args.batch
    log(f"trained {len(losses)} steps ({samples} samples) in {t_train:.1f} s: {samples / t_train:.2f} samples/s")
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    net.save(args.out)
    summary, rows = evaluate(net, eval_set, "fp32", log=log)
    summary_m, rows_m = evaluate(net, eval_set, "mixed", log=log)
    report = dict(train_scenes=args.train, eval_scenes=args.eval, n=args.n, epochs=args.epochs, batch=args.batch,
                  lr=args.lr, steps=len(losses), train_seconds=t_train, samples_per_s=samples / t_train,
                  generate_seconds=t_gen, loss_first=float(np.mean(losses[:20])), loss_last=float(np.mean(losses[-50:])),
                  loss_curve=[float(np.mean(losses[i:i + 50])) for i in range(0, len(losses), 50)],
                  eval_fp32=summary, eval_mixed=summary_m, parameters=net.num_parameters())
    log(json.dumps({k: v for k, v in report.items() if k != "loss_curve"}))
    if args.report:
        with open(args.report, "w") as f:
            json.dump(dict(report, rows_fp32=rows, rows_mixed=rows_m), f, indent=1)
    return report


def _eval_only(args, dev, log):
    net = UNet3D.load(args.out, device=dev)
    eval_set = generate(args.eval, args.n, seed0=900000 + args.seed * 1000003, device=dev, log=log)
    held_out = []
    for sched in args.schedules.split(","):
        for level in (int(v) for v in args.levels.split(",")):
            for prec in ("fp32", "mixed"):
                summary, _ = evaluate(net, eval_set, prec, schedule=sched, level=level, log=log)
                log(json.dumps(summary))
                held_out.append(summary)
    report = {}
    if args.report and os.path.exists(args.report):
        with open(args.report) as f:
            report = json.load(f)
    report["held_out"] = held_out
    report["held_out_command"] = ("python -m flub_gb300.learned --eval-only --eval %d --n %d --schedules %s "
                                  "--levels %s --report <report.json>" % (args.eval, args.n, args.schedules,
                                                                          args.levels))
    if args.report:
        with open(args.report, "w") as f:
            json.dump(report, f, indent=1)
    return report


if __name__ == "__main__":
    main()
