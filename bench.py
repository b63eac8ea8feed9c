#!/usr/bin/env python
"""Headline benchmark: batched differentiable MLS-MPM on one GB300.

Workload (the batching configuration): 64 independent envs, each its own 64^3
grid, particle counts log-uniform in [2,000, 30,000] (seeded), cube or
ellipsoid objects, von Mises yield stress U[30, 80], 22 random-walk capsules
per env; 10 env steps x 50 substeps, forward and forward+backward (adjoint with
per-env-step checkpoints and substep recomputation), each env step replayed as
a CUDA graph.  A step = one full rollout forward + loss + backward.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Metric: particle-substeps/s (forward+backward; forward-only and the plain
per-env sequential path are reported beside it).  Under torchrun every rank
runs its own replica batch (no collective on the data path; weak scaling).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-substeps/s fwd & fwd+bwd, batched vs plain, 1 GB300 @1e-3 tol; p50/p99"
UNIT = "particle-substeps/s"
N_ENVS, SUBSTEPS, ENV_STEPS = 64, 50, 10
SERVING_SUBSTEPS = 50
MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--envs", type=int, default=N_ENVS)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--substeps", type=int, default=SUBSTEPS, help="substeps per env step (profiling cases)")
    ap.add_argument("--env-steps", type=int, default=ENV_STEPS, help="env steps per rollout (profiling cases)")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-large", action="store_true")
    ap.add_argument("--no-render", action="store_true")
    ap.add_argument("--no-diff", action="store_true", help="skip the differentiation (config 1) leg")
    ap.add_argument("--no-overlap", action="store_true",
                    help="backward without recomputing env step k - 1 on a second stream during the adjoint of k")
    ap.add_argument("--no-tune", action="store_true", help="default launch shape instead of the autotuner's")
    ap.add_argument("--presorted", action="store_true",
                    help="particles handed over already ordered by grid cell (default: sampling order)")
    ap.add_argument("--serving-requests", type=int, default=200)
    ap.add_argument("--sort-every", type=int, default=1,
                    help="re-order particles by grid cell on the device every this many env steps (0: never)")
    return ap.parse_args()


# ------------------------------------------------------------------ helpers
def dist_setup(n_gpus):
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _all_reduce(x, world, op):
    """Reduce one scalar over the ranks: NCCL on the GPU (the benchmark),
    gloo on the CPU (the multi-process tests)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=getattr(dist.ReduceOp, op))
    return float(t.item())


def max_over_ranks(x, world):
    return _all_reduce(x, world, "MAX")


def sum_over_ranks(x, world):
    return _all_reduce(x, world, "SUM")


def weak_scaling_value(work, t_ms, steps, world):
    """Whole-job particle-substeps/s: the units all ranks processed over the
    slowest rank's time (each rank runs its own replica batch)."""
    t_max = max_over_ranks(t_ms, world)
    return sum_over_ranks(float(work), world) * steps / (t_max / 1e3), t_max


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index, self.proc, self.lines = index, None, []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), f[5:9]))
            except ValueError:
                continue
        if not rows:
            return None
        sm = sorted(r[0] for r in rows)
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[2]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": max(r[1] for r in rows), "reasons": sorted(reasons),
                "samples": len(rows)}


def peaks():
    try:
        with open(MEASURED_PEAKS) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# ------------------------------------------------------------- workloads
def build_batch(seed, n_envs, presorted=False):
    from dexdeform_gb300 import workloads as W
    return W.batch_envs(seed, n_envs=n_envs, steps=SUBSTEPS * ENV_STEPS, sort=presorted)


def targets_for(envs):
    rng = np.random.default_rng(12345)
    return [e.x + rng.normal(scale=0.01, size=e.x.shape).astype(np.float32) for e in envs]


# ---------------------------------------------------------------- our arm
def run_ours(args, rank, world, local):
    import torch
    from dexdeform_gb300.engine import BatchEngine, EnvSpec, Rollout
    from dexdeform_gb300 import _native as N

    dev = torch.device("cuda", local)
    envs = build_batch(rank, args.envs, args.presorted)
    n_total = sum(e.n for e in envs)
    work = n_total * SUBSTEPS * ENV_STEPS  # particle-substeps per rollout
    # two sets of kept grid slots: the backward recomputes env step k - 1
    # while the adjoint of env step k runs
    E = BatchEngine([EnvSpec.from_env(e) for e in envs], device=dev, grad=True, grid_slots=2 * SUBSTEPS + 2)
    R = Rollout(E, substeps=SUBSTEPS, env_steps=ENV_STEPS, overlap=not args.no_overlap, sort_every=args.sort_every)
    poses_h = E.pack_poses([e.poses[:, :, :3] for e in envs], [e.poses[:, :, 3:] for e in envs])
    R.poses.copy_(torch.from_numpy(poses_h))
    s0 = E.pack_state([e.state() for e in envs])
    R.sort_initial(s0)  # the launch shape is tuned on the order the rollout runs in
    tgt = E.pack_state([{"x": t, "v": np.zeros_like(t), "F": np.zeros((len(t), 3, 3), np.float32),
                         "C": np.zeros((len(t), 3, 3), np.float32)} for t in targets_for(envs)])
    counts = torch.zeros(E.n_particles, device=dev)
    for e, env in enumerate(envs):
        counts[E.p_off[e]:E.p_off[e] + env.n] = 1.0 / env.n
    g_final = torch.zeros_like(s0)
    from dexdeform_gb300.autotune import tune
    tuned = (E.tile_size, E.grid_ctas) if args.no_tune else tune(E, R.stored(0), R.poses[:4], use_cache=False)

    def loss_grad(final):
        # L = sum_e mean_p |x - target|^2 ; dL/dx = 2 (x - target) / n_e
        d = (final[0:3] - tgt[0:3]) * counts
        g_final[0:3] = 2.0 * d
        return (d * (final[0:3] - tgt[0:3])).sum()

    def step():
        final = R.forward(s0)
        loss = loss_grad(final)
        g0 = R.backward(g_final)
        return loss, g0

    def fwd_step():
        return R.forward(s0, keep_last=False)

    # ----- warm-up (captures the graphs)
    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    launches0 = E.launches
    # ----- timed fwd+bwd
    per_step = []
    with ClockSampler(local) as clk:
        barrier(world)
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
        ev[0].record()
        for k in range(args.steps):
            step()
            ev[k + 1].record()
        torch.cuda.synchronize()
        barrier(world)
    gpu_launches = E.launches - launches0
    per_step = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    t_ms = ev[0].elapsed_time(ev[-1])
    value, t_ms_max = weak_scaling_value(work, t_ms, args.steps, world)
    work_all = sum_over_ranks(float(work), world)
    # ----- forward only
    for _ in range(3):
        fwd_step()
    torch.cuda.synchronize()
    barrier(world)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        fwd_step()
    e1.record()
    torch.cuda.synchronize()
    barrier(world)
    fwd_ms = max_over_ranks(e0.elapsed_time(e1), world)
    fwd_value = work_all * args.steps / (fwd_ms / 1e3)
    # ----- end to end: inputs from pinned host, result back to host
    s0_h = s0.cpu().pin_memory()
    poses_pin = torch.from_numpy(poses_h).pin_memory()
    g0_h = torch.empty_like(s0_h).pin_memory()
    bg_h = torch.empty(R.bgrad.shape, dtype=torch.float32).pin_memory()
    loss_h = torch.empty(1, dtype=torch.float32).pin_memory()
    s0_dev = torch.empty_like(s0)

    def e2e_step():
        s0_dev.copy_(s0_h, non_blocking=True)
        R.poses.copy_(poses_pin, non_blocking=True)
        final = R.forward(s0_dev)
        loss = loss_grad(final)
        g0 = R.backward(g_final)
        g0_h.copy_(g0, non_blocking=True)
        bg_h.copy_(R.bgrad, non_blocking=True)
        loss_h.copy_(loss.reshape(1), non_blocking=True)

    e2e_step()
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    e0.record()
    for _ in range(args.steps):
        e2e_step()
    e1.record()
    torch.cuda.synchronize()
    host_ms = (time.perf_counter() - t0) * 1e3
    barrier(world)
    e2e_ms = max_over_ranks(max(e0.elapsed_time(e1), host_ms), world)
    e2e_value = work_all * args.steps / (e2e_ms / 1e3)
    h2d = s0_h.numel() * 4 + poses_pin.numel() * 4
    d2h = g0_h.numel() * 4 + bg_h.numel() * 4 + 4

    # ----- locality: distinct stencil bases per warp of 32 particles, in the
    # caller's sampling order, right after a sort, and after an env step of
    # drift (the last checkpoint, never re-sorted)
    locality = {"sampling_order": bases_per_warp(E, s0), "sorted": bases_per_warp(E, R.stored(0)),
                f"after_{SUBSTEPS}_substeps": bases_per_warp(E, R.stored(ENV_STEPS))}
    # ----- per-kernel timing (eager, CUDA events on the launching stream)
    kt, cells = kernel_times(E, R, s0, g_final)
    roof = roofline(E, kt, cells)
    err = E.error_word()
    overlapped = R.overlap

    plain = None if (args.no_plain or rank != 0) else plain_rates(envs, dev)
    dropin = None if (args.no_plain or rank != 0) else plain_rates(envs, dev, backend="batched")
    cpu = None if (args.no_cpu or rank != 0 or world > 1) else cpu_baseline(envs)
    del R, E
    serving = None if (args.no_serving or world > 1) else serving_leg(dev, seed=rank, n_req=args.serving_requests)
    # the same requests arriving three times as fast: above the server's
    # capacity, so the throughput is the capacity and latency includes queueing
    serving_sat = None if (args.no_serving or world > 1) else serving_leg(dev, seed=rank, n_req=args.serving_requests,
                                                                         rate_hz=60.0)
    large = None if (args.no_large or world > 1) else large_env_leg(dev)
    diff = None if (args.no_diff or world > 1) else differentiation_leg(dev)
    rend = None if (args.no_render or world > 1) else render_leg(dev, cpu=not args.no_cpu)

    if rank == 0:
        ps = sorted(per_step)
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded, workloads.batch_envs)",
            "config": {"workload": f"batch: {len(envs)} envs x 64^3 grid, log-uniform 2k-30k particles, 22 capsules/env, "
                                   f"{ENV_STEPS} env steps x {SUBSTEPS} substeps, fwd+bwd with per-env-step "
                                   "checkpoints, CUDA graphs",
                       "n_envs": len(envs), "particles_per_replica": n_total, "substeps": SUBSTEPS * ENV_STEPS,
                       "dx": 1 / 64, "dt": 5e-5, "parallelism": f"replicas x{world}",
                       "launch_shape": {"tile_size": tuned[0], "grid_ctas": tuned[1],
                                        "source": "default" if args.no_tune else "autotune"},
                       "particle_order": ("presorted by grid cell" if args.presorted else "sampling order") +
                                         (f"; device sort every {args.sort_every} env step(s), inside the timed "
                                          "region" if args.sort_every else "; no device sort"),
                       "backward": ("recompute of env step k-1 on a second stream during the adjoint of env step k"
                                    if overlapped else "recompute, then adjoint, per env step"),
                       "l2": "inputs larger than L2 (per-step state traffic ~4 GB >> 129 MB L2)"},
            "fwd": {"value": fwd_value, "unit": UNIT, "ms_per_step": fwd_ms / args.steps},
            "latency_ms": {"p50": ps[len(ps) // 2], "p99": ps[min(len(ps) - 1, int(math.ceil(0.99 * len(ps))) - 1)],
                           "what": "one fwd+bwd rollout of the whole batch"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": int(gpu_launches),
            "roofline": roof,
            "kernels_us": {k: round(v, 2) for k, v in kt.items()},
            "locality": {k: round(v, 2) for k, v in locality.items()},
            "error_word": err,
        }
        if dropin is not None:
            out["simulator_dropin"] = dropin
        if plain is not None:
            out["plain"] = plain
            out["batched_vs_plain"] = {"fwd": fwd_value / plain["fwd"], "fwd_bwd": value / plain["fwd_bwd"]}
        if cpu is not None:
            out["cpu_baseline"] = cpu
        if serving is not None:
            out["serving"] = serving
        if serving_sat is not None:
            out["serving_saturated"] = serving_sat
        if large is not None:
            out["large_env"] = large
        if diff is not None:
            out["differentiation"] = diff
        if rend is not None:
            out["render"] = rend
        out["clocks"] = clk.summary()
        print(json.dumps(out))


def bases_per_warp(E, state):
    """Mean number of distinct stencil base cells among 32 consecutive
    particles of an env (what the warp pre-reduction of the scatters sees)."""
    x = state[0:3].cpu().numpy()
    out = []
    for e, sp in enumerate(E.specs):
        o = E.p_off[e]
        b = np.floor(x[:, o:o + sp.n] / sp.dx - 0.5).astype(np.int64)
        key = (b[0] * 4096 + b[1]) * 4096 + b[2]
        w = (sp.n // 32) * 32
        if w:
            k = np.sort(key[:w].reshape(-1, 32), axis=1)
            out.append((1 + (np.diff(k, axis=1) != 0).sum(1)).astype(np.float64))
    return float(np.concatenate(out).mean()) if out else 0.0


def kernel_times(E, R, s0, g_final):
    """Average device time (us) of each kernel over one env step, from CUDA
    events around eager launches on the current stream: the forward pass
    (alternating grid slots, each grid update clearing the other), the
    recompute of the backward (P2G writing the tape, grid slots kept), then
    the adjoint."""
    import torch
    from dexdeform_gb300 import _native as N
    L, sp = E.lib, N.stream_ptr()
    T = R.T
    acc = {}

    def timed(name, fn):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        acc.setdefault(name, []).append((a, b))

    ring, ck = R.ring, R.ckpt
    # the particle sort of an env-step boundary (sort + state permute, then
    # the material), and the gradient's way back through it, as a rollout
    # runs them once per env step
    if R._sorted:
        # the first boundary sorts the caller's sampling order (a random
        # permutation); later ones re-sort the end of an env step (50
        # substeps of drift: nearly in order)
        perm = E.identity_perm(1)[0]
        mat = torch.empty_like(E.mat)
        timed("sort_initial", lambda: E.sort(R.src, ring[1], perm))
        timed("permute_grad_initial", lambda: E.permute(perm, ring[1], ring[2], inverse=True))
        drifted = R.stored(R.S) if R.S > 1 else ck[0]
        timed("sort", lambda: E.sort(drifted, ring[1], perm))
        timed("permute_material", lambda: E.permute(perm, E.mat, mat))
        timed("permute_grad", lambda: E.permute(perm, ring[1], ring[2], inverse=True))
    E.use_material(R.material(0))

    def pass_(sts, kept):
        """One env step of the fused sequence: P2G, grid update, then T - 1 x
        (G2P fused with the next P2G, grid update), then G2P."""
        def take(t):
            if kept:
                return 2 + t, -1
            slot = E.fslot
            E.fslot ^= 1
            return slot, slot ^ 1
        sfx = "_tape" if kept else ""
        gname = "grid_op_keep" if kept else "grid_op"
        slot, clear = take(0)
        tp = (lambda t: N.ptr(R._tape(t))) if kept else (lambda t: None)
        timed("p2g" + sfx, lambda: N.check(L.dexmpm_p2g(E._bp, slot, N.ptr(sts[0]), N.ptr(sts[1]), tp(0), sp), "p2g"))
        timed(gname, lambda: N.check(L.dexmpm_grid_op(E._bp, slot, clear, N.ptr(R.poses[0]), N.ptr(R.poses[1]), sp),
                                     "grid_op"))
        for t in range(T - 1):
            nslot, clear = take(t + 1)
            timed("g2p2g" + sfx, lambda: N.check(L.dexmpm_g2p2g(E._bp, slot, nslot, N.ptr(sts[t]), N.ptr(sts[t + 1]),
                                                                N.ptr(sts[t + 2]), tp(t + 1), sp), "g2p2g"))
            timed(gname, lambda: N.check(L.dexmpm_grid_op(E._bp, nslot, clear, N.ptr(R.poses[t + 1]),
                                                          N.ptr(R.poses[t + 2]), sp), "grid_op"))
            slot = nslot
        timed("g2p", lambda: N.check(L.dexmpm_g2p(E._bp, slot, N.ptr(sts[T - 1]), N.ptr(sts[T]), sp), "g2p"))

    pass_([ck[0]] + [ring[t] for t in range(1, T + 1)], kept=False)   # forward pass
    pass_([ck[0]] + [ring[t] for t in range(1, T + 1)], kept=True)    # recompute of the backward
    torch.cuda.synchronize()
    cells = float(E.block_count[2:2 + T].double().mean()) * 64  # active cells per substep
    # the adjoint as BatchEngine.run_adjoint runs it: G2P adjoint of the last
    # substep, then per substep the grid adjoint and the P2G adjoint, fused
    # with the previous substep's G2P adjoint for all but the first
    gn, g = R.gbuf[1], R.gbuf[0]
    gn.copy_(g_final)
    sts = [ck[0]] + [ring[t] for t in range(1, T + 1)]
    timed("g2p_grad", lambda: N.check(L.dexmpm_g2p_grad(E._bp, 1 + T, N.ptr(sts[T - 1]), N.ptr(sts[T]), N.ptr(gn),
                                                        N.ptr(g), sp), "g2p_grad"))
    for s in range(T - 1, -1, -1):
        slot = 2 + s
        pz, pn = R.poses[s], R.poses[s + 1]
        timed("grid_op_grad", lambda: N.check(L.dexmpm_grid_op_grad(E._bp, slot, N.ptr(pz), N.ptr(pn),
                                                                    N.ptr(R.bgrad[s]), N.ptr(R.bgrad[s + 1]), sp),
                                              "grid_op_grad"))
        if s > 0:
            timed("p2g2g_grad", lambda: N.check(L.dexmpm_p2g_g2p_grad(E._bp, slot, slot - 1, N.ptr(sts[s]),
                                                                      N.ptr(sts[s - 1]), N.ptr(gn), N.ptr(g),
                                                                      N.ptr(gn), N.ptr(R._tape(s)), sp),
                                                "p2g2g_grad"))
        else:
            timed("p2g_grad", lambda: N.check(L.dexmpm_p2g_grad(E._bp, slot, N.ptr(sts[0]), N.ptr(gn), N.ptr(g),
                                                                N.ptr(R._tape(0)), sp), "p2g_grad"))
        gn, g = g, gn
    torch.cuda.synchronize()
    return {k: 1e3 * sum(a.elapsed_time(b) for a, b in v) / len(v) for k, v in acc.items()}, cells


# Algorithmic bytes per particle (N) and per cell of the active blocks (A)
# for each kernel: particle state read/written once, grid float4 cells once.
ALG_BYTES = {
    "sort_initial": (236, 0),  # as "sort", from a random order
    "permute_grad_initial": (196, 0),
    "sort": (236, 0),          # x read, key + rank written and read, perm written and segment-sorted; 24 planes
                               # gathered (96 B read, 96 B written, perm read)
    "permute_material": (44, 0),  # 5 material planes gathered, perm read
    "permute_grad": (196, 0),  # 24 gradient planes scattered back, perm read
    "p2g": (152, 16),          # x v F C + m vol mu lam yield read, F' written; m,mv scattered
    "p2g_tape": (284, 16),     # as p2g, plus the 33-plane tape written (recompute of the backward)
    "g2p2g": (164, 32),        # x, F + material read, x v C and F' written; v_out gathered, m,mv scattered
    "g2p2g_tape": (296, 32),   # as g2p2g, plus the tape written
    "grid_op": (0, 48),        # (mv, m) read, v_out written, the previous substep's cells cleared
    "grid_op_keep": (0, 32),   # (mv, m) read, v_out written (slot kept for the adjoint)
    "g2p": (72, 16),           # x read, x v C written; v_out gathered
    "g2p_grad": (96, 32),      # x, v', dL/d(x v C)' read, dL/dx written; v_out read, dL/dv_out scattered
    "grid_op_grad": (0, 80),   # (mv, m), dL/dv_out read, dL/d(mv, m) written, dL/dv_out and the slot zeroed
    "p2g_grad": (392, 16),     # x v F C + material + tape + dL/dF', dL/dx read, dL/d(x v F C) written; dL/d(mv,m) gathered
    "p2g2g_grad": (356, 48),   # p2g_grad's reads, dL/dF written; x of the previous state read, its dL/dx written;
                               # dL/d(mv,m) and v_out gathered, dL/dv_out scattered
}


# DRAM bytes (read + write) per particle of one launch, from ncu captures
# on the 64-env batch (654,552 particles, 5 substeps per env step; the fused
# kernels' on device-sorted input with the segment limit of 12)
NCU_DRAM_BYTES_PER_PARTICLE = {"p2g_grad": 236.910592e6 / 654552, "g2p2g_tape": 142.285376e6 / 654552,
                               "g2p2g": 63.428544e6 / 654552, "p2g2g_grad": 232.012544e6 / 654552}
# L2 reduction traffic and the busy fraction of the L2 atomic units of one
# launch, from an ncu capture on the same batch and input:
# (lts__t_requests_op_red.sum, lts__t_sectors_op_red.sum,
#  lts__d_atomic_input_cycles_active.avg.pct_of_peak_sustained_elapsed)
NCU_L2_RED = {"g2p2g": (2156514, 3752499, 8.13), "g2p2g_tape": (2158644, 3754360, 7.76),
              "p2g2g_grad": (2167977, 3771161, 5.50)}

# what limits each dominant kernel function, from its ncu capture on the same
# batch (--set full): issue-active and DRAM throughput percentages, warps
# active, and the reading of the stall counters
NCU_LIMITER = {
    "k_g2p2g": {"issue_active_pct": {"tape": 60.5, "forward": 60.9}, "dram_throughput_pct": {"tape": 19.9, "forward": 9.4},
                "warps_active_pct": 33.1,
                "reading": "instruction issue: G2P gather, SVD, return mapping and the 27-node scatter; "
                           "long-scoreboard the top stall",
                "source": "profiles/k_g2p2g_batch64.md"},
    "k_p2g2g_grad": {"issue_active_pct": 50.7, "dram_throughput_pct": 25.1, "warps_active_pct": 28.8,
                     "reading": "latency: streamed planes and dependent stress/SVD adjoint arithmetic at 20 "
                                "warps per SM",
                     "source": "profiles/k_p2g2g_grad_batch64.md"},
}

# kernel function of each timed launch variant (the forward pass and the
# recompute launch the same function, the recompute with the tape written)
FUNCTION = {"sort_initial": "dexmpm_sort", "permute_grad_initial": "k_permute", "sort": "dexmpm_sort",
            "permute_material": "k_permute", "permute_grad": "k_permute", "p2g": "k_p2g", "p2g_tape": "k_p2g", "g2p2g": "k_g2p2g", "g2p2g_tape": "k_g2p2g",
            "grid_op": "k_grid_op", "grid_op_keep": "k_grid_op", "g2p": "k_g2p", "g2p_grad": "k_g2p_grad",
            "grid_op_grad": "k_grid_op_grad", "p2g_grad": "k_p2g_grad", "p2g2g_grad": "k_p2g2g_grad"}


# launches per fwd+bwd substep (forward pass + recompute + adjoint; the first
# P2G and last G2P of an env step of SUBSTEPS substeps stand alone)
def launches_per_substep(T):
    # (the initial sort and its gradient map run once per rollout of
    # ENV_STEPS env steps, the others once per later env step)
    S = ENV_STEPS
    return {"sort_initial": 1 / (T * S), "permute_grad_initial": 1 / (T * S), "sort": (S - 1) / (T * S),
            "permute_material": 1 / T, "permute_grad": (S - 1) / (T * S), "p2g": 1 / T, "p2g_tape": 1 / T,
            "g2p2g": 1 - 1 / T, "g2p2g_tape": 1 - 1 / T, "grid_op": 1, "grid_op_keep": 1, "g2p": 2 / T,
            "g2p_grad": 1 / T, "grid_op_grad": 1, "p2g_grad": 1 / T, "p2g2g_grad": 1 - 1 / T}


def roofline(E, kt, cells):
    """Roofline of the dominant kernel function: the one with the largest
    device time per fwd+bwd substep, its launch variants combined (achieved =
    the variants' algorithmic bytes / their device time, both weighted by
    launches per substep)."""
    peak, src = peaks()
    w = launches_per_substep(SUBSTEPS)
    n = sum(s.n for s in E.specs)
    per_fn, bytes_fn, launches_fn, traffic_fn, variants = {}, {}, {}, {}, {}
    for k, us in kt.items():
        f = FUNCTION[k]
        bp, bc = ALG_BYTES[k]
        per_fn[f] = per_fn.get(f, 0.0) + us * w[k]
        bytes_fn[f] = bytes_fn.get(f, 0.0) + (bp * n + bc * cells) * w[k]
        launches_fn[f] = launches_fn.get(f, 0.0) + w[k]
        if k in NCU_DRAM_BYTES_PER_PARTICLE and traffic_fn.get(f, 0.0) is not None:
            traffic_fn[f] = traffic_fn.get(f, 0.0) + NCU_DRAM_BYTES_PER_PARTICLE[k] * n * w[k]
        else:
            traffic_fn[f] = None
        variants.setdefault(f, {})[k] = {"us": round(us, 2), "launches_per_substep": round(w[k], 4),
                                         "alg_bytes": int(bp * n + bc * cells)}
    top = max(per_fn, key=per_fn.get)
    total = sum(per_fn.values())
    achieved = bytes_fn[top] / (per_fn[top] * 1e-6) / 1e9
    L = launches_fn[top]
    out = {"kernel": top, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
           "frac": achieved / peak, "peak_source": src, "alg_bytes_per_launch": int(bytes_fn[top] / L),
           "avg_launch_us": per_fn[top] / L, "share_of_substep": per_fn[top] / total,
           "traffic": int(traffic_fn[top] / L) if traffic_fn.get(top) is not None else None,
           "variants": variants[top],
           "traffic_note": "dram__bytes_read.sum + dram__bytes_write.sum of ncu captures of each launch variant on "
                           "the same 64-env batch (654,552 particles, 5 substeps per env step), per particle x n, "
                           "averaged over the variants by launches per substep; profiles/k_<kernel>_batch64.md"}
    if top in NCU_LIMITER:
        out["limiter"] = NCU_LIMITER[top]
    red = [NCU_L2_RED[k] for k in variants[top] if k in NCU_L2_RED]
    if red:
        out["atomics"] = {"l2_red_requests_per_launch": int(np.mean([r[0] for r in red])),
                          "l2_red_sectors_per_launch": int(np.mean([r[1] for r in red])),
                          "l2_atomic_unit_busy_pct": round(float(np.mean([r[2] for r in red])), 2),
                          "source": "ncu lts__t_requests_op_red / lts__t_sectors_op_red / "
                                    "lts__d_atomic_input_cycles_active (profiles/l2_atomics_batch64.md)"}
    return out


def serving_leg(dev, seed=0, n_req=200, rate_hz=20.0):
    """Continuous-batching server on the serving workload: Poisson arrivals,
    grids 48/64/96^3, particles log-uniform in [2,000, 50,000], horizons
    uniform in [5, 100] env steps x 50 substeps, 30% gradient requests, HBM
    admission within 180 GB.  Latency = completion - arrival (queueing
    included); throughput = particle-substeps served / wall time.  Six short
    requests are served first, untimed, as a warm-up."""
    import torch
    from dexdeform_gb300.serving import Server, latency_stats, poisson_requests
    # warm-up: a few short requests of every kind load the kernels and fill
    # the allocator's pools before the measured run
    warm = poisson_requests(seed=seed + 1000, n=6, rate_hz=1000.0, h_lo=1, h_hi=2, grad_frac=0.5,
                            substeps=SERVING_SUBSTEPS)
    Server(substeps=SERVING_SUBSTEPS, hbm_budget_bytes=180 * 2 ** 30, device=dev).run(warm)
    torch.cuda.synchronize(dev)
    reqs = poisson_requests(seed=seed, n=n_req, rate_hz=rate_hz, substeps=SERVING_SUBSTEPS)
    base = torch.cuda.memory_allocated(dev)
    torch.cuda.reset_peak_memory_stats(dev)
    srv = Server(substeps=SERVING_SUBSTEPS, hbm_budget_bytes=180 * 2 ** 30, device=dev)
    t0 = time.perf_counter()
    done = srv.run(reqs)
    torch.cuda.synchronize(dev)
    wall = time.perf_counter() - t0
    st = latency_stats(done)
    return {"value": srv.work / wall, "unit": UNIT, "p50_s": st["p50_s"], "p99_s": st["p99_s"],
            "mean_s": st["mean_s"], "requests": len(done), "grad_requests": int(sum(r.grad for r in reqs)),
            "rate_hz": rate_hz, "wall_s": round(wall, 3), "rounds": srv.rounds,
            "breakdown": srv.breakdown(wall),
            "peak_hbm_gb": round((torch.cuda.max_memory_allocated(dev) - base) / 2 ** 30, 3),
            "hbm_budget_gb": 180, "what": "Poisson arrivals, 48/64/96^3 grids, 2k-50k particles in sampling order "
                                          "(sorted by grid cell on the device each round), horizons 5-100 env "
                                          "steps x 50 substeps, 30% gradient requests; continuous batching"}


def differentiation_leg(dev, env_steps=20, substeps=50):
    """The differentiation form on config 1 through the autograd path
    (torch_wrapper.GradModel): 20,000 particles in an ellipsoid, a 24-joint
    hand of 22 capsules driven by 24 joint-velocity controls N(0, 0.1) for 20
    env steps x 50 substeps, checkpoint per env step, loss = mean squared
    distance to a seeded target cloud; loss.backward() gives the gradients
    wrt every control and the initial state.  Whole rollouts (forward, loss,
    backward) timed with CUDA events after two warm-up rollouts."""
    import torch
    from dexdeform_gb300 import workloads as W
    from dexdeform_gb300.hand import N_BODIES, SyntheticHand, default_qpos
    from dexdeform_gb300.torch_wrapper import GradModel
    hand = SyntheticHand(base_pos=(0.5, 0.2, 0.47), action_scale=0.05)
    env = W.make_env(11, 20000, "ellipsoid", grid=64, dt=5e-5, center=(0.5, 0.11, 0.5), extent=(0.12, 0.06, 0.09),
                     nb=N_BODIES, steps=2, sort=False, name="config1")
    env.body_tfsr, env.body_args = hand.body_shapes()
    rng = np.random.default_rng(0)
    actions = torch.tensor(rng.normal(scale=0.1, size=(env_steps, 24)), dtype=torch.float32, device=dev)
    target = torch.tensor(env.x + rng.normal(scale=0.01, size=env.x.shape).astype(np.float32), device=dev)
    model = GradModel(env, hand, substeps)
    q0 = default_qpos()
    s0 = model.sim.E.pack_state([env.state()])

    def rollout():
        a = actions.clone().requires_grad_(True)
        st = s0.clone().requires_grad_(True)
        model.zero_grad()
        model.reset(q0, st)
        for k in range(env_steps):
            obs = model.forward(k, a[k])
        loss = ((obs[0][:, :3] - target) ** 2).sum(1).mean()
        loss.backward()
        return a.grad

    for _ in range(2):
        rollout()
    torch.cuda.synchronize()
    reps = 3
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ev[0].record()
    for _ in range(reps):
        g = rollout()
    ev[1].record()
    torch.cuda.synchronize()
    ms = ev[0].elapsed_time(ev[1]) / reps
    assert model.sim.E.error_word() == 0 and bool(torch.isfinite(g).all())
    work = env.n * env_steps * substeps
    return {"value": work / (ms * 1e-3), "unit": UNIT, "ms_per_rollout": round(ms, 3),
            "what": "config 1 through GradModel: 20,000 particles (sampling order, sorted on the device each env "
                    "step), 24 joint-velocity controls x 20 env steps x 50 substeps, 22 capsules, forward + loss + "
                    "backward to every control and the initial state"}


def large_env_leg(dev, substeps=100, env_steps=10):
    """Large single env: 128^3 grid, 300,000 particles in two stacked cubes
    (yield 40 / 120), 22 capsules + a palm box, 10 env steps x 100 substeps
    forward+backward with per-env-step checkpoints and substep recomputation.
    Peak device memory of the run and achieved GB/s per kernel (algorithmic
    bytes / CUDA-event time)."""
    import torch
    from dexdeform_gb300 import workloads as W
    from dexdeform_gb300.engine import BatchEngine, EnvSpec, Rollout
    env = W.large_env(0, steps=substeps * env_steps, sort=False)
    base = torch.cuda.memory_allocated(dev)
    torch.cuda.reset_peak_memory_stats(dev)
    E = BatchEngine([EnvSpec.from_env(env)], device=dev, grad=True, grid_slots=2 * substeps + 2)
    R = Rollout(E, substeps=substeps, env_steps=env_steps)
    R.poses.copy_(torch.from_numpy(E.pack_poses([env.poses[:, :, :3]], [env.poses[:, :, 3:]])))
    s0 = E.pack_state([env.state()])
    g = torch.zeros_like(s0)
    g[0:3] = 1.0 / env.n
    for _ in range(2):
        R.forward(s0)
        R.backward(g)
    torch.cuda.synchronize(dev)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 2
    a.record()
    for _ in range(reps):
        R.forward(s0)
        R.backward(g)
    b.record()
    torch.cuda.synchronize(dev)
    ms = a.elapsed_time(b) / reps
    kt, cells = kernel_times(E, R, s0, g)
    peak = torch.cuda.max_memory_allocated(dev) - base
    kern = {}
    for k, us in kt.items():
        bp, bc = ALG_BYTES[k]
        kern[k] = {"us": round(us, 2), "GB/s": round((bp * env.n + bc * cells) / (us * 1e-6) / 1e9, 1)}
    out = {"value": env.n * substeps * env_steps / (ms / 1e3), "unit": UNIT, "ms_per_rollout": round(ms, 2),
           "particles": env.n, "grid": list(env.grid_dim), "substeps": substeps * env_steps,
           "peak_hbm_gb": round(peak / 2 ** 30, 3), "active_cells_per_substep": int(cells), "kernels": kern,
           "error_word": E.error_word(),
           "what": "128^3, 300k particles (two cubes, yield 40/120), 22 capsules + palm box, 10 x 100 substeps "
                   "fwd+bwd, per-env-step checkpoints + recompute"}
    del R, E
    torch.cuda.empty_cache()
    return out


def render_leg(dev, cpu=True):
    """Renderer at the reference's defaults (mpm/renderer.py:17-27: 168^3
    voxels, 512 x 512, spp 3, 2 bounces, bake size 7, inv_dx 150) on a 20,000
    particle scene: device time of one frame (volume bake + path tracing,
    CUDA events), and the CPU restatement on a 128 x 128 frame of the same
    scene (OpenMP, all host cores), both as pixels/s."""
    import torch
    from dexdeform_gb300 import workloads as W
    from dexdeform_gb300.renderer import Renderer
    sc = W.render_scene(0, n=20000, voxel=168, image=(512, 512), inv_dx=150.0, spp=3, max_ray_depth=2)
    r = Renderer(spp=3, voxel_res=(168, 168, 168), image_res=(512, 512), max_ray_depth=2, inv_dx=150.0)
    r.setRT(sc["cam_rot"].reshape(3, 3), sc["cam_pos"])
    x = torch.tensor(sc["x"], device=dev)
    col = torch.tensor(sc["color"], device=dev)
    bodies = [torch.tensor(sc[k], device=dev) for k in ("body_pos", "body_rot", "body_tfsr", "body_args")]

    def frame():
        r.bake(x, col)
        return r.trace(*bodies, sc["ground"], seed=0)

    frame()
    torch.cuda.synchronize(dev)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 3
    a.record()
    for _ in range(reps):
        r.bake(x, col)
        r.trace(*bodies, sc["ground"], seed=0)
    b.record()
    torch.cuda.synchronize(dev)
    ms = a.elapsed_time(b) / reps
    out = {"ms_per_frame": round(ms, 3), "pixels_per_s": 512 * 512 / (ms / 1e3), "image": [512, 512], "spp": 3,
           "max_ray_depth": 2, "voxels": [168] * 3, "particles": 20000,
           "what": "volume bake + path tracing per frame (device time incl. the host copy of the image)"}
    if cpu:
        from oracle import oracle as O
        small = W.render_scene(0, n=20000, voxel=168, image=(128, 128), inv_dx=150.0, spp=3, max_ray_depth=2)
        t0 = time.perf_counter()
        _, sdf, colv = O.particle_sdf("oracle", small["x"], small["color"], small["bbox_min"], 7, small["voxel"], 150.0)
        t1 = time.perf_counter()
        O.render("oracle", small, sdf, colv)
        t2 = time.perf_counter()
        out["cpu_baseline"] = {"pixels_per_s": 128 * 128 / (t2 - t1), "bake_s": round(t1 - t0, 3),
                               "cores": os.cpu_count(), "kind": "port",
                               "sample": "CPU restatement (oracle/render_oracle.c, OpenMP over pixels), 128 x 128 "
                                         "frame of the same scene; bake single-threaded"}
    return out


def plain_rates(envs, dev, sample_every=8, backend="reference"):
    """Plain per-env sequential path: the reference's schedule (per-substep
    calls, full per-substep state storage) through the drop-in MPMSimulator,
    one env at a time, for a sample of the batch's envs.  backend
    "reference": the reference-compatible launchers (memsets + four kernels
    per substep); "batched": the same schedule on the batched kernels."""
    import torch
    from dexdeform_gb300.simulator import MPMSimulator
    T = SUBSTEPS
    fwd_t = bwd_t = step_t = 0.0
    work = 0
    for env in envs[::sample_every]:
        sim = MPMSimulator(env.nb, n_particles=env.n, dx=env.dx, dt=env.dt, grid_size=(1, 1, 1), max_steps=T + 1,
                           substeps=T, gravity=(0, -1, 0), ground_friction=env.ground_friction, backend=backend)
        sim.init_particles(env.vol.astype(np.float64), env.mass.astype(np.float64), env.mu_lam_yield.astype(np.float64))
        sim.init_bodies(env.body_tfsr[:, 0], env.body_tfsr[:, 2], env.body_tfsr[:, 1], env.body_tfsr[:, 3],
                        env.body_args, None)
        st = env.state()
        pose0 = env.poses[0]
        sim.set_state(0, (st["x"], st["v"], st["F"], st["C"], *[p for p in pose0]))
        poses = torch.tensor(env.poses[:T + 1], device=dev)
        for rep in range(2):
            torch.cuda.synchronize()
            a, b, c = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            a.record()
            for f in range(T):
                sim.set_pose(sim.states[f + 1], poses[f + 1, :, :3], poses[f + 1, :, 3:])
                sim.substep(f, clear_grad=True)
            b.record()
            sim.states[T].x_grad.t.normal_()
            for f in range(T - 1, -1, -1):
                sim.substep_grad(f)
            c.record()
            torch.cuda.synchronize()
        fwd_t += a.elapsed_time(b) / 1e3
        bwd_t += a.elapsed_time(c) / 1e3
        work += env.n * T
        if backend == "batched":
            # MPMSimulator.step: the env step's substeps as one fused sequence
            sim.action_scales = np.full((env.nb, 6), 0.01, np.float32)
            act = np.zeros((env.nb, 6), np.float32)
            for _ in range(2):  # both orders of the states (the step swaps two), each captured once
                sim.step(act)
            torch.cuda.synchronize()
            a.record()
            for _ in range(4):
                sim.step(act)
            b.record()
            torch.cuda.synchronize()
            step_t += a.elapsed_time(b) / 4e3
        del sim
    out = {"fwd": work / fwd_t, "fwd_bwd": work / bwd_t, "unit": UNIT,
           "what": f"reference schedule through MPMSimulator (backend {backend!r}), one env at a time, "
                   f"{len(envs[::sample_every])} sampled envs x 1 env step"}
    if step_t > 0:
        out["step"] = work / step_t
    return out


def median_env(envs):
    """The env of median particle count: the CPU sample of the batch."""
    return sorted(envs, key=lambda e: e.n)[len(envs) // 2]


def cpu_rollout(env, substeps):
    """One rollout of one env on the FP64 C restatement (oracle/, OpenMP over
    particles and cells, all host cores) in the reference's schedule: the
    forward storing every substep's state (mpm/simulator.py:561-571), a loss
    gradient on the final positions, then the chained substep adjoints
    (mpm/simulator.py:573-585).  Returns the seconds it took."""
    from oracle import oracle as O
    O.set_svd_mode("reference")
    t0 = time.perf_counter()
    prm = O.SimParams(grid_dim=env.grid_dim, dx=env.dx, dt=env.dt, gravity=env.gravity,
                      ground_friction=env.ground_friction)
    o = O.CpuMPM("oracle", prm, O.Material(env.mass, env.vol, env.mu_lam_yield),
                 O.Bodies(env.body_tfsr, env.body_args))
    states = [env.state()]
    for t in range(substeps):
        states.append(o.substep(states[-1], env.pose(t), env.pose(t + 1)))
    g = {k: np.zeros_like(v, dtype=np.float64) for k, v in states[-1].items()}
    g["x"] = 2.0 * (states[-1]["x"] - env.x) / env.n
    for t in range(substeps - 1, -1, -1):
        g, _, _ = o.substep_grad(states[t], env.pose(t), env.pose(t + 1), states[t + 1]["v"], g)
    return time.perf_counter() - t0


def cpu_baseline(envs):
    """The CPU baseline beside our line: one full rollout (all env steps x
    substeps, forward + backward) of the median env of the batch."""
    env = median_env(envs)
    T = SUBSTEPS * ENV_STEPS
    dt = cpu_rollout(env, T)
    return {"value": env.n * T / dt, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "sample": f"1 env of the batch (median size, {env.n} particles, {env.name}) x {ENV_STEPS} env steps x "
                      f"{SUBSTEPS} substeps, fwd+bwd in the reference's schedule (every substep state stored), "
                      f"FP64 C restatement with OpenMP", "seconds": round(dt, 2)}


# ---------------------------------------------------------- reference arm
def run_reference(args, rank, world):
    """The reference path is CUDA-only (mpm/csrc/integrator.cu); its CPU
    implementation here is the FP64 C restatement of its kernels (oracle/),
    run in its schedule on the host cores.  Each step is a bounded sample of
    the batch workload: one full rollout (all env steps x substeps, forward +
    backward) of the batch's median env.  The reference's own kernels built
    for the host (oracle/_ref) need the reference tree to compile, which the
    GPU hosts do not have."""
    if rank != 0:
        return
    envs = build_batch(0, args.envs, args.presorted)
    env = median_env(envs)
    T = SUBSTEPS * ENV_STEPS
    times = []
    for k in range(args.warmup + args.steps):
        dt = cpu_rollout(env, T)
        if k >= args.warmup:
            times.append(dt)
    sec = float(np.mean(times))
    value = env.n * T / sec
    sample = (f"1 env of the batch (median size, {env.n} particles, {env.name}) x {ENV_STEPS} env steps x "
              f"{SUBSTEPS} substeps, fwd+bwd in the reference's schedule (every substep state stored)")
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, workloads.batch_envs)",
           "impl": "reference",
           "config": {"workload": f"batch sample: {sample}",
                      "note": "the reference path is CUDA-only; its CPU implementation is the FP64 C restatement "
                              "of its kernels (oracle/), OpenMP over all host cores; each step is one full rollout "
                              "of the sampled env, timed whole"},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": os.cpu_count(), "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    global SUBSTEPS, ENV_STEPS
    args = parse()
    SUBSTEPS, ENV_STEPS = args.substeps, args.env_steps
    if args.impl == "reference":
        rank = int(os.environ.get("RANK", "0"))
        world = int(os.environ.get("WORLD_SIZE", "1"))
        run_reference(args, rank, world)
        return
    rank, world, local = dist_setup(args.gpus)
    run_ours(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
