"""Launch-shape autotuner for the batched kernels.

Picks the particle tile size (CTA size of the particle kernels) and the number
of persistent CTAs of the grid kernels for a given batch by timing a few
forward substeps (and, for gradient engines, their adjoint) of each candidate
on the batch itself, launched as a rollout launches them, with CUDA events on
the launching stream.  Results are cached in
memory and in a JSON file keyed by (grid size, particle-count bucket, number
of envs bucket, gradient or not), so a shape is tuned once per process or
machine.
"""
from __future__ import annotations

import json
import math
import os
from typing import Dict, Optional, Tuple

import torch

from .engine import BatchEngine, sm_count


def candidates_for(E: BatchEngine):
    """Particle tile sizes x persistent grid CTAs of 2, 4 and 8 per SM of the
    engine's device."""
    sms = sm_count(E.device)
    return [(t, c) for t in (64, 128, 256) for c in (sms * 2, sms * 4, sms * 8)]


_CACHE: Dict[str, Tuple[int, int]] = {}
CACHE_FILE = os.environ.get("DEXMPM_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache",
                                                              "dexmpm_autotune.json"))


def key_for(E: BatchEngine) -> str:
    g = max(max(s.grid_dim) for s in E.specs)
    n = sum(s.n for s in E.specs)
    return f"g{g}-n{2 ** int(math.log2(max(n, 1)))}-e{2 ** int(math.log2(len(E.specs)))}-grad{int(E.grad)}"


def _load_file():
    try:
        with open(CACHE_FILE) as f:
            _CACHE.update({k: tuple(v) for k, v in json.load(f).items()})
    except (OSError, ValueError):
        pass


def _save_file():
    try:
        os.makedirs(os.path.dirname(CACHE_FILE), exist_ok=True)
        with open(CACHE_FILE, "w") as f:
            json.dump(_CACHE, f)
    except OSError:
        pass


def tune(E: BatchEngine, state: torch.Tensor, poses: torch.Tensor, reps: int = 3, use_cache: bool = True,
         candidates=None, rounds: int = 3) -> Tuple[int, int]:
    """Time each candidate (tile_size, grid_ctas) on `state` (a state slot of
    E) with poses (>= 2 rows of [n_bodies][8]); apply and return the best."""
    key = key_for(E)
    if candidates is None:
        candidates = candidates_for(E)
    if use_cache:
        if not _CACHE:
            _load_file()
        if key in _CACHE:
            E.retune(*_CACHE[key])
            return _CACHE[key]
    # a short rollout piece as the Rollout runs it: T substeps with each G2P
    # fused with the next P2G, and (gradient engines with kept grid slots)
    # their adjoint with each P2G adjoint fused with the previous G2P adjoint
    T = 3
    scratch = list(E.new_slots(T))
    sts = [state] + scratch
    pz = torch.stack([poses[min(i, poses.shape[0] - 1)] for i in range(T + 1)])
    kept = E.grad and E.n_grid_slots >= T + 2
    tapes = E.new_tape(T) if kept else None
    g_slots = E.new_slots(2) if E.grad else None
    bg = torch.zeros((T + 1,) + tuple(poses.shape[1:]), device=E.device)
    best, best_t = None, math.inf
    for tile, ctas in candidates:
        E.retune(tile, ctas)

        def run():
            if kept:
                E.run_substeps(sts, pz, kept=True, tapes=tapes)
                E.run_adjoint(sts, g_slots[0], g_slots[1], pz, bg, tapes=tapes)
            elif E.grad:
                E.substep(state, scratch[0], poses[0], poses[1])
                E.substep_grad(state, scratch[0], g_slots[0], g_slots[1], poses[0], poses[1], bg[0], bg[1])
            else:
                E.run_substeps(sts, pz)

        run()
        torch.cuda.synchronize()
        t = math.inf
        for _ in range(rounds):  # the best of a few timed rounds, against clock and neighbour noise
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            for _ in range(reps):
                run()
            b.record()
            torch.cuda.synchronize()
            t = min(t, a.elapsed_time(b) / reps)
        if t < best_t:
            best, best_t = (tile, ctas), t
    E.retune(*best)
    _CACHE[key] = best
    if use_cache:
        _save_file()
    return best
