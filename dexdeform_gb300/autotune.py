"""Launch-shape autotuner for the batched kernels.

Picks the particle tile size (CTA size of the particle kernels) and the number
of persistent CTAs of the grid kernels for a given batch by timing a few
forward (and, for gradient engines, adjoint) substeps of each candidate on the
batch itself, with CUDA events on the launching stream.  Results are cached in
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

from .engine import SM_COUNT, BatchEngine

CANDIDATES = [(t, c) for t in (64, 128, 256) for c in (SM_COUNT * 2, SM_COUNT * 4, SM_COUNT * 8)]
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
         candidates=CANDIDATES) -> Tuple[int, int]:
    """Time each candidate (tile_size, grid_ctas) on `state` (a state slot of
    E) with poses (>= 2 rows of [n_bodies][8]); apply and return the best."""
    key = key_for(E)
    if use_cache:
        if not _CACHE:
            _load_file()
        if key in _CACHE:
            E.retune(*_CACHE[key])
            return _CACHE[key]
    scratch = E.new_slots(2)
    g_slots = E.new_slots(2) if E.grad else None
    bg = torch.zeros((2,) + tuple(poses.shape[1:]), device=E.device)
    # gradient engines with kept grid slots run the adjoint on the slot the
    # forward filled, as a rollout does
    kept = 2 if (E.grad and E.n_grid_slots > 2) else None
    best, best_t = None, math.inf
    for tile, ctas in candidates:
        E.retune(tile, ctas)

        def run():
            if E.grad:
                E.substep(state, scratch[0], poses[0], poses[1], slot=kept)
                E.substep_grad(state, scratch[0], g_slots[0], g_slots[1], poses[0], poses[1], bg[0], bg[1],
                               slot=kept)
            else:
                E.substep(state, scratch[0], poses[0], poses[1])

        run()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            run()
        b.record()
        torch.cuda.synchronize()
        t = a.elapsed_time(b) / reps
        if t < best_t:
            best, best_t = (tile, ctas), t
    E.retune(*best)
    _CACHE[key] = best
    if use_cache:
        _save_file()
    return best
