"""Continuous-batching request loop for rollouts and gradient rollouts.

Requests (an env, a horizon in env steps, optionally a gradient) arrive over
time.  The server admits them while their device footprint fits the HBM budget,
keeps every admitted request's state resident on the device, and advances all
running requests together one env step (``substeps`` substeps) per round:

  * forward-phase requests (rollouts, and gradient requests before their
    horizon) form one batch: the particle states are gathered into a
    BatchEngine arena (one launch for all requests, dexmpm_copy_segments),
    ordered by grid cell on the device, stepped, and scattered back in the
    requests' own order; gradient requests keep a checkpoint per env step;
  * backward-phase requests (gradient requests past their horizon) form a
    second batch that runs one env step of the adjoint (recompute from the
    checkpoint, reverse substeps) per round, on its own CUDA stream so that
    it overlaps the forward batch on the device.

Requests may hand over their particles in any order (Server(sort=True)
re-orders every round's gathered particles by grid cell, with their material
and incoming gradients, and maps the results back).

Membership changes at round boundaries (a request that arrives while others
run joins at the next round; a finished request leaves and frees its memory).
Each phase has one engine sized to a capacity: a membership change re-lays it
out in place (new env, tile and block tables, material and body shapes copied
on the stream, no new buffers, no host wait); it is rebuilt, larger, only when
a membership outgrows it.  A membership that stays for `capture_after` rounds
is captured as a CUDA graph and replayed while it lasts.  Results do not
depend on co-scheduling: envs never interact, and a request computes the same
substeps in the same order alone or in the mix.
"""
from __future__ import annotations

import collections
import ctypes
import math
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np
import torch

from . import _native as N
from .engine import BatchEngine, Capacity, EnvSpec, footprint_bytes, pack_poses, run_graph

# one DexSegment (include/dexmpm.h)
_SEGMENT = np.dtype([("other", "<u8"), ("other_stride", "<i4"), ("offset", "<i4"), ("count", "<i4"),
                     ("pad", "<i4")])


def copy_segments(blocks, planes: int, buf: torch.Tensor, buf_stride: int, mode: int):
    """Copy many blocks of `planes` planes between their own tensors and one
    shared buffer in one launch (dexmpm_copy_segments): blocks = [(tensor at
    the block's first plane, its plane stride, column offset in buf, count)].
    The segment table is a host array the library passes in the launch
    parameters."""
    if not blocks:
        return
    table = np.zeros(len(blocks), _SEGMENT)
    for i, (t, stride, offset, count) in enumerate(blocks):
        table[i] = (t.data_ptr(), stride, offset, count, 0)
    N.check(N.load().dexmpm_copy_segments(table.ctypes.data_as(ctypes.c_void_p), len(blocks), planes, N.ptr(buf),
                                          buf_stride, mode, int(table["count"].max()), N.stream_ptr()),
            "dexmpm_copy_segments")


@dataclass
class Request:
    rid: int
    env: object                 # workloads.Env (poses for horizon * substeps substeps)
    horizon: int                # env steps
    grad: bool = False
    arrival: float = 0.0        # seconds on the server clock
    # filled by the server
    admitted: Optional[float] = None
    finished: Optional[float] = None
    result: Optional[dict] = None
    step: int = 0               # env steps done (forward), then adjoint steps done
    phase: str = "queued"       # queued | forward | backward | done

    @property
    def spec(self) -> EnvSpec:
        return EnvSpec.from_env(self.env)

    def footprint(self, substeps):
        return footprint_bytes([self.spec], n_slots=2, grad=self.grad, substeps=substeps,
                               env_steps=self.horizon if self.grad else 0)


class _Resident:
    """Device-resident state of one admitted request."""

    def __init__(self, req: Request, substeps: int, device):
        env = req.env
        self.n = env.n
        f = dict(dtype=torch.float32, device=device)
        st = env.state()
        buf = np.zeros((24, env.n), np.float32)
        buf[0:3], buf[3:6] = st["x"].T, st["v"].T
        buf[6:15], buf[15:24] = st["F"].reshape(env.n, 9).T, st["C"].reshape(env.n, 9).T
        self.state = torch.tensor(buf, **f)
        mat = np.zeros((5, env.n), np.float32)
        mat[0], mat[1], mat[2:5] = env.mass, env.vol, np.asarray(env.mu_lam_yield, np.float32).T
        self.mat = torch.tensor(mat, **f)   # mass, vol, mu, lambda, yield stress
        n_sub = req.horizon * substeps
        self.poses = torch.tensor(pack_poses(env.poses[:n_sub + 1, :, :3], env.poses[:n_sub + 1, :, 3:]), **f)
        self.ckpt = [self.state.clone()] if req.grad else None
        self.grad = None
        self.bgrad = torch.zeros_like(self.poses) if req.grad else None


class _Arena:
    """One phase's BatchEngine (forward, or adjoint with kept grid slots) with
    its round buffers, sized to a capacity and re-laid out for each new
    membership, plus the CUDA graphs of the current membership.

    With `sort`, a round orders the gathered particles by grid cell on the
    device first (BatchEngine.sort; material and incoming gradients permuted
    the same way), steps them in that order and maps the results back, so
    that requests may hand over their particles in any order."""

    def __init__(self, capacity: Capacity, substeps: int, grad: bool, device, tile_size: int, use_graphs: bool,
                 capture_after: int, sort: bool = True):
        self.E = BatchEngine([], device=device, grad=grad, tile_size=tile_size,
                             grid_slots=substeps + 2 if grad else 2, capacity=capacity)
        self.T = substeps
        nb = self.E.capacity.bodies
        # slot 0 and the gradient are gathered into and the kernels write the
        # rest before reading them: no zero fill
        self.slot = self.E.new_slots(self.T + 1, zero=False)
        self.poses = torch.zeros((self.T + 1, nb, 8), device=device)
        if grad:
            self.gbuf = self.E.new_slots(2, zero=False)
            self.tape = self.E.new_tape(self.T, zero=False)
            self.bgrad = torch.zeros((self.T + 1, nb, 8), device=device)
        self.sort = sort
        E = self.E
        if sort:
            self.ident = E.identity_perm(1)[0]
            self.perm = self.ident.clone()
            self.srt = E.new_slots(1, zero=False)[0]      # state 0 in cell order
            self.mat_s = torch.empty_like(E.mat)           # material in cell order
            E.use_material(self.mat_s)
            if grad:
                self.gsrt = E.new_slots(1, zero=False)[0]  # incoming gradient in cell order
        # where a round leaves its result in the requests' order
        self.out = self.slot[0] if sort else self.slot[self.T]
        self.use_graphs = use_graphs
        self.capture_after = max(1, int(capture_after))
        self.key = None
        self.graphs = {}
        self.uses = {}

    def assign(self, reqs: List[Request], resident: Dict[int, "_Resident"]) -> bool:
        """Lay the engine out for these requests (True when that changed the
        layout); the material planes are copied from the residents."""
        key = tuple(r.rid for r in reqs)
        if key == self.key:
            return False
        E = self.E
        E.relayout([r.spec for r in reqs], material=False)
        for e, r in enumerate(reqs):
            o = E.p_off[e]
            E.mat[:, o:o + r.env.n].copy_(resident[r.rid].mat)
        if self.sort:
            # the sort writes the envs' entries; the rest stays the identity
            self.perm.copy_(self.ident)
        self.key = key
        self.graphs.clear()
        self.uses.clear()
        return True

    def _states(self):
        """The round's states: sorted state 0, then the substeps' slots."""
        first = self.srt if self.sort else self.slot[0]
        return [first] + [self.slot[s] for s in range(1, self.T + 1)]

    def _order(self):
        E = self.E
        E.sort(self.slot[0], self.srt, self.perm)
        E.permute(self.perm, E.mat, self.mat_s)

    def _forward(self):
        E = self.E
        if self.sort:
            self._order()
        E.run_substeps(self._states(), self.poses)
        if self.sort:
            E.permute(self.perm, self.slot[self.T], self.slot[0], inverse=True)

    def _backward(self):
        E = self.E
        g_next = self.gbuf[1]
        if self.sort:
            self._order()
            E.permute(self.perm, self.gbuf[1], self.gsrt)
            g_next = self.gsrt
        sts = self._states()
        E.run_substeps(sts, self.poses, kept=True, tapes=self.tape)
        out = E.run_adjoint(sts, g_next, self.gbuf[0], self.poses, self.bgrad, tapes=self.tape)
        if self.sort:
            E.permute(self.perm, out, self.gbuf[1], inverse=True)
        elif out is not self.gbuf[1]:
            self.gbuf[1].copy_(out)

    def run(self, kind: str) -> bool:
        """Run the round's launch sequence; True when it was captured as a
        new CUDA graph.  A membership's rounds run eagerly until its
        capture_after-th, which is captured (many memberships last a round or
        two while requests arrive and leave); later ones replay the graph."""
        self.uses[kind] = self.uses.get(kind, 0) + 1
        before = len(self.graphs)
        run_graph(self.E, self.graphs, kind, self._forward if kind == "fwd" else self._backward,
                  self.use_graphs and self.uses[kind] >= self.capture_after)
        return len(self.graphs) > before


class Server:
    """Continuous-batching MPM server on one GPU."""

    def __init__(self, substeps=50, hbm_budget_bytes=180 * 2 ** 30, device="cuda", tile_size=128,
                 use_graphs=True, max_inflight_rounds=3, capture_after=8, growth=1.25, sort=True):
        self.T = substeps
        self.budget = int(hbm_budget_bytes)
        self.device = torch.device(device)
        self.tile_size = tile_size
        self.use_graphs = use_graphs
        self.queue: collections.deque = collections.deque()
        self.running: Dict[int, Request] = {}
        self.resident: Dict[int, _Resident] = {}
        self.done: List[Request] = []
        self.in_use = 0
        # one engine per phase (False: forward, True: adjoint), grown by
        # `growth` beyond the membership that outgrew it
        self.arenas: Dict[bool, _Arena] = {}
        self.capture_after = capture_after
        self.growth = float(growth)
        self.sort = sort
        self.s_fwd = torch.cuda.Stream(device=self.device)
        self.s_bwd = torch.cuda.Stream(device=self.device)
        self.rounds = 0
        self.work = 0  # particle-substeps processed
        # rounds queued on the device ahead of the host: each holds an event
        # and the requests it finished and batches it used (kept alive until
        # the event has passed, so their memory is not reused under it)
        self.max_inflight = max(1, int(max_inflight_rounds))
        self._round_reqs: List[Request] = []
        self._round_batches: list = []
        # where the time goes: engines built, re-laid out and graphs captured
        # (host seconds), and per round the device time of the state gathers,
        # the substeps and the scatters on each stream (CUDA events, read at
        # the end of run)
        self.engine_builds = 0
        self.relayouts = 0
        self.host_relayout_s = 0.0
        self.graph_captures = 0
        self.host_build_s = 0.0
        self.host_capture_s = 0.0
        self._events: list = []

    # ---------------------------------------------------------- admission
    def submit(self, req: Request):
        if req.footprint(self.T) > self.budget:
            raise ValueError(f"request {req.rid} needs {req.footprint(self.T)} bytes > budget {self.budget}")
        if req.env.poses.shape[0] < req.horizon * self.T + 1:
            raise ValueError(f"request {req.rid}: poses for {req.horizon * self.T} substeps required")
        req.phase = "queued"
        self.queue.append(req)

    def _admit(self, now):
        while self.queue:
            r = self.queue[0]
            need = r.footprint(self.T)
            if self.in_use + need > self.budget:
                break
            self.queue.popleft()
            self.in_use += need
            r.admitted = now
            r.phase = "forward"
            self.running[r.rid] = r
            self.resident[r.rid] = _Resident(r, self.T, self.device)

    def _batch(self, reqs, grad):
        a = self.arenas.get(grad)
        need = Capacity.of([r.spec for r in reqs], self.tile_size)
        if a is None or not a.E.capacity.holds(need):
            t0 = time.perf_counter()
            # room for every admitted request that can join this phase (all
            # of them forward, the gradient requests backward), so that the
            # arena is not regrown at each admission
            can_join = [r.spec for r in self.running.values() if r.grad or not grad]
            cap = need.union(Capacity.of(can_join, self.tile_size)).scaled(self.growth)
            if a is not None:
                cap = cap.union(a.E.capacity)
            a = _Arena(cap, self.T, grad, self.device, self.tile_size, self.use_graphs, self.capture_after, self.sort)
            self.arenas[grad] = a
            self.engine_builds += 1
            self.host_build_s += time.perf_counter() - t0
        t0 = time.perf_counter()
        if a.assign(reqs, self.resident):
            self.relayouts += 1
            self.host_relayout_s += time.perf_counter() - t0
        return a

    # -------------------------------------------------------------- round
    def _mark(self):
        ev = torch.cuda.Event(enable_timing=True)
        ev.record()
        return ev

    def _run_batch(self, b, kind):
        t0 = time.perf_counter()
        if b.run(kind):
            self.graph_captures += 1
            self.host_capture_s += time.perf_counter() - t0

    def _forward_round(self, reqs):
        b = self._batch(reqs, grad=False)
        self._round_batches.append(b)
        E = b.E
        ev = [self._mark()]
        # every request's state and poses into the engine: one launch each
        res_ = [self.resident[r.rid] for r in reqs]
        np_, nb8 = E.n_particles, b.poses.shape[1] * 8
        copy_segments([(res.state, r.env.n, E.p_off[e], r.env.n) for e, (r, res) in enumerate(zip(reqs, res_))],
                      N.STATE_PLANES, b.slot[0], np_, N.SEGMENTS_GATHER)
        copy_segments([(res.poses[r.step * self.T], r.env.nb * 8, E.body_off[e] * 8, r.env.nb * 8)
                       for e, (r, res) in enumerate(zip(reqs, res_)) if r.env.nb],
                      self.T + 1, b.poses, nb8, N.SEGMENTS_GATHER)
        ev.append(self._mark())
        self._run_batch(b, "fwd")
        ev.append(self._mark())
        copy_segments([(res.state, r.env.n, E.p_off[e], r.env.n) for e, (r, res) in enumerate(zip(reqs, res_))],
                      N.STATE_PLANES, b.out, np_, N.SEGMENTS_SCATTER)
        for r, res in zip(reqs, res_):
            if r.grad:
                res.ckpt.append(res.state.clone())
            self.work += r.env.n * self.T
        ev.append(self._mark())
        self._events.append(("fwd", ev))

    def _backward_round(self, reqs):
        b = self._batch(reqs, grad=True)
        self._round_batches.append(b)
        E = b.E
        ev = [self._mark()]
        b.gbuf[1].zero_()
        res_ = [self.resident[r.rid] for r in reqs]
        ks = [r.horizon - 1 - r.step for r in reqs]  # the env step being differentiated
        for r, res in zip(reqs, res_):
            if res.grad is None:  # loss gradient of the final state: d/dx of mean |x|^2
                res.grad = torch.zeros_like(res.state)
                res.grad[0:3] = 2.0 * res.ckpt[-1][0:3] / r.env.n
        np_, nb8 = E.n_particles, b.poses.shape[1] * 8
        rows = list(enumerate(zip(reqs, res_, ks)))
        copy_segments([(res.ckpt[k], r.env.n, E.p_off[e], r.env.n) for e, (r, res, k) in rows],
                      N.STATE_PLANES, b.slot[0], np_, N.SEGMENTS_GATHER)
        copy_segments([(res.grad, r.env.n, E.p_off[e], r.env.n) for e, (r, res, k) in rows],
                      N.STATE_PLANES, b.gbuf[1], np_, N.SEGMENTS_GATHER)
        copy_segments([(res.poses[k * self.T], r.env.nb * 8, E.body_off[e] * 8, r.env.nb * 8)
                       for e, (r, res, k) in rows if r.env.nb], self.T + 1, b.poses, nb8, N.SEGMENTS_GATHER)
        b.bgrad.zero_()
        ev.append(self._mark())
        self._run_batch(b, "bwd")
        ev.append(self._mark())
        copy_segments([(res.grad, r.env.n, E.p_off[e], r.env.n) for e, (r, res, k) in rows],
                      N.STATE_PLANES, b.gbuf[1], np_, N.SEGMENTS_SCATTER)
        copy_segments([(res.bgrad[k * self.T], r.env.nb * 8, E.body_off[e] * 8, r.env.nb * 8)
                       for e, (r, res, k) in rows if r.env.nb], self.T + 1, b.bgrad, nb8,
                      N.SEGMENTS_SCATTER_ADD)
        for r in reqs:
            self.work += r.env.n * self.T
        ev.append(self._mark())
        self._events.append(("bwd", ev))

    def step(self, now):
        """Admit what fits, run one round, retire finished requests."""
        self._admit(now)
        fwd = [r for r in self.running.values() if r.phase == "forward"]
        bwd = [r for r in self.running.values() if r.phase == "backward"]
        if not fwd and not bwd:
            return False
        main = torch.cuda.current_stream(self.device)
        if fwd:
            self.s_fwd.wait_stream(main)
            with torch.cuda.stream(self.s_fwd):
                self._forward_round(fwd)
        if bwd:
            self.s_bwd.wait_stream(main)
            with torch.cuda.stream(self.s_bwd):
                self._backward_round(bwd)
        main.wait_stream(self.s_fwd)
        main.wait_stream(self.s_bwd)
        for r in fwd:
            r.step += 1
            if r.step == r.horizon:
                if r.grad:
                    r.phase, r.step = "backward", 0
                else:
                    self._finish(r, now)
        for r in bwd:
            r.step += 1
            if r.step == r.horizon:
                self._finish(r, now)
        self.rounds += 1
        return True

    def _finish(self, r, now):
        res = self.resident[r.rid]
        out = {"state": res.state}
        if r.grad:
            out["grad_state0"] = res.grad
            out["grad_poses"] = res.bgrad
        r.result = out
        r.phase = "done"
        r._resident = res  # released with the round's event
        self._round_reqs.append(r)
        self.done.append(r)
        del self.running[r.rid]
        del self.resident[r.rid]
        self.in_use -= r.footprint(self.T)

    def run(self, requests: List[Request], clock=None, max_rounds=100000):
        """Serve requests (sorted by arrival) on a wall clock starting now;
        returns the finished requests with latencies in seconds.  The host
        runs up to max_inflight_rounds rounds ahead of the device; a
        request's completion time is taken when the event recorded after
        its last round has passed."""
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0
        inflight = collections.deque()
        stream = torch.cuda.current_stream(self.device)

        def retire(block):
            while inflight and (block or inflight[0][0].query()):
                ev, reqs, _ = inflight.popleft()
                ev.synchronize()
                t = now()
                for r in reqs:
                    r.finished = t
                    r._resident = None
                block = False

        rounds = 0
        while (pending or self.queue or self.running) and rounds < max_rounds:
            while pending and pending[0].arrival <= now():
                self.submit(pending.popleft())
            self._round_reqs, self._round_batches = [], []
            if not self.step(now()):
                retire(block=bool(inflight))
                if pending and not inflight:
                    time.sleep(max(0.0, min(0.005, pending[0].arrival - now())))
                continue
            ev = torch.cuda.Event()
            ev.record(stream)
            inflight.append((ev, self._round_reqs, self._round_batches))
            retire(block=len(inflight) > self.max_inflight)
            retire(block=False)
            rounds += 1
        while inflight:
            retire(block=True)
        return self.done


    def breakdown(self, wall_s: float) -> dict:
        """Where the serving time went (call after run): device seconds of the
        state gathers, the substeps and the scatters per stream, their busy
        fraction of the wall time, and the host time spent building engines
        building engines, re-laying them out and capturing graphs."""
        out = {"wall_s": round(wall_s, 3), "rounds": self.rounds, "engine_builds": self.engine_builds,
               "relayouts": self.relayouts, "graph_captures": self.graph_captures,
               "host_build_s": round(self.host_build_s, 3), "host_relayout_s": round(self.host_relayout_s, 3),
               "host_capture_s": round(self.host_capture_s, 3)}
        for kind in ("fwd", "bwd"):
            g = c = sc = 0.0
            n = 0
            for k, ev in self._events:
                if k != kind:
                    continue
                g += ev[0].elapsed_time(ev[1]) / 1e3
                c += ev[1].elapsed_time(ev[2]) / 1e3
                sc += ev[2].elapsed_time(ev[3]) / 1e3
                n += 1
            out[kind] = {"rounds": n, "gather_s": round(g, 3), "substeps_s": round(c, 3), "scatter_s": round(sc, 3),
                         "busy_frac": round((g + c + sc) / wall_s, 3) if wall_s > 0 else None}
        return out


def latency_stats(done: List[Request]):
    lat = np.array([r.finished - r.arrival for r in done if r.finished is not None])
    if lat.size == 0:
        return None
    return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean()), "n": int(lat.size)}


def poisson_requests(seed=0, n=32, rate_hz=20.0, grids=(48, 64, 96), n_lo=2000, n_hi=50000, h_lo=5, h_hi=100,
                     grad_frac=0.3, substeps=50, horizon_scale=1.0, sort=False):
    """Seeded serving workload: Poisson arrivals, grids 48/64/96^3, particles
    log-uniform in [n_lo, n_hi], horizons uniform in [h_lo, h_hi] env steps
    (scaled by horizon_scale), grad_frac of the requests ask for gradients.
    Particles in sampling order (sort=False) or presorted by grid cell."""
    from . import workloads as W
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += rng.exponential(1.0 / rate_hz)
        g = int(rng.choice(grids))
        npart = int(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi))))
        h = max(1, int(round(rng.integers(h_lo, h_hi + 1) * horizon_scale)))
        grad = bool(rng.random() < grad_frac)
        if rng.random() < 0.5:
            env = W.make_env(seed * 100000 + i, npart, "cube", grid=g, center=(0.5, 0.16, 0.5), extent=0.18,
                             steps=h * substeps, sort=sort, name=f"req{i}")
        else:
            env = W.make_env(seed * 100000 + i, npart, "ellipsoid", grid=g, center=(0.5, 0.13, 0.5),
                             extent=(0.12, 0.06, 0.09), steps=h * substeps, sort=sort, name=f"req{i}")
        out.append(Request(rid=i, env=env, horizon=h, grad=grad, arrival=t))
    return out
