"""Differentiable rollouts: the hand-written adjoint behind torch.autograd.

Mirror of DexDeform's mpm/torch_wrapper.py (GradModel.diff_forward,
:107-144) with a different memory model: the reference keeps every
substep's state (mpm/simulator.py:206) and replays substep_grad over them; here
an env step is one autograd node (EnvStep) that saves only its input state
(the per-env-step checkpoint) and, in backward, recomputes its T substeps from
it into a ring buffer and runs the adjoint kernels in reverse.  The forward and
the backward of an env step are CUDA graphs replayed on every call.

Gradients flow to the input state (all 24 planes) and to the per-substep body
poses (T+1 rows: row 0 is the pose at the env step's start, rows 1..T the
poses the step drives), so any torch code producing the poses -- e.g. hand
forward kinematics of joint-velocity controls -- is differentiated through.
"""
from __future__ import annotations

import ctypes
import gc
from typing import Optional, Sequence

import numpy as np
import torch

from . import _native as N
from .engine import BatchEngine, EnvSpec, run_graph


def pack_pose_tensor(pos: torch.Tensor, rot: torch.Tensor) -> torch.Tensor:
    """(..., nb, 3), (..., nb, 4) -> (..., nb, 8) = p.xyz, 0, q.wxyz (differentiable)."""
    return torch.cat([pos, torch.zeros_like(pos[..., :1]), rot], -1)


class DiffSim:
    """Differentiable batched simulator core: T substeps per env step.  The
    adjoint recomputes the env step from its input state into a ring of T+1
    state slots, keeping each substep's grid slot, then runs the adjoint
    kernels in reverse on those slots.  With `sort` (default) each call first
    orders the particles by grid cell on the device (BatchEngine.sort) and
    maps the results back: states and gradients go in and out in the
    caller's order."""

    def __init__(self, specs: Sequence[EnvSpec], substeps: int, device="cuda", tile_size=128, use_graphs=True,
                 capsule_grad="reference", sort=True):
        self.T = int(substeps)
        self.E = BatchEngine(specs, device=device, grad=True, tile_size=tile_size, capsule_grad=capsule_grad,
                             grid_slots=self.T + 2)
        self.nb = max(self.E.n_bodies, 1)
        self.ring = self.E.new_slots(self.T + 1)
        self.gbuf = self.E.new_slots(2)
        self.tape = self.E.new_tape(self.T)
        dev = self.E.device
        self.poses = torch.zeros((self.T + 1, self.nb, 8), device=dev)
        self.bgrad = torch.zeros((self.T + 1, self.nb, 8), device=dev)
        self.use_graphs = use_graphs
        self.sort = bool(sort)
        self.src = self.E.new_slots(1)[0]   # input state, caller's order
        self.io = self.E.new_slots(1)[0]    # output state / gradient, caller's order
        if self.sort:
            self.perm = self.E.identity_perm(1)[0]
            self.mat = self.E.mat.clone()
        self._g = {}

    def _prepare(self):
        """ring[0] = the input state in the order the substeps run in."""
        E = self.E
        if self.sort:
            E.sort(self.src, self.ring[0], self.perm)
            E.permute(self.perm, E.mat, self.mat)
            E.use_material(self.mat)
        else:
            self.ring[0].copy_(self.src)
            E.use_material()

    # eager bodies of the two graphs
    def _fwd(self):
        self._prepare()
        self.E.run_substeps([self.ring[s] for s in range(self.T + 1)], self.poses)
        if self.sort:
            self.E.permute(self.perm, self.ring[self.T], self.io, inverse=True)
        else:
            self.io.copy_(self.ring[self.T])

    def _bwd(self):
        E = self.E
        self._prepare()
        if self.sort:
            E.permute(self.perm, self.io, self.gbuf[1])
        else:
            self.gbuf[1].copy_(self.io)
        E.run_substeps([self.ring[s] for s in range(self.T + 1)], self.poses, kept=True, tapes=self.tape)
        out = E.run_adjoint([self.ring[s] for s in range(self.T + 1)], self.gbuf[1], self.gbuf[0], self.poses,
                            self.bgrad, tapes=self.tape)
        if self.sort:
            E.permute(self.perm, out, self.io, inverse=True)
        else:
            self.io.copy_(out)

    def forward(self, state: torch.Tensor, poses: torch.Tensor) -> torch.Tensor:
        self.src.copy_(state)
        self.poses.copy_(poses)
        run_graph(self.E, self._g, "fwd", self._fwd, self.use_graphs)
        return self.io.clone()

    def backward(self, state: torch.Tensor, poses: torch.Tensor, g_out: torch.Tensor):
        self.src.copy_(state)
        self.poses.copy_(poses)
        self.io.copy_(g_out)
        self.bgrad.zero_()
        run_graph(self.E, self._g, "bwd", self._bwd, self.use_graphs)
        return self.io.clone(), self.bgrad.clone()


class EnvStep(torch.autograd.Function):
    """state_out = T substeps of state_in under poses (T+1, nb, 8)."""

    @staticmethod
    def forward(ctx, sim: DiffSim, state: torch.Tensor, poses: torch.Tensor):
        ctx.sim = sim
        ctx.save_for_backward(state.detach(), poses.detach())
        return sim.forward(state.detach(), poses.detach())

    @staticmethod
    def backward(ctx, g_out):
        state, poses = ctx.saved_tensors
        g_state, g_poses = ctx.sim.backward(state, poses, g_out.contiguous())
        g_poses[..., 3] = 0.0
        return None, g_state, g_poses


def env_step(sim: DiffSim, state: torch.Tensor, poses: torch.Tensor) -> torch.Tensor:
    return EnvStep.apply(sim, state, poses)


# ------------------------------------------------------------- loss hooks
class _Dist(torch.autograd.Function):
    """Particle-to-body signed distances (integrator.cu:188-237) through the
    compute_dist launcher, with its adjoint."""

    @staticmethod
    def forward(ctx, x, pos, rot, tfsr, args):
        L = N.load()
        n, nb = x.shape[0], pos.shape[0]
        x, pos, rot = x.detach().contiguous(), pos.detach().contiguous(), rot.detach().contiguous()
        d = torch.empty((n, nb), device=x.device)
        z = torch.zeros(1, device=x.device)
        N.check(L.compute_dist(N.ptr(x), N.ptr(pos), N.ptr(rot), N.ptr(tfsr), N.ptr(args), N.ptr(d), nb, N.ptr(z),
                               N.ptr(z), N.ptr(z), N.ptr(z), 0, n, N.stream_ptr()), "compute_dist")
        ctx.save_for_backward(x, pos, rot, tfsr, args)
        return d

    @staticmethod
    def backward(ctx, gd):
        x, pos, rot, tfsr, args = ctx.saved_tensors
        L = N.load()
        gx, gp, gr = torch.zeros_like(x), torch.zeros_like(pos), torch.zeros_like(rot)
        gd = gd.contiguous()
        N.check(L.compute_dist(N.ptr(x), N.ptr(pos), N.ptr(rot), N.ptr(tfsr), N.ptr(args), N.ptr(gd), pos.shape[0],
                               N.ptr(gx), N.ptr(gp), N.ptr(gr), N.ptr(gd), 1, x.shape[0], N.stream_ptr()),
                "compute_dist")
        return gx, gp, gr, None, None


def dists(x, pos, rot, tfsr, args):
    return _Dist.apply(x, pos, rot, tfsr, args)


class _GridMass(torch.autograd.Function):
    """Grid mass of particles (integrator.cu:239-310) through particle2mass."""

    @staticmethod
    def forward(ctx, x, mass, grid_dim, dx, ids, obj):
        L = N.load()
        x = x.detach().contiguous()
        g = torch.zeros(int(np.prod(grid_dim)), device=x.device)
        gd = (ctypes.c_int * 3)(*grid_dim)
        low = torch.zeros(3, dtype=torch.int32, device=x.device)
        N.check(L.particle2mass(N.ptr(x), N.ptr(mass), N.ptr(low), ctypes.cast(gd, ctypes.c_void_p), dx, 1.0 / dx,
                                N.ptr(g), N.ptr(g), N.ptr(x), N.ptr(ids), obj, 0, x.shape[0], N.stream_ptr()),
                "particle2mass")
        ctx.save_for_backward(x, mass, ids)
        ctx.meta = (tuple(grid_dim), dx, obj)
        return g.reshape(grid_dim)

    @staticmethod
    def backward(ctx, gg):
        x, mass, ids = ctx.saved_tensors
        grid_dim, dx, obj = ctx.meta
        L = N.load()
        gx = torch.zeros_like(x)
        gg = gg.contiguous().reshape(-1)
        gd = (ctypes.c_int * 3)(*grid_dim)
        low = torch.zeros(3, dtype=torch.int32, device=x.device)
        N.check(L.particle2mass(N.ptr(x), N.ptr(mass), N.ptr(low), ctypes.cast(gd, ctypes.c_void_p), dx, 1.0 / dx,
                                N.ptr(gg), N.ptr(gg), N.ptr(gx), N.ptr(ids), obj, 1, x.shape[0], N.stream_ptr()),
                "particle2mass")
        return gx, None, None, None, None, None


def grid_mass(x, mass, grid_dim, dx, ids=None, obj=-1):
    ids = torch.zeros(x.shape[0], dtype=torch.int32, device=x.device) if ids is None else ids
    return _GridMass.apply(x, mass, tuple(grid_dim), float(dx), ids, obj)


# ---------------------------------------------------------------- GradModel
class GradModel:
    """Mirror of mpm/torch_wrapper.py:7-184 for one environment driven by a
    hand (dexdeform_gb300.hand.SyntheticHand) under joint-velocity control.

    forward(s, action) advances env step s (substeps of the DiffSim) and
    returns the observation tuple of mpm/torch_wrapper.py:54-77:
    (particles (n, 6 + nb) = x | v | distances to every body, tool state
    (nb, 7), and the grid mass when return_grid is set).  loss.backward()
    runs the adjoint through every env step (set_obs_grad is what autograd
    does with the observation gradients).

    With use_graphs the hand's kinematics of each env step (a few hundred
    small tensor operations forward and as many backward) run as CUDA graphs
    (torch.cuda.make_graphed_callables), one per env step index and
    requires-grad pattern of its inputs; the MPM env steps replay their own
    graphs in DiffSim.  A graphed step's outputs live in its graph's memory:
    run a rollout's backward before the next rollout's forward reaches that
    env step again (the reference's training loop does)."""

    def __init__(self, env, hand, substeps, return_grid=(), device="cuda", use_graphs=True,
                 capsule_grad="reference", sort=True):
        self.env = env
        self.hand = hand
        self.device = torch.device(device)
        self.sim = DiffSim([EnvSpec.from_env(env)], substeps, device=device, use_graphs=use_graphs,
                           capsule_grad=capsule_grad, sort=sort)
        E = self.sim.E
        self.n, self.nb = env.n, env.nb
        self.tfsr = torch.tensor(env.body_tfsr, device=self.device)
        self.args = torch.tensor(env.body_args, device=self.device)
        self.mass = torch.tensor(env.mass, device=self.device)
        self.return_grid = tuple(return_grid)
        self.substeps = substeps
        self.use_graphs = use_graphs and self.device.type == "cuda"
        self._fk_graphs = {}
        self.zero_grad()

    def zero_grad(self, return_grid=None, **kw):
        if return_grid is not None:
            self.return_grid = tuple(return_grid)
        self.state = None
        self.qpos = None
        self.last_pose = None

    def reset(self, qpos: torch.Tensor, state0: Optional[torch.Tensor] = None):
        """Initial joint angles and particle state (SoA slot, or the env's)."""
        E = self.sim.E
        self.qpos = qpos
        pos, rot = self.hand.fk(qpos)
        self.last_pose = pack_pose_tensor(pos, rot)
        self.state = state0 if state0 is not None else E.pack_state([self.env.state()])
        return self.get_obs()

    def particles(self, state=None):
        st = self.state if state is None else state
        n = self.n
        return st[0:3, :n].t(), st[3:6, :n].t()

    def get_obs(self):
        x, v = self.particles()
        pose = self.last_pose
        d = dists(x.contiguous(), pose[:, :3].contiguous(), pose[:, 4:].contiguous(), self.tfsr, self.args)
        out = [torch.cat([x, v, d], 1), torch.cat([pose[:, :3], pose[:, 4:]], 1)]
        for _ in self.return_grid:
            out.append(grid_mass(x.contiguous(), self.mass, self.env.grid_dim, self.env.dx))
        return tuple(out)

    def _joint_velocity_poses(self, s, q, action):
        """Poses of the env step's substeps (substeps, nb, 8) and the final
        joint angles, through the hand's joint-velocity kinematics."""
        T = self.substeps

        def fk(q, a):
            pos, rot, q_last = self.hand.joint_velocity_poses(q, a, T)
            return pack_pose_tensor(pos, rot), q_last

        if not (self.use_graphs and torch.is_grad_enabled() and (q.requires_grad or action.requires_grad)):
            return fk(q, action)  # no gradient wanted: plain forward
        key = (s, q.requires_grad, action.requires_grad, tuple(q.shape), tuple(action.shape), q.dtype, action.dtype)
        g = self._fk_graphs.get(key)
        if g is None:
            sample = (q.detach().clone().requires_grad_(q.requires_grad),
                      action.detach().clone().requires_grad_(action.requires_grad))
            # no garbage collection while the graphs are captured: a finalizer
            # that calls CUDA (an event, stream or graph of an object going
            # out of scope) would invalidate the capture
            enabled = gc.isenabled()
            gc.disable()
            try:
                g = self._fk_graphs[key] = torch.cuda.make_graphed_callables(fk, sample)
            finally:
                if enabled:
                    gc.enable()
        return g(q, action)

    def forward(self, s, action, *past_obs):
        packed, q_last = self._joint_velocity_poses(s, self.qpos, action)
        poses = torch.cat([self.last_pose[None], packed], 0)
        self.state = env_step(self.sim, self.state, poses)
        self.qpos = q_last
        self.last_pose = poses[-1]
        return self.get_obs()

    def set_obs_grad(self, obs, grads):
        """Add observation gradients (the reference's set_obs_grad) by
        back-propagating them through the autograd graph."""
        torch.autograd.backward([o for o in obs], [g for g in grads])
