"""Drop-in mirror of DexDeform's mpm/simulator.py (MPMSimulator, State,
TempState, rigid_body_motion) on libdexmpm.so.

Same constructor arguments, state tuples, per-substep ``states`` list and
substep / substep_grad schedule (mpm/simulator.py:561-585).  Two backends:

* ``"batched"`` (default): the states live in the batched engine's layout
  (24 SoA planes per state, dexdeform_gb300.engine) and every substep runs the
  batched kernels -- fused SVD/stress/P2G with warp pre-reduction, the
  block-culled grid update, coalesced G2P; ``step`` fuses each G2P with the
  next P2G.  ``states[i].x`` etc. keep the interface of mpm/types.py's
  ``array`` (upload, download, zero, ``.t``) as strided views of the planes,
  so reads and writes convert between the caller's (n, 3) / (n, 3, 3) arrays
  and the planes only when a field is accessed.
* ``"reference"``: the reference-compatible launchers of include/dexmpm.h
  (AoS arrays, dense grid), launch for launch the reference's schedule.

Both keep the reference's memory model (one state per substep, gradients
accumulated into ``states[i].*_grad``).  Differences: no yacs config (keyword
arguments, ``cfg`` accepted and ignored except for ``gravity`` /
``ground_friction`` attributes), and device-side pose copies (``set_pose``
accepts device tensors without a host round trip).

For throughput (many environments, checkpointed gradients, CUDA graphs) use
dexdeform_gb300.engine / dexdeform_gb300.torch_wrapper.
"""
from __future__ import annotations

import ctypes
from types import SimpleNamespace

import numpy as np
import torch

from . import _native as N

GRID_LOWER_ZERO = np.zeros((1, 3), np.int32)  # mpm/simulator.py:16


def rigid_body_motion(states, actions):
    """mpm/simulator.py:19-43: integrate 6-D twists (T, B, 6) from poses
    (pos (B,3), q (B,4) wxyz) into per-substep poses (T,B,3), (T,B,4)."""
    T, B = actions.shape[:2]
    pos, q = states
    pos = pos[None, :].expand(T, -1, -1).reshape(-1, 3)
    q = q[None, :].expand(T, -1, -1).reshape(-1, 4)
    actions = actions.reshape(-1, 6)
    rot = actions[:, 3:]
    w = torch.sqrt((rot * rot).sum(axis=-1, keepdims=True) + 1e-16)
    dq = torch.cat((torch.cos(w / 2), (rot / torch.clamp(w, 1e-7, 1e9)) * torch.sin(w / 2)), 1)
    next_pos = pos + actions[:, :3]
    t = q[:, :, None] * dq[:, None, :]
    qw = t[:, 0, 0] - t[:, 1, 1] - t[:, 2, 2] - t[:, 3, 3]
    qx = t[:, 0, 1] + t[:, 1, 0] - t[:, 2, 3] + t[:, 3, 2]
    qy = t[:, 0, 2] + t[:, 1, 3] + t[:, 2, 0] - t[:, 3, 1]
    qz = t[:, 0, 3] - t[:, 1, 2] + t[:, 2, 1] + t[:, 3, 0]
    out = torch.stack([qw, qx, qy, qz], 1)
    next_rot = out / torch.linalg.norm(out, dim=-1, keepdims=True)
    return next_pos.reshape(T, B, 3), next_rot.reshape(T, B, 4)


class DeviceArray:
    """Device buffer with the interface of mpm/types.py:294-400 ``array``
    (upload / download / zero / data_ptr), held as a torch tensor."""

    def __init__(self, shape, dtype=torch.float32, device="cuda"):
        self.t = torch.zeros(shape, dtype=dtype, device=device)

    @classmethod
    def of(cls, tensor: torch.Tensor) -> "DeviceArray":
        """A DeviceArray over an existing contiguous tensor (a view)."""
        assert tensor.is_contiguous()
        a = cls.__new__(cls)
        a.t = tensor
        return a

    @property
    def data_ptr(self):
        return ctypes.c_void_p(self.t.data_ptr())

    @property
    def shape(self):
        return tuple(self.t.shape)

    def upload(self, arr, strict=False):
        a = torch.as_tensor(np.asarray(arr) if not isinstance(arr, torch.Tensor) else arr)
        a = a.to(self.t.dtype).reshape((-1,) + self.shape[1:])
        n = a.shape[0]
        if strict:
            assert n == self.shape[0]
        assert n <= self.shape[0], f"{n} {self.shape[0]}"
        self.t[:n].copy_(a, non_blocking=False)

    upload_async = upload

    def download(self, n=None, device="numpy", stream=None):
        src = self.t if n is None else self.t[:n]
        if device == "numpy":
            return src.detach().cpu().numpy().copy()
        return src.detach().to(device).clone()

    def zero(self, stream=None):
        self.t.zero_()

    zero_async = zero

    def cuda_add(self, values, stream=None):
        v = torch.as_tensor(values, dtype=self.t.dtype, device=self.t.device).reshape((-1,) + self.shape[1:])
        self.t[:v.shape[0]].add_(v)


class PlaneArray:
    """One per-particle field of one state held in SoA planes (the batched
    engine's slot layout), with the interface of mpm/types.py:294-400
    ``array``: ``.t`` is an (n, 3) or (n, 3, 3) strided view of the planes
    (reads and writes go to the planes); upload / download / zero /
    cuda_add act through it.  There is no AoS device pointer."""

    def __init__(self, planes: torch.Tensor, shape):
        self.planes = planes      # (width, stride) view of a state slot
        self._shape = tuple(shape)

    @property
    def t(self):
        v = self.planes[:, :self._shape[0]].t()
        return v.view(self._shape) if len(self._shape) == 3 else v

    @property
    def shape(self):
        return self._shape

    @property
    def data_ptr(self):
        raise N.DexError("state fields of the batched backend are SoA planes: use .t (or backend='reference')")

    def upload(self, arr, strict=False):
        a = torch.as_tensor(np.asarray(arr) if not isinstance(arr, torch.Tensor) else arr)
        a = a.to(device=self.planes.device, dtype=torch.float32).reshape((-1,) + self._shape[1:])
        n = a.shape[0]
        if strict:
            assert n == self._shape[0]
        assert n <= self._shape[0], f"{n} {self._shape[0]}"
        self.t[:n].copy_(a)

    upload_async = upload

    def download(self, n=None, device="numpy", stream=None):
        src = self.t if n is None else self.t[:n]
        if device == "numpy":
            return src.detach().cpu().numpy().copy()
        return src.detach().to(device).contiguous()

    def zero(self, stream=None):
        self.planes.zero_()

    zero_async = zero

    def cuda_add(self, values, stream=None):
        v = torch.as_tensor(values, dtype=torch.float32, device=self.planes.device).reshape((-1,) + self._shape[1:])
        self.t[:v.shape[0]].add_(v)


class TempState:
    """mpm/simulator.py:46-85: dense scratch grid and per-particle SVD temps
    (full=False: only what the loss hooks use -- the batched backend keeps
    its grids in the engine)."""

    def __init__(self, n_particles, grid_dim, n_bodies, full=True):
        g = int(grid_dim[0] * grid_dim[1] * grid_dim[2])
        A = DeviceArray
        self.grid_m, self.grid_m_grad = A((g,)), A((g,))
        self.grid_lower = DeviceArray((1, 3), dtype=torch.int32)
        if not full:
            return
        self.grid_v_in, self.grid_v_out = A((g, 3)), A((g, 3))
        self.grid_v_in_grad, self.grid_v_out_grad = A((g, 3)), A((g, 3))
        self.grid_body_v_in = A((g * (n_bodies + 1), 3))
        self.F, self.U, self.V, self.sig = A((n_particles, 3, 3)), A((n_particles, 3, 3)), A((n_particles, 3, 3)), \
            A((n_particles, 3))
        self.F_grad, self.U_grad, self.V_grad, self.sig_grad = A((n_particles, 3, 3)), A((n_particles, 3, 3)), \
            A((n_particles, 3, 3)), A((n_particles, 3))

    def clear(self, stream=None):
        self.grid_m.zero()
        self.grid_v_in.zero()
        self.grid_v_out.zero()

    def clear_grad(self, stream=None):
        for a in (self.grid_v_in_grad, self.grid_v_out_grad, self.grid_m_grad, self.sig_grad, self.F_grad,
                  self.U_grad, self.V_grad):
            a.zero()


class State:
    """mpm/simulator.py:88-145: one substep's particle and body state (+grads),
    AoS device arrays (the reference backend)."""

    def __init__(self, n_particles, n_bodies):
        self.n_particles, self.n_bodies = int(n_particles), n_bodies
        A = DeviceArray
        self.x, self.v, self.F, self.C = A((n_particles, 3)), A((n_particles, 3)), A((n_particles, 3, 3)), \
            A((n_particles, 3, 3))
        self.x_grad, self.v_grad, self.F_grad, self.C_grad = A((n_particles, 3)), A((n_particles, 3)), \
            A((n_particles, 3, 3)), A((n_particles, 3, 3))
        nb = max(n_bodies, 1)
        self.body_pos, self.body_rot = A((nb, 3)), A((nb, 4))
        self.body_pos_grad, self.body_rot_grad = A((nb, 3)), A((nb, 4))

    def get_state(self, n=None):
        return (self.x.download(n), self.v.download(n), self.F.download(n).reshape(-1, 3, 3),
                self.C.download(n).reshape(-1, 3, 3), self.body_pos.download(), self.body_rot.download())

    def set_state(self, state):
        self.x.upload(state[0])
        self.v.upload(state[1])
        self.F.upload(np.asarray(state[2]).reshape(-1, 3, 3))
        self.C.upload(np.asarray(state[3]).reshape(-1, 3, 3))
        if self.n_bodies:
            self.body_pos.upload(state[4])
            self.body_rot.upload(state[5])

    def clear_grad(self, stream=None):
        for a in (self.x_grad, self.v_grad, self.F_grad, self.C_grad, self.body_pos_grad, self.body_rot_grad):
            a.zero()


class SoAState(State):
    """One substep's state in the batched backend: particle fields and their
    gradients are PlaneArray views of state slot `index` of the simulator's
    SoA storage (x 0-2, v 3-5, F 6-14, C 15-23); body poses as in State."""

    def __init__(self, sim, index):
        self.n_particles, self.n_bodies = sim.max_particles, sim.n_bodies
        self.index = index
        self.slot, self.gslot = sim._soa[index], sim._soa_grad[index]
        n = sim.max_particles
        P = PlaneArray
        self.x, self.v = P(self.slot[0:3], (n, 3)), P(self.slot[3:6], (n, 3))
        self.F, self.C = P(self.slot[6:15], (n, 3, 3)), P(self.slot[15:24], (n, 3, 3))
        self.x_grad, self.v_grad = P(self.gslot[0:3], (n, 3)), P(self.gslot[3:6], (n, 3))
        self.F_grad, self.C_grad = P(self.gslot[6:15], (n, 3, 3)), P(self.gslot[15:24], (n, 3, 3))
        nb = max(sim.n_bodies, 1)
        A = DeviceArray
        # rows of the simulator's pose tables, so that an env step writes the
        # poses of all its substeps in one copy
        self.body_pos, self.body_rot = A.of(sim._bpos[index]), A.of(sim._brot[index])
        self.body_pos_grad, self.body_rot_grad = A((nb, 3)), A((nb, 4))


class MPMSimulator:
    """mpm/simulator.py:151-634."""

    def __init__(self, n_bodies, cfg=None, ground_friction=0., gravity=(0., -1., 0.), n_particles=20000,
                 dx=1. / 64, dt=0.0001, grid_size=(1., 1., 1.), max_steps=30, substeps=20, yield_stress=30.,
                 vol=(1. / 64 / 2) ** 2, mass=(1. / 64 / 2) ** 2, E=5000., nu=0.2, backend="batched"):
        N.require_cuda()
        self.lib = N.load()
        assert backend in ("batched", "reference")
        self.backend = backend
        self._cfg = SimpleNamespace(gravity=tuple(getattr(cfg, "gravity", gravity)),
                                    ground_friction=float(getattr(cfg, "ground_friction", ground_friction)))
        self.dx, self.inv_dx, self.dt = float(dx), 1.0 / float(dx), float(dt)
        self.max_particles = self.n_particles = int(n_particles)
        self.n_bodies = n_bodies
        self.substeps = substeps
        grid_dim = np.ceil(np.array(grid_size) / self.dx / 4).astype(int) * 4  # mpm/simulator.py:181
        self.grid_dim = (ctypes.c_int * 3)(*[int(g) for g in grid_dim])
        self.grid_length = int(np.prod(grid_dim))
        self.n_grid = int(grid_dim[0])
        self.gravity = DeviceArray((1, 3))
        self.particle_vol = DeviceArray((self.n_particles,))
        self.particle_mass = DeviceArray((self.n_particles,))
        self.particle_mu_lam_yield = DeviceArray((self.n_particles, 3))
        self.particle_ids = DeviceArray((self.n_particles,), dtype=torch.int32)
        self.particle_color = DeviceArray((self.n_particles,), dtype=torch.int32)  # 0xRRGGBB per particle
        self.dists = DeviceArray((self.n_particles * max(n_bodies, 1),))
        self.dists_grad = DeviceArray((self.n_particles * max(n_bodies, 1),))
        self.body_type_mu_softness_round = DeviceArray((max(n_bodies, 1), 4))
        self.body_args = DeviceArray((max(n_bodies, 1), 4))
        batched = backend == "batched"
        self.temp = TempState(self.n_particles, grid_dim, self.n_bodies, full=not batched)
        self.max_steps = max_steps
        if batched:
            stride = max(32, (self.n_particles + 31) // 32 * 32)
            self._soa = torch.zeros((max_steps, N.STATE_PLANES, stride), device="cuda")
            self._soa_grad = torch.zeros_like(self._soa)
            nb = max(n_bodies, 1)
            self._bpos = torch.zeros((max_steps, nb, 3), device="cuda")
            self._brot = torch.zeros((max_steps, nb, 4), device="cuda")
            self._graphs = {}
            self._row_index = {}
            self.states = [SoAState(self, i) for i in range(max_steps)]
            self._pose = torch.zeros((substeps + 1, nb, 8), device="cuda")
            self._bgrad = torch.zeros((2, nb, 8), device="cuda")
            self._E = None  # batched engine, built on first use (material and bodies are set after __init__)
        else:
            self.states = [State(self.n_particles, n_bodies) for _ in range(max_steps)]
        self.stream0 = torch.cuda.current_stream()
        self.stream1 = torch.cuda.current_stream()
        mu, lam = E / (2 * (1 + nu)), E * nu / ((1 + nu) * (1 - 2 * nu))
        self.init_particles(np.zeros(self.n_particles) + vol, np.zeros(self.n_particles) + mass,
                            np.zeros((self.n_particles, 3)) + np.array([mu, lam, yield_stress]))
        self.object_id = None
        self.torch_scale = None
        self.cur = 0
        self.action_scales = None

    # ------------------------------------------------------------- helpers
    def _sp(self):
        return N.stream_ptr()

    def _run(self, rc, what):
        N.check(rc, what)

    # ------------------------------------------------------ batched engine
    def _invalidate(self):
        """Material, bodies or the particle count changed: the batched engine
        is rebuilt on its next use."""
        if getattr(self, "backend", "reference") == "batched":
            self._E = None
            self._graphs = {}

    def _engine(self):
        """One-env BatchEngine over the SoA storage (plane stride of
        max_particles), from the simulator's current material and bodies."""
        if self._E is None:
            from .engine import BatchEngine, EnvSpec
            n, nb = self.n_particles, self.n_bodies
            mly = self.particle_mu_lam_yield.download(n)
            spec = EnvSpec(n=n, grid_dim=tuple(int(g) for g in self.grid_dim), dx=self.dx, dt=self.dt,
                           gravity=tuple(float(g) * 30 for g in self._cfg.gravity),
                           ground_friction=self.get_ground_friction(),
                           body_tfsr=self.body_type_mu_softness_round.download()[:nb],
                           body_args=self.body_args.download()[:nb], mass=self.particle_mass.download(n),
                           vol=self.particle_vol.download(n), mu_lam_yield=mly,
                           ground_height=self.get_ground_height())
            self._E = BatchEngine([spec], grad=True, stride=self._soa.shape[-1])
            assert self._E.n_particles == self._soa.shape[-1]
            self._gtmp = self._E.new_slots(1)[0]
        return self._E

    def _pack_pose(self, state, out):
        """Body pose of a state in the engine's [n_bodies][8] layout."""
        nb = self.n_bodies
        if nb:
            out[:nb, :3].copy_(state.body_pos.t[:nb])
            out[:nb, 4:].copy_(state.body_rot.t[:nb])
        return out

    # ------------------------------------------------------- state access
    def clear_grad(self, max_steps):
        for i in range(max_steps):
            self.states[i].clear_grad()

    def get_state(self, index):
        st = self.states[index].get_state(self.n_particles)
        return tuple(st[:4]) + tuple(np.r_[a, b] for a, b in zip(st[4], st[5]))

    def set_state(self, index, state):
        state = [np.float32(i) for i in state]
        if int(len(state[0])) != self.n_particles:
            self._invalidate()
        self.n_particles = int(len(state[0]))
        pos = np.float32([i[:3] for i in state[4:]]).reshape(-1, 3)
        rot = np.float32([i[3:] for i in state[4:]]).reshape(-1, 4)
        self.states[index].set_state(state[:4] + [pos, rot])
        self.cur = index

    def set_object_id(self, object_id):
        self.object_id = object_id
        assert len(object_id) == self.n_particles
        self.particle_ids.upload(np.int32(object_id))

    def get_object_id(self, device):
        assert device == "numpy"
        return self.object_id

    def set_color(self, inp):
        """Packed 0xRRGGBB colors for the renderer (mpm/simulator.py:263-266)."""
        color = self.particle_color.download(self.n_particles)
        color[:] = inp
        self.particle_color.upload(color)

    def set_softness(self, softness):
        pp = self.body_type_mu_softness_round.download()
        pp[:, 2] = softness
        self.body_type_mu_softness_round.upload(pp)
        self._invalidate()

    def get_softness(self):
        return self.body_type_mu_softness_round.download()[:, 2]

    def get_x(self, index, device="numpy"):
        return self.states[index].x.download(self.n_particles, device=device)

    def get_v(self, index, device="numpy"):
        return self.states[index].v.download(self.n_particles, device=device)

    def get_tool_state(self, index=0, device=None):
        pos, rot = self.states[index].body_pos.download(), self.states[index].body_rot.download()
        state = [i for i in np.concatenate((pos, rot), axis=1)]
        return state if device == "numpy" else [torch.tensor(i).to(device) for i in state]

    def set_tool_state(self, index, pose):
        pose = np.array(pose)
        assert pose.shape == (self.n_bodies, 7)
        self.states[index].body_pos.upload(pose[:, :3])
        self.states[index].body_rot.upload(pose[:, 3:7])

    def get_action_scales(self):
        return np.array(self.action_scales)

    def init_particles(self, vol, mass, mu_lam_yield):
        assert vol.shape == (self.n_particles,) and mass.shape == (self.n_particles,)
        assert mu_lam_yield.shape == (self.n_particles, 3)
        self.particle_vol.upload(vol)
        self.particle_mass.upload(mass)
        self.particle_mu_lam_yield.upload(mu_lam_yield)
        self.gravity.upload(np.float32([np.array(self._cfg.gravity) * 30]))  # mpm/simulator.py:385
        self.temp.grid_lower.upload(GRID_LOWER_ZERO)
        self._invalidate()

    def init_bodies(self, types, softness, mu, round, args, action_scales, pos=None, rot=None):
        assert len(mu) == len(args) == self.n_bodies
        self.body_type_mu_softness_round.upload(
            np.stack((np.float32(types), np.float32(mu), np.float32(softness), np.float32(round)), 1).reshape(-1, 4))
        self.body_args.upload(np.float32(args))
        self.action_scales = action_scales
        self._invalidate()
        if pos is not None:
            self.states[0].body_pos.upload(np.array(pos).reshape(self.n_bodies, 3))
        if rot is not None:
            self.states[0].body_rot.upload(np.array(rot).reshape(self.n_bodies, 4))

    def sync(self):
        torch.cuda.current_stream().synchronize()

    def get_ground_friction(self):
        return float(self._cfg.ground_friction)

    def get_ground_height(self):
        return 3.0

    # ------------------------------------------------------------ kernels
    def compute_svd(self, state, temp):
        self._run(self.lib.compute_svd(state.F.data_ptr, state.C.data_ptr, temp.F.data_ptr, temp.U.data_ptr,
                                       temp.V.data_ptr, temp.sig.data_ptr, self.dt, self.n_particles, self._sp()),
                  "compute_svd")

    def compute_svd_grad(self, state, temp):
        self._run(self.lib.compute_svd_grad(state.F.data_ptr, state.C.data_ptr, temp.U.data_ptr, temp.V.data_ptr,
                                            temp.sig.data_ptr, temp.F_grad.data_ptr, temp.U_grad.data_ptr,
                                            temp.V_grad.data_ptr, temp.sig_grad.data_ptr, state.F_grad.data_ptr,
                                            state.C_grad.data_ptr, self.dt, self.n_particles, self._sp()),
                  "compute_svd_grad")

    def p2g(self, s1, temp, s2):
        self._run(self.lib.p2g(s1.x.data_ptr, s1.v.data_ptr, self.particle_mass.data_ptr, self.particle_vol.data_ptr,
                               temp.F.data_ptr, temp.U.data_ptr, temp.sig.data_ptr, temp.V.data_ptr, s1.C.data_ptr,
                               self.particle_mu_lam_yield.data_ptr, temp.grid_lower.data_ptr,
                               ctypes.cast(self.grid_dim, ctypes.c_void_p), self.dx, self.inv_dx, self.dt,
                               s2.F.data_ptr, temp.grid_v_in.data_ptr, temp.grid_m.data_ptr, self.n_particles,
                               self._sp()), "p2g")

    def p2g_grad(self, s1, temp, s2):
        self._run(self.lib.p2g_grad(
            s1.x.data_ptr, s1.v.data_ptr, self.particle_mass.data_ptr, self.particle_vol.data_ptr, temp.F.data_ptr,
            temp.U.data_ptr, temp.sig.data_ptr, temp.V.data_ptr, s1.C.data_ptr, self.particle_mu_lam_yield.data_ptr,
            temp.grid_lower.data_ptr, ctypes.cast(self.grid_dim, ctypes.c_void_p), self.dx, self.inv_dx, self.dt,
            s2.F.data_ptr, temp.grid_v_in.data_ptr, temp.grid_m.data_ptr, s1.x_grad.data_ptr, s1.v_grad.data_ptr,
            temp.F_grad.data_ptr, s1.C_grad.data_ptr, temp.U_grad.data_ptr, temp.sig_grad.data_ptr,
            temp.V_grad.data_ptr, s2.F_grad.data_ptr, temp.grid_v_in_grad.data_ptr, temp.grid_m_grad.data_ptr,
            self.n_particles, self._sp()), "p2g_grad")

    def grid_op(self, s1, temp, s2):
        self._run(self.lib.grid_op_v2(
            temp.grid_m.data_ptr, temp.grid_v_in.data_ptr, temp.grid_body_v_in.data_ptr, temp.grid_lower.data_ptr,
            self.gravity.data_ptr, s1.body_pos.data_ptr, s1.body_rot.data_ptr, s2.body_pos.data_ptr,
            s2.body_rot.data_ptr, self.body_type_mu_softness_round.data_ptr, self.body_args.data_ptr, self.dx,
            self.inv_dx, self.dt, self.get_ground_friction(), temp.grid_v_out.data_ptr,
            ctypes.cast(self.grid_dim, ctypes.c_void_p), self.n_bodies, self._sp()), "grid_op_v2")

    def grid_op_grad(self, s1, temp, s2):
        self._run(self.lib.grid_op_v2_grad(
            temp.grid_m.data_ptr, temp.grid_v_in.data_ptr, temp.grid_body_v_in.data_ptr, temp.grid_lower.data_ptr,
            self.gravity.data_ptr, s1.body_pos.data_ptr, s1.body_rot.data_ptr, s2.body_pos.data_ptr,
            s2.body_rot.data_ptr, self.body_type_mu_softness_round.data_ptr, self.body_args.data_ptr,
            temp.grid_m_grad.data_ptr, temp.grid_v_in_grad.data_ptr, s1.body_pos_grad.data_ptr,
            s1.body_rot_grad.data_ptr, s2.body_pos_grad.data_ptr, s2.body_rot_grad.data_ptr, self.dx, self.inv_dx,
            self.dt, self.get_ground_friction(), temp.grid_v_out.data_ptr, temp.grid_v_out_grad.data_ptr,
            ctypes.cast(self.grid_dim, ctypes.c_void_p), self.n_bodies, self._sp()), "grid_op_v2_grad")

    def g2p(self, s1, temp, s2):
        self._run(self.lib.g2p(s1.x.data_ptr, temp.grid_v_out.data_ptr, temp.grid_lower.data_ptr, self.dx,
                               self.inv_dx, self.dt, ctypes.cast(self.grid_dim, ctypes.c_void_p), s2.v.data_ptr,
                               self.get_ground_height(), s2.C.data_ptr, s2.x.data_ptr, self.n_particles,
                               self._sp()), "g2p")

    def g2p_grad(self, s1, temp, s2):
        self._run(self.lib.g2p_grad(s1.x.data_ptr, temp.grid_v_out.data_ptr, temp.grid_lower.data_ptr, self.dx,
                                    self.inv_dx, self.dt, ctypes.cast(self.grid_dim, ctypes.c_void_p),
                                    s2.v.data_ptr, self.get_ground_height(), s2.C.data_ptr, s2.x.data_ptr,
                                    self.n_particles, s1.x_grad.data_ptr, temp.grid_v_out_grad.data_ptr,
                                    s2.v_grad.data_ptr, s2.C_grad.data_ptr, s2.x_grad.data_ptr, self._sp()),
                  "g2p_grad")

    # ----------------------------------------------------------- schedule
    def set_pose(self, state, pos, rot, stream=None):
        state.body_pos.upload(pos)
        state.body_rot.upload(rot)

    def substep(self, f, clear_grad=False):
        """mpm/simulator.py:561-571"""
        if self.backend == "batched":
            cur, nxt = self.states[f], self.states[f + 1]
            E = self._engine()
            E.substep(cur.slot, nxt.slot, self._pack_pose(cur, self._pose[0]), self._pack_pose(nxt, self._pose[1]))
            if clear_grad:
                nxt.clear_grad()
            return
        temp, cur, nxt = self.temp, self.states[f], self.states[f + 1]
        temp.clear()
        self.compute_svd(cur, temp)
        self.p2g(cur, temp, nxt)
        self.grid_op(cur, temp, nxt)
        self.g2p(cur, temp, nxt)
        if clear_grad:
            nxt.clear_grad()

    def substep_grad(self, f):
        """mpm/simulator.py:573-585: the gradients of state f + 1 back to
        state f and to both body poses, added to what they hold."""
        if self.backend == "batched":
            cur, nxt = self.states[f], self.states[f + 1]
            E = self._engine()
            bg = self._bgrad
            bg.zero_()
            E.substep_grad(cur.slot, nxt.slot, nxt.gslot, self._gtmp, self._pack_pose(cur, self._pose[0]),
                           self._pack_pose(nxt, self._pose[1]), bg[0], bg[1])
            cur.gslot.add_(self._gtmp)
            nb = self.n_bodies
            if nb:
                cur.body_pos_grad.t[:nb].add_(bg[0, :nb, :3])
                cur.body_rot_grad.t[:nb].add_(bg[0, :nb, 4:])
                nxt.body_pos_grad.t[:nb].add_(bg[1, :nb, :3])
                nxt.body_rot_grad.t[:nb].add_(bg[1, :nb, 4:])
            return
        temp, cur, nxt = self.temp, self.states[f], self.states[f + 1]
        temp.clear()
        temp.clear_grad()
        self.compute_svd(cur, temp)
        self.p2g(cur, temp, nxt)
        self.grid_op(cur, temp, nxt)
        self.g2p_grad(cur, temp, nxt)
        self.grid_op_grad(cur, temp, nxt)
        self.p2g_grad(cur, temp, nxt)
        self.compute_svd_grad(cur, temp)

    # ------------------------------------------------------- loss hooks
    def _aos(self, state, n=None):
        """(x, x_grad) device pointers of the first n particles of a state for
        the AoS loss-hook launchers, and a finisher that adds an AoS x
        gradient back (batched backend: contiguous copies of the planes)."""
        if self.backend != "batched":
            return state.x.data_ptr, state.x_grad.data_ptr, lambda: None
        n = self.n_particles if n is None else int(n)
        x = state.x.t[:n].contiguous()
        gx = torch.zeros_like(x)
        self._aos_keep = (x, gx)

        def finish():
            state.x_grad.t[:n].add_(gx)
        return ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(gx.data_ptr()), finish

    def get_dists(self, f, grad=None, device="cuda:0"):
        """mpm/simulator.py:294-321 (compute_dist, integrator.cu:188-237)."""
        state = self.states[f]
        need_grad = grad is not None
        if need_grad:
            assert grad.shape == (self.n_particles, self.n_bodies)
            self.dists_grad.t[:grad.numel()].copy_(torch.as_tensor(grad).reshape(-1))
        x_ptr, gx_ptr, finish = self._aos(state)
        self._run(self.lib.compute_dist(x_ptr, state.body_pos.data_ptr, state.body_rot.data_ptr,
                                        self.body_type_mu_softness_round.data_ptr, self.body_args.data_ptr,
                                        self.dists.data_ptr, self.n_bodies, gx_ptr,
                                        state.body_pos_grad.data_ptr, state.body_rot_grad.data_ptr,
                                        self.dists_grad.data_ptr, int(need_grad), self.n_particles, self._sp()),
                  "compute_dist")
        if need_grad:
            finish()
        if not need_grad:
            return self.dists.download(self.n_particles * self.n_bodies, device=device).reshape(-1, self.n_bodies)

    def compute_grid_mass(self, f, id=-1, device="numpy", backward_grad=None):
        """mpm/simulator.py:323-351 (particle2mass, integrator.cu:239-310)."""
        need_grad = backward_grad is not None
        if isinstance(f, int):
            n_particles, state = self.n_particles, self.states[f]
        else:
            f = f.detach().cpu().numpy() if isinstance(f, torch.Tensor) else f
            assert f.shape[-1] == 3 and id == -1
            state = self.states[-1]
            state.x.upload(np.float32(f))
            n_particles = len(f)
            if need_grad:
                state.clear_grad()
        if need_grad:
            self.temp.grid_m_grad.t.copy_(torch.as_tensor(backward_grad).reshape(-1))
        self.temp.grid_m.zero()
        x_ptr, gx_ptr, finish = self._aos(state, n_particles)
        self._run(self.lib.particle2mass(x_ptr, self.particle_mass.data_ptr, self.temp.grid_lower.data_ptr,
                                         ctypes.cast(self.grid_dim, ctypes.c_void_p), self.dx, self.inv_dx,
                                         self.temp.grid_m.data_ptr, self.temp.grid_m_grad.data_ptr,
                                         gx_ptr, self.particle_ids.data_ptr, id, int(need_grad),
                                         n_particles, self._sp()), "particle2mass")
        if need_grad:
            finish()
        if not need_grad:
            return self.temp.grid_m.download(device=device).reshape(*list(self.grid_dim))

    # --------------------------------------------------------- env step
    def download_pos_rot(self, cur, device):
        pos, rot = self.states[cur].body_pos.download(), self.states[cur].body_rot.download()
        return (torch.tensor(pos, device=device, dtype=torch.float32),
                torch.tensor(rot, device=device, dtype=torch.float32))

    def compute_forward_kinematics(self, f, action, pos_rot=None):
        """mpm/simulator.py:597-624: per-substep poses from a 6-D action per body."""
        device = "cpu" if not isinstance(action, torch.Tensor) else action.device
        pos, rot = self.download_pos_rot(f, device) if pos_rot is None else pos_rot
        action = torch.as_tensor(np.asarray(action, np.float32) if not isinstance(action, torch.Tensor) else action,
                                 dtype=torch.float32, device=device)
        if self.torch_scale is None:
            self.torch_scale = torch.tensor(np.array(self.action_scales), device=device, dtype=torch.float32)
        self.torch_scale = self.torch_scale.to(device)
        action = action.reshape(-1, 6).clamp(-1., 1.) * self.torch_scale
        steps = torch.arange(self.substeps, device=device)[:, None, None] + 1
        pos, rot = rigid_body_motion((pos, rot), action[None, :].expand(self.substeps, -1, -1) * steps / self.substeps)
        return pos, rot, (pos, rot)

    def step(self, action, pos_rot=None):
        """mpm/simulator.py:626-634 (batched backend: the env step's substeps
        in one fused sequence, each G2P fused with the next P2G)."""
        pos, rot, _ = self.compute_forward_kinematics(self.cur, action, pos_rot=pos_rot)
        if self.backend == "batched":
            # the substeps' poses into their states' rows in one copy each, the
            # engine's pose table gathered from the rows, and the env step's
            # launches replayed as a CUDA graph (one per order of the states,
            # which the swap below alternates)
            T, nb = self.substeps, self.n_bodies
            rows = tuple(self.states[f].index for f in range(T + 1))
            idx = self._row_index.get(rows)
            if idx is None:
                idx = self._row_index[rows] = torch.tensor(rows, device="cuda")
            if nb:
                f32 = dict(dtype=torch.float32, device="cuda")
                self._bpos.index_copy_(0, idx[1:], torch.as_tensor(pos).to(**f32).reshape(T, nb, 3))
                self._brot.index_copy_(0, idx[1:], torch.as_tensor(rot).to(**f32).reshape(T, nb, 4))
                self._pose[:T + 1, :nb, :3] = self._bpos.index_select(0, idx)[:, :nb]
                self._pose[:T + 1, :nb, 4:] = self._brot.index_select(0, idx)[:, :nb]
            from .engine import run_graph
            E = self._engine()
            slots = [self.states[f].slot for f in range(T + 1)]
            run_graph(E, self._graphs, ("step", rows), lambda: E.run_substeps(slots, self._pose[:T + 1]))
        else:
            for f in range(self.substeps):
                self.set_pose(self.states[f + 1], pos[f], rot[f])
            for f in range(self.substeps):
                self.substep(f)
        self.sync()
        self.states[0], self.states[self.substeps] = self.states[self.substeps], self.states[0]
