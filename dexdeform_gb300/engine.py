"""Batched MLS-MPM engine: device buffers, grid slots and checkpointed rollouts.

A ``BatchEngine`` owns the device memory of a batch of environments (particle
state slots in SoA planes, grid slots with active-block lists, body shapes)
and launches the kernels of libdexmpm.so through its C ABI.  Forward
substeps alternate grid slots 0 and 1; an engine built with more slots lets a
recomputed env step keep one grid slot per substep, which its adjoint then
reads instead of recomputing P2G and the grid update.  A ``Rollout`` runs env
steps of ``T`` substeps forward with one checkpoint per env step and
back-propagates by recomputing each env step's substeps from its checkpoint,
each env step captured once as a CUDA graph and replayed.

Layouts (see include/dexmpm.h): state slot = 24 planes x n_particles
(x 0-2, v 3-5, F 6-14, C 15-23); poses [n_bodies][8] = p.xyz, 0, q.wxyz.
"""
from __future__ import annotations

import ctypes
import gc
import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import _native as N

TAPE_PLANES = N.TAPE_PLANES
MATERIAL_PLANES = 5  # mass, vol, mu, lambda, yield stress


def sm_count(device=None) -> int:
    """Streaming multiprocessors of the device (152 on a GB300): the
    persistent grid kernels and the autotuner's candidates are sized from it."""
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    return int(torch.cuda.get_device_properties(dev).multi_processor_count)


@dataclass
class EnvSpec:
    """Static description of one environment (mpm/simulator.py:152-226 state
    that never changes during a rollout)."""
    n: int
    grid_dim: tuple
    dx: float
    dt: float
    gravity: tuple
    ground_friction: float
    body_tfsr: np.ndarray     # (nb, 4) type, friction, softness, round
    body_args: np.ndarray     # (nb, 4)
    mass: np.ndarray          # (n,)
    vol: np.ndarray           # (n,)
    mu_lam_yield: np.ndarray  # (n, 3)
    ground_height: float = 3.0

    @property
    def nb(self):
        return int(self.body_args.shape[0])

    @classmethod
    def from_env(cls, env) -> "EnvSpec":
        return cls(n=env.n, grid_dim=tuple(env.grid_dim), dx=env.dx, dt=env.dt, gravity=tuple(env.gravity),
                   ground_friction=env.ground_friction, body_tfsr=env.body_tfsr, body_args=env.body_args,
                   mass=env.mass, vol=env.vol, mu_lam_yield=env.mu_lam_yield)


def pack_poses(pos: np.ndarray, rot: np.ndarray) -> np.ndarray:
    """(..., nb, 3) positions and (..., nb, 4) wxyz quaternions -> (..., nb, 8)."""
    out = np.zeros(pos.shape[:-1] + (8,), np.float32)
    out[..., :3] = pos
    out[..., 4:] = rot
    return out


def footprint_bytes(specs: Sequence[EnvSpec], n_slots: int = 2, grad: bool = False, substeps: int = 0,
                    env_steps: int = 0) -> int:
    """Device bytes a batch needs (used by admission control): grid slots
    (2, plus one per substep of an env step with gradients), state slots,
    checkpoints, the SVD tape of one env step (gradients) and poses."""
    n = sum(s.n for s in specs)
    blocks = sum((s.grid_dim[0] // 4) * (s.grid_dim[1] // 4) * (s.grid_dim[2] // 4) for s in specs)
    nb = sum(s.nb for s in specs)
    grid_slots = 2 + (substeps if grad else 0)
    b = blocks * 64 * 32 * grid_slots + blocks * 8 * grid_slots + blocks * 4
    b += blocks * 64 * 32 if grad else 0
    slots = n_slots + ((env_steps + 1) + (substeps + 1) + 2 if grad else 0)
    b += slots * 24 * 4 * n + 5 * 4 * n
    b += substeps * TAPE_PLANES * 4 * n if grad else 0
    b += (env_steps * substeps + 1) * nb * 32 * (2 if grad else 1)
    return int(b)


@dataclass(frozen=True)
class Capacity:
    """Table sizes a BatchEngine is built for: particles per state plane, 4^3
    grid blocks per grid slot (the slots' stride), bodies, particle tiles and
    envs.  An engine re-laid out for another set of envs (BatchEngine.relayout)
    keeps its buffers while the new layout fits."""
    particles: int = 0
    blocks: int = 0
    bodies: int = 0
    tiles: int = 0
    envs: int = 0

    @classmethod
    def of(cls, specs: Sequence[EnvSpec], tile_size: int) -> "Capacity":
        n = blk = nb = tiles = 0
        for s in specs:
            n += s.n
            blk += (s.grid_dim[0] // 4) * (s.grid_dim[1] // 4) * (s.grid_dim[2] // 4)
            nb += s.nb
            tiles += -(-s.n // tile_size)
        return cls(particles=n, blocks=blk, bodies=nb, tiles=tiles, envs=len(specs))

    def holds(self, other: "Capacity") -> bool:
        return all(getattr(self, k) >= getattr(other, k) for k in self.__dataclass_fields__)

    def union(self, other: "Capacity") -> "Capacity":
        return Capacity(**{k: max(getattr(self, k), getattr(other, k)) for k in self.__dataclass_fields__})

    def scaled(self, factor: float) -> "Capacity":
        return Capacity(**{k: int(math.ceil(getattr(self, k) * factor)) for k in self.__dataclass_fields__})


def plan_layout(specs: Sequence[EnvSpec], tile_size: int) -> dict:
    """Host-side layout of a batch: particle / block / body offsets per env,
    particle tiles (env, first particle) that never straddle envs, as an
    (n_tiles, 2) int32 array, the owning env of every grid block and its
    coordinates in that env's grid of 4^3 blocks (bx << 20 | by << 10 | bz,
    int32), and the DexEnv descriptors."""
    envs = (N.DexEnv * len(specs))()
    p_off, blk_off, body_off, tiles, nblk, xyz = [], [], [], [], [], []
    p = blk = body = 0
    for e, s in enumerate(specs):
        nbx, nby, nbz = (g // 4 for g in s.grid_dim)
        E = envs[e]
        E.p_off, E.n, E.blk_off, E.body_off = p, s.n, blk, body
        E.gx, E.gy, E.gz = s.grid_dim
        E.n_bodies = s.nb
        E.dx, E.inv_dx, E.dt, E.ground_friction = s.dx, 1.0 / s.dx, s.dt, s.ground_friction
        E.gravity[:] = list(s.gravity)
        E.ground_height = s.ground_height
        p_off.append(p)
        blk_off.append(blk)
        body_off.append(body)
        first = np.arange(0, s.n, tile_size, dtype=np.int32)
        tiles.append(np.stack([np.full_like(first, e), first], 1))
        nblk.append(nbx * nby * nbz)
        assert max(nbx, nby, nbz) < 1024, "at most 1,023 blocks of 4 cells per axis"
        bx, by, bz = np.meshgrid(np.arange(nbx, dtype=np.int32), np.arange(nby, dtype=np.int32),
                                 np.arange(nbz, dtype=np.int32), indexing="ij")
        xyz.append(((bx << 20) | (by << 10) | bz).reshape(-1))
        p += s.n
        blk += nbx * nby * nbz
        body += s.nb
    tiles = np.concatenate(tiles) if tiles else np.zeros((0, 2), np.int32)
    block_env = np.repeat(np.arange(len(specs), dtype=np.int32), nblk)
    block_xyz = np.concatenate(xyz) if xyz else np.zeros(0, np.int32)
    return dict(envs=envs, tiles=tiles, block_env=block_env, block_xyz=block_xyz, p_off=p_off, blk_off=blk_off,
                body_off=body_off, n_blocks=blk, n_bodies=body, n_particles=p)


class BatchEngine:
    def __init__(self, specs: Sequence[EnvSpec], device="cuda", tile_size: int = 128,
                 grid_ctas: Optional[int] = None, n_slots: int = 2, grad: bool = False,
                 capsule_grad: str = "reference", grid_slots: int = 2, stride: int = 0,
                 capacity: Optional[Capacity] = None):
        """grid_slots: 2 for forward use; 2 + T lets Rollout / DiffSim keep the
        grids of a recomputed env step of T substeps for the adjoint.
        capsule_grad: "reference" drops the capsule-normal term of the body
        pose gradient as the reference does; "exact" keeps it.  stride: at
        least this many entries per state plane (the planes of a caller's
        storage sized for more particles than the envs hold now).  capacity:
        size the tables and grid slots for at least this much, so that
        relayout can later move the engine to other envs without new
        buffers."""
        N.require_cuda()
        self.lib = N.load()
        self.device = torch.device(device)
        self.tile_size = int(tile_size)
        assert self.tile_size in (64, 128, 256)
        self.grad = grad
        self._check_specs(specs)
        need = Capacity.of(specs, self.tile_size)
        cap = need if capacity is None else need.union(capacity)
        n_real = max(cap.particles, int(stride))
        self.n_particles = max(32, ((n_real + 31) // 32) * 32)
        self.capacity = Capacity(particles=self.n_particles, blocks=max(cap.blocks, 1), bodies=max(cap.bodies, 1),
                                 tiles=max(cap.tiles, 1), envs=max(cap.envs, 1))
        # grid slots hold capacity.blocks blocks each (their stride), whatever
        # the current layout uses
        self.n_blocks = self.capacity.blocks
        dev = self.device
        f32 = dict(dtype=torch.float32, device=dev)
        i32 = dict(dtype=torch.int32, device=dev)
        C, Np = self.capacity, self.n_particles
        self.envs_t = torch.zeros(C.envs * ctypes.sizeof(N.DexEnv), dtype=torch.uint8, device=dev)
        self.tiles_t = torch.zeros((C.tiles, 2), **i32)
        self.block_env_t = torch.zeros(C.blocks, **i32)
        self.block_xyz_t = torch.zeros(C.blocks, **i32)
        # material planes: mass, vol, mu, lambda, yield stress
        self.mat = torch.zeros((MATERIAL_PLANES, self.n_particles), **f32)
        self.mass, self.vol, self.mly = self.mat[0], self.mat[1], self.mat[2:5]
        self.body_shape = torch.zeros((C.bodies, 8), **f32)
        cells = self.n_blocks * 64
        self.n_grid_slots = K = max(2, int(grid_slots))
        # grids, gradient grids and flags are zeroed by dexmpm_reset below
        self.grid = torch.empty((K, cells, 4), **f32)
        self.vout = torch.empty((K, cells, 4), **f32)
        self.vout_grad = torch.empty((cells, 4), **f32) if grad else None
        self.in_grad = torch.empty((cells, 4), **f32) if grad else None
        self.block_flag = torch.empty((K, self.n_blocks), **i32)
        self.block_list = torch.zeros((K, self.n_blocks), **i32)
        self.block_count = torch.zeros(K, **i32)
        self.done_counter = torch.zeros(1, **i32)
        self.error = torch.zeros(1, **i32)
        self.states = torch.zeros((n_slots, N.STATE_PLANES, Np), **f32)
        self.grid_ctas = int(grid_ctas or sm_count(self.device) * 4)
        b = N.DexBatch()
        b.n_particles, b.n_blocks = Np, self.n_blocks
        b.tile_size, b.grid_ctas = self.tile_size, self.grid_ctas
        assert capsule_grad in ("reference", "exact")
        b.flags = N.FLAG_EXACT_CAPSULE_GRAD if capsule_grad == "exact" else 0
        b.n_slots = K
        b.envs, b.tiles, b.block_env = self.envs_t.data_ptr(), self.tiles_t.data_ptr(), self.block_env_t.data_ptr()
        b.mass, b.vol, b.mu_lam_yield = self.mass.data_ptr(), self.vol.data_ptr(), self.mly.data_ptr()
        b.grid, b.vout = self.grid.data_ptr(), self.vout.data_ptr()
        b.vout_grad = self.vout_grad.data_ptr() if grad else None
        b.in_grad = self.in_grad.data_ptr() if grad else None
        b.block_flag, b.block_list = self.block_flag.data_ptr(), self.block_list.data_ptr()
        b.block_count, b.done_counter = self.block_count.data_ptr(), self.done_counter.data_ptr()
        b.body_shape, b.error = self.body_shape.data_ptr(), self.error.data_ptr()
        b.block_xyz = self.block_xyz_t.data_ptr()
        self.batch = b
        self._bp = ctypes.byref(b)
        self.fslot = 0          # grid slot of the next forward substep (0 or 1)
        self.launches = 0
        self._sortw = None      # scratch of the particle sort, allocated on first use
        self._write_layout(specs, material=True, staged=False)
        N.check(self.lib.dexmpm_reset(self._bp, N.stream_ptr()), "dexmpm_reset")

    @staticmethod
    def _check_specs(specs):
        for s in specs:
            assert all(g % 4 == 0 and g >= 8 for g in s.grid_dim), "grid dims must be multiples of 4"
            if s.nb > N.MAX_BODIES:
                raise N.DexError(f"{s.nb} bodies > {N.MAX_BODIES} per env")

    def _upload(self, dst: torch.Tensor, src: np.ndarray, staged: bool):
        t = torch.from_numpy(np.require(src, requirements=["C", "W"]))
        if staged:
            # through pinned memory, ordered on the current stream: the host
            # does not wait for the device work queued ahead of the copy
            dst.copy_(t.pin_memory(), non_blocking=True)
        else:
            dst.copy_(t)

    def _write_layout(self, specs, material: bool, staged: bool):
        L = plan_layout(specs, self.tile_size)
        self.specs = list(specs)
        self.p_off, self.blk_off, self.body_off = L["p_off"], L["blk_off"], L["body_off"]
        self.n_bodies, self.used_blocks = L["n_bodies"], L["n_blocks"]
        tiles = L["tiles"]
        if len(specs):
            self._upload(self.envs_t[:ctypes.sizeof(N.DexEnv) * len(specs)],
                         np.frombuffer(bytes(L["envs"]), np.uint8), staged)
        if len(tiles):
            self._upload(self.tiles_t[:len(tiles)], tiles, staged)
        if L["n_blocks"]:
            self._upload(self.block_env_t[:L["n_blocks"]], L["block_env"], staged)
            self._upload(self.block_xyz_t[:L["n_blocks"]], L["block_xyz"], staged)
        if self.n_bodies:
            shapes = np.zeros((self.n_bodies, 8), np.float32)
            for e, s in enumerate(self.specs):
                if s.nb:
                    shapes[self.body_off[e]:self.body_off[e] + s.nb, :4] = s.body_tfsr
                    shapes[self.body_off[e]:self.body_off[e] + s.nb, 4:] = s.body_args
            self._upload(self.body_shape[:self.n_bodies], shapes, staged)
        if material:
            mat = np.zeros((MATERIAL_PLANES, L["n_particles"]), np.float32)
            for e, s in enumerate(self.specs):
                o = self.p_off[e]
                mat[0, o:o + s.n] = s.mass
                mat[1, o:o + s.n] = s.vol
                mat[2:5, o:o + s.n] = np.asarray(s.mu_lam_yield, np.float32).T
            if L["n_particles"]:
                self._upload(self.mat[:, :L["n_particles"]], mat, staged)
        b = self.batch
        b.n_envs, b.n_tiles, b.n_bodies = len(self.specs), len(tiles), self.n_bodies

    def fits(self, specs: Sequence[EnvSpec]) -> bool:
        """True when relayout(specs) can keep this engine's buffers."""
        return self.capacity.holds(Capacity.of(specs, self.tile_size))

    def relayout(self, specs: Sequence[EnvSpec], material: bool = True):
        """Move the engine to another set of envs within its capacity: rewrite
        the env, tile and block tables (owner and coordinates of each block),
        the body shapes and (material=True)
        the material planes, on the current stream through pinned staging, so
        that the host does not wait.  The grid slots stay: every slot's active
        blocks are cleared by the launch that consumes it, so a slot left in
        use by the last forward substep is still cleared by the next one.
        CUDA graphs captured before this call hold the old launch shapes and
        must not be replayed after it.  With material=False the caller writes
        mass, vol, mu, lambda, yield stress into mat itself."""
        self._check_specs(specs)
        if not self.fits(specs):
            raise N.DexError(f"layout of {len(specs)} envs exceeds the engine's capacity {self.capacity}")
        self._write_layout(specs, material=material, staged=self.device.type == "cuda")

    # ------------------------------------------------------------ material
    def use_material(self, mat: Optional[torch.Tensor] = None):
        """Material planes (MATERIAL_PLANES, n_particles) the next launches
        read: mass, vol, mu, lambda, yield stress in the particle order of the
        states they step (None: the engine's own, in the specs' order).  The
        pointers are copied into each launch, so CUDA graphs captured after
        this call keep them."""
        m = self.mat if mat is None else mat
        assert m.shape == (MATERIAL_PLANES, self.n_particles) and m.is_contiguous()
        b = self.batch
        b.mass, b.vol, b.mu_lam_yield = m[0].data_ptr(), m[1].data_ptr(), m[2].data_ptr()

    # ------------------------------------------------------ particle order
    def identity_perm(self, n: int = 1) -> torch.Tensor:
        """n permutations of the engine's particles, each the identity."""
        return torch.arange(self.n_particles, dtype=torch.int32, device=self.device).repeat(n, 1)

    def _sort_work(self):
        if self._sortw is None:
            dev, i32 = self.device, torch.int32
            cells = self.n_blocks * 64
            t = {"cell_count": torch.zeros(cells, dtype=i32, device=dev),
                 "cell_start": torch.zeros(cells, dtype=i32, device=dev),
                 "block_total": torch.zeros(self.n_blocks, dtype=i32, device=dev),
                 "block_base": torch.zeros(self.n_blocks, dtype=i32, device=dev),
                 "block_flag": torch.zeros(self.n_blocks, dtype=i32, device=dev),
                 "block_list": torch.zeros(self.n_blocks, dtype=i32, device=dev),
                 "rank": torch.zeros(self.n_particles, dtype=i32, device=dev),
                 "key": torch.zeros(self.n_particles, dtype=i32, device=dev),
                 "partial": torch.zeros(N.sort_partials(self.n_blocks), dtype=i32, device=dev),
                 "counters": torch.zeros(4, dtype=i32, device=dev)}
            w = N.DexSortWork()
            for k, v in t.items():
                setattr(w, k, v.data_ptr())
            self._sortw = (t, w, ctypes.byref(w))
        return self._sortw[2]

    def sort(self, s: torch.Tensor, sorted_s: torch.Tensor, perm: torch.Tensor):
        """Order every env's particles of state slot s by grid block, cell and
        previous index: perm[i] = index in s of the particle that goes to i,
        sorted_s = s gathered by perm.  perm's entries beyond the envs'
        particles are left as they are (start from identity_perm)."""
        assert perm.dtype == torch.int32 and perm.numel() == self.n_particles
        N.check(self.lib.dexmpm_sort(self._bp, self._sort_work(), N.ptr(s), N.ptr(sorted_s), N.ptr(perm),
                                     N.stream_ptr()), "dexmpm_sort")
        self.launches += 7

    def permute(self, perm: torch.Tensor, src: torch.Tensor, dst: torch.Tensor, inverse: bool = False):
        """dst = src gathered by perm (dst[.., i] = src[.., perm[i]]), or with
        inverse scattered back (dst[.., perm[i]] = src[.., i]); planes of
        n_particles 32-bit values (floats or int32)."""
        n = self.n_particles
        assert src.shape[-1] == n and dst.shape == src.shape and src.is_contiguous() and dst.is_contiguous()
        assert src.element_size() == 4 and dst.element_size() == 4
        planes = src.numel() // n
        N.check(self.lib.dexmpm_permute(N.ptr(perm), N.ptr(src), N.ptr(dst), n, planes, int(inverse),
                                        N.stream_ptr()), "dexmpm_permute")
        self.launches += 1

    # ----------------------------------------------------------- state I/O
    def new_slots(self, n: int, zero: bool = True) -> torch.Tensor:
        """n state slots; zero=False leaves them uninitialised (for slots every
        particle's planes are written into before they are read)."""
        f = torch.zeros if zero else torch.empty
        return f((n, N.STATE_PLANES, self.n_particles), dtype=torch.float32, device=self.device)

    def new_tape(self, n: int, zero: bool = True) -> torch.Tensor:
        """n tape slots (the per-particle SVD and stress a recomputed forward
        P2G stores for its adjoint)."""
        f = torch.zeros if zero else torch.empty
        return f((n, TAPE_PLANES, self.n_particles), dtype=torch.float32, device=self.device)

    def pack_state(self, per_env: Sequence[dict]) -> torch.Tensor:
        """Host dicts (x, v (n,3); F, C (n,3,3)) -> one device slot (24, Np)."""
        buf = np.zeros((N.STATE_PLANES, self.n_particles), np.float32)
        for e, st in enumerate(per_env):
            o, n = self.p_off[e], self.specs[e].n
            buf[0:3, o:o + n] = np.asarray(st["x"], np.float32).T
            buf[3:6, o:o + n] = np.asarray(st["v"], np.float32).T
            buf[6:15, o:o + n] = np.asarray(st["F"], np.float32).reshape(n, 9).T
            buf[15:24, o:o + n] = np.asarray(st["C"], np.float32).reshape(n, 9).T
        return torch.from_numpy(buf).to(self.device)

    def unpack_state(self, slot: torch.Tensor) -> List[dict]:
        buf = slot.detach().cpu().numpy()
        out = []
        for e, s in enumerate(self.specs):
            o, n = self.p_off[e], s.n
            out.append({"x": buf[0:3, o:o + n].T.copy(), "v": buf[3:6, o:o + n].T.copy(),
                        "F": buf[6:15, o:o + n].T.reshape(n, 3, 3).copy(),
                        "C": buf[15:24, o:o + n].T.reshape(n, 3, 3).copy()})
        return out

    def pack_poses(self, per_env_pos: Sequence[np.ndarray], per_env_rot: Sequence[np.ndarray]) -> np.ndarray:
        """Per-env (..., nb, 3)/(..., nb, 4) -> (..., n_bodies, 8) host array."""
        lead = np.asarray(per_env_pos[0]).shape[:-2]
        out = np.zeros(lead + (max(self.n_bodies, 1), 8), np.float32)
        for e, s in enumerate(self.specs):
            if s.nb:
                o = self.body_off[e]
                out[..., o:o + s.nb, :] = pack_poses(np.asarray(per_env_pos[e]), np.asarray(per_env_rot[e]))
        return out

    # ------------------------------------------------------------ kernels
    def substep(self, s: torch.Tensor, s_next: torch.Tensor, pose: torch.Tensor, next_pose: torch.Tensor,
                slot: Optional[int] = None, tape: Optional[torch.Tensor] = None):
        """One forward substep (P2G, grid update, G2P) of every env.  Without
        `slot` it uses the forward slot pair (alternating, each clearing the
        other); with `slot` (>= 2) it fills that grid slot and keeps it for the
        adjoint of this substep.  `tape` (a slot of new_tape) receives the SVD
        and stress of every particle for that adjoint."""
        if slot is None:
            slot, clear = self.fslot, self.fslot ^ 1
            self.fslot ^= 1
        else:
            assert 2 <= slot < self.n_grid_slots
            clear = -1
        N.check(self.lib.dexmpm_substep(self._bp, slot, clear, N.ptr(s), N.ptr(s_next), N.ptr(pose),
                                        N.ptr(next_pose), N.ptr(tape), N.stream_ptr()), "dexmpm_substep")
        self.launches += 3
        return slot

    def run_substeps(self, sts: Sequence[torch.Tensor], poses: torch.Tensor, kept: bool = False,
                     tapes: Optional[torch.Tensor] = None, slot_base: int = 2):
        """T = len(sts) - 1 forward substeps from sts[0] to sts[T] (sts[t], 0 < t
        < T, hold the intermediate states; sts[t] and sts[t + 2] may be one
        buffer), with body poses poses[0..T].  The G2P of every substep but
        the last is fused with the next substep's P2G.  Slots: the forward
        pair (kept=False) or slot slot_base + t kept for the adjoint of substep
        t (kept=True), with tapes[t] written when given."""
        T = len(sts) - 1
        if T < 1:
            return
        L, bp, sp = self.lib, self._bp, N.stream_ptr()

        def take(t):
            if kept:
                assert 2 <= slot_base and slot_base + t < self.n_grid_slots
                return slot_base + t, -1
            slot = self.fslot
            self.fslot ^= 1
            return slot, slot ^ 1

        def tape(t):
            return N.ptr(tapes[t]) if tapes is not None else None

        slot, clear = take(0)
        N.check(L.dexmpm_p2g(bp, slot, N.ptr(sts[0]), N.ptr(sts[1]), tape(0), sp), "dexmpm_p2g")
        N.check(L.dexmpm_grid_op(bp, slot, clear, N.ptr(poses[0]), N.ptr(poses[1]), sp), "dexmpm_grid_op")
        for t in range(T - 1):
            nslot, clear = take(t + 1)
            N.check(L.dexmpm_g2p2g(bp, slot, nslot, N.ptr(sts[t]), N.ptr(sts[t + 1]), N.ptr(sts[t + 2]), tape(t + 1),
                                   sp), "dexmpm_g2p2g")
            N.check(L.dexmpm_grid_op(bp, nslot, clear, N.ptr(poses[t + 1]), N.ptr(poses[t + 2]), sp),
                    "dexmpm_grid_op")
            slot = nslot
        N.check(L.dexmpm_g2p(bp, slot, N.ptr(sts[T - 1]), N.ptr(sts[T]), sp), "dexmpm_g2p")
        self.launches += 2 * T + 1

    def substep_grad(self, s, s_next, g_next, g, pose, next_pose, bgrad, next_bgrad, slot: Optional[int] = None,
                     tape: Optional[torch.Tensor] = None):
        """Adjoint of one substep: G2P, grid and P2G adjoints.  With `slot` the
        grid slot left by that substep's forward is used (and cleared);
        without, P2G and the grid update are recomputed from s first.  With
        `tape` (written by that forward) the SVD is read, not recomputed.
        g (gradient of s) is overwritten."""
        assert self.grad, "engine built without gradient buffers"
        sp = N.stream_ptr()
        if slot is None:
            slot, clear = self.fslot, self.fslot ^ 1
            self.fslot ^= 1
            N.check(self.lib.dexmpm_p2g(self._bp, slot, N.ptr(s), None, None, sp), "dexmpm_p2g")
            tape = None
            N.check(self.lib.dexmpm_grid_op(self._bp, slot, clear, N.ptr(pose), N.ptr(next_pose), sp),
                    "dexmpm_grid_op")
            self.launches += 2
        N.check(self.lib.dexmpm_substep_grad(self._bp, slot, N.ptr(s), N.ptr(s_next), N.ptr(g_next), N.ptr(g),
                                             N.ptr(pose), N.ptr(next_pose), N.ptr(bgrad), N.ptr(next_bgrad),
                                             N.ptr(tape), sp),
                "dexmpm_substep_grad")
        self.launches += 3

    def run_adjoint(self, sts: Sequence[torch.Tensor], g_next: torch.Tensor, g: torch.Tensor, poses: torch.Tensor,
                    bgrad: torch.Tensor, tapes: Optional[torch.Tensor] = None, slot_base: int = 2) -> torch.Tensor:
        """Adjoint of the T = len(sts) - 1 substeps that run_substeps(kept=True)
        ran from sts[0] (grid slots slot_base..slot_base+T-1, tapes[t] when given), from the
        gradient of sts[T] in g_next; g is scratch of the same shape.  The P2G
        adjoint of every substep but the first is fused with the G2P adjoint
        of the substep before it.  Returns the buffer (g_next or g) that holds
        the gradient of sts[0]; body-pose gradients of poses[t] are added to
        bgrad[t].  Clears the slots."""
        assert self.grad, "engine built without gradient buffers"
        T = len(sts) - 1
        assert T >= 1 and 2 <= slot_base and slot_base + T <= self.n_grid_slots
        L, bp, sp = self.lib, self._bp, N.stream_ptr()

        def tape(t):
            return N.ptr(tapes[t]) if tapes is not None else None

        b0 = slot_base
        s = T - 1
        N.check(L.dexmpm_g2p_grad(bp, b0 + s, N.ptr(sts[s]), N.ptr(sts[s + 1]), N.ptr(g_next), N.ptr(g), sp),
                "dexmpm_g2p_grad")
        for s in range(T - 1, -1, -1):
            N.check(L.dexmpm_grid_op_grad(bp, b0 + s, N.ptr(poses[s]), N.ptr(poses[s + 1]), N.ptr(bgrad[s]),
                                          N.ptr(bgrad[s + 1]), sp), "dexmpm_grid_op_grad")
            if s > 0:
                # gradients: of state s + 1 in g_next, of state s in g; the x
                # gradient of state s - 1 goes to g_next
                N.check(L.dexmpm_p2g_g2p_grad(bp, b0 + s, b0 + s - 1, N.ptr(sts[s]), N.ptr(sts[s - 1]),
                                              N.ptr(g_next), N.ptr(g), N.ptr(g_next), tape(s), sp),
                        "dexmpm_p2g_g2p_grad")
            else:
                N.check(L.dexmpm_p2g_grad(bp, b0, N.ptr(sts[0]), N.ptr(g_next), N.ptr(g), tape(0), sp),
                        "dexmpm_p2g_grad")
            g_next, g = g, g_next
        self.launches += 2 * T + 1
        return g_next

    def clear_slots(self, first: int, last: int):
        """Make grid slots [first, last) clean (their adjoint will not run)."""
        N.check(self.lib.dexmpm_clear_slots(self._bp, int(first), int(last), N.stream_ptr()), "dexmpm_clear_slots")
        self.launches += 1

    def retune(self, tile_size: int, grid_ctas: int):
        """Change the particle tile size and the persistent grid-kernel CTA
        count (launch shape only; no buffer changes)."""
        assert tile_size in (64, 128, 256) and grid_ctas > 0
        tiles = plan_layout(self.specs, tile_size)["tiles"]
        self.tile_size, self.grid_ctas = int(tile_size), int(grid_ctas)
        if len(tiles) > self.tiles_t.shape[0]:
            self.tiles_t = torch.zeros((len(tiles), 2), dtype=torch.int32, device=self.device)
            self.capacity = Capacity(**{**self.capacity.__dict__, "tiles": len(tiles)})
        if len(tiles):
            self.tiles_t[:len(tiles)].copy_(torch.from_numpy(tiles))
        b = self.batch
        b.tiles, b.n_tiles, b.tile_size, b.grid_ctas = self.tiles_t.data_ptr(), len(tiles), self.tile_size, \
            self.grid_ctas

    def error_word(self) -> int:
        out = ctypes.c_int32(0)
        N.check(self.lib.dexmpm_get_error(self._bp, ctypes.byref(out), N.stream_ptr()), "dexmpm_get_error")
        return int(out.value)

    def active_blocks(self, slot: int) -> int:
        return int(self.block_count[slot].item())

    def grid_mass(self, slot: int) -> float:
        return float(self.grid[slot, :, 3].double().sum())


class Rollout:
    """Env steps of T substeps over a BatchEngine, with per-env-step
    checkpoints (grad mode) and substep recomputation in the backward pass.
    When the engine has T + 2 grid slots, the recomputed substeps keep their
    grids and the adjoint reads them; otherwise the adjoint recomputes P2G and
    the grid update per substep.  With kept grids, the forward pass runs its
    last env step the way the backward would recompute it (kept slots, tape),
    so the backward of that env step needs no recompute.  With 2 T + 2 grid
    slots (and `overlap`), the backward keeps two sets of slots, tapes and
    state rings and recomputes env step k - 1 on a second stream while the
    adjoint of env step k runs.  Each env step's forward, recompute and
    adjoint are captured as CUDA graphs on first use and replayed afterwards.

    Particle order (`sort_every` > 0): at the start of every sort_every-th
    env step the particles are re-ordered on the device by grid cell
    (BatchEngine.sort) -- the first from the caller's order -- so that the
    scatters pre-reduce well whatever order the caller hands over and however
    the particles drift.  Checkpoint k is stored in env step k's order with
    that order's material; the end state of an env step followed by a sort
    goes to a scratch slot first.  The backward maps the gradient of each
    sorted checkpoint back through the permutation.  forward() takes and
    returns states in the caller's order, backward() takes and returns
    gradients in it; `order(k)` gives the caller's index of every particle of
    checkpoint k."""

    def __init__(self, engine: BatchEngine, substeps: int, env_steps: int, use_graphs: bool = True,
                 overlap: bool = True, sort_every: int = 1):
        self.E = engine
        self.T, self.S = int(substeps), int(env_steps)
        self.use_graphs = use_graphs
        dev = engine.device
        nb = max(engine.n_bodies, 1)
        self.poses = torch.zeros((self.S * self.T + 1, nb, 8), dtype=torch.float32, device=dev)
        self.keep_grids = engine.n_grid_slots >= self.T + 2
        self.overlap = bool(overlap) and engine.grad and engine.n_grid_slots >= 2 * self.T + 2
        self.sort_every = max(0, int(sort_every))
        self.tape = None
        if engine.grad:
            self.ckpt = engine.new_slots(self.S + 1)
            self.ring = engine.new_slots(self.T + 1)
            self.gbuf = engine.new_slots(2)
            if self.keep_grids:
                self.tape = engine.new_tape(self.T)
            self.bgrad = torch.zeros((self.S * self.T + 1, nb, 8), dtype=torch.float32, device=dev)
        else:
            self.ckpt = engine.new_slots(2)
            self.ring = engine.new_slots(2)
        # slot sets of the overlapped backward: (first kept grid slot, state ring, tape)
        self._sets = [(2, self.ring, self.tape)]
        if self.overlap:
            self._sets.append((2 + self.T, engine.new_slots(self.T + 1), engine.new_tape(self.T)))
            self._side = torch.cuda.Stream(device=dev)
        self._fwd_graphs, self._bwd_graphs = {}, {}
        self._kept_live = False  # slots 2..T+1 and the tape hold the last env step's forward
        # particle order: sorted boundaries, their permutations, the material
        # and the caller's indices in each sorted order
        self._sorted = [k for k in range(self.S) if self.sort_every and k % self.sort_every == 0]
        if self._sorted:
            m = len(self._sorted)
            self.src = engine.new_slots(1)[0]    # the caller's initial state
            self.tail = engine.new_slots(1)[0]   # end of an env step that a sort follows
            self.out = engine.new_slots(1)[0]    # the final state in the caller's order
            self.perm = engine.identity_perm(m)
            self.orders = engine.identity_perm(m)
            self.mats = torch.zeros((m,) + tuple(engine.mat.shape), dtype=torch.float32, device=dev)

    # ------------------------------------------------------- particle order
    def _sidx(self, k: int) -> int:
        """Index (into perm, orders, mats) of the last sorted boundary <= k, or -1."""
        j = -1
        for i, b in enumerate(self._sorted):
            if b <= k:
                j = i
        return j

    def material(self, k: int) -> torch.Tensor:
        """Material planes in the particle order of env step k."""
        j = self._sidx(k)
        return self.E.mat if j < 0 else self.mats[j]

    def order(self, k: int) -> Optional[torch.Tensor]:
        """Caller's index of each particle of checkpoint k (k = S: the final
        state); None when the order is the caller's."""
        j = self._sidx(min(k, self.S - 1))
        return None if j < 0 else self.orders[j]

    def _sort_boundary(self, k: int, pre: torch.Tensor):
        """Sorted boundary k: checkpoint k = pre (the end of env step k - 1,
        or the caller's state) in the new order, with its permutation, the
        material in that order and the caller's indices."""
        E, j = self.E, self._sorted.index(k)
        E.sort(pre, self._ckpt(k), self.perm[j])
        E.permute(self.perm[j], self.E.mat if j == 0 else self.mats[j - 1], self.mats[j])
        if j == 0:
            self.orders[0].copy_(self.perm[0])
        else:
            E.permute(self.perm[j], self.orders[j - 1], self.orders[j])

    def _end(self, k: int) -> torch.Tensor:
        """Where the forward of env step k leaves its final state."""
        return self.tail if (k + 1 < self.S and (k + 1) in self._sorted) else self._ckpt(k + 1)

    # ------------------------------------------------------------- forward
    def _ckpt(self, k):
        return self.ckpt[k] if self.E.grad else self.ckpt[k % 2]

    def _forward_step(self, k: int):
        """Env step k: (sort) ckpt[k] -> its end through T substeps (two ring
        buffers for the intermediate states)."""
        T = self.T
        if k in self._sorted:
            self._sort_boundary(k, self.src if k == 0 else self.tail)
        self.E.use_material(self.material(k))
        sts = [self._ckpt(k)] + [self.ring[t % 2] for t in range(1, T)] + [self._end(k)]
        self.E.run_substeps(sts, self.poses[k * T:k * T + T + 1])

    def _forward_step_kept(self, k: int):
        """Env step k (the last) as the backward recomputes it: states into
        the ring, grids kept in slots 2..T+1, the tape written; result in
        ckpt[k+1]."""
        T = self.T
        if k in self._sorted:
            self._sort_boundary(k, self.src if k == 0 else self.tail)
        self.E.use_material(self.material(k))
        sts = [self.ckpt[k]] + [self.ring[t] for t in range(1, T)] + [self.ckpt[k + 1]]
        self.E.run_substeps(sts, self.poses[k * T:k * T + T + 1], kept=True, tapes=self.tape)

    def forward_step(self, k: int):
        self._run(self._fwd_graphs, k, self._forward_step)

    def sort_initial(self, state0: torch.Tensor):
        """Checkpoint 0 and its material from the caller's state0 (eager),
        e.g. to tune launch shapes on the order the rollout will run."""
        if 0 in self._sorted:
            self.src.copy_(state0)
            self._sort_boundary(0, self.src)
        else:
            self._ckpt(0).copy_(state0)
        self.E.use_material(self.material(0))

    def forward(self, state0: Optional[torch.Tensor] = None, keep_last: bool = True):
        """Run the S env steps from state0 (the caller's order; None: the
        state of the previous call).  keep_last (gradient engines with kept
        grids): run the last env step as the backward would recompute it, for
        a backward that follows; pass False for forward-only use.  Returns
        the final state in the caller's order."""
        if state0 is not None:
            (self.src if 0 in self._sorted else self._ckpt(0)).copy_(state0)
        keep = keep_last and self.E.grad and self.keep_grids and self.S > 0
        if self._kept_live:
            self.E.clear_slots(2, 2 + self.T)  # a kept forward whose backward was not taken
            self._kept_live = False
        for k in range(self.S - 1 if keep else self.S):
            self.forward_step(k)
        if keep:
            k = self.S - 1
            run_graph(self.E, self._fwd_graphs, ("kept", k), lambda: self._forward_step_kept(k), self.use_graphs)
            self._kept_live = True
        return self._to_caller(self._ckpt(self.S), self.S, self.out if self._sorted else None)

    def _to_caller(self, st: torch.Tensor, k: int, out: Optional[torch.Tensor]):
        o = self.order(k)
        if o is None:
            return st
        self.E.permute(o, st, out, inverse=True)
        return out

    def stored(self, k: int) -> torch.Tensor:
        """Checkpoint k as stored: in env step k's particle order."""
        return self._ckpt(k)

    def state(self, k: int) -> torch.Tensor:
        """Checkpoint k (the state at the start of env step k; k = S is the
        final state) in the caller's order.  Without gradients only the last
        two are kept."""
        if not self.E.grad:
            assert k >= self.S - 1, "forward-only rollouts keep the last two checkpoints"
        st = self._ckpt(k)
        return self._to_caller(st, k, torch.empty_like(st))

    # ------------------------------------------------------------ backward
    def _end_for_adjoint(self, k: int, ring) -> torch.Tensor:
        """The end state of env step k in its own order: the checkpoint after
        it, unless a sort followed (then the recompute left it in ring[T])."""
        return ring[self.T] if (k + 1 < self.S and (k + 1) in self._sorted) else self.ckpt[k + 1]

    def _unsort_grad(self, k: int):
        """Gradient of checkpoint k (gbuf[1]) -> gradient of what was sorted
        into it (the end of env step k - 1, or the caller's state)."""
        if k in self._sorted:
            j = self._sorted.index(k)
            self.E.permute(self.perm[j], self.gbuf[1], self.gbuf[0], inverse=True)
            self.gbuf[1].copy_(self.gbuf[0])

    def _backward_step(self, k: int, recompute: bool = True):
        """Gradient of ckpt[k] from the gradient of the end of env step k (in
        gbuf[1]): recompute the T states of env step k into the ring (keeping
        each substep's grid slot when there are enough slots) unless the
        forward kept them, then run the adjoint substeps in reverse; then back
        through the sort of boundary k.  Result in gbuf[1]."""
        T, E = self.T, self.E
        E.use_material(self.material(k))
        if recompute and self.keep_grids:
            sts = [self.ckpt[k]] + [self.ring[t] for t in range(1, T + 1)]
            E.run_substeps(sts, self.poses[k * T:k * T + T + 1], kept=True, tapes=self.tape)
        elif recompute:
            src = self.ckpt[k]
            for s in range(T):
                t = k * T + s
                E.substep(src, self.ring[s + 1], self.poses[t], self.poses[t + 1])
                src = self.ring[s + 1]
        end = self._end_for_adjoint(k, self.ring)
        if self.keep_grids:
            sts = [self.ckpt[k]] + [self.ring[s] for s in range(1, T)] + [end]
            out = E.run_adjoint(sts, self.gbuf[1], self.gbuf[0], self.poses[k * T:k * T + T + 1],
                                self.bgrad[k * T:k * T + T + 1], tapes=self.tape)
            if out is not self.gbuf[1]:
                self.gbuf[1].copy_(out)
            self._unsort_grad(k)
            return
        g_next, g = self.gbuf[1], self.gbuf[0]
        for s in range(T - 1, -1, -1):
            t = k * T + s
            cur = self.ckpt[k] if s == 0 else self.ring[s]
            nxt = end if s == T - 1 else self.ring[s + 1]
            E.substep_grad(cur, nxt, g_next, g, self.poses[t], self.poses[t + 1], self.bgrad[t],
                           self.bgrad[t + 1], tape=self._tape(s))
            g_next, g = g, g_next
        if T % 2 == 1:
            self.gbuf[1].copy_(self.gbuf[0])
        self._unsort_grad(k)

    def _tape(self, s):
        return None if self.tape is None else self.tape[s]

    def backward_step(self, k: int):
        if self._kept_live and k == self.S - 1:
            run_graph(self.E, self._bwd_graphs, ("kept", k), lambda: self._backward_step(k, recompute=False),
                      self.use_graphs)
            self._kept_live = False  # the adjoint cleared the kept slots
        else:
            if self._kept_live:
                self.E.clear_slots(2, 2 + self.T)
                self._kept_live = False
            self._run(self._bwd_graphs, k, self._backward_step)

    def backward(self, g_final: torch.Tensor, on_boundary=None):
        """Back-propagate g_final (gradient of the final state, caller's
        order).  on_boundary(k, g) may add loss gradients of the state at
        boundary k in place; g is in the particle order of env step k - 1
        (order(k - 1) maps it to the caller's; the caller's order for k = 0).
        Returns the gradient of the initial state in the caller's order;
        body-pose gradients land in bgrad."""
        assert self.E.grad
        self.bgrad.zero_()
        o = self.order(self.S)
        if o is None:
            self.gbuf[1].copy_(g_final)
        else:
            self.E.permute(o, g_final.contiguous(), self.gbuf[1])
        if self.overlap and self.S > 1:
            self._backward_overlapped(on_boundary)
            return self.gbuf[1]
        for k in range(self.S - 1, -1, -1):
            self.backward_step(k)
            if on_boundary is not None:
                on_boundary(k, self.gbuf[1])
        return self.gbuf[1]

    # ------------------------------------------------- overlapped backward
    def _set_of(self, k: int):
        """Slot set of env step k: the last env step uses set 0 (where the
        kept forward left it), earlier ones alternate."""
        return self._sets[(self.S - 1 - k) % 2]

    def _recompute(self, k: int):
        """Env step k recomputed from ckpt[k] into its slot set (states in the
        set's ring, grids kept, tape written)."""
        T = self.T
        base, ring, tape = self._set_of(k)
        self.E.use_material(self.material(k))
        sts = [self.ckpt[k]] + [ring[t] for t in range(1, T + 1)]
        self.E.run_substeps(sts, self.poses[k * T:k * T + T + 1], kept=True, tapes=tape, slot_base=base)

    def _adjoint(self, k: int):
        """Adjoint of env step k from its slot set; gradient of the end of
        env step k in gbuf[1] in, gradient of what precedes ckpt[k] (back
        through the sort of boundary k) in gbuf[1] out."""
        T = self.T
        base, ring, tape = self._set_of(k)
        self.E.use_material(self.material(k))
        sts = [self.ckpt[k]] + [ring[t] for t in range(1, T)] + [self._end_for_adjoint(k, ring)]
        out = self.E.run_adjoint(sts, self.gbuf[1], self.gbuf[0], self.poses[k * T:k * T + T + 1],
                                 self.bgrad[k * T:k * T + T + 1], tapes=tape, slot_base=base)
        if out is not self.gbuf[1]:
            self.gbuf[1].copy_(out)
        self._unsort_grad(k)

    def _backward_overlapped(self, on_boundary):
        """Env steps S-1 .. 0: the adjoint of env step k on the current stream
        while env step k - 1 is recomputed into the other slot set on a side
        stream.  The recompute of k - 1 starts after everything issued before
        the adjoint of k (so the adjoint of k + 1, the last user of that set,
        is done); the adjoint of k waits for the recompute of k."""
        main, side = torch.cuda.current_stream(), self._side
        k = self.S - 1
        if self._kept_live:
            self._kept_live = False  # the adjoint below consumes the kept slots
        else:
            run_graph(self.E, self._bwd_graphs, ("rec", k), lambda: self._recompute(k), self.use_graphs)
        ready = None
        for k in range(self.S - 1, -1, -1):
            nxt = None
            if k > 0:
                side.wait_stream(main)
                with torch.cuda.stream(side):
                    run_graph(self.E, self._bwd_graphs, ("rec", k - 1), lambda: self._recompute(k - 1),
                              self.use_graphs)
                nxt = torch.cuda.Event()
                nxt.record(side)
            if ready is not None:
                main.wait_event(ready)
            run_graph(self.E, self._bwd_graphs, ("adj", k), lambda: self._adjoint(k), self.use_graphs)
            if on_boundary is not None:
                on_boundary(k, self.gbuf[1])
            ready = nxt
        main.wait_stream(side)

    # -------------------------------------------------------------- graphs
    def _run(self, cache, k, fn):
        run_graph(self.E, cache, k, lambda: fn(k), self.use_graphs)


def run_graph(E: BatchEngine, cache: dict, key, fn, use_graphs: bool = True):
    """Run fn (a fixed launch sequence) through a CUDA graph cached under
    (key, forward slot parity).  The first call runs fn eagerly -- that is
    the call's work -- and captures it; later calls replay it.  The host-side
    slot parity and launch counter advance as the eager run advanced them."""
    if not use_graphs:
        fn()
        return
    entry = cache.get((key, E.fslot))
    if entry is None:
        f0, l0 = E.fslot, E.launches
        fn()
        torch.cuda.synchronize()
        df, dl = E.fslot ^ f0, E.launches - l0
        f1 = E.fslot
        g = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        # no garbage collection during the capture: a finalizer that calls
        # CUDA (an event or graph of an object going out of scope) would
        # invalidate it
        enabled = gc.isenabled()
        gc.disable()
        try:
            with torch.cuda.stream(side):
                g.capture_begin()
                fn()
                g.capture_end()
        finally:
            if enabled:
                gc.enable()
        torch.cuda.current_stream().wait_stream(side)
        E.fslot, E.launches = f1, l0 + dl
        cache[(key, f1)] = (g, df, dl)
        return
    g, df, dl = entry
    g.replay()
    E.fslot ^= df
    E.launches += dl
