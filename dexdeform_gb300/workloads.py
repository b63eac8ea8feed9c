"""Seeded synthetic workloads for the MLS-MPM substep.

The reference's demonstrations and env assets are not part of this build, so
every workload is generated here from a seed with the shapes, sizes and value
ranges of the benchmark configurations:

* ``plain_env``   -- one env, 64^3 grid, 5,000 particles in a 0.2 cube, 22
  random-walk capsules (the plain forward configuration).
* ``batch_envs``  -- 64 envs with log-uniform particle counts in
  [2,000, 30,000], cube or ellipsoid objects, yield stress U[30, 80].
* ``large_env``   -- 128^3 grid, 300,000 particles in two stacked cubes with
  yield stresses 40 and 120, 22 capsules plus a palm box.

Material defaults follow mpm/simulator.py:152-170 and mpm/cuda_env.py:88
(E=5e3, nu=0.2, softness 666, body friction 0.9).  Particle mass equals particle
volume (density 1), the object volume split evenly over its particles.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

SOFTNESS = 666.0      # mpm/cuda_env.py:88
BODY_FRICTION = 0.9   # mpm/cuda_env.py:40
GRAVITY_SCALE = 30.0  # mpm/simulator.py:385


def lame(E=5e3, nu=0.2):
    """mpm/simulator.py:211-212"""
    return E / (2 * (1 + nu)), E * nu / ((1 + nu) * (1 - 2 * nu))


@dataclass
class Env:
    """One environment: particle state, material, bodies and per-substep poses."""
    grid_dim: tuple
    dx: float
    dt: float
    gravity: tuple
    ground_friction: float
    x: np.ndarray            # (n,3) float32
    v: np.ndarray            # (n,3)
    F: np.ndarray            # (n,3,3)
    C: np.ndarray            # (n,3,3)
    mass: np.ndarray         # (n,)
    vol: np.ndarray          # (n,)
    mu_lam_yield: np.ndarray  # (n,3)
    body_tfsr: np.ndarray    # (nb,4): type, friction, softness, round
    body_args: np.ndarray    # (nb,4)
    poses: np.ndarray        # (T+1, nb, 7): pos xyz, quat wxyz per substep boundary
    name: str = ""

    @property
    def n(self):
        return int(self.x.shape[0])

    @property
    def nb(self):
        return int(self.body_args.shape[0])

    def state(self):
        return {"x": self.x.copy(), "v": self.v.copy(), "F": self.F.copy(), "C": self.C.copy()}

    def pose(self, t):
        p = self.poses[t]
        return p[:, :3].copy(), p[:, 3:].copy()


# ------------------------------------------------------------------ shapes
def sample_cube(rng, n, center, side):
    c = np.asarray(center, np.float64)
    s = np.broadcast_to(np.asarray(side, np.float64), (3,))
    return (c + (rng.random((n, 3)) - 0.5) * s).astype(np.float32), float(np.prod(s))


def sample_ellipsoid(rng, n, center, semi):
    semi = np.asarray(semi, np.float64)
    out = np.empty((0, 3))
    while out.shape[0] < n:
        p = rng.random((2 * n, 3)) * 2 - 1
        p = p[(p * p).sum(1) <= 1.0]
        out = np.concatenate([out, p], 0)
    vol = 4.0 / 3.0 * math.pi * float(np.prod(semi))
    return (np.asarray(center) + out[:n] * semi).astype(np.float32), vol


def cell_sort(x, dx, block=4):
    """Order particles by (4^3 block, cell) so that neighbouring particles are
    adjacent in memory; returns the permutation."""
    c = np.floor(x / dx - 0.5).astype(np.int64)
    b = c // block
    key = (((b[:, 0] * 4096 + b[:, 1]) * 4096 + b[:, 2]) * 64
           + ((c[:, 0] % block) * block + (c[:, 1] % block)) * block + (c[:, 2] % block))
    return np.argsort(key, kind="stable")


# ------------------------------------------------------------------ bodies
def capsules(rng, nb, r_range=(0.008, 0.02), h_range=(0.02, 0.05)):
    tfsr = np.zeros((nb, 4), np.float32)
    tfsr[:, 0] = 1.0                      # capsule
    tfsr[:, 1] = BODY_FRICTION
    tfsr[:, 2] = SOFTNESS
    args = np.zeros((nb, 4), np.float32)
    args[:, 0] = rng.uniform(*r_range, nb)
    args[:, 1] = rng.uniform(*h_range, nb)
    return tfsr, args


def _qmul(a, b):
    w1, x1, y1, z1 = a[..., 0], a[..., 1], a[..., 2], a[..., 3]
    w2, x2, y2, z2 = b[..., 0], b[..., 1], b[..., 2], b[..., 3]
    return np.stack([w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2, w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2,
                     w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2, w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2], -1)


def random_walk_poses(rng, nb, steps, dt, lo, hi, vmax=0.5, wmax=4.0, v0=(0.0, -0.3, 0.0)):
    """Seeded random-walk rigid poses, (steps+1, nb, 7).  Linear speed is
    capped at ``vmax`` and angular speed at ``wmax`` rad/s."""
    pos = rng.uniform(lo, hi, (nb, 3))
    q = rng.normal(size=(nb, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    vel = np.asarray(v0, np.float64) + rng.normal(scale=0.1, size=(nb, 3))
    ang = rng.normal(scale=1.0, size=(nb, 3))
    out = np.zeros((steps + 1, nb, 7), np.float64)
    out[0, :, :3], out[0, :, 3:] = pos, q
    for t in range(steps):
        vel += rng.normal(scale=0.05, size=(nb, 3))
        sp = np.linalg.norm(vel, axis=1, keepdims=True)
        vel *= np.minimum(1.0, vmax / np.maximum(sp, 1e-12))
        ang += rng.normal(scale=0.2, size=(nb, 3))
        wn = np.linalg.norm(ang, axis=1, keepdims=True)
        ang *= np.minimum(1.0, wmax / np.maximum(wn, 1e-12))
        pos = pos + vel * dt
        th = np.linalg.norm(ang, axis=1, keepdims=True) * dt
        axis = ang / np.maximum(np.linalg.norm(ang, axis=1, keepdims=True), 1e-12)
        dq = np.concatenate([np.cos(th / 2), axis * np.sin(th / 2)], 1)
        q = _qmul(q, dq)
        q /= np.linalg.norm(q, axis=1, keepdims=True)
        out[t + 1, :, :3], out[t + 1, :, 3:] = pos, q
    return out.astype(np.float32)


# ------------------------------------------------------------------- envs
def make_env(seed, n, shape="cube", grid=64, dt=5e-5, yield_stress=50.0, center=None,
             extent=0.2, nb=22, steps=50, ground_friction=0.9, E=5e3, nu=0.2,
             sort=True, name="") -> Env:
    rng = np.random.default_rng(seed)
    dx = 1.0 / grid
    if center is None:
        center = (0.5, 0.05 + (extent / 2 if shape == "cube" else 0.06), 0.5)
    if shape == "cube":
        x, volume = sample_cube(rng, n, center, extent)
        top = center[1] + extent / 2
    else:
        semi = np.broadcast_to(np.asarray(extent, np.float64), (3,))
        x, volume = sample_ellipsoid(rng, n, center, semi)
        top = center[1] + float(semi[1])
    if sort:
        x = x[cell_sort(x, dx)]
    mu, lam = lame(E, nu)
    pv = volume / max(n, 1)
    tfsr, args = capsules(rng, nb)
    c = np.asarray(center)
    poses = random_walk_poses(rng, nb, steps, dt, lo=(c[0] - 0.12, top - 0.02, c[2] - 0.12),
                              hi=(c[0] + 0.12, top + 0.06, c[2] + 0.12))
    eye = np.broadcast_to(np.eye(3, dtype=np.float32), (n, 3, 3)).copy()
    return Env(grid_dim=(grid, grid, grid), dx=dx, dt=dt, gravity=(0.0, -1.0 * GRAVITY_SCALE, 0.0),
               ground_friction=ground_friction, x=x, v=np.zeros((n, 3), np.float32), F=eye,
               C=np.zeros((n, 3, 3), np.float32), mass=np.full(n, pv, np.float32),
               vol=np.full(n, pv, np.float32),
               mu_lam_yield=np.tile(np.float32([mu, lam, yield_stress]), (n, 1)),
               body_tfsr=tfsr, body_args=args, poses=poses, name=name)


def plain_env(seed=0, steps=50, n=5000):
    """Plain forward: 64^3, 5,000 particles in a 0.2 cube centred (0.5,0.15,0.5)."""
    return make_env(seed, n, "cube", grid=64, center=(0.5, 0.15, 0.5), extent=0.2, steps=steps,
                    name="plain-fwd-64^3-5k")


def batch_envs(seed=0, n_envs=64, steps=50, n_lo=2000, n_hi=30000, grid=64, sort=True):
    """Batching: log-uniform particle counts, cube or ellipsoid, yield U[30,80].
    sort=False keeps each object's particles in sampling order (random
    positions, as an object sampler hands them over)."""
    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(math.log(n_lo), math.log(n_hi), n_envs)).astype(int)
    shapes = rng.integers(0, 2, n_envs)
    ys = rng.uniform(30.0, 80.0, n_envs)
    envs = []
    for e in range(n_envs):
        if shapes[e] == 0:
            envs.append(make_env(seed * 1000 + e + 1, int(counts[e]), "cube", grid=grid,
                                 center=(0.5, 0.15, 0.5), extent=0.2, yield_stress=float(ys[e]),
                                 steps=steps, sort=sort, name=f"cube{e}"))
        else:
            envs.append(make_env(seed * 1000 + e + 1, int(counts[e]), "ellipsoid", grid=grid,
                                 center=(0.5, 0.11, 0.5), extent=(0.12, 0.06, 0.09),
                                 yield_stress=float(ys[e]), steps=steps, sort=sort, name=f"ellipsoid{e}"))
    return envs


def large_env(seed=0, steps=100, n=300000, sort=True):
    """Large: 128^3, dt 2.5e-5, two stacked cubes (yield 40 / 120), 22 capsules + palm box.
    sort=False keeps the sampling order (the two cubes one after the other)."""
    rng = np.random.default_rng(seed)
    grid, dt = 128, 2.5e-5
    dx = 1.0 / grid
    n1 = n // 2
    x1, v1 = sample_cube(rng, n1, (0.5, 0.15, 0.5), 0.2)
    x2, v2 = sample_cube(rng, n - n1, (0.5, 0.35, 0.5), 0.2)
    x = np.concatenate([x1, x2])
    ys = np.concatenate([np.full(n1, 40.0), np.full(n - n1, 120.0)]).astype(np.float32)
    if sort:
        order = cell_sort(x, dx)
        x, ys = x[order], ys[order]
    mu, lam = lame()
    pv = (v1 + v2) / n
    tfsr, args = capsules(rng, 23)
    tfsr[22] = (0.0, BODY_FRICTION, SOFTNESS, 0.0)   # palm box, half extents
    args[22] = (0.06, 0.01, 0.05, 0.0)
    poses = random_walk_poses(rng, 23, steps, dt, lo=(0.38, 0.43, 0.38), hi=(0.62, 0.5, 0.62))
    mly = np.stack([np.full(n, mu), np.full(n, lam), ys], 1).astype(np.float32)
    eye = np.broadcast_to(np.eye(3, dtype=np.float32), (n, 3, 3)).copy()
    return Env(grid_dim=(grid,) * 3, dx=dx, dt=dt, gravity=(0.0, -GRAVITY_SCALE, 0.0),
               ground_friction=0.9, x=x, v=np.zeros((n, 3), np.float32), F=eye,
               C=np.zeros((n, 3, 3), np.float32), mass=np.full(n, pv, np.float32),
               vol=np.full(n, pv, np.float32), mu_lam_yield=mly, body_tfsr=tfsr, body_args=args,
               poses=poses, name="large-128^3-300k")


def tiny_env(seed=0, n=256, grid=32, nb=4, steps=4, dt=1e-4, shape="cube"):
    """Small case for golden fixtures and quick parity checks."""
    if shape == "cube":
        return make_env(seed, n, "cube", grid=grid, dt=dt, center=(0.5, 0.2, 0.5), extent=0.2, nb=nb,
                        steps=steps, name=f"tiny{grid}")
    return make_env(seed, n, "ellipsoid", grid=grid, dt=dt, center=(0.5, 0.15, 0.5),
                    extent=(0.12, 0.06, 0.09), nb=nb, steps=steps, name=f"tiny{grid}e")


def random_rotations(rng, n):
    """n uniformly random proper rotations (normalised Gaussian quaternions)."""
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    return np.stack([np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
                     np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
                     np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1)], 1)


def perturb_state(env: Env, seed=1, v_scale=0.5, c_scale=5.0, f_scale=0.05, f_mode="separated"):
    """A non-rest state for adjoint checks: random v and C, and F away from
    the identity (F = I puts the SVD at its degenerate point).
    f_mode "separated": F = U diag(s) V^T with random rotations U, V and
    singular values s = 1 + f_scale (k + u), k = 1, 0, -1, u ~ U[-1/4, 1/4],
    so that every gap is at least f_scale / 2 (nearly equal singular values
    make the SVD adjoint -- the reference's and this one -- divide FP32
    rounding by their squared difference).  "gaussian": F = I + f_scale N(0,
    1) entrywise (the states of the committed oracle fixtures)."""
    rng = np.random.default_rng(seed)
    st = env.state()
    n = st["F"].shape[0]
    st["v"] = (rng.normal(size=st["v"].shape) * v_scale).astype(np.float32)
    st["C"] = (rng.normal(size=st["C"].shape) * c_scale).astype(np.float32)
    if f_mode == "gaussian":
        st["F"] = (np.eye(3) + rng.normal(size=st["F"].shape) * f_scale).astype(np.float32)
        return st
    assert f_mode == "separated"
    s = 1.0 + f_scale * (np.array([1.0, 0.0, -1.0]) + rng.uniform(-0.25, 0.25, (n, 3)))
    U, V = random_rotations(rng, n), random_rotations(rng, n)
    st["F"] = np.einsum("nij,nj,nkj->nik", U, s, V).astype(np.float32)
    return st


def render_scene(seed=0, n=3000, voxel=32, image=(64, 64), inv_dx=64.0, spp=2, max_ray_depth=2, nb=5):
    """Seeded renderer input: a colored particle cube (packed 0xRRGGBB), nb - 1
    capsules and a box above it, a camera looking down at it, and the
    renderer settings (mpm/renderer.py:17-27 defaults where they apply)."""
    from .renderer import intrinsic, lookat
    rng = np.random.default_rng(seed)
    x = (np.array([0.5, 0.15, 0.5]) + rng.uniform(-0.1, 0.1, (n, 3))).astype(np.float32)
    color = (rng.integers(0, 256, (n, 3)) * np.array([1 << 16, 1 << 8, 1])).sum(1).astype(np.int32)
    xl = np.floor(x.astype(np.float32) * np.float32(inv_dx) - 6) / np.float32(inv_dx)
    bbox_min = xl.min(0).astype(np.float32)
    vox = (voxel,) * 3 if np.isscalar(voxel) else tuple(voxel)
    bbox_max = (bbox_min + np.asarray(vox, np.float32) / np.float32(inv_dx)).astype(np.float32)
    tfsr, args = capsules(rng, nb, r_range=(0.02, 0.04), h_range=(0.05, 0.1))
    tfsr[nb - 1] = (0.0, BODY_FRICTION, SOFTNESS, 0.0)   # a box
    args[nb - 1] = (0.04, 0.01, 0.03, 0.0)
    pos = np.stack([rng.uniform(0.42, 0.58, nb), rng.uniform(0.27, 0.33, nb), rng.uniform(0.42, 0.58, nb)], 1)
    q = rng.normal(size=(nb, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    R, T = lookat((0.5, 0.2, 0.5), 0.5, 0.3, 1.2)
    return {"x": x, "color": color, "bbox_min": bbox_min, "bbox_max": bbox_max, "voxel": vox, "inv_dx": inv_dx,
            "bake": 7, "body_pos": pos.astype(np.float32), "body_rot": q.astype(np.float32),
            "body_tfsr": np.asarray(tfsr, np.float32), "body_args": np.asarray(args, np.float32),
            "cam_rot": np.asarray(R, np.float32).reshape(9), "cam_pos": np.asarray(T, np.float32),
            "cam_intr": intrinsic((image[0], image[1], 3)).astype(np.float32).reshape(9), "image": tuple(image),
            "sdf_threshold": 0.414, "visualize_shape": 1, "max_ray_depth": max_ray_depth, "spp": spp,
            "ground": 0.03, "seed": seed, "light": np.array([1.0, 1.0, 0.0], np.float32)}
