"""Headless renderer with the interface of mpm/renderer.py:14-169.

``Renderer.render(simulator, state)`` bakes the particles into a signed
distance volume (``particle_sdf``) and path-traces the ground, the bodies and
that volume (``render``) with the library's CUDA kernels, returning an
(H, W, 4) array of RGB and depth, as the reference does.  The Open3D helpers
of the reference (point clouds and GL windows, mpm/renderer.py:171-226) need
a graphics stack and are not provided; the image is a device buffer copied to
the host.
"""
from __future__ import annotations

import ctypes
import math
from typing import Optional, Sequence

import numpy as np
import torch

from . import _native as N

EMPTY_VOXEL = (1 << 33) - 1  # unreached voxel: distance code 511, white (mpm/renderer.py:64-65)


def euler_sxyz(ai: float, aj: float, ak: float) -> np.ndarray:
    """Rotation matrix of static-axis Euler angles about x, then y, then z
    (R = Rz(ak) Ry(aj) Rx(ai)), the convention of the reference's lookat
    (mpm/renderer.py:225, transforms3d 'sxyz')."""
    ca, sa, cb, sb, cc, sc = math.cos(ai), math.sin(ai), math.cos(aj), math.sin(aj), math.cos(ak), math.sin(ak)
    rx = np.array([[1, 0, 0], [0, ca, -sa], [0, sa, ca]])
    ry = np.array([[cb, 0, sb], [0, 1, 0], [-sb, 0, cb]])
    rz = np.array([[cc, -sc, 0], [sc, cc, 0], [0, 0, 1]])
    return rz @ ry @ rx


def lookat(center, theta, phi, radius):
    """Camera rotation and position at `radius` behind `center`
    (mpm/renderer.py:224-228)."""
    R = euler_sxyz(theta, phi, 0.0)
    back = R.dot(np.array([0.0, 0.0, radius]))
    return R, np.asarray(center, dtype=float) - back


def intrinsic(image_res, fov=0.23) -> np.ndarray:
    """Pixel (u, v, 1) -> camera ray (mpm/renderer.py:68-74)."""
    return np.array([-np.array([2 * fov / image_res[1], 0, -fov - 1e-5]),
                     -np.array([0, 2 * fov / image_res[1], -fov - 1e-5]),
                     [0, 0, 1]])


class Renderer:
    """Mirror of mpm/renderer.py's Renderer (constructor arguments, camera
    helpers, bake_particles, render, get_int, get_ext)."""

    def __init__(self, cfg=None, spp=3, voxel_res=(168, 168, 168), image_res=(512, 512), max_ray_depth=2,
                 light_direction=(1., 1., 0.), sdf_threshold=0.414, bake_size=7, inv_dx=150., ground_height=None,
                 device="cuda"):
        self.spp, self.max_ray_depth, self.sdf_threshold = int(spp), int(max_ray_depth), float(sdf_threshold)
        self.bake_size, self.inv_dx = int(bake_size), float(inv_dx)
        self.light = tuple(float(v) for v in light_direction)
        self.ground_height = ground_height
        self.device = torch.device(device)
        self.voxel_res = tuple(int(v) for v in voxel_res)
        self.image_res = (int(image_res[0]), int(image_res[1]), 3)
        nvox = int(np.prod(self.voxel_res))
        npix = self.image_res[0] * self.image_res[1]
        dev = self.device
        self.volume = torch.full((nvox,), EMPTY_VOXEL, dtype=torch.int64, device=dev)
        self.sdf_volume = torch.zeros(nvox, device=dev)
        self.sdf_volume2 = torch.zeros(nvox, device=dev)
        self.color_volume = torch.zeros((nvox, 3), device=dev)
        self.bbox_min = torch.zeros(3, device=dev)
        self.bbox_max = torch.zeros(3, device=dev)
        self.camera_rot = torch.zeros(9, device=dev)
        self.camera_pos = torch.zeros(3, device=dev)
        self.camera_intrinsic = torch.zeros(9, device=dev)
        self.light_direction = torch.tensor(self.light, dtype=torch.float32, device=dev)
        self.color_buffer = torch.zeros((npix, 3), device=dev)
        self.depth_buffer = torch.zeros(npix, device=dev)
        self._vdim = (ctypes.c_int * 3)(*self.voxel_res)
        self._idim = (ctypes.c_int * 3)(*self.image_res)
        self.render_seed = 0
        self.center, self.theta, self.phi, self.radius = (0.5, 0.2, 0.5), 0., 0., 3
        self.lookat(self.center, self.theta, self.phi, self.radius)

    # --------------------------------------------------------------- camera
    def initialize_camera(self, rot, pos):
        self.camera_intrinsic.copy_(torch.tensor(intrinsic(self.image_res).reshape(9), dtype=torch.float32))
        self.camera_rot.copy_(torch.tensor(np.asarray(rot, dtype=np.float64).reshape(9), dtype=torch.float32))
        self.camera_pos.copy_(torch.tensor(np.asarray(pos, dtype=np.float64).reshape(3), dtype=torch.float32))

    def lookat(self, center=(0.5, 0.2, 0.5), theta=0., phi=0., radius=3):
        self.setRT(*lookat(center, theta, phi, radius))
        self.center, self.theta, self.phi, self.radius = center, theta, phi, radius

    def setRT(self, R, T):
        self.initialize_camera(R, T)

    def get_int(self, image_res=None):
        return np.linalg.inv(intrinsic(image_res or self.image_res))

    def get_ext(self):
        T = np.eye(4)
        T[:3, :3] = self.camera_rot.cpu().numpy().reshape(3, 3)
        T[:3, 3] = self.camera_pos.cpu().numpy()
        return np.linalg.inv(T)

    # ---------------------------------------------------------------- bake
    def bake(self, x: torch.Tensor, color: torch.Tensor):
        """Bake particles x (n, 3) with packed 0xRRGGBB colors (n,) into the
        volume; its box starts 6 voxels below the particles' lower corner
        (mpm/renderer.py:93-100)."""
        n = int(x.shape[0])
        xl = torch.floor(x.float() * self.inv_dx - 6) / self.inv_dx
        lo = xl.min(0).values if n > 0 else torch.zeros(3, device=self.device)
        self.bbox_min.copy_(lo)
        self.bbox_max.copy_(lo + torch.tensor(self.voxel_res, dtype=torch.float32, device=self.device) / self.inv_dx)
        self.volume.fill_(EMPTY_VOXEL)
        xc = x.float().contiguous()
        cc = color.to(torch.int32).contiguous()
        N.check(N.load().particle_sdf(N.ptr(self.volume), N.ptr(xc), N.ptr(cc), N.ptr(self.bbox_min),
                                      N.ptr(self.bbox_max), self.bake_size, self._vdim, self.inv_dx,
                                      N.ptr(self.sdf_volume), N.ptr(self.color_volume), N.ptr(self.sdf_volume2), n,
                                      N.stream_ptr()), "particle_sdf")

    def bake_particles(self, simulator, state, stream=None):
        n = simulator.n_particles
        x = state.x.t[:n] if hasattr(state.x, "t") else state.x[:n]
        self.bake(x, simulator.particle_color.t[:n])

    # -------------------------------------------------------------- render
    def trace(self, body_pos: torch.Tensor, body_rot: torch.Tensor, body_tfsr: torch.Tensor, body_args: torch.Tensor,
              ground_height: float, visualize_shape: bool = True, spp: Optional[int] = None,
              max_ray_depth: Optional[int] = None, seed: Optional[int] = None) -> np.ndarray:
        """Path-trace the scene with the current volume and camera; returns
        (H, W, 4) = RGB and depth."""
        nb = int(body_pos.shape[0])
        bp, br = body_pos.float().contiguous(), body_rot.float().contiguous()
        bt, ba = body_tfsr.float().contiguous(), body_args.float().contiguous()
        s = self.render_seed if seed is None else int(seed)
        N.check(N.load().render(N.ptr(self.sdf_volume), N.ptr(self.bbox_min), N.ptr(self.bbox_max),
                                N.ptr(self.color_volume), N.ptr(bp), N.ptr(br), N.ptr(bt), N.ptr(ba),
                                N.ptr(self.camera_rot), N.ptr(self.camera_pos), N.ptr(self.camera_intrinsic),
                                N.ptr(self.color_buffer), N.ptr(self.depth_buffer), self.sdf_threshold, self._vdim,
                                nb, bool(visualize_shape), self._idim,
                                self.max_ray_depth if max_ray_depth is None else int(max_ray_depth),
                                self.spp if spp is None else int(spp), float(ground_height), s,
                                N.ptr(self.light_direction), N.stream_ptr()), "render")
        if seed is None:
            self.render_seed += 1
        H, W = self.image_res[:2]
        color = self.color_buffer.cpu().numpy().reshape(H, W, 3)
        depth = self.depth_buffer.cpu().numpy().reshape(H, W)
        return np.concatenate((color, depth[..., None]), -1)

    def render(self, simulator, state, stream=None, **kwargs):
        """mpm/renderer.py:121-158: bake, then trace the first
        n_bodies * primitive bodies; `shape` toggles the volume."""
        self.bake_particles(simulator, state, stream)
        primitive = kwargs.get("primitive", 1)
        nb = simulator.n_bodies * primitive
        ground = (simulator.get_ground_height() * simulator.dx if self.ground_height is None else self.ground_height)
        return self.trace(state.body_pos.t[:nb], state.body_rot.t[:nb], simulator.body_type_mu_softness_round.t[:nb],
                          simulator.body_args.t[:nb], ground, bool(kwargs.get("shape", 1)), kwargs.get("spp"),
                          kwargs.get("max_ray_depth"))
