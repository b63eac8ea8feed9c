"""CPU checkers for DexDeform's MLS-MPM substep.  TEST INFRASTRUCTURE ONLY.

Two backends share one driver that replays the reference's per-substep
schedule (mpm/simulator.py:561-571 forward, :573-585 backward):

* ``"oracle"`` -- ``oracle/mpm_oracle.c``, an FP64 restatement of the reference
  kernels (built into ``oracle/_build/libmpm_oracle.so``).
* ``"ref"``    -- the reference's own ``mpm/csrc/integrator.cu`` compiled as host
  C++ (``oracle/_ref/libref_host.so``, FP32, kernel bodies run serially).  Only
  buildable where the reference tree exists; used to pin the oracle and to
  generate the committed golden fixtures.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module; the product never does.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libmpm_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref_host.so")

_P = ctypes.c_void_p
_libs: dict = {}


def _load(path):
    if path not in _libs:
        if not os.path.isfile(path):
            raise FileNotFoundError(f"{path} is missing: run oracle/build_oracle.sh "
                                    f"(or oracle/build_ref_host.sh for the reference build)")
        _libs[path] = ctypes.CDLL(path)
    return _libs[path]


def ref_available() -> bool:
    return os.path.isfile(REF_SO)


def _ptr(a: np.ndarray):
    assert a.flags.c_contiguous
    return a.ctypes.data_as(_P)


@dataclass
class SimParams:
    """Physical and grid parameters of one environment (reference defaults:
    mpm/simulator.py:152-170, gravity scaled by 30 at :385)."""
    grid_dim: tuple = (64, 64, 64)
    dx: float = 1.0 / 64
    dt: float = 5e-5
    gravity: tuple = (0.0, -30.0, 0.0)
    ground_friction: float = 0.9
    ground_height: float = 3.0


@dataclass
class Material:
    mass: np.ndarray          # (n,)
    vol: np.ndarray           # (n,)
    mu_lam_yield: np.ndarray  # (n, 3)


@dataclass
class Bodies:
    type_friction_softness_round: np.ndarray  # (nb, 4)
    args: np.ndarray                          # (nb, 4)

    @property
    def n(self):
        return int(self.args.shape[0])


class _Temp:
    def __init__(self, dt, n, gdim, nb):
        g = int(np.prod(gdim))
        z = lambda *s: np.zeros(s, dtype=dt)
        self.grid_m, self.grid_mv, self.grid_v_out = z(g), z(g, 3), z(g, 3)
        self.grid_m_grad, self.grid_v_in_grad, self.grid_v_out_grad = z(g), z(g, 3), z(g, 3)
        self.grid_body_v_in = z(g * (nb + 1), 3)
        self.F, self.U, self.V, self.sig = z(n, 3, 3), z(n, 3, 3), z(n, 3, 3), z(n, 3)
        self.F_grad, self.U_grad, self.V_grad, self.sig_grad = z(n, 3, 3), z(n, 3, 3), z(n, 3, 3), z(n, 3)

    def clear(self):
        self.grid_m[:] = 0
        self.grid_mv[:] = 0
        self.grid_v_out[:] = 0

    def clear_grad(self):
        for a in (self.grid_m_grad, self.grid_v_in_grad, self.grid_v_out_grad, self.F_grad,
                  self.U_grad, self.V_grad, self.sig_grad):
            a[:] = 0


class CpuMPM:
    """One environment stepped on the CPU by a checker backend.

    States are dicts with x, v (n,3), F, C (n,3,3); poses are (pos (nb,3),
    rot (nb,4) as w,x,y,z)."""

    def __init__(self, backend: str, params: SimParams, mat: Material, bodies: Bodies):
        assert backend in ("oracle", "ref")
        self.backend = backend
        self.dtype = np.float64 if backend == "oracle" else np.float32
        self.lib = _load(ORACLE_SO if backend == "oracle" else REF_SO)
        self.p = params
        self.n = int(mat.mass.shape[0])
        self.nb = bodies.n
        c = lambda a: np.ascontiguousarray(a, dtype=self.dtype)
        self.mass, self.vol, self.mly = c(mat.mass), c(mat.vol), c(mat.mu_lam_yield)
        self.tfsr, self.bargs = c(bodies.type_friction_softness_round), c(bodies.args)
        self.gdim = np.ascontiguousarray(params.grid_dim, dtype=np.int32)
        self.gravity = c(params.gravity)
        self.grid_lower = np.zeros(3, dtype=np.int32)
        self.temp = _Temp(self.dtype, self.n, params.grid_dim, self.nb)
        self.dx = float(params.dx)
        self.inv_dx = 1.0 / self.dx
        self.dt = float(params.dt)

    # ------------------------------------------------------------ helpers
    def _c(self, a):
        return np.ascontiguousarray(a, dtype=self.dtype)

    def _f(self, v):
        return ctypes.c_double(v) if self.backend == "oracle" else ctypes.c_float(v)

    # ------------------------------------------------------ kernel steps
    def compute_svd(self, F, C):
        t, L = self.temp, self.lib
        if self.backend == "oracle":
            L.orc_compute_svd(ctypes.c_int(self.n), _ptr(F), _ptr(C), self._f(self.dt),
                              _ptr(t.F), _ptr(t.U), _ptr(t.V), _ptr(t.sig))
        else:
            L.compute_svd(_ptr(F), _ptr(C), _ptr(t.F), _ptr(t.U), _ptr(t.V), _ptr(t.sig),
                          self._f(self.dt), ctypes.c_int(self.n), _P(0))

    def p2g(self, x, v, C, outF):
        t, L = self.temp, self.lib
        if self.backend == "oracle":
            L.orc_p2g(ctypes.c_int(self.n), _ptr(x), _ptr(v), _ptr(self.mass), _ptr(self.vol),
                      _ptr(t.F), _ptr(t.U), _ptr(t.sig), _ptr(t.V), _ptr(C), _ptr(self.mly),
                      _ptr(self.gdim), self._f(self.dx), self._f(self.inv_dx), self._f(self.dt),
                      _ptr(outF), _ptr(t.grid_mv), _ptr(t.grid_m))
        else:
            L.p2g(_ptr(x), _ptr(v), _ptr(self.mass), _ptr(self.vol), _ptr(t.F), _ptr(t.U),
                  _ptr(t.sig), _ptr(t.V), _ptr(C), _ptr(self.mly), _ptr(self.grid_lower),
                  _ptr(self.gdim), self._f(self.dx), self._f(self.inv_dx), self._f(self.dt),
                  _ptr(outF), _ptr(t.grid_mv), _ptr(t.grid_m), ctypes.c_int(self.n), _P(0))

    def grid_op(self, pose, npose):
        t, L = self.temp, self.lib
        bp, br = self._c(pose[0]), self._c(pose[1])
        nbp, nbr = self._c(npose[0]), self._c(npose[1])
        if self.backend == "oracle":
            L.orc_grid_op(_ptr(self.gdim), _ptr(t.grid_m), _ptr(t.grid_mv), _ptr(t.grid_body_v_in),
                          _ptr(self.gravity), ctypes.c_int(self.nb), _ptr(bp), _ptr(br), _ptr(nbp),
                          _ptr(nbr), _ptr(self.tfsr), _ptr(self.bargs), self._f(self.dx),
                          self._f(self.inv_dx), self._f(self.dt), self._f(self.p.ground_friction),
                          _ptr(t.grid_v_out))
        else:
            L.grid_op_v2(_ptr(t.grid_m), _ptr(t.grid_mv), _ptr(t.grid_body_v_in), _ptr(self.grid_lower),
                         _ptr(self.gravity), _ptr(bp), _ptr(br), _ptr(nbp), _ptr(nbr), _ptr(self.tfsr),
                         _ptr(self.bargs), self._f(self.dx), self._f(self.inv_dx), self._f(self.dt),
                         self._f(self.p.ground_friction), _ptr(t.grid_v_out), _ptr(self.gdim),
                         ctypes.c_int(self.nb), _P(0))

    def g2p(self, x, out_v, out_C, out_x):
        t, L = self.temp, self.lib
        if self.backend == "oracle":
            L.orc_g2p(ctypes.c_int(self.n), _ptr(x), _ptr(t.grid_v_out), _ptr(self.gdim),
                      self._f(self.dx), self._f(self.inv_dx), self._f(self.dt),
                      self._f(self.p.ground_height), _ptr(out_v), _ptr(out_C), _ptr(out_x))
        else:
            L.g2p(_ptr(x), _ptr(t.grid_v_out), _ptr(self.grid_lower), self._f(self.dx),
                  self._f(self.inv_dx), self._f(self.dt), _ptr(self.gdim), _ptr(out_v),
                  self._f(self.p.ground_height), _ptr(out_C), _ptr(out_x), ctypes.c_int(self.n), _P(0))

    # ----------------------------------------------------------- schedule
    def substep(self, st: dict, pose, npose) -> dict:
        """mpm/simulator.py:561-571: clear, compute_svd, p2g, grid_op, g2p."""
        x, v, F, C = (self._c(st[k]) for k in ("x", "v", "F", "C"))
        out = {k: np.zeros_like(x if k in "xv" else F) for k in ("x", "v", "F", "C")}
        self.temp.clear()
        self.compute_svd(F, C)
        self.p2g(x, v, C, out["F"])
        self.grid_op(pose, npose)
        self.g2p(x, out["v"], out["C"], out["x"])
        return out

    def substep_grad(self, st: dict, pose, npose, next_v, g_next: dict):
        """mpm/simulator.py:573-585: recompute svd/p2g/grid_op, then g2p_grad,
        grid_op_grad, p2g_grad, compute_svd_grad.  Returns the gradients of the
        current state (fresh arrays) and of the two body poses."""
        t, L = self.temp, self.lib
        x, v, F, C = (self._c(st[k]) for k in ("x", "v", "F", "C"))
        nv = self._c(next_v)
        gx_n, gv_n, gF_n, gC_n = (self._c(g_next[k]) for k in ("x", "v", "F", "C"))
        g = {k: np.zeros_like(x if k in "xv" else F) for k in ("x", "v", "F", "C")}
        nb = self.nb
        bpg, brg = np.zeros((nb, 3), self.dtype), np.zeros((nb, 4), self.dtype)
        nbpg, nbrg = np.zeros((nb, 3), self.dtype), np.zeros((nb, 4), self.dtype)
        bp, br = self._c(pose[0]), self._c(pose[1])
        nbp, nbr = self._c(npose[0]), self._c(npose[1])
        scratchF = np.zeros_like(F)
        t.clear()
        t.clear_grad()
        self.compute_svd(F, C)
        self.p2g(x, v, C, scratchF)
        self.grid_op(pose, npose)
        f = self._f
        if self.backend == "oracle":
            L.orc_g2p_grad(ctypes.c_int(self.n), _ptr(x), _ptr(t.grid_v_out), _ptr(self.gdim), f(self.dx),
                           f(self.inv_dx), f(self.dt), _ptr(nv), f(self.p.ground_height), _ptr(g["x"]),
                           _ptr(t.grid_v_out_grad), _ptr(gv_n), _ptr(gC_n), _ptr(gx_n))
            L.orc_grid_op_grad(_ptr(self.gdim), _ptr(t.grid_m), _ptr(t.grid_mv), _ptr(t.grid_body_v_in),
                               _ptr(self.gravity), ctypes.c_int(nb), _ptr(bp), _ptr(br), _ptr(nbp), _ptr(nbr),
                               _ptr(self.tfsr), _ptr(self.bargs), _ptr(t.grid_m_grad), _ptr(t.grid_v_in_grad),
                               _ptr(bpg), _ptr(brg), _ptr(nbpg), _ptr(nbrg), f(self.dx), f(self.inv_dx),
                               f(self.dt), f(self.p.ground_friction), _ptr(t.grid_v_out_grad))
            L.orc_p2g_grad(ctypes.c_int(self.n), _ptr(x), _ptr(v), _ptr(self.mass), _ptr(self.vol), _ptr(t.F),
                           _ptr(t.U), _ptr(t.sig), _ptr(t.V), _ptr(C), _ptr(self.mly), _ptr(self.gdim),
                           f(self.dx), f(self.inv_dx), f(self.dt), _ptr(g["x"]), _ptr(g["v"]), _ptr(t.F_grad),
                           _ptr(g["C"]), _ptr(t.U_grad), _ptr(t.sig_grad), _ptr(t.V_grad), _ptr(gF_n),
                           _ptr(t.grid_v_in_grad), _ptr(t.grid_m_grad))
            L.orc_compute_svd_grad(ctypes.c_int(self.n), _ptr(F), _ptr(C), _ptr(t.U), _ptr(t.V), _ptr(t.sig),
                                   _ptr(t.F_grad), _ptr(t.U_grad), _ptr(t.V_grad), _ptr(t.sig_grad),
                                   _ptr(g["F"]), _ptr(g["C"]), f(self.dt))
        else:
            n = ctypes.c_int(self.n)
            L.g2p_grad(_ptr(x), _ptr(t.grid_v_out), _ptr(self.grid_lower), f(self.dx), f(self.inv_dx), f(self.dt),
                       _ptr(self.gdim), _ptr(nv), f(self.p.ground_height), _ptr(np.zeros_like(gC_n)),
                       _ptr(np.zeros_like(gx_n)), n, _ptr(g["x"]), _ptr(t.grid_v_out_grad), _ptr(gv_n),
                       _ptr(gC_n), _ptr(gx_n), _P(0))
            L.grid_op_v2_grad(_ptr(t.grid_m), _ptr(t.grid_mv), _ptr(t.grid_body_v_in), _ptr(self.grid_lower),
                              _ptr(self.gravity), _ptr(bp), _ptr(br), _ptr(nbp), _ptr(nbr), _ptr(self.tfsr),
                              _ptr(self.bargs), _ptr(t.grid_m_grad), _ptr(t.grid_v_in_grad), _ptr(bpg),
                              _ptr(brg), _ptr(nbpg), _ptr(nbrg), f(self.dx), f(self.inv_dx), f(self.dt),
                              f(self.p.ground_friction), _ptr(t.grid_v_out), _ptr(t.grid_v_out_grad),
                              _ptr(self.gdim), ctypes.c_int(nb), _P(0))
            L.p2g_grad(_ptr(x), _ptr(v), _ptr(self.mass), _ptr(self.vol), _ptr(t.F), _ptr(t.U), _ptr(t.sig),
                       _ptr(t.V), _ptr(C), _ptr(self.mly), _ptr(self.grid_lower), _ptr(self.gdim), f(self.dx),
                       f(self.inv_dx), f(self.dt), _ptr(scratchF), _ptr(t.grid_mv), _ptr(t.grid_m),
                       _ptr(g["x"]), _ptr(g["v"]), _ptr(t.F_grad), _ptr(g["C"]), _ptr(t.U_grad),
                       _ptr(t.sig_grad), _ptr(t.V_grad), _ptr(gF_n), _ptr(t.grid_v_in_grad),
                       _ptr(t.grid_m_grad), n, _P(0))
            L.compute_svd_grad(_ptr(F), _ptr(C), _ptr(t.U), _ptr(t.V), _ptr(t.sig), _ptr(t.F_grad),
                               _ptr(t.U_grad), _ptr(t.V_grad), _ptr(t.sig_grad), _ptr(g["F"]), _ptr(g["C"]),
                               f(self.dt), n, _P(0))
        return g, (bpg, brg), (nbpg, nbrg)

    # ------------------------------------------------------- loss hooks
    def compute_dist(self, x, pose):
        """integrator.cu:188-237 forward: (n, nb) signed distances (oracle only)."""
        assert self.backend == "oracle"
        x = self._c(x)
        d = np.zeros((self.n, self.nb), np.float64)
        z = np.zeros(1)
        self.lib.orc_compute_dist(ctypes.c_int(self.n), _ptr(x), ctypes.c_int(self.nb), _ptr(self._c(pose[0])),
                                  _ptr(self._c(pose[1])), _ptr(self.tfsr), _ptr(self.bargs), _ptr(d),
                                  ctypes.c_int(0), _ptr(z), _ptr(z), _ptr(z), _ptr(z))
        return d

    def compute_dist_grad(self, x, pose, dist_grad):
        assert self.backend == "oracle"
        x = self._c(x)
        gx = np.zeros_like(x)
        gp, gr = np.zeros((self.nb, 3)), np.zeros((self.nb, 4))
        z = np.zeros(1)
        self.lib.orc_compute_dist(ctypes.c_int(self.n), _ptr(x), ctypes.c_int(self.nb), _ptr(self._c(pose[0])),
                                  _ptr(self._c(pose[1])), _ptr(self.tfsr), _ptr(self.bargs), _ptr(z),
                                  ctypes.c_int(1), _ptr(self._c(dist_grad)), _ptr(gx), _ptr(gp), _ptr(gr))
        return gx, gp, gr

    def particle2mass(self, x, ids=None, obj=-1):
        assert self.backend == "oracle"
        x = self._c(x)
        gm = np.zeros(int(np.prod(self.p.grid_dim)))
        ids = np.zeros(self.n, np.int32) if ids is None else np.ascontiguousarray(ids, np.int32)
        z = np.zeros(1)
        self.lib.orc_particle2mass(ctypes.c_int(self.n), _ptr(x), _ptr(self.mass), _ptr(self.gdim),
                                   self._f(self.dx), self._f(self.inv_dx), _ptr(gm), _ptr(z), _ptr(z),
                                   _ptr(ids), ctypes.c_int(obj), ctypes.c_int(0))
        return gm.reshape(self.p.grid_dim)

    def particle2mass_grad(self, x, grid_m_grad, ids=None, obj=-1):
        assert self.backend == "oracle"
        x = self._c(x)
        gx = np.zeros_like(x)
        ids = np.zeros(self.n, np.int32) if ids is None else np.ascontiguousarray(ids, np.int32)
        z = np.zeros(1)
        self.lib.orc_particle2mass(ctypes.c_int(self.n), _ptr(x), _ptr(self.mass), _ptr(self.gdim),
                                   self._f(self.dx), self._f(self.inv_dx), _ptr(z),
                                   _ptr(self._c(grid_m_grad).reshape(-1)), _ptr(gx), _ptr(ids),
                                   ctypes.c_int(obj), ctypes.c_int(1))
        return gx


def svd3(A: np.ndarray):
    """FP64 restatement of svd3 (mpm/csrc/svd.h:390-413) on a batch (n,3,3)."""
    lib = _load(ORACLE_SO)
    A = np.ascontiguousarray(A, np.float64).reshape(-1, 3, 3)
    U, V, s = np.zeros_like(A), np.zeros_like(A), np.zeros((A.shape[0], 3))
    for i in range(A.shape[0]):
        lib.orc_svd3(_ptr(A[i]), _ptr(U[i]), _ptr(s[i]), _ptr(V[i]))
    return U, s, V


def set_svd_mode(mode: str):
    """``"reference"`` (default): the reference's svd3 restated exactly.
    ``"exact"``: converged FP64 Jacobi with the same conventions."""
    _load(ORACLE_SO).orc_set_svd_mode(ctypes.c_int({"reference": 0, "exact": 1}[mode]))


def set_capsule_grad(mode: str):
    """``"reference"`` (default): the reference's capsule adjoint, which drops
    the capsule-normal term.  ``"exact"``: its true derivative."""
    _load(ORACLE_SO).orc_set_capsule_grad(ctypes.c_int({"reference": 0, "exact": 1}[mode]))


# --------------------------------------------------------------- renderer
def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _pp(a):
    return a.ctypes.data_as(_P)


def particle_sdf(backend, x, color, bbox_min, bake, gdim, inv_dx):
    """Volume bake of mpm/csrc/integrator.cu:1911-1933 (bake, unpack, two
    smoothing passes) on the CPU.  Returns (packed volume int64, sdf, color
    (n, 3)).  backend "oracle" (render_oracle.c) or "ref" (the reference's own
    code built for the host)."""
    x, color, lo = _f32(x), _i32(color), _f32(bbox_min)
    g = (ctypes.c_int * 3)(*[int(v) for v in gdim])
    nv = int(np.prod(gdim))
    vol = np.full(nv, (1 << 33) - 1, np.int64)
    sdf, tmp = np.zeros(nv, np.float32), np.zeros(nv, np.float32)
    colv = np.zeros((nv, 3), np.float32)
    n = int(x.shape[0])
    if backend == "oracle":
        L = _load(ORACLE_SO)
        L.orc_particle_sdf(_pp(vol), _pp(x), _pp(color), _pp(lo), ctypes.c_int(bake), g, ctypes.c_float(inv_dx),
                           _pp(sdf), _pp(colv), _pp(tmp), ctypes.c_int(n))
    else:
        L = _load(REF_SO)
        hi = _f32(lo + np.asarray(gdim, np.float32) / np.float32(inv_dx))
        L.particle_sdf(_pp(vol), _pp(x), _pp(color), _pp(lo), _pp(hi), ctypes.c_int(bake), g,
                       ctypes.c_float(inv_dx), _pp(sdf), _pp(colv), _pp(tmp), ctypes.c_int(n), None)
    return vol, sdf, colv


def render(backend, sc, sdf, colv):
    """Path-traced image of integrator.cu:1287-1436 on the CPU for a scene
    dict (workloads.render_scene); returns (color (H, W, 3), depth (H, W))."""
    H, W = sc["image"]
    col, dep = np.zeros((H * W, 3), np.float32), np.zeros(H * W, np.float32)
    arrs = [_f32(sdf), _f32(sc["bbox_min"]), _f32(sc["bbox_max"]), _f32(colv), _f32(sc["body_pos"]),
            _f32(sc["body_rot"]), _f32(sc["body_tfsr"]), _f32(sc["body_args"]), _f32(sc["cam_rot"]),
            _f32(sc["cam_pos"]), _f32(sc["cam_intr"])]
    g = (ctypes.c_int * 3)(*[int(v) for v in sc["voxel"]])
    im = (ctypes.c_int * 3)(H, W, 3)
    light = _f32(sc["light"])
    nb = int(sc["body_pos"].shape[0])
    args = [*[_pp(a) for a in arrs], _pp(col), _pp(dep), ctypes.c_float(sc["sdf_threshold"]), g, ctypes.c_int(nb)]
    tail = [ctypes.c_int(int(sc["max_ray_depth"])), ctypes.c_int(int(sc["spp"])), ctypes.c_float(sc["ground"]),
            ctypes.c_int(int(sc["seed"])), _pp(light)]
    if backend == "oracle":
        _load(ORACLE_SO).orc_render(*args, ctypes.c_int(int(sc["visualize_shape"])), im, *tail)
    else:
        _load(REF_SO).render(*args, ctypes.c_bool(bool(sc["visualize_shape"])), im, *tail, None)
    return col.reshape(H, W, 3), dep.reshape(H, W)
