"""Host build of the product's FP32 arithmetic (tests/native/math_host.cpp,
which includes dexdeform_gb300/csrc/mpm_math.cuh) for CPU-side checks."""
import ctypes
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None


def load():
    global _lib
    if _lib is None:
        out = os.path.join(tempfile.mkdtemp(prefix="dexmpm_host_"), "libmath_host.so")
        subprocess.run(["g++", "-O2", "-fPIC", "-shared", os.path.join(HERE, "native", "math_host.cpp"), "-o", out],
                       check=True)
        _lib = ctypes.CDLL(out)
    return _lib


def _p(a):
    assert a.flags.c_contiguous and a.dtype == np.float32
    return a.ctypes.data_as(ctypes.c_void_p)


def f32(a):
    return np.ascontiguousarray(a, np.float32)


def svd(F, C=None, dt=0.0):
    L = load()
    F = f32(F)
    n = F.shape[0]
    C = f32(np.zeros_like(F) if C is None else C)
    U, V, Ft = (np.zeros((n, 3, 3), np.float32) for _ in range(3))
    s, d = np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32)
    L.host_svd(ctypes.c_int(n), _p(F), _p(C), ctypes.c_float(dt), _p(U), _p(s), _p(d), _p(V), _p(Ft))
    return U, s, d, V, Ft


def constitutive(F, C, dt, mly):
    L = load()
    F, C, mly = f32(F), f32(C), f32(mly)
    n = F.shape[0]
    nF, P = np.zeros((n, 3, 3), np.float32), np.zeros((n, 3, 3), np.float32)
    J = np.zeros(n, np.float32)
    L.host_constitutive(ctypes.c_int(n), _p(F), _p(C), ctypes.c_float(dt), _p(mly), _p(nF), _p(P), _p(J))
    return nF, P, J


def svd_backward(U, sig, d, V, gU, gs, gV, gdirect):
    """The product's SVD adjoint (mpm_math.cuh svd_backward) on the host."""
    L = load()
    U, sig, d, V, gU, gs, gV, gdirect = (f32(a) for a in (U, sig, d, V, gU, gs, gV, gdirect))
    out = np.zeros_like(gdirect)
    L.host_svd_backward(ctypes.c_int(U.shape[0]), _p(U), _p(sig), _p(d), _p(V), _p(gU), _p(gs), _p(gV), _p(gdirect),
                        _p(out))
    return out


def stress_backward(F, C, dt, mly, gP, gF):
    """dL/dF_tmp of the product's return mapping and stress (mpm_math.cuh
    plastic_stress_backward); returns it with F_tmp and the yield flags."""
    L = load()
    F, C, mly, gP, gF = (f32(a) for a in (F, C, mly, gP, gF))
    n = F.shape[0]
    out, Ft = np.zeros_like(F), np.zeros_like(F)
    y = np.zeros(n, np.int32)
    L.host_stress_backward(ctypes.c_int(n), _p(F), _p(C), ctypes.c_float(dt), _p(mly), _p(gP), _p(gF), _p(out),
                           _p(Ft), y.ctypes.data_as(ctypes.c_void_p))
    return out, Ft, y.astype(bool)


def surely_elastic(d, mu, ys):
    """The return mapping's logarithm-free elastic test (mpm_math.cuh)."""
    L = load()
    d, ys = f32(d), f32(ys)
    out = np.zeros(d.shape[0], np.int32)
    L.host_surely_elastic(ctypes.c_int(d.shape[0]), _p(d), ctypes.c_float(mu), _p(ys),
                          out.ctypes.data_as(ctypes.c_void_p))
    return out.astype(bool)


def substep(env, st, t):
    """One forward substep of workloads.Env `env` from state dict st at substep t."""
    L = load()
    n = env.n
    out = {k: np.zeros_like(f32(st[k])) for k in ("x", "v", "F", "C")}
    pose = np.zeros((env.nb, 8), np.float32)
    npose = np.zeros((env.nb, 8), np.float32)
    pose[:, :3], pose[:, 4:] = env.poses[t][:, :3], env.poses[t][:, 3:]
    npose[:, :3], npose[:, 4:] = env.poses[t + 1][:, :3], env.poses[t + 1][:, 3:]
    shapes = f32(np.concatenate([env.body_tfsr, env.body_args], 1))
    g = env.grid_dim
    L.host_substep(ctypes.c_int(n), _p(f32(st["x"])), _p(f32(st["v"])), _p(f32(st["F"])), _p(f32(st["C"])),
                   _p(f32(env.mass)), _p(f32(env.vol)), _p(f32(env.mu_lam_yield)), ctypes.c_int(g[0]),
                   ctypes.c_int(g[1]), ctypes.c_int(g[2]), ctypes.c_float(env.dx), ctypes.c_float(env.dt),
                   _p(f32(env.gravity)), ctypes.c_float(env.ground_friction), ctypes.c_int(env.nb), _p(pose),
                   _p(npose), _p(shapes), _p(out["x"]), _p(out["v"]), _p(out["F"]), _p(out["C"]))
    return out


def block_cull(pose, shapes, blk, dx):
    """(may, touched) per case of the block culling test (see math_host.cpp)."""
    L = load()
    pose, shapes = f32(pose), f32(shapes)
    blk = np.ascontiguousarray(blk, np.int32)
    n = pose.shape[0]
    may, touched = np.zeros(n, np.int32), np.zeros(n, np.int32)
    L.host_block_cull(ctypes.c_int(n), _p(pose), _p(shapes), blk.ctypes.data_as(ctypes.c_void_p), ctypes.c_float(dx),
                      may.ctypes.data_as(ctypes.c_void_p), touched.ctypes.data_as(ctypes.c_void_p))
    return may.astype(bool), touched.astype(bool)
