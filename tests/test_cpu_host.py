"""CPU tests: the C ABI library loads and exports what include/dexmpm.h
declares, struct layouts agree with the header, the product's FP32 arithmetic
(host build of mpm_math.cuh) against the FP64 oracle, and host-side logic."""
import ctypes
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT, oracle_sim, rel


def header_functions():
    text = open(os.path.join(ROOT, "include", "dexmpm.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol(native_lib):
    from dexdeform_gb300 import _native as N
    names = header_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(native_lib, n), n
    assert sorted(N.EXPORTED) == names
    assert native_lib.dexmpm_version().startswith(b"dexmpm")


def test_struct_layouts_match_header():
    from dexdeform_gb300 import _native as N
    src = os.path.join(tempfile.mkdtemp(), "l.c")
    with open(src, "w") as f:
        f.write('#include <stdio.h>\n#include <stddef.h>\n#include "dexmpm.h"\nint main(){'
                'printf("%zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(DexEnv), offsetof(DexEnv, gravity), '
                'sizeof(DexBatch), offsetof(DexBatch, grid), offsetof(DexBatch, block_count), '
                'offsetof(DexBatch, error), sizeof(DexSortWork), offsetof(DexSortWork, partial)); '
                'printf("%zu %zu %zu\\n", offsetof(DexBatch, block_xyz), sizeof(DexSegment), '
                'offsetof(DexSegment, count)); return 0;}\n')
    exe = src[:-2]
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True)
    got = [int(v) for v in subprocess.run([exe], capture_output=True, text=True).stdout.split()]
    want = [ctypes.sizeof(N.DexEnv), N.DexEnv.gravity.offset, ctypes.sizeof(N.DexBatch), N.DexBatch.grid.offset,
            N.DexBatch.block_count.offset, N.DexBatch.error.offset, ctypes.sizeof(N.DexSortWork),
            N.DexSortWork.partial.offset, N.DexBatch.block_xyz.offset, ctypes.sizeof(N.DexSegment),
            N.DexSegment.count.offset]
    assert got == want


def test_product_svd_against_fp64(oracle_mod):
    import host_math as H
    rng = np.random.default_rng(0)
    for scale in (0.0, 1e-4, 1e-2, 0.3, 1.0):
        F = (np.eye(3) + rng.normal(size=(500, 3, 3)) * scale).astype(np.float32)
        U, s, d, V, _ = H.svd(F)
        st = np.linalg.svd(F.astype(np.float64), compute_uv=False)
        st[:, 2] *= np.sign(np.linalg.det(F.astype(np.float64)))
        rec = np.einsum("nij,nj,nkj->nik", U.astype(np.float64), s.astype(np.float64), V.astype(np.float64))
        assert np.abs(rec - F).max() < 5e-6 * max(1.0, scale * 4)
        assert np.allclose(np.linalg.det(U), 1, atol=2e-6) and np.allclose(np.linalg.det(V), 1, atol=2e-6)
        if scale == 0.0:
            assert (U == np.eye(3)).all() and (V == np.eye(3)).all() and (s == 1).all() and (d == 0).all()
        else:
            # sigma - 1 to (near) full FP32 relative precision
            assert np.abs(d - (st - 1)).max() <= 2e-6 * np.abs(st - 1).max() + 1e-7 * (scale > 0.2)
        # same conventions as the reference's svd3
        oracle_mod.set_svd_mode("exact")
        _, so, _ = oracle_mod.svd3(F.astype(np.float64))
        oracle_mod.set_svd_mode("reference")
        assert np.abs(s - so).max() < 1e-5 * max(1.0, 4 * scale)


def test_product_stress_is_cancellation_free(oracle_mod):
    """Stress from the product arithmetic vs an FP64 evaluation of the
    reference formula 2 mu (F' - U V^T) F'^T + lam J (J-1) I."""
    import host_math as H
    rng = np.random.default_rng(1)
    n = 400
    F = (np.eye(3) + rng.normal(size=(n, 3, 3)) * 1e-3).astype(np.float32)
    C = (rng.normal(size=(n, 3, 3)) * 0.5).astype(np.float32)
    mly = np.tile(np.float32([2083.33, 1388.89, 50.0]), (n, 1))
    dt = 5e-5
    nF, P, J = H.constitutive(F, C, dt, mly)
    Ft = np.einsum("nij,njk->nik", np.eye(3) + dt * C.astype(np.float64), F.astype(np.float64))
    oracle_mod.set_svd_mode("exact")
    U, s, V = oracle_mod.svd3(Ft)
    oracle_mod.set_svd_mode("reference")
    R = np.einsum("nij,nkj->nik", U, V)
    Jd = np.prod(s, 1)
    Pd = 2 * 2083.33 * np.einsum("nij,nkj->nik", Ft - R, Ft) + (1388.89 * Jd * (Jd - 1))[:, None, None] * np.eye(3)
    assert rel(P, Pd) < 1e-5
    assert rel(J, Jd) < 1e-7


def test_svd_adjoint_matches_expanded_formula():
    """The product's compact SVD adjoint (one reciprocal per singular-value
    pair, U M V^T) against the reference's expanded form in FP64
    (integrator.cu:131-159): F = 1/clamp_gap(sigma_j^2 - sigma_i^2) off the
    diagonal, u = F o (U^T gU - gU^T U), v = F o (V^T gV - gV^T V),
    gF = gF_direct + U u S V^T + U diag(gs) V^T + U S v V^T, including
    equal singular values (zero gaps, where clamp_gap gives +1e-6 for both
    orders) and tiny gaps."""
    import host_math as H
    rng = np.random.default_rng(4)
    n = 600

    def rot(k):
        q = rng.normal(size=(k, 4))
        q /= np.linalg.norm(q, axis=1, keepdims=True)
        w, x, y, z = q.T
        return np.stack([np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
                         np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
                         np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1)], 1)

    U, V = rot(n).astype(np.float32), rot(n).astype(np.float32)
    d = (rng.normal(size=(n, 3)) * 0.05).astype(np.float32)
    d[:100] = 0.0                                  # at rest: all gaps zero
    d[100:200, 1] = d[100:200, 0]                  # one repeated singular value
    d[200:300, 2] = d[200:300, 1] + 1e-7           # a tiny gap
    sig = (1.0 + d.astype(np.float64)).astype(np.float32)
    gU, gV, gd = (rng.normal(size=(n, 3, 3)).astype(np.float32) for _ in range(3))
    gs = rng.normal(size=(n, 3)).astype(np.float32)
    out = H.svd_backward(U, sig, d, V, gU, gs, gV, gd)

    def clamp_gap(a):
        return np.where(a >= 0, np.maximum(a, 1e-6), np.minimum(a, -1e-6))

    Ud, Vd, dd, sd = (a.astype(np.float64) for a in (U, V, d, sig))
    gap = (dd[:, None, :] - dd[:, :, None]) * (sd[:, None, :] + sd[:, :, None])  # [n, i, j]: (d_j - d_i)(s_j + s_i)
    F = np.where(np.eye(3, dtype=bool)[None], 0.0, 1.0 / clamp_gap(gap))
    UtgU = np.einsum("nki,nkj->nij", Ud, gU)
    VtgV = np.einsum("nki,nkj->nij", Vd, gV)
    u_in = F * (UtgU - np.swapaxes(UtgU, 1, 2))
    v_in = F * (VtgV - np.swapaxes(VtgV, 1, 2))
    S = np.einsum("ni,ij->nij", sd, np.eye(3))
    G = np.einsum("nij,njk->nik", u_in, S) + np.einsum("nij,njk->nik", S, v_in) + \
        np.einsum("ni,ij->nij", gs.astype(np.float64), np.eye(3))
    ref = gd + np.einsum("nij,njk,nlk->nil", Ud, G, Vd)
    for sl in (slice(0, 100), slice(100, 200), slice(200, 300), slice(300, n)):
        assert rel(out[sl], ref[sl]) < 2e-6, sl


def _stress_objective(Ft, gP, gF, mu, lam, ys, sig_clip=0.05, norm_eps=1e-8):
    """<gP, P(Ft)> + <gF, newF(Ft)> in FP64 for one F_tmp: the reference's von
    Mises projection (integrator.cu:42-67) and fixed-corotated stress
    2 mu (newF - R) newF^T + lam J (J - 1) I (integrator.cu:364-371)."""
    U, s, Vt = np.linalg.svd(Ft)
    e = np.log(np.where(s >= sig_clip, s, sig_clip))
    eh = e - e.mean()
    ehn = np.sqrt(eh @ eh + norm_eps)
    dg = ehn - ys / (2 * mu)
    nF = U @ np.diag(np.exp(e - dg * eh / ehn)) @ Vt if dg > 0 else Ft
    R = U @ Vt
    J = np.linalg.det(nF)
    P = 2 * mu * (nF - R) @ nF.T + lam * J * (J - 1) * np.eye(3)
    return float((gP * P).sum() + (gF * nF).sum())


def test_stress_adjoint_matches_finite_differences():
    """The product's adjoint of the return mapping and stress (worked in the
    frame of the SVD) against central differences of the FP64 objective
    <gP, P(F_tmp)> + <gF, newF(F_tmp)>, for states that do not yield and
    states that yield, with well-separated singular values."""
    import host_math as H
    rng = np.random.default_rng(6)
    n = 120
    F = np.zeros((n, 3, 3), np.float32)
    for k in range(n):
        while True:
            A = np.eye(3) + rng.normal(size=(3, 3)) * (0.02 if k < n // 2 else 0.15)
            sv = np.linalg.svd(A, compute_uv=False)
            if np.linalg.det(A) > 0.3 and np.min(np.abs(np.diff(sv))) > 2e-3:
                break
        F[k] = A
    C = np.zeros_like(F)
    mu, lam = 2083.33, 1388.89
    ys = np.where(np.arange(n) < n // 2, 1e4, 20.0)      # first half cannot yield, second half yields
    mly = np.stack([np.full(n, mu), np.full(n, lam), ys], 1).astype(np.float32)
    gP = rng.normal(size=(n, 3, 3)).astype(np.float32)
    gF = (rng.normal(size=(n, 3, 3)) * 1e3).astype(np.float32)
    out, Ft, yielded = H.stress_backward(F, C, 0.0, mly, gP, gF)
    assert not yielded[:n // 2].any() and yielded[n // 2:].mean() > 0.8
    eps = 1e-6
    for k in range(n):
        Fk = Ft[k].astype(np.float64)
        fd = np.zeros((3, 3))
        for i in range(3):
            for j in range(3):
                dF = np.zeros((3, 3))
                dF[i, j] = eps
                fd[i, j] = (_stress_objective(Fk + dF, gP[k], gF[k], mu, lam, float(mly[k, 2]))
                            - _stress_objective(Fk - dF, gP[k], gF[k], mu, lam, float(mly[k, 2]))) / (2 * eps)
        assert rel(out[k], fd) < 2e-5, (k, bool(yielded[k]), rel(out[k], fd))


def test_elastic_pretest_never_skips_a_yield():
    """The return mapping decides "not yielded" without logarithms when a
    bound on the deviatoric log strain is inside the yield radius; it must
    never say so for a state whose exact (FP64) test yields, and it should
    say so for most states well inside the surface."""
    import host_math as H
    rng = np.random.default_rng(8)
    n = 200000
    mu = 2083.33
    ys = rng.uniform(30, 80, n)
    r = ys / (2 * mu)
    # deviatoric directions scaled to 0.5x .. 1.5x the yield radius, plus a
    # volumetric part and some large strains
    dirs = rng.normal(size=(n, 3))
    dirs -= dirs.mean(1, keepdims=True)
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    scale = rng.uniform(0.5, 1.5, n) * r
    d = dirs * scale[:, None] + rng.normal(size=(n, 1)) * 0.02
    d[: n // 10] *= 20.0
    d = np.clip(d, -0.9, 3.0).astype(np.float32)
    sure = H.surely_elastic(d, mu, ys)
    e = np.log1p(d.astype(np.float64))
    eh = e - e.mean(1, keepdims=True)
    dg = np.sqrt((eh * eh).sum(1) + 1e-8) - ys.astype(np.float32).astype(np.float64) / (2 * np.float32(mu))
    assert not (sure & (dg > 0)).any()
    inside = (dg < -0.05 * r) & (np.abs(d).max(1) < 0.1)   # small strains well inside the surface
    assert sure[inside].mean() > 0.95


def test_host_substep_matches_oracle_off_rest(oracle_mod):
    """The product arithmetic (host build) for one substep from a non-rest
    state meets the 1e-5 bar against the FP64 oracle."""
    import host_math as H
    from dexdeform_gb300 import workloads as W
    env = W.tiny_env(0, n=256, grid=32, nb=6, steps=2, dt=1e-4)
    st = W.perturb_state(env, v_scale=0.1, c_scale=1.0, f_scale=0.02)
    oracle_mod.set_svd_mode("exact")
    a = oracle_sim(oracle_mod, env).substep(st, env.pose(0), env.pose(1))
    oracle_mod.set_svd_mode("reference")
    b = H.substep(env, st, 0)
    for k in ("x", "v", "F", "C"):
        assert rel(b[k], a[k]) < 1e-5, k


def test_layout_plan_and_footprint():
    from dexdeform_gb300 import workloads as W
    from dexdeform_gb300.engine import EnvSpec, footprint_bytes, plan_layout
    envs = W.batch_envs(0, n_envs=7, steps=2, n_lo=100, n_hi=900)
    specs = [EnvSpec.from_env(e) for e in envs]
    for tile in (64, 128, 256):
        L = plan_layout(specs, tile)
        seen = np.zeros(sum(s.n for s in specs), np.int32)
        for e, first in L["tiles"]:
            n = min(tile, specs[e].n - first)
            assert 0 <= first < specs[e].n and n > 0
            seen[L["p_off"][e] + first:L["p_off"][e] + first + n] += 1
        assert (seen == 1).all()
        assert len(L["block_env"]) == sum((s.grid_dim[0] // 4) ** 3 for s in specs)
        assert all(L["block_env"][L["blk_off"][e]] == e for e in range(len(specs)))
        # block coordinates: the block index within the env decomposes as
        # (bx * nby + by) * nbz + bz
        xyz = L["block_xyz"]
        for e, sp in enumerate(specs):
            nby, nbz = sp.grid_dim[1] // 4, sp.grid_dim[2] // 4
            local = np.arange(len(xyz))[L["block_env"] == e] - L["blk_off"][e]
            c = xyz[L["block_env"] == e]
            assert (((c >> 20) * nby + ((c >> 10) & 1023)) * nbz + (c & 1023) == local).all()
    a = footprint_bytes(specs)
    b = footprint_bytes(specs, grad=True, substeps=50, env_steps=10)
    assert 0 < a < b


def test_capacity_covers_the_layout_it_is_computed_from():
    """Capacity.of counts what plan_layout lays out (particles, blocks,
    bodies, tiles, envs), and a capacity holds a layout exactly when every
    count fits: what BatchEngine.relayout checks before it keeps its buffers."""
    from dexdeform_gb300 import workloads as W
    from dexdeform_gb300.engine import Capacity, EnvSpec, plan_layout
    envs = W.batch_envs(3, n_envs=6, steps=2, n_lo=100, n_hi=900)
    specs = [EnvSpec.from_env(e) for e in envs]
    for tile in (64, 128, 256):
        L = plan_layout(specs, tile)
        c = Capacity.of(specs, tile)
        assert (c.particles, c.blocks, c.bodies, c.tiles, c.envs) == (
            L["n_particles"], L["n_blocks"], L["n_bodies"], len(L["tiles"]), len(specs))
    c = Capacity.of(specs, 128)
    part = Capacity.of(specs[:3], 128)
    assert c.holds(part) and not part.holds(c) and c.holds(c)
    assert c.union(part) == c and part.union(c) == c
    g = part.scaled(1.25)
    assert g.holds(part) and g.blocks == -(-part.blocks * 5 // 4)
    # one count over is enough to not fit
    assert not c.holds(Capacity(**{**c.__dict__, "bodies": c.bodies + 1}))
    assert Capacity.of([], 128) == Capacity()


def test_workloads_are_seeded_and_in_range():
    from dexdeform_gb300 import workloads as W
    a, b = W.batch_envs(0, n_envs=16, steps=5), W.batch_envs(0, n_envs=16, steps=5)
    assert all(np.array_equal(x.x, y.x) and np.array_equal(x.poses, y.poses) for x, y in zip(a, b))
    counts = np.array([e.n for e in a])
    assert counts.min() >= 2000 and counts.max() <= 30000
    for e in a:
        assert 30.0 <= e.mu_lam_yield[0, 2] <= 80.0
        r, h = e.body_args[:, 0], e.body_args[:, 1]
        assert (r >= 0.008).all() and (r <= 0.02).all() and (h >= 0.02).all() and (h <= 0.05).all()
        v = np.linalg.norm(np.diff(e.poses[:, :, :3], axis=0), axis=-1) / e.dt
        assert v.max() <= 0.5 + 1e-3
        q = np.linalg.norm(e.poses[:, :, 3:], axis=-1)
        assert np.abs(q - 1).max() < 1e-5


def test_block_culling_never_skips_a_touching_body():
    """The grid kernels skip a body for a whole 4^3 block when a distance
    bound at the block centre proves no cell of the block is in contact.
    Check the bound against the contact activation at all 64 cells, for
    capsules and boxes, unit and non-unit quaternions, several softness
    values and rounding radii."""
    rng = np.random.default_rng(7)
    n, dx = 60000, 1.0 / 64
    pose = np.zeros((n, 8), np.float32)
    pose[:, :3] = rng.uniform(0.3, 0.7, (n, 3))
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    q *= rng.choice([1.0, 1.0, 1.0, 0.9, 1.15], size=(n, 1))
    pose[:, 4:] = q
    shapes = np.zeros((n, 8), np.float32)
    shapes[:, 0] = rng.integers(0, 2, n)
    shapes[:, 1] = 0.9
    shapes[:, 2] = rng.choice([666.0, 50.0, 5000.0, 0.0], n)
    shapes[:, 3] = rng.choice([0.0, 0.005], n)
    cap = shapes[:, 0] == 1
    shapes[cap, 4] = rng.uniform(0.008, 0.02, cap.sum())
    shapes[cap, 5] = rng.uniform(0.02, 0.05, cap.sum())
    shapes[~cap, 4:7] = rng.uniform(0.01, 0.05, ((~cap).sum(), 3))
    blk = (np.floor(pose[:, :3] / dx / 4) * 4 + 4 * rng.integers(-3, 3, (n, 3))).astype(np.int32)
    import host_math as H
    may, touched = H.block_cull(pose, shapes, blk, dx)
    assert not np.any(touched & ~may)
    assert touched.sum() > 1000 and (~may).sum() > 0.3 * n


def test_fused_adjoint_entry_checks_arguments(native_lib):
    """dexmpm_p2g_g2p_grad rejects a missing or gradient-less batch, aliased
    gradient buffers and bad slots before any CUDA call, and returns OK
    without a launch for a batch with no particle tiles (the descriptor's
    pointers are placeholders that are never dereferenced on these paths)."""
    import ctypes
    from dexdeform_gb300 import _native as N
    one = ctypes.c_void_p(1)
    two, three, four = ctypes.c_void_p(2), ctypes.c_void_p(3), ctypes.c_void_p(4)
    b = N.DexBatch()
    for f, _ in N.DexBatch._fields_:
        if f not in ("n_envs", "n_particles", "n_tiles", "n_blocks", "n_bodies", "tile_size", "grid_ctas", "flags",
                     "n_slots", "pad0", "pad1", "pad2"):
            setattr(b, f, 4096)  # 16-byte aligned, as the float4 buffers must be
    b.n_envs, b.n_particles, b.n_tiles, b.n_blocks, b.n_bodies = 1, 32, 1, 8, 0
    b.tile_size, b.grid_ctas, b.n_slots = 128, 8, 6
    f = native_lib.dexmpm_p2g_g2p_grad
    bp = ctypes.byref(b)
    ARG = 1
    assert f(None, 3, 2, one, two, three, four, one, None, None) == ARG                   # no batch
    assert f(bp, 3, 2, one, two, three, four, four, None, None) == ARG                    # g_prev == g
    assert f(bp, 3, 2, one, two, three, three, one, None, None) == ARG                    # g == g_next
    assert f(bp, 3, 3, one, two, three, four, one, None, None) == ARG                     # same slot
    assert f(bp, 6, 2, one, two, three, four, one, None, None) == ARG                     # slot out of range
    assert f(bp, 3, 2, None, two, three, four, one, None, None) == ARG                    # no state
    b.vout_grad = None
    assert f(bp, 3, 2, one, two, three, four, one, None, None) == ARG                     # no gradient grids
    b.vout_grad = 4096
    b.n_tiles = 0
    assert f(bp, 3, 2, one, two, three, four, three, None, None) == 0                     # g_prev may be g_next


def test_copy_segments_checks_arguments(native_lib):
    """dexmpm_copy_segments rejects bad counts and modes before any CUDA
    call, and returns OK without a launch when there is nothing to copy."""
    import ctypes
    f = native_lib.dexmpm_copy_segments
    one = ctypes.c_void_p(1)
    ARG = 1
    assert f(one, -1, 24, one, 100, 0, 10, None) == ARG          # negative segment count
    assert f(one, 2, 24, one, 100, 3, 10, None) == ARG           # unknown mode
    assert f(None, 2, 24, one, 100, 0, 10, None) == ARG          # no table
    assert f(None, 0, 24, None, 100, 0, 10, None) == 0           # nothing to copy
    assert f(one, 2, 24, one, 100, 1, 0, None) == 0              # empty segments


def test_render_launchers_reject_bad_arguments(native_lib):
    """Argument checks of particle_sdf / render run before any CUDA call."""
    import ctypes
    P = None
    g = (ctypes.c_int * 3)(8, 8, 8)
    bad = (ctypes.c_int * 3)(0, 8, 8)
    im = (ctypes.c_int * 3)(4, 4, 3)
    one = ctypes.c_void_p(1)  # never dereferenced: rejected before use
    assert native_lib.particle_sdf(P, one, one, one, one, 7, g, 64.0, one, one, one, 10, P) != 0
    assert native_lib.particle_sdf(one, one, one, one, one, 7, bad, 64.0, one, one, one, 10, P) != 0
    args = [one] * 13
    assert native_lib.render(*args, 0.4, g, 65, True, im, 2, 1, 0.0, 0, one, P) != 0   # > 64 bodies
    assert native_lib.render(*args, 0.4, g, 1, True, im, 2, 0, 0.0, 0, one, P) != 0    # spp 0
    assert native_lib.render(*args[:11], P, one, 0.4, g, 1, True, im, 2, 1, 0.0, 0, one, P) != 0  # no color buffer


def test_sort_entry_points_check_arguments(native_lib):
    """dexmpm_sort / dexmpm_permute reject bad arguments before any CUDA call
    and return OK without a launch when there is nothing to move."""
    import ctypes
    from dexdeform_gb300 import _native as N
    one, two = ctypes.c_void_p(1), ctypes.c_void_p(2)
    b = N.DexBatch()
    b.n_envs, b.n_particles, b.n_tiles, b.n_blocks, b.tile_size = 1, 32, 1, 8, 128
    b.envs, b.tiles = 1, 1
    w = N.DexSortWork()
    for f, _ in N.DexSortWork._fields_:
        setattr(w, f, 4096)  # never dereferenced: every call below is refused first
    sort, perm = native_lib.dexmpm_sort, native_lib.dexmpm_permute
    assert sort(None, ctypes.byref(w), one, two, one, None) == N.ERR_ARG          # no batch
    assert sort(ctypes.byref(b), None, one, two, one, None) == N.ERR_ARG          # no scratch
    assert sort(ctypes.byref(b), ctypes.byref(w), one, one, one, None) == N.ERR_ARG  # in place
    w.rank = None
    assert sort(ctypes.byref(b), ctypes.byref(w), one, two, one, None) == N.ERR_ARG  # incomplete scratch
    w.rank = 4096
    w.cell_count = 4100
    assert sort(ctypes.byref(b), ctypes.byref(w), one, two, one, None) == N.ERR_ARG  # cell counts read as int2
    w.cell_count, w.block_total = 4096, 4104
    assert sort(ctypes.byref(b), ctypes.byref(w), one, two, one, None) == N.ERR_ARG  # block totals read as int4
    assert perm(one, one, one, 32, 24, 0, None) == N.ERR_ARG                        # in place
    assert perm(None, one, two, 32, 24, 0, None) == N.ERR_ARG                       # no permutation
    assert perm(one, one, two, -1, 24, 0, None) == N.ERR_ARG                        # negative size
    assert perm(one, one, two, 0, 24, 0, None) == N.OK                              # nothing to move


def test_batch_launchers_refuse_unaligned_vector_buffers(native_lib):
    """The kernels read and write the grid slots, their velocities and
    adjoints, the body shapes and the poses as float4: a buffer that does not
    start on a 16-byte boundary is refused with DEXMPM_ERR_ARG before any CUDA
    call (with no particle tiles an accepted call returns OK unlaunched)."""
    import ctypes
    from dexdeform_gb300 import _native as N
    b = N.DexBatch()
    b.n_envs, b.n_particles, b.n_tiles, b.n_blocks, b.n_bodies = 1, 32, 0, 8, 1
    b.tile_size, b.grid_ctas, b.n_slots = 128, 1, 2
    for f, t in N.DexBatch._fields_:
        if t is ctypes.c_void_p:
            setattr(b, f, 4096)  # never dereferenced
    s, t = ctypes.c_void_p(8192), ctypes.c_void_p(12288)
    g2p, g2p_grad = native_lib.dexmpm_g2p, native_lib.dexmpm_g2p_grad
    assert g2p(ctypes.byref(b), 0, s, t, None) == N.OK
    assert g2p_grad(ctypes.byref(b), 0, s, t, s, t, None) == N.OK
    for field in ("grid", "vout", "body_shape"):
        setattr(b, field, 4104)
        assert g2p(ctypes.byref(b), 0, s, t, None) == N.ERR_ARG, field
        setattr(b, field, 4096)
    for field in ("vout_grad", "in_grad"):
        setattr(b, field, 4104)
        assert g2p_grad(ctypes.byref(b), 0, s, t, s, t, None) == N.ERR_ARG, field
        assert g2p(ctypes.byref(b), 0, s, t, None) == N.OK  # the forward does not use it
        setattr(b, field, 4096)
    odd = ctypes.c_void_p(8200)
    assert native_lib.dexmpm_grid_op(ctypes.byref(b), 0, -1, odd, s, None) == N.ERR_ARG
    assert native_lib.dexmpm_grid_op(ctypes.byref(b), 0, -1, s, odd, None) == N.ERR_ARG
    assert native_lib.dexmpm_grid_op_grad(ctypes.byref(b), 0, odd, s, s, t, None) == N.ERR_ARG
    assert native_lib.dexmpm_grid_op_grad(ctypes.byref(b), 0, s, odd, s, t, None) == N.ERR_ARG
    # the allocation-free entry point, on an otherwise valid 8^3 env with one body
    e = N.DexEnv()
    e.n, e.gx, e.gy, e.gz, e.n_bodies = 32, 8, 8, 8, 1
    e.dx, e.inv_dx, e.dt = 0.125, 8.0, 1e-4
    one = ctypes.c_void_p(4096)
    f = native_lib.dexmpm_substep_noalloc
    assert f(ctypes.byref(e), one, s, one, one, one, odd, one, one, one, None) == N.ERR_ARG  # body shapes
    assert f(ctypes.byref(e), one, s, one, one, one, one, odd, one, one, None) == N.ERR_ARG  # pose
    assert f(ctypes.byref(e), one, s, one, one, one, one, one, odd, one, None) == N.ERR_ARG  # next pose


def test_product_modules_import():
    """Every module of the package imports on a machine without a GPU (no
    CUDA call at import time)."""
    import importlib
    import pkgutil
    import dexdeform_gb300
    names = [m.name for m in pkgutil.iter_modules(dexdeform_gb300.__path__)]
    assert {"engine", "serving", "simulator", "torch_wrapper", "shadow_hand", "hand"} <= set(names)
    for name in names:
        importlib.import_module(f"dexdeform_gb300.{name}")
