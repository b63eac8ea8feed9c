"""The FP64 oracle pinned against the reference's own kernels.

The golden fixtures in tests/golden were produced by DexDeform's
mpm/csrc/integrator.cu itself (compiled for the host, run serially; see
tests/golden/make_golden.py).  The reference computes in FP32, so the
tolerances below are the reference's own FP32 rounding distance from an FP64
evaluation of the same formulas:
  * state after a substep from a non-rest state: ~2e-5 relative in v and C;
  * from the rest state (F = I) v and C are dominated by the stress of
    F - U V^T, a difference of nearly equal FP32 numbers: ~5e-4 relative in v
    and up to ~3e-3 in C (the affine velocity field is itself nearly zero
    there, so its rounding noise is a large fraction of it);
  * adjoint of one substep: ~1e-5 (state gradients), ~2e-4 (body poses).
A transliteration error shows up as O(1) relative error, far above these.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_env, oracle_sim, rel


@pytest.mark.parametrize("name", ["ref_forward_32.npz", "ref_forward_box_32.npz"])
def test_oracle_forward_matches_reference_golden(oracle_mod, name):
    env, z = golden_env(os.path.join(GOLDEN, name))
    o = oracle_sim(oracle_mod, env)
    keep = [int(k) for k in z["keep"]]
    st = env.state()
    for t in range(max(keep)):
        st = o.substep(st, env.pose(t), env.pose(t + 1))
        if t + 1 in keep:
            for k in ("x", "F"):
                assert rel(z[f"s{t + 1}_{k}"], st[k]) < 1e-6, (t + 1, k)
            assert rel(z[f"s{t + 1}_v"], st["v"]) < 2e-3, (t + 1, "v")
            assert rel(z[f"s{t + 1}_C"], st["C"]) < 5e-3, (t + 1, "C")


@pytest.mark.parametrize("name", ["ref_grad_32.npz", "ref_grad_box_32.npz"])
def test_oracle_adjoint_matches_reference_golden(oracle_mod, name):
    env, z = golden_env(os.path.join(GOLDEN, name))
    o = oracle_sim(oracle_mod, env)
    st = {k: z[f"in_{k}"] for k in ("x", "v", "F", "C")}
    nxt = o.substep(st, env.pose(0), env.pose(1))
    for k in ("x", "F"):
        assert rel(z[f"next_{k}"], nxt[k]) < 1e-6, k
    for k in ("v", "C"):
        assert rel(z[f"next_{k}"], nxt[k]) < 2e-4, k
    g, (bp, br), (nbp, nbr) = o.substep_grad(st, env.pose(0), env.pose(1), z["next_v"],
                                             {k: z[f"gnext_{k}"] for k in ("x", "v", "F", "C")})
    for k in ("x", "v", "F", "C"):
        assert rel(z[f"g_{k}"], g[k]) < 2e-4, k
    for a, b in ((z["bpos_grad"], bp), (z["brot_grad"], br), (z["nbpos_grad"], nbp), (z["nbrot_grad"], nbr)):
        assert rel(a, b) < 2e-3


def test_oracle_against_live_reference_build(oracle_mod):
    """Where the reference host build exists (oracle/_ref), check fresh seeds."""
    if not oracle_mod.ref_available():
        pytest.skip("oracle/_ref not built (no reference tree here)")
    from dexdeform_gb300 import workloads as W
    for seed in (11, 12):
        env = W.tiny_env(seed, n=192, grid=32, nb=5, steps=3, dt=1e-4)
        st = W.perturb_state(env, seed=seed, v_scale=0.1, c_scale=1.0, f_scale=0.02)
        o, r = oracle_sim(oracle_mod, env), oracle_sim(oracle_mod, env, "ref")
        a = o.substep(st, env.pose(0), env.pose(1))
        b = r.substep(st, env.pose(0), env.pose(1))
        for k in ("x", "v", "F", "C"):
            assert rel(b[k], a[k]) < 2e-4, (seed, k)
        rng = np.random.default_rng(seed)
        gn = {k: rng.normal(size=st[k].shape).astype(np.float32) for k in st}
        ga, *_ = o.substep_grad(st, env.pose(0), env.pose(1), a["v"], gn)
        gb, *_ = r.substep_grad(st, env.pose(0), env.pose(1), a["v"].astype(np.float32), gn)
        for k in ("x", "v", "F", "C"):
            assert rel(gb[k], ga[k]) < 2e-4, (seed, k)


def test_oracle_svd_conventions(oracle_mod):
    rng = np.random.default_rng(0)
    A = np.eye(3) + rng.normal(size=(300, 3, 3)) * 0.4
    A[:20] = np.eye(3)
    A[20:40, :, 0] *= -1  # reflections: negative determinant
    for mode in ("reference", "exact"):
        oracle_mod.set_svd_mode(mode)
        U, s, V = oracle_mod.svd3(A)
        oracle_mod.set_svd_mode("reference")
        rec = np.einsum("nij,nj,nkj->nik", U, s, V)
        tol = 1e-5 if mode == "reference" else 1e-12
        assert np.abs(rec - A).max() < tol * 10
        assert np.allclose(np.linalg.det(U), 1, atol=1e-6) and np.allclose(np.linalg.det(V), 1, atol=1e-6)
        assert (np.abs(s[:, 0]) >= np.abs(s[:, 1]) - 1e-9).all() and (np.abs(s[:, 1]) >= np.abs(s[:, 2]) - 1e-9).all()
        assert (s[:, :2] >= -1e-12).all()
        assert (np.sign(s[:, 2]) == np.sign(np.linalg.det(A))).all()


def test_oracle_loss_hooks_adjoint_by_finite_differences(oracle_mod):
    """compute_dist / particle2mass adjoints (integrator.cu:188-310) against
    central differences of their own forward."""
    from dexdeform_gb300 import workloads as W
    env = W.tiny_env(2, n=32, grid=32, nb=3, steps=1, dt=1e-4)
    o = oracle_sim(oracle_mod, env)
    x = env.x.astype(np.float64)
    pose = env.pose(0)
    rng = np.random.default_rng(0)
    gd = rng.normal(size=(env.n, env.nb))
    gx, gp, gr = o.compute_dist_grad(x, pose, gd)
    eps = 1e-6
    for (p, c) in [(0, 0), (5, 1), (17, 2)]:
        xp, xm = x.copy(), x.copy()
        xp[p, c] += eps
        xm[p, c] -= eps
        fd = ((o.compute_dist(xp, pose) - o.compute_dist(xm, pose)) * gd).sum() / (2 * eps)
        assert abs(fd - gx[p, c]) < 1e-5 * max(1, abs(fd))
    gm = rng.normal(size=env.grid_dim)
    gxm = o.particle2mass_grad(x, gm)
    for (p, c) in [(1, 0), (9, 2)]:
        xp, xm = x.copy(), x.copy()
        xp[p, c] += eps
        xm[p, c] -= eps
        fd = ((o.particle2mass(xp) - o.particle2mass(xm)) * gm).sum() / (2 * eps)
        assert abs(fd - gxm[p, c]) < 1e-4 * max(1, abs(fd))


def test_render_oracle_matches_reference_fixture(oracle_mod):
    """The renderer restatement (oracle/render_oracle.c) against the
    reference's own particle_sdf and render run on the host with the shared
    counter-based generator: bit-identical volume, image and depth."""
    from conftest import render_fixture, sha256
    sc, ref = render_fixture()
    vol, sdf, colv = oracle_mod.particle_sdf("oracle", sc["x"], sc["color"], sc["bbox_min"], sc["bake"], sc["voxel"],
                                             sc["inv_dx"])
    assert (sha256(vol) == ref["volume_sha256"]).all()
    assert (sha256(sdf) == ref["sdf_sha256"]).all() and (sha256(colv) == ref["color_sha256"]).all()
    img, dep = oracle_mod.render("oracle", sc, sdf, colv)
    assert np.array_equal(img, ref["image"]) and np.array_equal(dep, ref["depth"])
