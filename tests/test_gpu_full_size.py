"""Parity at the sizes the benchmark runs, through the production path
(BatchEngine + Rollout: fused kernels, kept grid slots, the SVD tape, CUDA
graphs and, for gradients, the overlapped backward), against the FP64 oracle.

* Batching configuration: the benchmark's own 64-env batch (64^3 grids,
  log-uniform 2k-30k particles, cubes and ellipsoids, yield U[30, 80]), in
  sampling order as the benchmark hands it over (the rollout sorts it on the
  device); the smallest, the median and the largest env are compared with the
  oracle.
* Large single env: 128^3 grid, dx 1/128, dt 2.5e-5, 300,000 particles in two
  stacked cubes of yield 40 and 120, 22 capsules and a palm box.

Forward bar: relative L2 error <= 1e-3 on x, v, F, C after full env steps of
50 substeps from the configurations' rest states, against the oracle with
FP32 state storage between substeps (the reference's storage format).
Adjoint bar: the gradients of the initial state (x, v, F, C) and of the body
poses against the oracle's chained substep adjoints (FP32 state storage),
within max(1e-3, 8 x the oracle's own FP32-vs-FP64-storage difference, 8 x
the difference between two GPU runs, 1.25 x the distance of the reference's
own FP32 kernels from the oracle on the same case), from a perturbed state (at F = I every singular value is exactly 1 and the
reference's SVD adjoint multiplies FP32 rounding by its clamped
1 / (sigma_j^2 - sigma_i^2) = 1e6 factors; away from rest the gradient is
well conditioned).
"""
import numpy as np
import pytest

from conftest import oracle_chain_adjoint, oracle_rollout, rel

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def cuda(native_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return native_lib


def _rollout(envs, T, S):
    from dexdeform_gb300.engine import BatchEngine, EnvSpec, Rollout
    E = BatchEngine([EnvSpec.from_env(e) for e in envs], grad=True, grid_slots=2 * T + 2)
    R = Rollout(E, substeps=T, env_steps=S)
    R.poses.copy_(torch.tensor(E.pack_poses([e.poses[:, :, :3] for e in envs], [e.poses[:, :, 3:] for e in envs]),
                               device="cuda")[:S * T + 1])
    return E, R


def _sampled(envs):
    """Indices of the smallest, the median and the largest env."""
    order = np.argsort([e.n for e in envs], kind="stable")
    return [int(order[0]), int(order[len(order) // 2]), int(order[-1])]


def _seeded_gradient(E, envs, seed):
    rng = np.random.default_rng(seed)
    per_env = []
    for e in envs:
        per_env.append({"x": rng.normal(size=(e.n, 3)).astype(np.float32),
                        "v": rng.normal(size=(e.n, 3)).astype(np.float32),
                        "F": rng.normal(size=(e.n, 3, 3)).astype(np.float32),
                        "C": rng.normal(size=(e.n, 3, 3)).astype(np.float32)})
    return per_env, E.pack_state(per_env)


def _gradients_twice(E, R, state0, g_final):
    """Forward + backward twice: the gradients of the first run and the GPU's
    own run-to-run spread (the float atomics add in a different order)."""
    out = []
    for _ in range(2):
        R.forward(state0)
        out.append((E.unpack_state(R.backward(g_final).clone()), R.bgrad.cpu().numpy()))
    assert E.error_word() == 0
    return out


def _check_adjoint(O, E, R, runs, envs, idx, st0, g_env, T, S, ref_pose=None, ref=None):
    """The GPU's gradients of the initial state and of the body poses against
    the oracle's chained adjoint with FP32 state storage.  The bar is set by
    the rounding sensitivities of the same quantity: d, the distance between
    the oracle's FP32- and FP64-storage gradients; e, the distance between
    two GPU runs (a body-pose gradient sums the contributions of thousands of
    grid nodes in FP32, in an order the atomics change); and r, how far the
    reference's own FP32 kernels land from the oracle on the same case.  The
    test holds the GPU to max(1e-3, 8 d, 8 e, 1.25 r), and the particles whose
    gradient is off by more than 5% of the field's RMS to under max(0.1%,
    2 x the reference's own fraction).  ref (per env of idx, from a fixture):
    {"distance": {field: r}, "outliers": {field: fraction}} with the fields
    x, v, F, C, "pose position", "pose rotation".  ref_pose (position,
    rotation gradients of the reference's own FP32 kernels on the same
    states, for a single env): r of the pose gradients computed here."""
    (g0, bg), (g0b, bgb) = runs
    for i, e in enumerate(idx):
        env = envs[e]
        rd = ref[i]["distance"] if ref is not None else {}
        rf = ref[i]["outliers"] if ref is not None else {}
        res = {}
        for storage in ("fp32", "fp64"):
            states = oracle_rollout(O, env, S * T, "exact", state=st0[e], storage=storage)
            res[storage] = oracle_chain_adjoint(O, env, [states[t] for t in range(S * T + 1)], g_env[e], "exact")
        (want, bp, br), (w64, bp64, br64) = res["fp32"], res["fp64"]
        for k in ("x", "v", "F", "C"):
            err, d, n, r = rel(g0[e][k], want[k]), rel(want[k], w64[k]), rel(g0[e][k], g0b[e][k]), rd.get(k, 0.0)
            assert err < max(1e-3, 8 * d, 8 * n, 1.25 * r), (env.name, env.n, k, err, d, n, r)
            dev = np.linalg.norm((g0[e][k] - want[k]).reshape(env.n, -1), axis=1)
            rms = np.sqrt((np.asarray(want[k]).reshape(env.n, -1) ** 2).sum(1).mean())
            frac = float((dev > 0.05 * rms).mean())
            assert frac < max(1e-3, 2 * rf.get(k, 0.0)), (env.name, k, frac, rf.get(k))
        o = E.body_off[e]
        for got, other, w, w2, what in ((bg[:, o:o + env.nb, :3], bgb[:, o:o + env.nb, :3], bp, bp64,
                                         "pose position"),
                                        (bg[:, o:o + env.nb, 4:], bgb[:, o:o + env.nb, 4:], br, br64,
                                         "pose rotation")):
            err, d, n = rel(got, w), rel(w, w2), rel(got, other)
            r = rd.get(what, 0.0)
            if ref_pose is not None:
                r = rel(ref_pose[0] if what == "pose position" else ref_pose[1], w)
            assert err < max(1e-3, 8 * d, 8 * n, 1.25 * r), (env.name, what, err, d, n, r)


def test_batch_config_full_size_forward(cuda, oracle_mod):
    """The benchmark batch, one env step of 50 substeps (the kept last env
    step of a gradient rollout, and the forward-only path), against the
    oracle for the smallest, median and largest env."""
    from dexdeform_gb300 import workloads as W
    T = 50
    envs = W.batch_envs(0, n_envs=64, steps=T, sort=False)  # sampling order: the rollout sorts
    assert sum(e.n for e in envs) > 600000
    E, R = _rollout(envs, T, 1)
    s0 = E.pack_state([e.state() for e in envs])
    kept = E.unpack_state(R.forward(s0).clone())
    plain = E.unpack_state(R.forward(s0, keep_last=False).clone())
    assert E.error_word() == 0
    for e in _sampled(envs):
        env = envs[e]
        want = oracle_rollout(oracle_mod, env, T, "exact")[T]
        for k in ("x", "v", "F", "C"):
            assert rel(kept[e][k], want[k]) < 1e-3, (env.name, env.n, k, rel(kept[e][k], want[k]))
            assert rel(plain[e][k], want[k]) < 1e-3, (env.name, env.n, k, rel(plain[e][k], want[k]))


def test_batch_config_full_size_adjoint(cuda, oracle_mod):
    """The benchmark batch, 3 env steps x 5 substeps forward + backward with
    the overlapped schedule (env step k - 1 recomputed on a second stream
    while the adjoint of env step k runs), from a perturbed state with a
    seeded gradient on every field of the final state.

    Here the gradient of the initial state is ill-conditioned in FP32 at a
    few particles whose singular values nearly coincide (the SVD adjoint
    divides by their squared difference): on the largest env one particle
    carries half of the distance between the reference's own FP32 kernels
    and the FP64 oracle, 5.3e-3 in x (tests/golden/ref_batch_adjoint.npz,
    tests/golden/make_ref_batch_adjoint.py).  The GPU is held to no further
    than the reference on every field and env."""
    import os
    from conftest import GOLDEN
    from dexdeform_gb300 import workloads as W
    T, S = 5, 3
    z = np.load(os.path.join(GOLDEN, "ref_batch_adjoint.npz"))
    assert int(z["substeps"]) == S * T and int(z["state_seed"]) == 7 and int(z["grad_seed"]) == 3
    envs = W.batch_envs(0, n_envs=64, steps=S * T, sort=False)
    idx = _sampled(envs)
    assert list(z["envs"]) == idx
    names = [str(f).replace("_", " ") for f in z["fields"]]
    ref = [{"distance": dict(zip(names, z["distance"][i])), "outliers": dict(zip(names, z["outlier_fraction"][i]))}
           for i in range(len(idx))]
    E, R = _rollout(envs, T, S)
    assert R.overlap
    st0 = [W.perturb_state(e, seed=7, v_scale=0.1, c_scale=1.0, f_scale=0.02) for e in envs]
    g_env, g_final = _seeded_gradient(E, envs, 3)
    runs = _gradients_twice(E, R, E.pack_state(st0), g_final)
    _check_adjoint(oracle_mod, E, R, runs, envs, idx, st0, g_env, T, S, ref=ref)


def test_large_config_forward(cuda, oracle_mod):
    """128^3, 300,000 particles, yield 40 / 120, capsules and a palm box: two
    env steps of 50 substeps, compared after each."""
    from dexdeform_gb300 import workloads as W
    T, S = 50, 2
    env = W.large_env(0, steps=S * T, sort=False)
    assert env.n == 300000 and env.grid_dim == (128, 128, 128) and env.dt == 2.5e-5
    assert (env.body_tfsr[:, 0] == 0).sum() == 1  # the palm box
    E, R = _rollout([env], T, S)
    s0 = E.pack_state([env.state()])
    R.forward(s0)
    got = {k: E.unpack_state(R.state(k))[0] for k in (1, 2)}
    assert E.error_word() == 0
    want = oracle_rollout(oracle_mod, env, S * T, "exact")
    for k in (1, 2):
        for f in ("x", "v", "F", "C"):
            assert rel(got[k][f], want[k * T][f]) < 1e-3, (k * T, f, rel(got[k][f], want[k * T][f]))


def test_large_config_adjoint(cuda, oracle_mod):
    """The large env, 2 env steps x 5 substeps forward + backward (overlapped
    schedule), from a perturbed state.

    Its body-pose gradients are ill-conditioned in FP32: a pose row sums, over
    every node a body touches, terms of order 1/dt (dt = 2.5e-5) from the
    body velocity, once as the current and once as the next pose of adjacent
    substeps, with opposite signs.  Measured: GPU 6.5e-3 (position) from the
    FP64 oracle, the same in every schedule (sorted or not, overlapped or not,
    any slot count); the reference's own FP32 kernels on the same states
    6.2e-2 (position) and 2.5e-2 (rotation)
    (tests/golden/ref_large_pose_grad.npz, tests/golden/make_ref_large_pose.py).
    The pose gradients are therefore held to no further from the oracle than
    the reference's own kernels."""
    import os
    from conftest import GOLDEN
    from dexdeform_gb300 import workloads as W
    T, S = 5, 2
    ref = np.load(os.path.join(GOLDEN, "ref_large_pose_grad.npz"))
    assert int(ref["substeps"]) == S * T and int(ref["state_seed"]) == 8 and int(ref["grad_seed"]) == 4
    env = W.large_env(0, steps=S * T, sort=False)
    E, R = _rollout([env], T, S)
    assert R.overlap
    st0 = [W.perturb_state(env, seed=8, v_scale=0.1, c_scale=1.0, f_scale=0.02)]
    g_env, g_final = _seeded_gradient(E, [env], 4)
    runs = _gradients_twice(E, R, E.pack_state(st0), g_final)
    _check_adjoint(oracle_mod, E, R, runs, [env], [0], st0, g_env, T, S,
                   ref_pose=(ref["pose_position"], ref["pose_rotation"]))
