"""Edge cases of the batched path on the GPU: a batch that holds an env with
no particles and an env with no bodies, through the production rollout
(device sort at every env step, kept slots, tape, overlapped backward).

* The empty env changes nothing for the others: every other env's final
  state, initial-state gradient and body-pose gradients equal those of the
  same rollout without it, within the schedule-equivalence bars (the float
  atomics add in another order in each run): states 2e-4, gradients 5e-4,
  or 4 x the spread of two identical runs where that is larger.
* The body-less env matches the FP64 oracle after 10 substeps from a
  perturbed state (1e-3).
* A batch of empty envs only runs and returns nothing to do.
"""
import numpy as np
import pytest

from conftest import oracle_rollout, rel, within_spread

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def cuda(native_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return native_lib


T, S = 5, 2


def _envs():
    from dexdeform_gb300 import workloads as W
    a = W.make_env(21, 1500, "cube", grid=32, center=(0.5, 0.2, 0.5), extent=0.25, nb=3, steps=S * T, sort=False)
    empty = W.make_env(22, 0, "cube", grid=32, nb=2, steps=S * T, sort=False)
    bodyless = W.make_env(23, 800, "ellipsoid", grid=48, center=(0.5, 0.15, 0.5), extent=(0.12, 0.06, 0.09), nb=0,
                          steps=S * T, sort=False)
    c = W.make_env(24, 2000, "cube", grid=32, center=(0.5, 0.25, 0.5), extent=0.3, nb=5, steps=S * T, sort=False)
    return [a, empty, bodyless, c]


def _seeded_gradient(env):
    """A gradient of the final state on every field, seeded by the env (so
    that it is the same whatever batch the env is in).  A uniform one (1 on
    every x and v) would leave the F and C gradients of a freely falling
    body as FP32 residues of cancelling node sums (sum_n N_n dpos_n = 0)."""
    rng = np.random.default_rng(1000 + int(env.n))
    return {"x": rng.normal(size=(env.n, 3)).astype(np.float32), "v": rng.normal(size=(env.n, 3)).astype(np.float32),
            "F": rng.normal(size=(env.n, 3, 3)).astype(np.float32),
            "C": rng.normal(size=(env.n, 3, 3)).astype(np.float32)}


def _run(envs):
    """Forward + backward of S env steps x T substeps; per env: final state,
    gradient of the initial state, body-pose gradients."""
    from dexdeform_gb300 import workloads as W
    from dexdeform_gb300.engine import BatchEngine, EnvSpec, Rollout
    E = BatchEngine([EnvSpec.from_env(e) for e in envs], grad=True, grid_slots=2 * T + 2)
    R = Rollout(E, substeps=T, env_steps=S)
    R.poses.copy_(torch.tensor(E.pack_poses([e.poses[:, :, :3] for e in envs], [e.poses[:, :, 3:] for e in envs]),
                               device="cuda")[:S * T + 1])
    s0 = E.pack_state([W.perturb_state(e, seed=9, v_scale=0.1, c_scale=1.0, f_scale=0.02) for e in envs])
    g = E.pack_state([_seeded_gradient(e) for e in envs])
    fin = E.unpack_state(R.forward(s0).clone())
    g0 = E.unpack_state(R.backward(g).clone())
    bg = R.bgrad.cpu().numpy()
    assert E.error_word() == 0
    return [(fin[e], g0[e], bg[:, E.body_off[e]:E.body_off[e] + envs[e].nb]) for e in range(len(envs))]


def test_empty_env_changes_nothing_for_the_others(cuda):
    envs = _envs()
    with_empty = _run(envs)
    without = _run([envs[0], envs[2], envs[3]])
    again = _run([envs[0], envs[2], envs[3]])  # the spread of two identical runs
    assert with_empty[1][0]["x"].shape == (0, 3) and with_empty[1][1]["x"].shape == (0, 3)
    for got, want, rep in zip([with_empty[0], with_empty[2], with_empty[3]], without, again):
        for k in ("x", "v", "F", "C"):
            within_spread((got[0][k], got[1][k]), (want[0][k], want[1][k]), (rep[0][k], rep[1][k]), (2e-4, 5e-4))
        if want[2].size:
            within_spread((got[2],), (want[2],), (rep[2],), (5e-4,))
    assert with_empty[2][2].size == 0  # no bodies, no pose gradients


def test_bodyless_env_matches_oracle(cuda, oracle_mod):
    from dexdeform_gb300.engine import BatchEngine, EnvSpec, Rollout
    envs = _envs()
    E = BatchEngine([EnvSpec.from_env(e) for e in envs])
    R = Rollout(E, substeps=S * T, env_steps=1)
    R.poses.copy_(torch.tensor(E.pack_poses([e.poses[:, :, :3] for e in envs], [e.poses[:, :, 3:] for e in envs]),
                               device="cuda")[:S * T + 1])
    from dexdeform_gb300 import workloads as W
    st = [W.perturb_state(e, seed=4, v_scale=0.1, c_scale=1.0, f_scale=0.02) for e in envs]
    fin = E.unpack_state(R.forward(E.pack_state(st)).clone())
    assert E.error_word() == 0
    want = oracle_rollout(oracle_mod, envs[2], S * T, "exact", state=st[2])[S * T]
    for k in ("x", "v", "F", "C"):
        assert rel(fin[2][k], want[k]) < 1e-3, k
    assert np.isfinite(fin[0]["x"]).all() and np.isfinite(fin[3]["x"]).all()


def test_batch_of_empty_envs(cuda):
    from dexdeform_gb300 import workloads as W
    from dexdeform_gb300.engine import BatchEngine, EnvSpec
    envs = [W.make_env(30 + i, 0, "cube", grid=32, nb=2, steps=2) for i in range(3)]
    E = BatchEngine([EnvSpec.from_env(e) for e in envs], grad=True, grid_slots=4)
    poses = torch.tensor(E.pack_poses([e.poses[:, :, :3] for e in envs], [e.poses[:, :, 3:] for e in envs]),
                         device="cuda")
    sts = E.new_slots(3)
    E.run_substeps(list(sts), poses, kept=True, tapes=E.new_tape(2))
    g = E.new_slots(2)
    bg = torch.zeros((3, max(E.n_bodies, 1), 8), device="cuda")
    E.run_adjoint(list(sts), g[0], g[1], poses, bg, tapes=E.new_tape(2))
    perm = E.identity_perm(1)[0]
    E.sort(sts[0], sts[1], perm)
    torch.cuda.synchronize()
    assert E.error_word() == 0 and E.active_blocks(2) == 0 and float(bg.abs().sum()) == 0.0
