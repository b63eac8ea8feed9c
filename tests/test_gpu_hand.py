"""The Shadow hand driving the MPM on the GPU: HandSimulator's state tuple and
env step (mpm/hand.py:183-210, :383-440) against the FP64 oracle, and the
gradient of a particle loss wrt the hand's joint-velocity controls through
GradModel against central differences.  The hand model is the committed one
parsed from the reference's MJCF (tests/golden/shadow_rh_model.npz), at the
reference envs' scale 2.5."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, oracle_rollout, rel

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SCALE = 2.5   # mpm/assets/env_cfgs/*.yml SIMULATOR.scale
ROOT = ((0.5, 0.16, 0.3), (0.0, 0.0, 0.0))  # hand base position / static-xyz Euler angles


@pytest.fixture(scope="module")
def cuda(native_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return native_lib


def _model():
    from dexdeform_gb300.shadow_hand import HandModel
    return HandModel.load(os.path.join(GOLDEN, "shadow_rh_model.npz")).scaled(SCALE)


def _object(seed, n):
    """An ellipsoid of particles under the hand's fingers."""
    from dexdeform_gb300 import workloads as W
    env = W.make_env(seed, n, "ellipsoid", grid=64, dt=5e-5, center=(0.5, 0.1, 0.68), extent=(0.14, 0.05, 0.12),
                     nb=1, steps=1, sort=False)
    return env


def test_hand_simulator_state_tuple_and_env_step(cuda, oracle_mod):
    """set_state places the 19 primitives by the kinematics of the tuple's base
    pose and joint angles; get_state returns the tuple; one env step (40
    substeps at quality 1) under joint-velocity + wrist actions moves the
    hand as JointVel_Fk says and the particles as the oracle does (<= 1e-3)."""
    from dexdeform_gb300 import workloads as W
    from dexdeform_gb300.shadow_hand import DEFAULT_INITIAL_QPOS, HandSimulator, ShadowHand, root_matrix
    model = _model()
    obj = _object(3, 3000)
    sim = HandSimulator([model], n_particles=obj.n, max_steps=64, root_frames=root_matrix(*ROOT),
                        gravity=(0.0, -1.0, 0.0), ground_friction=0.9)
    assert sim.n_bodies == 19 and sim.substeps == 40
    sim.init_particles(obj.vol.astype(np.float64), obj.mass.astype(np.float64), obj.mu_lam_yield.astype(np.float64))
    base = root_matrix(*ROOT)[None]
    q = DEFAULT_INITIAL_QPOS[None].copy()
    st = obj.state()
    sim.set_state(0, (st["x"], st["v"], st["F"], st["C"], base, q))
    got = sim.get_state(0)
    assert len(got) == 4 + 19 + 2
    assert np.array_equal(got[0], st["x"]) and np.allclose(got[-2], base) and np.allclose(got[-1], q)
    hand = ShadowHand(model, device="cuda")
    pos, rot = hand.forward_kinematics(torch.tensor(base, dtype=torch.float32, device="cuda")[None],
                                       torch.tensor(q, dtype=torch.float32, device="cuda")[None])
    poses0 = np.stack(got[4:4 + 19])
    assert np.abs(poses0[:, :3] - pos[0].cpu().numpy()).max() < 1e-6

    rng = np.random.default_rng(0)
    action = rng.uniform(-1, 1, (1, 26)).astype(np.float32)
    p_sub, r_sub, (nb, nq) = hand.joint_velocity_fk(torch.tensor(base, dtype=torch.float32, device="cuda"),
                                                    torch.tensor(q, dtype=torch.float32, device="cuda"),
                                                    torch.tensor(action, device="cuda"), sim.substeps)
    sim.step(action)
    end = sim.get_state(0)
    assert np.allclose(end[-2], nb.cpu().numpy(), atol=1e-6) and np.allclose(end[-1], nq.cpu().numpy(), atol=1e-6)
    assert sim._engine().error_word() == 0

    # the oracle, stepping the same per-substep poses
    T = sim.substeps
    poses = np.zeros((T + 1, 19, 7), np.float32)
    poses[0] = poses0
    poses[1:, :, :3] = p_sub.cpu().numpy()
    poses[1:, :, 3:] = r_sub.cpu().numpy()
    tfsr, args = hand.body_shapes(friction=0.9)
    env = W.Env(grid_dim=(64, 64, 64), dx=1 / 64, dt=sim.dt, gravity=(0.0, -30.0, 0.0), ground_friction=0.9,
                x=st["x"], v=st["v"], F=st["F"], C=st["C"], mass=obj.mass, vol=obj.vol, mu_lam_yield=obj.mu_lam_yield,
                body_tfsr=tfsr, body_args=args, poses=poses)
    want = oracle_rollout(oracle_mod, env, T, "exact")[T]
    for k, i in (("x", 0), ("v", 1), ("F", 2), ("C", 3)):
        assert rel(end[i], want[k]) < 1e-3, (k, rel(end[i], want[k]))
    # the hand was in contact: particles inside its primitives at the start
    sim.set_state(0, (st["x"], st["v"], st["F"], st["C"], base, q))
    d = sim.get_dists(0, device="numpy")
    assert d.shape == (obj.n, 19) and (d < 0).any()


def test_controls_gradient_real_hand_by_central_differences(cuda):
    """Joint-velocity controls of the Shadow hand's 20 actuators -> JointVel_Fk
    -> 19 primitive poses -> MPM, 3 env steps x 10 substeps; gradient of a
    particle-to-target loss wrt the controls against central differences
    (eps = 1e-3) on 12 random coordinates.  The exact capsule-normal
    derivative is used (the reference's adjoint drops it)."""
    from dexdeform_gb300.shadow_hand import DEFAULT_INITIAL_QPOS, ShadowHand, root_matrix
    from dexdeform_gb300.torch_wrapper import GradModel
    hand = ShadowHand(_model(), device="cuda", action_scale=np.full(26, 0.02)).set_base(root_matrix(*ROOT))
    env = _object(7, 3000)
    env.body_tfsr, env.body_args = hand.body_shapes()
    S, T = 3, 10
    rng = np.random.default_rng(0)
    actions = torch.tensor(rng.normal(scale=0.3, size=(S, 20)), dtype=torch.float32, device="cuda")
    target = torch.tensor(env.x + rng.normal(scale=0.01, size=env.x.shape).astype(np.float32), device="cuda")
    model = GradModel(env, hand, T, capsule_grad="exact")
    q0 = torch.tensor(DEFAULT_INITIAL_QPOS, dtype=torch.float32, device="cuda")

    def rollout(acts):
        model.zero_grad()
        model.reset(q0)
        for s in range(S):
            obs = model.forward(s, acts[s])
        x = obs[0][:, :3].double()
        return ((x - target.double()) ** 2).sum(1).mean()

    a = actions.clone().requires_grad_(True)
    rollout(a).backward()
    grad = a.grad.reshape(-1).clone()
    assert model.sim.E.error_word() == 0
    assert float(grad.abs().max()) > 0  # the hand drives the particles
    idx = rng.choice(S * 20, size=12, replace=False)
    eps = 1e-3
    fd = []
    with torch.no_grad():
        for i in idx:
            e = torch.zeros(S * 20, device="cuda")
            e[i] = eps
            e = e.reshape(S, 20)
            fd.append(float((rollout(actions + e) - rollout(actions - e)) / (2 * eps)))
    fd = np.array(fd)
    an = grad[idx].cpu().numpy()
    scale = np.abs(an).max()
    # the contact model is discontinuous (a body's influence on a node jumps
    # from 0 to 0.1 at the SDF threshold, integrator.cu:708-710): a 1e-3
    # control step flips a few nodes, which finite differences see and the
    # adjoint (the smooth branch's derivative) does not.  Measured here: 12
    # coordinates, correlation > 0.99, median error 0.06% and the largest
    # 14.5% of the gradient's scale; the bars of the full-size config-1 test
    assert np.corrcoef(fd, an)[0, 1] > 0.98, (fd, an)
    err = np.abs(fd - an) / scale
    assert np.median(err) < 0.05 and err.max() < 0.25, (fd, an)
