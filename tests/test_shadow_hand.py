"""Shadow-hand kinematics (dexdeform_gb300.shadow_hand) against the
reference's own hand code: fixtures written by tests/golden/make_shadow_fk.py
from DexDeform's mpm/mujoco_parser.py + mpm/hand.py (forward kinematics of the
19 collision primitives, JointVel_Fk with and without a wrist twist) and the
joint / actuator tables of mpm/robots/interface.py.  CPU only (pure torch).

Bars: positions within 1e-6 m and quaternions within 1e-6 (up to sign: q and
-q are one rotation) of the reference's FP32 results; tables equal to FP32
rounding; the parser, where the reference's MJCF is present, equal to the
committed model."""
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN

MJCF = {"rh": "right_hand", "lh": "left_hand"}
REF_ASSETS = os.path.join(os.environ.get("REF_ROOT", "/root/reference"), "mpm", "assets", "robots", "shadow")


def _q_close(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.minimum(np.abs(a - b).max(-1), np.abs(a + b).max(-1)).max()


def _load(mode):
    from dexdeform_gb300.shadow_hand import HandModel, ShadowHand
    z = np.load(os.path.join(GOLDEN, f"shadow_{mode}_fk.npz"))
    model = HandModel.load(os.path.join(GOLDEN, f"shadow_{mode}_model.npz"))
    return z, model, ShadowHand(model, device="cpu")


@pytest.mark.parametrize("mode", ["rh", "lh"])
def test_forward_kinematics_matches_reference(mode):
    z, model, hand = _load(mode)
    assert model.n_geoms == 19 and (model.geom_type == z["types"]).all()
    pos, rot = hand.forward_kinematics(torch.tensor(z["base"]), torch.tensor(z["q"]))
    assert np.abs(pos.numpy() - z["pos"]).max() < 1e-6
    assert _q_close(rot.numpy(), z["rot"]) < 1e-6


@pytest.mark.parametrize("mode", ["rh", "lh"])
def test_joint_velocity_control_matches_reference(mode):
    """JointVel_Fk from the default joint angles: 26 actions (joint velocities
    and a wrist twist) for one env step, then 20 (joints only) for the next."""
    z, model, hand = _load(mode)
    T = int(z["substeps"])
    base0, q0 = torch.tensor(z["root_frame"]), torch.tensor(z["q0"])
    p, r, (b, q) = hand.joint_velocity_fk(base0, q0, torch.tensor(z["a26"]), T)
    assert p.shape == (T, 19, 3) and r.shape == (T, 19, 4)
    assert np.abs(p.numpy() - z["pos26"]).max() < 1e-6 and _q_close(r.numpy(), z["rot26"]) < 1e-6
    assert np.abs(b.numpy() - z["base26"]).max() < 1e-6 and np.abs(q.numpy() - z["q26"]).max() < 1e-6
    p, r, (b, q) = hand.joint_velocity_fk(b, q, torch.tensor(z["a20"]), T)
    assert np.abs(p.numpy() - z["pos20"]).max() < 1e-6 and _q_close(r.numpy(), z["rot20"]) < 1e-6
    assert np.abs(q.numpy() - z["q20"]).max() < 1e-6


def test_tables_match_reference():
    from dexdeform_gb300 import shadow_hand as S
    z, model, hand = _load("rh")
    lo, hi = S.joint_limits()
    assert np.abs(lo - z["q_lower"]).max() < 1e-7 and np.abs(hi - z["q_upper"]).max() < 1e-7
    assert (S.actuator_of_joint() == z["action_map"]).all()
    assert np.abs(S.default_action_scale() - z["action_scale"]).max() < 1e-8
    assert np.abs(S.DEFAULT_INITIAL_QPOS - z["q0"][0]).max() < 1e-7
    tfsr, args = hand.body_shapes(friction=0.9)
    assert (tfsr[:, 0] == z["types"]).all() and np.abs(args[:, :3] - z["sizes"]).max() < 1e-7
    assert np.abs(S.default_root_frame(model) - z["root_frame"][0]).max() < 1e-6


@pytest.mark.parametrize("mode", ["rh", "lh"])
def test_parser_reproduces_committed_model(mode):
    path = os.path.join(REF_ASSETS, MJCF[mode], "shadow_hand.xml")
    if not os.path.isfile(path):
        pytest.skip("the reference's MJCF is not present")
    from dexdeform_gb300.shadow_hand import HandModel, parse_mjcf
    got = parse_mjcf(path)
    want = HandModel.load(os.path.join(GOLDEN, f"shadow_{mode}_model.npz"))
    for k in ("parent", "geom_joint", "geom_type"):
        assert (getattr(got, k) == getattr(want, k)).all(), k
    for k in ("M", "p", "axis", "G", "geom_size"):
        assert np.abs(getattr(got, k) - getattr(want, k)).max() < 1e-12, k
    assert got.geom_name == want.geom_name


def test_kinematics_is_differentiable():
    """Gradients of the geom poses wrt the joint angles and the base pose,
    against central differences in double precision."""
    from dexdeform_gb300.shadow_hand import HandModel, ShadowHand
    model = HandModel.load(os.path.join(GOLDEN, "shadow_rh_model.npz"))
    hand = ShadowHand(model, device="cpu", dtype=torch.float64)
    z = np.load(os.path.join(GOLDEN, "shadow_rh_fk.npz"))
    base = torch.tensor(z["base"][:1], dtype=torch.float64)
    q = torch.tensor(z["q"][:1], dtype=torch.float64, requires_grad=True)
    w = torch.linspace(-1, 1, 19 * 7, dtype=torch.float64).reshape(19, 7)

    def f(qq):
        p, r = hand.forward_kinematics(base, qq)
        return (torch.cat([p[0], r[0]], -1) * w).sum()

    f(q).backward()
    g = q.grad.clone()
    eps = 1e-6
    for i in range(0, 24, 5):
        e = torch.zeros_like(q)
        e[..., i] = eps
        fd = (f(q.detach() + e) - f(q.detach() - e)) / (2 * eps)
        assert abs(float(fd) - float(g[..., i])) < 1e-6 * max(1.0, abs(float(fd)))


def test_rotation_conversions_round_trip():
    from dexdeform_gb300.shadow_hand import axis_angle_to_matrix, matrix_to_quaternion, quaternion_to_matrix
    rng = np.random.default_rng(0)
    v = torch.tensor(rng.normal(size=(2000, 3)) * np.array([[1.0], [1e-5], [3.1]]).repeat(667, 0)[:2000],
                     dtype=torch.float64)
    R = axis_angle_to_matrix(v)
    eye = torch.eye(3, dtype=torch.float64)
    assert (R @ R.transpose(-1, -2) - eye).abs().max() < 1e-12
    q = matrix_to_quaternion(R)
    assert (q[:, 0] >= 0).all() and ((q * q).sum(-1) - 1).abs().max() < 1e-12
    assert (quaternion_to_matrix(q) - R).abs().max() < 1e-12
