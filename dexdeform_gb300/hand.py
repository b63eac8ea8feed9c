"""Differentiable hand kinematics producing per-substep capsule poses.

Mirrors the control path of mpm/hand.py (JointVel_Fk, :383-428): joint
velocity actions are integrated over the substeps of an env step
(q_k = q + a * scale * (k+1), clamped to joint limits) and forward kinematics
maps joint angles to the world poses of the collision capsules.  The Shadow
hand's MJCF tree (mpm/assets/robots/shadow, parsed by mpm/mujoco_parser.py with
pytorch3d / transforms3d, none of which is part of this build) is replaced by a
fixed 24-joint, 22-capsule hand of the same structure: 2 wrist joints, four
4-joint fingers (one with an extra metacarpal joint), a 5-joint thumb; capsules
on the palm and on every phalanx.  Pure torch, batched over envs and substeps.
"""
from __future__ import annotations

import math

import torch

# (name, parent index or -1, joint axis in parent frame, joint origin in parent frame, limits)
# Lengths in metres; the palm is ~9 cm long, fingers ~3-4 cm per two phalanges.
_J = []


def _add(name, parent, axis, origin, lo, hi):
    _J.append((name, parent, axis, origin, lo, hi))
    return len(_J) - 1


_wr2 = _add("WRJ2", -1, (0.0, 0.0, 1.0), (0.0, 0.0, 0.0), -0.5, 0.2)
_wr1 = _add("WRJ1", _wr2, (1.0, 0.0, 0.0), (0.0, 0.0, 0.0), -0.7, 0.5)
FINGER_BASES = {"FF": (-0.033, 0.095, 0.0), "MF": (-0.011, 0.099, 0.0), "RF": (0.011, 0.095, 0.0),
                "LF": (0.033, 0.086, 0.0)}
for f, base in FINGER_BASES.items():
    parent = _wr1
    if f == "LF":
        parent = _add("LFJ5", parent, (0.0, 0.57, 0.82), (0.033, 0.02, 0.0), 0.0, 0.785)
        base = (0.0, 0.066, 0.0)
    j4 = _add(f + "J4", parent, (0.0, 0.0, 1.0), base, -0.35, 0.35)
    j3 = _add(f + "J3", j4, (1.0, 0.0, 0.0), (0.0, 0.0, 0.0), -0.26, 1.57)
    j2 = _add(f + "J2", j3, (1.0, 0.0, 0.0), (0.0, 0.045, 0.0), 0.0, 1.57)
    _add(f + "J1", j2, (1.0, 0.0, 0.0), (0.0, 0.025, 0.0), 0.0, 1.57)
_t5 = _add("THJ5", _wr1, (0.0, 0.0, -1.0), (-0.034, 0.029, 0.009), -1.05, 1.05)
_t4 = _add("THJ4", _t5, (0.71, 0.0, 0.71), (0.0, 0.0, 0.0), 0.0, 1.22)
_t3 = _add("THJ3", _t4, (0.71, 0.0, 0.71), (0.0, 0.038, 0.0), -0.21, 0.21)
_t2 = _add("THJ2", _t3, (0.0, 0.0, 1.0), (0.0, 0.0, 0.0), -0.7, 0.7)
_t1 = _add("THJ1", _t2, (0.0, 0.0, 1.0), (0.0, 0.032, 0.0), -0.26, 1.57)

JOINTS = [j[0] for j in _J]
assert len(JOINTS) == 24

# capsules: (joint index frame, centre offset in that frame, radius, length); axis = frame y
_C = []
for f in FINGER_BASES:
    j3, j2, j1 = JOINTS.index(f + "J3"), JOINTS.index(f + "J2"), JOINTS.index(f + "J1")
    _C += [(j3, (0.0, 0.0225, 0.0), 0.0100, 0.045), (j2, (0.0, 0.0125, 0.0), 0.0095, 0.025),
           (j1, (0.0, 0.0130, 0.0), 0.0090, 0.026)]
_C += [(JOINTS.index("LFJ5"), (0.0, 0.033, 0.0), 0.011, 0.066)]
_C += [(_t4, (0.0, 0.019, 0.0), 0.013, 0.038), (_t2, (0.0, 0.016, 0.0), 0.011, 0.032),
       (_t1, (0.0, 0.014, 0.0), 0.010, 0.028)]
_C += [(_wr1, (x, 0.045, 0.0), 0.012, 0.05) for x in (-0.03, -0.01, 0.01, 0.03)]
_C += [(_wr1, (0.0, 0.015, 0.0), 0.012, 0.05), (_wr1, (0.0, 0.075, -0.01), 0.011, 0.06)]
N_BODIES = len(_C)
assert N_BODIES == 22


# The joints by depth in the tree: every joint of a level has its parent in
# an earlier level, so a level's joints are placed together.
def _levels():
    depth = []
    for name, parent, *_ in _J:
        depth.append(0 if parent < 0 else depth[parent] + 1)
    return [[j for j in range(len(_J)) if depth[j] == d] for d in range(max(depth) + 1)]


def _hamilton():
    """H with (a b)_i = sum_jk H[i, j, k] a_j b_k for quaternions w, x, y, z."""
    H = torch.zeros(4, 4, 4)
    for i, j, k, s in ((0, 0, 0, 1), (0, 1, 1, -1), (0, 2, 2, -1), (0, 3, 3, -1),
                       (1, 0, 1, 1), (1, 1, 0, 1), (1, 2, 3, 1), (1, 3, 2, -1),
                       (2, 0, 2, 1), (2, 1, 3, -1), (2, 2, 0, 1), (2, 3, 1, 1),
                       (3, 0, 3, 1), (3, 1, 2, 1), (3, 2, 1, -1), (3, 3, 0, 1)):
        H[i, j, k] = s
    return H


def _rotation_form():
    """R with rot(q)_ij = sum_kl R[i, j, k, l] q_k q_l for unit quaternions
    (the identity part of the rotation matrix written as |q|^2)."""
    R = torch.zeros(3, 3, 4, 4)
    w, x, y, z = 0, 1, 2, 3
    def put(i, j, terms):
        for k, l, s in terms:
            R[i, j, k, l] += s
    put(0, 0, ((w, w, 1), (x, x, 1), (y, y, -1), (z, z, -1)))
    put(1, 1, ((w, w, 1), (x, x, -1), (y, y, 1), (z, z, -1)))
    put(2, 2, ((w, w, 1), (x, x, -1), (y, y, -1), (z, z, 1)))
    put(0, 1, ((x, y, 2), (w, z, -2)))
    put(0, 2, ((x, z, 2), (w, y, 2)))
    put(1, 0, ((x, y, 2), (w, z, 2)))
    put(1, 2, ((y, z, 2), (w, x, -2)))
    put(2, 0, ((x, z, 2), (w, y, -2)))
    put(2, 1, ((y, z, 2), (w, x, 2)))
    return R


def _qmul(H, a, b):
    return torch.einsum("ijk,...j,...k->...i", H, a, b)


def _qrot(R, q, v):
    """Rotate v by the unit quaternion q."""
    return torch.einsum("ijkl,...k,...l,...j->...i", R, q, q, v)


class SyntheticHand:
    """24 joint angles -> 22 capsule world poses (pos, quat wxyz)."""

    def __init__(self, device="cuda", base_pos=(0.5, 0.2, 0.5), base_rot=(0.7071068, 0.7071068, 0.0, 0.0),
                 action_scale=0.01):
        self.device = torch.device(device)
        f = dict(dtype=torch.float32, device=self.device)
        self.axes = torch.tensor([j[2] for j in _J], **f)
        self.origins = torch.tensor([j[3] for j in _J], **f)
        self.lower = torch.tensor([j[4] for j in _J], **f)
        self.upper = torch.tensor([j[5] for j in _J], **f)
        self.parents = [j[1] for j in _J]
        self.cap_joint = [c[0] for c in _C]
        self.cap_off = torch.tensor([c[1] for c in _C], **f)
        self.radius = torch.tensor([c[2] for c in _C], **f)
        self.length = torch.tensor([c[3] for c in _C], **f)
        self.base_pos = torch.tensor(base_pos, **f)
        self.base_rot = torch.tensor(base_rot, **f)
        self.action_scale = action_scale
        self.H, self.R = _hamilton().to(**f), _rotation_form().to(**f)
        self.unit_axes = self.axes / torch.linalg.norm(self.axes, dim=-1, keepdim=True)
        # per level: its joints, and where each one's parent sits in the
        # running table of world poses (row 0 the base, then the levels in order)
        row = {}
        self.level_joints, self.level_parent_rows = [], []
        n = 1
        for js in _levels():
            self.level_joints.append(torch.tensor(js, dtype=torch.long, device=self.device))
            self.level_parent_rows.append(torch.tensor([0 if _J[j][1] < 0 else row[_J[j][1]] for j in js],
                                                       dtype=torch.long, device=self.device))
            for j in js:
                row[j] = n
                n += 1
        self.cap_rows = torch.tensor([row[j] for j in self.cap_joint], dtype=torch.long, device=self.device)

    def body_shapes(self):
        """(22, 4) type friction softness round, (22, 4) args (radius, length)."""
        import numpy as np
        from .workloads import BODY_FRICTION, SOFTNESS
        tfsr = np.zeros((N_BODIES, 4), np.float32)
        tfsr[:, 0], tfsr[:, 1], tfsr[:, 2] = 1.0, BODY_FRICTION, SOFTNESS
        args = np.zeros((N_BODIES, 4), np.float32)
        args[:, 0] = self.radius.cpu().numpy()
        args[:, 1] = self.length.cpu().numpy()
        return tfsr, args

    def fk(self, q):
        """q (..., 24) -> pos (..., 22, 3), rot (..., 22, 4).  Joint j's world
        frame is its parent's composed with the joint's offset (translation
        origin_j in the parent frame) and rotation (angle q_j about axis_j);
        a capsule sits at an offset in its joint's frame.  The joints of one
        depth of the tree are done together."""
        lead = q.shape[:-1]
        Q = self.base_rot.expand(*lead, 1, 4)   # world rotations, row 0 the base
        P = self.base_pos.expand(*lead, 1, 3)   # world positions
        for js, rows in zip(self.level_joints, self.level_parent_rows):
            pq, pp = Q.index_select(-2, rows), P.index_select(-2, rows)
            h = q.index_select(-1, js)[..., None] * 0.5
            local = torch.cat([torch.cos(h), torch.sin(h) * self.unit_axes[js]], -1)
            P = torch.cat([P, pp + _qrot(self.R, pq, self.origins[js].expand(pq.shape[:-1] + (3,)))], -2)
            Q = torch.cat([Q, _qmul(self.H, pq, local)], -2)
        cq, cp = Q.index_select(-2, self.cap_rows), P.index_select(-2, self.cap_rows)
        pos = cp + _qrot(self.R, cq, self.cap_off.expand(cq.shape[:-1] + (3,)))
        return pos, cq

    def joint_velocity_poses(self, q0, action, substeps):
        """mpm/hand.py:383-428 for a fixed base: q_k = clamp(q0 + a*scale*(k+1)),
        k = 0..substeps-1.  q0 (..., 24), action (..., 24) in [-1, 1].
        Returns poses (substeps, ..., 22, 3/4) and the final joint angles."""
        a = action.clamp(-1.0, 1.0) * self.action_scale
        k = torch.arange(1, substeps + 1, device=q0.device, dtype=q0.dtype).reshape(-1, *([1] * q0.dim()))
        q = torch.max(torch.min(q0.unsqueeze(0) + a.unsqueeze(0) * k, self.upper), self.lower)
        pos, rot = self.fk(q)
        return pos, rot, q[-1]


def default_qpos(device="cuda"):
    q = torch.zeros(24, device=device)
    q[JOINTS.index("FFJ3")] = q[JOINTS.index("MFJ3")] = q[JOINTS.index("RFJ3")] = 0.3
    q[JOINTS.index("THJ4")] = 0.6
    return q
