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


def _qmul(a, b):
    aw, ax, ay, az = a.unbind(-1)
    bw, bx, by, bz = b.unbind(-1)
    return torch.stack([aw * bw - ax * bx - ay * by - az * bz, aw * bx + ax * bw + ay * bz - az * by,
                        aw * by - ax * bz + ay * bw + az * bx, aw * bz + ax * by - ay * bx + az * bw], -1)


def _qrot(q, v):
    qv = q[..., 1:]
    uv = torch.cross(qv, v, dim=-1)
    uuv = torch.cross(qv, uv, dim=-1)
    return v + 2.0 * (q[..., :1] * uv + uuv)


def _axis_angle(axis, angle):
    axis = axis / torch.linalg.norm(axis)
    h = angle[..., None] * 0.5
    return torch.cat([torch.cos(h), torch.sin(h) * axis], -1)


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
        """q (..., 24) -> pos (..., 22, 3), rot (..., 22, 4)."""
        lead = q.shape[:-1]
        qs = [None] * len(_J)
        ps = [None] * len(_J)
        base_q = self.base_rot.expand(*lead, 4)
        base_p = self.base_pos.expand(*lead, 3)
        for j, (name, parent, axis, origin, lo, hi) in enumerate(_J):
            pq = base_q if parent < 0 else qs[parent]
            pp = base_p if parent < 0 else ps[parent]
            ps[j] = pp + _qrot(pq, self.origins[j].expand(*lead, 3))
            qs[j] = _qmul(pq, _axis_angle(self.axes[j], q[..., j]))
        pos = torch.stack([ps[j] + _qrot(qs[j], self.cap_off[c].expand(*lead, 3))
                           for c, j in enumerate(self.cap_joint)], -2)
        rot = torch.stack([qs[j] for j in self.cap_joint], -2)
        return pos, rot

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
