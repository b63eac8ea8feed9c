"""Shadow-hand kinematics for the batched MPM: the hand model read from its
MJCF, batched forward kinematics of its collision geometry, and the
joint-velocity control law.  Pure torch (differentiable), batched over
substeps and hands.

Mirrors, in DexDeform (sizhe-li/DexDeform):
  * mpm/mujoco_parser.py:385-550 ``prepare`` -- which bodies, joints and
    collision geoms make up the hand, and their frames (``parse_mjcf``);
  * mpm/hand.py:347-381 ``hand_forward_kinematics`` -- joint frames
    base @ M_j @ [R(axis_j q_j) | p_j] down the tree, geom frames on top
    (``ShadowHand.forward_kinematics``);
  * mpm/hand.py:383-428 ``JointVel_Fk`` and :20-65 ``rigid_body_motion_hand``
    (``ShadowHand.joint_velocity_fk``, ``wrist_motion``);
  * the joint / actuator tables of mpm/robots/interface.py (below).
The reference computes the rotations with pytorch3d and transforms3d; here
they are written from their formulas (Rodrigues' rotation, the quaternion
product, and the branch-selected matrix-to-quaternion conversion).
"""
from __future__ import annotations

import math
import os
import xml.etree.ElementTree as ET
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from .simulator import MPMSimulator

# ------------------------------------------------------------------ tables
# Joint order of the hand's 24 joints (mpm/robots/interface.py:13-38): the
# index of a joint in q.
JOINTS = ["robot0:WRJ1", "robot0:WRJ0",
          "robot0:FFJ3", "robot0:FFJ2", "robot0:FFJ1", "robot0:FFJ0",
          "robot0:MFJ3", "robot0:MFJ2", "robot0:MFJ1", "robot0:MFJ0",
          "robot0:RFJ3", "robot0:RFJ2", "robot0:RFJ1", "robot0:RFJ0",
          "robot0:LFJ4", "robot0:LFJ3", "robot0:LFJ2", "robot0:LFJ1", "robot0:LFJ0",
          "robot0:THJ4", "robot0:THJ3", "robot0:THJ2", "robot0:THJ1", "robot0:THJ0"]

# The 20 actuators in action order: (name, driven joints, control range in
# radians) (mpm/robots/interface.py:67-110).  A coupled actuator drives two
# joints, each over half its range.
ACTUATORS: List[Tuple[str, Tuple[str, ...], float, float]] = [
    ("WRJ1", ("WRJ1",), -0.4887, 0.1396), ("WRJ0", ("WRJ0",), -0.6981, 0.4887),
    ("FFJ3", ("FFJ3",), -0.3491, 0.3491), ("FFJ2", ("FFJ2",), 0.0, 1.5708), ("FFJ1", ("FFJ1", "FFJ0"), 0.0, 3.1416),
    ("MFJ3", ("MFJ3",), -0.3491, 0.3491), ("MFJ2", ("MFJ2",), 0.0, 1.5708), ("MFJ1", ("MFJ1", "MFJ0"), 0.0, 3.1416),
    ("RFJ3", ("RFJ3",), -0.3491, 0.3491), ("RFJ2", ("RFJ2",), 0.0, 1.5708), ("RFJ1", ("RFJ1", "RFJ0"), 0.0, 3.1416),
    ("LFJ4", ("LFJ4",), 0.0, 0.7854), ("LFJ3", ("LFJ3",), -0.3491, 0.3491), ("LFJ2", ("LFJ2",), 0.0, 1.5708),
    ("LFJ1", ("LFJ1", "LFJ0"), 0.0, 3.1416),
    ("THJ4", ("THJ4",), -1.0472, 1.0472), ("THJ3", ("THJ3",), 0.0, 1.2217), ("THJ2", ("THJ2",), -0.2094, 0.2094),
    ("THJ1", ("THJ1",), -0.5236, 0.5236), ("THJ0", ("THJ0",), -1.5708, 0.0)]

# Initial joint angles of the "default" hand configuration
# (mpm/robots/interface.py:40-65), in JOINTS order.
DEFAULT_INITIAL_QPOS = np.array([
    -0.16514339750464327, -0.31973286565062153,
    0.14340512546557435, 0.32028208333591573, 0.7126053607727917, 0.6705281001412586,
    0.000246444303701037, 0.3152655251085491, 0.7659800313729842, 0.7323156897425923,
    0.00038520700007378114, 0.36743546201985233, 0.7119514095008576, 0.6699446327514138,
    0.0525442258033891, -0.13615534724474673, 0.39872030433433003, 0.7415570009679252, 0.704096378652974,
    0.003673823825070126, 0.5506291436028695, -0.014515151997119306, -0.0015229223564485414,
    -0.7894883021600622])

ROOT_BODY = "robot0:hand mount"
N_ACTUATORS = len(ACTUATORS)


def joint_limits() -> Tuple[np.ndarray, np.ndarray]:
    """Per-joint limits: the driving actuator's range split over the joints it
    drives (mpm/robots/interface.py:121-125)."""
    lo, hi = np.zeros(len(JOINTS)), np.zeros(len(JOINTS))
    for _, joints, a, b in ACTUATORS:
        for j in joints:
            k = JOINTS.index("robot0:" + j)
            lo[k], hi[k] = a / len(joints), b / len(joints)
    return lo, hi


def actuator_of_joint() -> np.ndarray:
    """Actuator index driving each joint (mpm/robots/interface.py:133-144)."""
    out = np.zeros(len(JOINTS), np.int64)
    for a, (_, joints, _, _) in enumerate(ACTUATORS):
        for j in joints:
            out[JOINTS.index("robot0:" + j)] = a
    return out


def default_action_scale(fixed_base: bool = False) -> np.ndarray:
    """mpm/hand.py:104-110: joint velocity 0.33 * 0.002 rad per substep per
    unit action; wrist translation 0.01 and rotation 0.015 per env step."""
    s = [0.33 * 0.002] * N_ACTUATORS
    return np.array(s + ([0.0] * 6 if fixed_base else [0.01] * 3 + [0.015] * 3))


# ------------------------------------------------------ rotation formulas
def _rx(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[1.0, 0.0, 0.0], [0.0, c, -s], [0.0, s, c]])


def _ry(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[c, 0.0, s], [0.0, 1.0, 0.0], [-s, 0.0, c]])


def _rz(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])


def euler_xyz(e) -> np.ndarray:
    """MJCF ``euler`` attribute (the parser's convention, mpm/mujoco_parser.py:16-40):
    R = Rx(e0) Ry(e1) Rz(e2)."""
    return _rx(e[0]) @ _ry(e[1]) @ _rz(e[2])


def quat_matrix_np(q) -> np.ndarray:
    """Rotation of a (not necessarily unit) quaternion w, x, y, z
    (mpm/mujoco_parser.py:43-66; identity for a zero quaternion)."""
    w, x, y, z = (float(v) for v in q)
    n = w * w + x * x + y * y + z * z
    if n <= np.finfo(np.float64).eps:
        return np.eye(3)
    s = 2.0 / n
    return np.array([[1 - s * (y * y + z * z), s * (x * y - w * z), s * (x * z + w * y)],
                     [s * (x * y + w * z), 1 - s * (x * x + z * z), s * (y * z - w * x)],
                     [s * (x * z - w * y), s * (y * z + w * x), 1 - s * (x * x + y * y)]])


def axis_angle_quat_np(axis, angle) -> np.ndarray:
    """Unit quaternion of a rotation by `angle` about `axis` (normalised)."""
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    q = np.concatenate([[math.cos(angle / 2)], math.sin(angle / 2) * a])
    return q / np.linalg.norm(q)


def homogeneous(pos, rot) -> np.ndarray:
    m = np.eye(4)
    m[:3, :3] = rot
    m[:3, 3] = pos
    return m


def axis_angle_to_matrix(v: torch.Tensor) -> torch.Tensor:
    """(..., 3) rotation vectors (axis * angle, axis not necessarily unit:
    the angle is the vector's norm) -> (..., 3, 3), Rodrigues' formula
    R = I + a [v]x + b [v]x^2 with a = sin t / t, b = (1 - cos t) / t^2
    (their series below t = 1e-4)."""
    t2 = (v * v).sum(-1)
    t = torch.sqrt(t2.clamp_min(1e-30))
    small = t2 < 1e-8
    a = torch.where(small, 1.0 - t2 / 6.0, torch.sin(t) / t)
    b = torch.where(small, 0.5 - t2 / 24.0, (1.0 - torch.cos(t)) / t2.clamp_min(1e-30))
    x, y, z = v.unbind(-1)
    zero = torch.zeros_like(x)
    K = torch.stack([zero, -z, y, z, zero, -x, -y, x, zero], -1).reshape(v.shape[:-1] + (3, 3))
    eye = torch.eye(3, dtype=v.dtype, device=v.device).expand(K.shape)
    return eye + a[..., None, None] * K + b[..., None, None] * (K @ K)


def homogeneous_row(like: torch.Tensor, lead) -> torch.Tensor:
    """The bottom row (0, 0, 0, 1) of homogeneous matrices, shaped lead + (1,
    4), made on like's device (no host copy, so that it can be captured in a
    CUDA graph)."""
    row = (torch.arange(4, device=like.device) == 3).to(like.dtype)
    return row.expand(tuple(lead) + (1, 4))


def quaternion_to_matrix(q: torch.Tensor) -> torch.Tensor:
    """(..., 4) quaternions w, x, y, z (any norm) -> (..., 3, 3) rotations."""
    w, x, y, z = q.unbind(-1)
    s = 2.0 / (q * q).sum(-1)
    return torch.stack([1 - s * (y * y + z * z), s * (x * y - w * z), s * (x * z + w * y),
                        s * (x * y + w * z), 1 - s * (x * x + z * z), s * (y * z - w * x),
                        s * (x * z - w * y), s * (y * z + w * x), 1 - s * (x * x + y * y)],
                       -1).reshape(q.shape[:-1] + (3, 3))


def matrix_to_quaternion(m: torch.Tensor) -> torch.Tensor:
    """(..., 3, 3) rotations -> (..., 4) unit quaternions w, x, y, z with
    w >= 0.  Of the four closed forms (each divides by one of 4w, 4x, 4y, 4z)
    the one with the largest divisor is taken, so every branch used is well
    conditioned."""
    m00, m01, m02 = m[..., 0, 0], m[..., 0, 1], m[..., 0, 2]
    m10, m11, m12 = m[..., 1, 0], m[..., 1, 1], m[..., 1, 2]
    m20, m21, m22 = m[..., 2, 0], m[..., 2, 1], m[..., 2, 2]
    t = torch.stack([1 + m00 + m11 + m22, 1 + m00 - m11 - m22, 1 - m00 + m11 - m22, 1 - m00 - m11 + m22], -1)
    r = torch.sqrt(t.clamp_min(1e-12))  # 2|w|, 2|x|, 2|y|, 2|z| of the four forms
    c = torch.stack([
        torch.stack([r[..., 0] * r[..., 0], m21 - m12, m02 - m20, m10 - m01], -1) / (2 * r[..., 0:1]),
        torch.stack([m21 - m12, r[..., 1] * r[..., 1], m01 + m10, m02 + m20], -1) / (2 * r[..., 1:2]),
        torch.stack([m02 - m20, m01 + m10, r[..., 2] * r[..., 2], m12 + m21], -1) / (2 * r[..., 2:3]),
        torch.stack([m10 - m01, m02 + m20, m12 + m21, r[..., 3] * r[..., 3]], -1) / (2 * r[..., 3:4])], -2)
    pick = torch.nn.functional.one_hot(t.argmax(-1), 4).to(m.dtype)
    q = (c * pick[..., None]).sum(-2)
    return torch.where(q[..., :1] < 0, -q, q)


def quat_multiply(a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """Hamilton product a b of quaternions w, x, y, z."""
    aw, ax, ay, az = a.unbind(-1)
    bw, bx, by, bz = b.unbind(-1)
    return torch.stack([aw * bw - ax * bx - ay * by - az * bz, aw * bx + ax * bw + ay * bz - az * by,
                        aw * by - ax * bz + ay * bw + az * bx, aw * bz + ax * by - ay * bx + az * bw], -1)


# --------------------------------------------------------------- the MJCF
@dataclass
class HandModel:
    """The kinematic tree and collision geometry of one hand.
    parent[j]: parent joint of joint j (-1: the tree's root joint, whose body
    frame is the base pose); M[j]: 4x4 transform from the parent joint's frame
    to joint j's body frame; p[j], axis[j]: joint position and (unnormalised)
    axis in that body frame.  Geoms g: attached to joint geom_joint[g] with
    frame G[g] (capsules turned so that their axis is y, the SDF's);
    geom_type 0 box / 1 capsule; geom_size: box half extents / capsule
    (radius, half length), scaled."""
    parent: np.ndarray      # (24,) int
    M: np.ndarray           # (24, 4, 4)
    p: np.ndarray           # (24, 3)
    axis: np.ndarray        # (24, 3)
    geom_joint: np.ndarray  # (G,) int
    G: np.ndarray           # (G, 4, 4)
    geom_type: np.ndarray   # (G,) int
    geom_size: np.ndarray   # (G, 3)
    geom_name: List[str]
    frames: Dict[str, np.ndarray]  # hand mount, forearm and wrist body frames

    @property
    def n_geoms(self) -> int:
        return int(self.G.shape[0])

    def order(self) -> List[int]:
        """Joints in an order where every parent comes first."""
        done, out = set(), []
        while len(out) < len(JOINTS):
            for j in range(len(JOINTS)):
                if j not in done and (self.parent[j] < 0 or self.parent[j] in done):
                    done.add(j)
                    out.append(j)
        return out

    def save(self, path: str):
        np.savez(path, parent=self.parent, M=self.M, p=self.p, axis=self.axis, geom_joint=self.geom_joint, G=self.G,
                 geom_type=self.geom_type, geom_size=self.geom_size, geom_name=np.array(self.geom_name),
                 **{"frame:" + k: v for k, v in self.frames.items()})

    @classmethod
    def load(cls, path: str) -> "HandModel":
        z = np.load(path)
        return cls(parent=z["parent"], M=z["M"], p=z["p"], axis=z["axis"], geom_joint=z["geom_joint"], G=z["G"],
                   geom_type=z["geom_type"], geom_size=z["geom_size"], geom_name=[str(s) for s in z["geom_name"]],
                   frames={k[6:]: z[k] for k in z.files if k.startswith("frame:")})


def _read_xml(path: str) -> ET.Element:
    """Parse an MJCF file with its <include file=...> elements replaced by
    the included files' top-level children (paths relative to the including
    file)."""
    root = ET.parse(path).getroot()
    base = os.path.dirname(os.path.abspath(path))
    for parent in list(root.iter()):
        kids = list(parent)
        for i, child in enumerate(kids):
            if child.tag != "include":
                continue
            inc = _read_xml(os.path.join(base, child.get("file")))
            parent.remove(child)
            for k, sub in enumerate(list(inc)):
                parent.insert(i + k, sub)
    return root


def _apply_defaults(root: ET.Element):
    """Fill attributes from the <default class=...> templates: an element's
    own class, then the childclass of its nearest ancestor that has one
    (attributes already set are kept)."""
    templates = {}
    d = root.find("default")
    if d is not None:
        for cls in d.findall("default"):
            templates[cls.get("class")] = {c.tag: dict(c.attrib) for c in cls}

    def fill(el, tpl):
        for k, v in tpl.get(el.tag, {}).items():
            if k not in el.attrib:
                el.set(k, v)

    def walk(el, inherited):
        for ch in el:
            if ch.get("class") in templates:
                fill(ch, templates[ch.get("class")])
            cc = ch.get("childclass")
            if inherited is not None:
                fill(ch, inherited)
            walk(ch, templates.get(cc, inherited) if cc else inherited)

    wb = root.find("worldbody")
    if wb is not None:
        walk(wb, None)


def _frame(el: ET.Element, scale: float) -> np.ndarray:
    """Pose of an MJCF element in its parent's frame (pos scaled; rotation
    from euler, axisangle or quat; mpm/mujoco_parser.py:420-435)."""
    pos = np.fromstring(el.get("pos", "0 0 0"), sep=" ") * scale
    if "euler" in el.attrib:
        rot = euler_xyz(np.fromstring(el.get("euler"), sep=" "))
    elif "axisangle" in el.attrib:
        aa = np.fromstring(el.get("axisangle"), sep=" ")
        rot = quat_matrix_np(axis_angle_quat_np(aa[:3], aa[3]))
    elif "quat" in el.attrib:
        rot = quat_matrix_np(np.fromstring(el.get("quat"), sep=" "))
    else:
        rot = np.eye(3)
    return homogeneous(pos, rot)


def parse_mjcf(path: str, scale: float = 1.0, root_body: str = ROOT_BODY) -> HandModel:
    """Read the hand's kinematic tree and collision geoms (group 4, not
    meshes) from its MJCF (e.g. DexDeform's
    mpm/assets/robots/shadow/right_hand/shadow_hand.xml)."""
    root = _read_xml(path)
    _apply_defaults(root)
    start = next((b for b in root.find("worldbody").iter("body") if b.get("name") == root_body), None)
    if start is None:
        raise ValueError(f"no body {root_body!r} in {path}")
    nj = len(JOINTS)
    parent = np.full(nj, -2, np.int64)
    M = np.tile(np.eye(4), (nj, 1, 1))
    p, axis = np.zeros((nj, 3)), np.zeros((nj, 3))
    g_joint, g_mat, g_type, g_size, g_name = [], [], [], [], []
    frames = {}
    cap_turn = homogeneous(np.zeros(3), _rx(math.pi / 2))

    def visit(body, anchor, acc, world):
        """anchor: joint whose frame the body hangs from (-1: none yet);
        acc: transform from that frame to this body's parent frame; world:
        the body's parent frame from the root (for the named frames)."""
        mat = _frame(body, scale)
        acc = acc @ mat
        name = body.get("name", "")
        if name in ("robot0:hand mount", "robot0:forearm", "robot0:wrist"):
            frames[name] = mat
        joints = [j for j in body.findall("joint") if j.get("name") in JOINTS]
        if len(joints) > 1:
            raise ValueError(f"body {name} has {len(joints)} hand joints (open chains only)")
        if joints:
            j = JOINTS.index(joints[0].get("name"))
            if joints[0].get("type", "hinge") != "hinge":
                raise ValueError(f"{joints[0].get('name')}: only hinge joints")
            parent[j] = anchor
            M[j] = acc if anchor >= 0 else np.eye(4)  # the root joint's body frame is the base pose
            p[j] = np.fromstring(joints[0].get("pos", "0 0 0"), sep=" ")
            axis[j] = np.fromstring(joints[0].get("axis", "0 0 1"), sep=" ")
            anchor, acc = j, np.eye(4)
        for g in body.findall("geom"):
            if g.get("group", "") != "4" or g.get("mesh") or g.get("type", "sphere") not in ("box", "capsule"):
                continue
            if anchor < 0:
                raise ValueError(f"collision geom {g.get('name')} above the hand's first joint")
            gm = _frame(g, scale) if g.get("pos") else np.eye(4)
            if g.get("type") == "capsule":
                gm = gm @ cap_turn
            size = [float(v) * scale for v in g.get("size").split()]
            g_joint.append(anchor)
            g_mat.append(acc @ gm)
            g_type.append(1 if g.get("type") == "capsule" else 0)
            g_size.append((size + [0.0, 0.0, 0.0])[:3])
            g_name.append(g.get("name", ""))
        for ch in body.findall("body"):
            visit(ch, anchor, acc, world)

    visit(start, -1, np.eye(4), np.eye(4))
    if (parent == -2).any():
        missing = [JOINTS[j] for j in np.nonzero(parent == -2)[0]]
        raise ValueError(f"joints not found below {root_body}: {missing}")
    return HandModel(parent=parent, M=M, p=p, axis=axis, geom_joint=np.array(g_joint), G=np.array(g_mat),
                     geom_type=np.array(g_type), geom_size=np.array(g_size), geom_name=g_name, frames=frames)


def default_root_frame(model: HandModel) -> np.ndarray:
    """The base pose the reference derives from the MJCF when no hand pose is
    configured (mpm/mujoco_parser.py:383-386 root pose, mpm/hand.py:606-607):
    root @ hand mount @ wrist."""
    root = homogeneous(np.array([1.0, 1.25, 0.15]), euler_xyz([math.pi / 2, 0.0, math.pi]))
    return root @ model.frames["robot0:hand mount"] @ model.frames["robot0:wrist"]


def root_matrix(pos, rot_euler) -> np.ndarray:
    """Base pose from a position and static-xyz Euler angles (mpm/hand.py:612-613)."""
    r = np.asarray(rot_euler, np.float64)
    return homogeneous(np.asarray(pos, np.float64), _rz(r[2]) @ _ry(r[1]) @ _rx(r[0]))


# ------------------------------------------------------------ kinematics
class ShadowHand:
    """Batched, differentiable forward kinematics of one or more identical
    hands and the joint-velocity control law."""

    def __init__(self, model: HandModel, device="cuda", dtype=torch.float32, action_scale=None,
                 fixed_base: bool = False):
        self.model = model
        self.device = torch.device(device)
        f = dict(dtype=dtype, device=self.device)
        self.M = torch.tensor(model.M, **f)
        self.p = torch.tensor(model.p, **f)
        self.axis = torch.tensor(model.axis, **f)
        self.G = torch.tensor(model.G, **f)
        self.geom_joint = torch.tensor(model.geom_joint, dtype=torch.long, device=self.device)
        self._order = model.order()
        # the joints by depth in the tree, each level with the rows of its
        # parents in the running table of frames (row 0 the base, then the
        # levels in order), and each joint's row at the end
        depth = {}
        for j in self._order:
            par = int(model.parent[j])
            depth[j] = 0 if par < 0 else depth[par] + 1
        row, n = {}, 1
        self._levels = []
        for d in range(max(depth.values()) + 1):
            js = [j for j in self._order if depth[j] == d]
            rows = [0 if model.parent[j] < 0 else row[int(model.parent[j])] for j in js]
            self._levels.append((torch.tensor(js, dtype=torch.long, device=self.device),
                                 torch.tensor(rows, dtype=torch.long, device=self.device),
                                 torch.tensor([int(model.parent[j]) >= 0 for j in js], device=self.device)))
            for j in js:
                row[j] = n
                n += 1
        self._rows = torch.tensor([row[j] for j in range(len(JOINTS))], dtype=torch.long, device=self.device)
        lo, hi = joint_limits()
        self.lower, self.upper = torch.tensor(lo, **f), torch.tensor(hi, **f)
        self.action_map = torch.tensor(actuator_of_joint(), dtype=torch.long, device=self.device)
        self.action_scale = torch.tensor(default_action_scale(fixed_base) if action_scale is None else action_scale,
                                         **f)

    @property
    def n_geoms(self) -> int:
        return self.model.n_geoms

    def body_shapes(self, friction: float = 0.9, softness: float = 666.0, n_hands: int = 1):
        """Body shape tables of the geoms for the MPM engine: (nb, 4) type,
        friction, softness, round and (nb, 4) args -- box half extents, or
        capsule (radius, half length) (mpm/cuda_env.py:76-92)."""
        m = self.model
        tfsr = np.zeros((m.n_geoms, 4), np.float32)
        tfsr[:, 0], tfsr[:, 1], tfsr[:, 2] = m.geom_type, friction, softness
        args = np.zeros((m.n_geoms, 4), np.float32)
        args[:, :3] = m.geom_size
        args[m.geom_type == 1, 2] = 0.0
        return np.tile(tfsr, (n_hands, 1)), np.tile(args, (n_hands, 1))

    # the hand interface GradModel drives (joint angles at a fixed base pose)
    def set_base(self, base):
        """Fixed base pose (4, 4) of fk / joint_velocity_poses."""
        self.base = torch.as_tensor(np.asarray(base) if not isinstance(base, torch.Tensor) else base,
                                    dtype=self.M.dtype, device=self.device)
        return self

    def fk(self, q: torch.Tensor):
        """Joint angles (24,) at the fixed base -> geom positions (G, 3) and
        quaternions (G, 4)."""
        pos, rot = self.forward_kinematics(self.base[None, None], q[None, None])
        return pos[0], rot[0]

    def joint_velocity_poses(self, q0: torch.Tensor, action: torch.Tensor, substeps: int):
        """JointVel_Fk at the fixed base for actions (20,): per-substep geom
        poses (substeps, G, 3) / (substeps, G, 4) and the final angles (24,)."""
        pos, rot, (_, q) = self.joint_velocity_fk(self.base[None], q0[None], action[None], substeps)
        return pos, rot, q[0]

    def joint_frames(self, base: torch.Tensor, q: torch.Tensor) -> torch.Tensor:
        """base (..., 4, 4) root-joint body frames, q (..., 24) joint angles ->
        (..., 24, 4, 4) joint frames."""
        R = axis_angle_to_matrix(self.axis * q[..., None])            # (..., 24, 3, 3)
        T = torch.cat([torch.cat([R, self.p.expand(R.shape[:-1])[..., None]], -1),
                       homogeneous_row(R, R.shape[:-2])], -2)           # (..., 24, 4, 4)
        # joint j's frame: its parent's frame @ M_j @ T_j, or base @ T_j at
        # the root; the joints of one depth of the tree are done together
        frames = base[..., None, :, :]                                  # (..., 1, 4, 4), row 0 the base
        for js, rows, has_parent in self._levels:
            src = frames.index_select(-3, rows)
            src = torch.where(has_parent[:, None, None], src @ self.M[js], src)
            frames = torch.cat([frames, src @ T.index_select(-3, js)], -3)
        return frames.index_select(-3, self._rows)

    def forward_kinematics(self, base: torch.Tensor, q: torch.Tensor):
        """mpm/hand.py:347-381: base (S, H, 4, 4), q (S, H, 24) -> geom
        positions (S, H * G, 3) and unit quaternions w, x, y, z with w >= 0
        (S, H * G, 4)."""
        J = self.joint_frames(base, q)
        geom = J[..., self.geom_joint, :, :] @ self.G                # (S, H, G, 4, 4)
        geom = geom.reshape(base.shape[0], -1, 4, 4)
        return geom[..., :3, 3], matrix_to_quaternion(geom[..., :3, :3])

    def wrist_motion(self, base: torch.Tensor, twist: torch.Tensor, substeps: int) -> torch.Tensor:
        """mpm/hand.py:20-65: base (H, 4, 4) moved by a twist (H, 6) (already
        scaled) spread over the substeps: substep k adds (k + 1) / substeps
        of the translation and of the rotation vector (applied in the world
        frame) -> (substeps, H, 4, 4)."""
        k = (torch.arange(substeps, device=base.device, dtype=base.dtype) + 1) / substeps
        a = twist[None] * k[:, None, None]                               # (S, H, 6)
        st = base[None].expand(substeps, -1, -1, -1)
        pos = st[..., :3, 3] + a[..., :3]
        q = matrix_to_quaternion(st[..., :3, :3])
        rot = a[..., 3:]
        w = torch.sqrt((rot * rot).sum(-1, keepdim=True) + 1e-16)
        dq = torch.cat([torch.cos(w / 2), rot / w.clamp(1e-7, 1e9) * torch.sin(w / 2)], -1)
        out = quat_multiply(dq, q)
        out = out / torch.linalg.norm(out, dim=-1, keepdim=True)
        R = quaternion_to_matrix(out)
        top = torch.cat([R, pos[..., None]], -1)
        return torch.cat([top, homogeneous_row(base, top.shape[:-2])], -2)

    def joint_velocity_fk(self, base: torch.Tensor, q: torch.Tensor, actions: torch.Tensor, substeps: int):
        """mpm/hand.py:383-428 (JointVel_Fk): actions (H, 20) joint velocities
        in [-1, 1], or (H, 26) with a wrist twist; q_k = clamp(q + a (k + 1))
        per substep k; returns geom positions (S, H * G, 3), quaternions
        (S, H * G, 4) and the final (base (H, 4, 4), q (H, 24))."""
        H = base.shape[0]
        if actions.shape[-1] == N_ACTUATORS + 6:
            nb = self.wrist_motion(base, actions[..., -6:] * self.action_scale[-6:], substeps)
        else:
            nb = base[None].expand(substeps, H, 4, 4)
        a = (actions[..., :N_ACTUATORS].clamp(-1.0, 1.0) * self.action_scale[:N_ACTUATORS])[..., self.action_map]
        k = torch.arange(substeps, device=q.device, dtype=q.dtype)[:, None, None] + 1
        nq = torch.max(torch.min(q[None] + a[None] * k, self.upper), self.lower)
        pos, rot = self.forward_kinematics(nb, nq)
        return pos, rot, (nb[-1], nq[-1])


def _scaled(model: HandModel, s: float) -> HandModel:
    """The model parsed with `scale` s instead of 1 (body and geom positions
    and geom sizes scale; joint positions do not, as in the parser)."""
    M, G = model.M.copy(), model.G.copy()
    M[:, :3, 3] *= s
    G[:, :3, 3] *= s
    frames = {}
    for k, v in model.frames.items():
        f = v.copy()
        f[:3, 3] *= s
        frames[k] = f
    return HandModel(parent=model.parent.copy(), M=M, p=model.p.copy(), axis=model.axis.copy(),
                     geom_joint=model.geom_joint.copy(), G=G, geom_type=model.geom_type.copy(),
                     geom_size=model.geom_size * s, geom_name=list(model.geom_name), frames=frames)


HandModel.scaled = _scaled


# ------------------------------------------------------------ simulator
class HandSimulator(MPMSimulator):
    """Drop-in mirror of mpm/hand.py:68-456 ``HandSimulator``: the MPM
    simulator (MPMSimulator, batched backend by default) driven by one or two
    Shadow hands under joint-velocity control.

    The state tuple of env-step boundaries carries the hands' base poses
    (n_hands, 4, 4) and joint angles (n_hands, 24) after the particle fields
    and body poses (mpm/hand.py:183-210); set_state runs the kinematics to
    place the 19 collision primitives of each hand.  compute_forward_kinematics
    is JointVel_Fk (mpm/hand.py:383-428), so step(action) takes actions of
    (n_hands, 20) joint velocities, or (n_hands, 26) with a wrist twist.

    models: one HandModel per hand (left before right for two hands, the
    reference's primitive order), already at the env's scale."""

    def __init__(self, models: Sequence[HandModel], quality: float = 1.0, n_particles: int = 10000,
                 hand_friction: float = 0.9, action_scale=None, fixed_base: bool = False, device="cuda",
                 root_frames=None, max_steps: int = 1024, **sim_kwargs):
        dt = 0.5e-4 / quality
        dx = 1.0 / (64 * quality)
        substeps = int(np.ceil(2e-3 / dt))
        self.models = list(models)
        self.n_hands = len(self.models)
        self.device = torch.device(device)
        self.hands = [ShadowHand(m, device=device, action_scale=action_scale, fixed_base=fixed_base)
                      for m in self.models]
        n_bodies = int(sum(m.n_geoms for m in self.models))
        super().__init__(n_bodies, n_particles=n_particles, dt=dt, dx=dx, substeps=substeps, max_steps=max_steps,
                         **sim_kwargs)
        self.n_joints_per_hand = len(JOINTS)
        self.n_actuators_per_hand = N_ACTUATORS
        tf, ar = zip(*[h.body_shapes(friction=hand_friction) for h in self.hands])
        tfsr, args = np.concatenate(tf), np.concatenate(ar)
        self.init_bodies(tfsr[:, 0], tfsr[:, 2], tfsr[:, 1], tfsr[:, 3], args, None)
        self.base_pose: List[Optional[torch.Tensor]] = [None] * self.max_steps
        self.joint_rot: List[Optional[torch.Tensor]] = [None] * self.max_steps
        rf = (np.stack([default_root_frame(m) for m in self.models]) if root_frames is None
              else np.asarray(root_frames, np.float64).reshape(self.n_hands, 4, 4))
        self.base_pose[0] = torch.tensor(rf, dtype=torch.float32, device=self.device)
        self.joint_rot[0] = torch.tensor(np.tile(DEFAULT_INITIAL_QPOS, (self.n_hands, 1)), dtype=torch.float32,
                                         device=self.device)

    # ---------------------------------------------------------- kinematics
    def hand_forward_kinematics(self, base_pose: torch.Tensor, q: torch.Tensor):
        """mpm/hand.py:347-381: base_pose (S, n_hands, 4, 4), q (S, n_hands,
        24) -> primitive positions (S, n_bodies, 3) and quaternions (S,
        n_bodies, 4)."""
        out = [h.forward_kinematics(base_pose[:, i:i + 1], q[:, i:i + 1]) for i, h in enumerate(self.hands)]
        return torch.cat([o[0] for o in out], 1), torch.cat([o[1] for o in out], 1)

    def JointVel_Fk(self, f, actions, pos_rot=None):
        """mpm/hand.py:383-428: per-substep primitive poses of env step f under
        joint-velocity actions; stores the hands' pose at f + substeps."""
        base, q = (self.base_pose[f], self.joint_rot[f]) if pos_rot is None else pos_rot
        actions = torch.as_tensor(np.asarray(actions, np.float32) if not isinstance(actions, torch.Tensor) else actions,
                                  dtype=torch.float32, device=self.device)
        assert actions.shape[0] == self.n_hands
        res = [h.joint_velocity_fk(base[i:i + 1], q[i:i + 1], actions[i:i + 1], self.substeps)
               for i, h in enumerate(self.hands)]
        pos = torch.cat([r[0] for r in res], 1)
        rot = torch.cat([r[1] for r in res], 1)
        nb = torch.cat([r[2][0] for r in res], 0)
        nq = torch.cat([r[2][1] for r in res], 0)
        self.base_pose[f + self.substeps] = nb
        self.joint_rot[f + self.substeps] = nq
        return pos, rot, (nb, nq)

    def compute_forward_kinematics(self, f, action, pos_rot=None):
        return self.JointVel_Fk(f, action, pos_rot=pos_rot)

    def download_pos_rot(self, cur, device):
        """mpm/hand.py:162-167: the hands' pose of state 0 (later ones reset)."""
        assert cur == 0
        for i in range(1, len(self.base_pose)):
            self.base_pose[i] = self.joint_rot[i] = None
        return self.base_pose[cur].to(device), self.joint_rot[cur].to(device)

    # -------------------------------------------------------- state tuple
    def get_state(self, index):
        """mpm/hand.py:183-187: (x, v, F, C, per-body poses ..., base poses
        (n_hands, 4, 4), joint angles (n_hands, 24))."""
        assert index % self.substeps == 0
        return super().get_state(index) + (self.base_pose[index].detach().cpu().numpy(),
                                           self.joint_rot[index].detach().cpu().numpy())

    def set_state(self, index, state):
        """mpm/hand.py:189-210: particles from the tuple, bodies placed by the
        kinematics of its base poses and joint angles."""
        assert index % self.substeps == 0
        self.base_pose[index] = torch.tensor(np.asarray(state[-2]), dtype=torch.float32, device=self.device)
        self.joint_rot[index] = torch.tensor(np.asarray(state[-1]), dtype=torch.float32, device=self.device)
        pos, rot = self.hand_forward_kinematics(self.base_pose[index][None], self.joint_rot[index][None])
        pose = np.concatenate([pos[0].detach().cpu().numpy(), rot[0].detach().cpu().numpy()], 1)
        super().set_state(index, tuple(np.float32(s) for s in state[:4]) + tuple(pose))

    def step(self, action, pos_rot=None):
        """mpm/hand.py:437-440: one env step, then the hands' pose at its end
        becomes the pose of state 0."""
        super().step(action, pos_rot)
        self.base_pose[0] = self.base_pose[self.substeps]
        self.joint_rot[0] = self.joint_rot[self.substeps]
