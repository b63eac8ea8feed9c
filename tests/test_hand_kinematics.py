"""The synthetic 24-joint hand's kinematics (dexdeform_gb300.hand), computed
one depth of the joint tree at a time, against a joint-by-joint restatement
of the same chain in FP64 (each joint's world frame: the parent's, moved by
the joint's origin and turned by the joint's angle about its axis; capsules
at offsets in their joint's frame).  Values to FP32 rounding (1e-6), and the
gradients of a random projection of the poses wrt the joint angles (5e-5).
CPU only."""
import torch

from dexdeform_gb300 import hand as Hm


def _qmul(a, b):
    aw, ax, ay, az = a.unbind(-1)
    bw, bx, by, bz = b.unbind(-1)
    return torch.stack([aw * bw - ax * bx - ay * by - az * bz, aw * bx + ax * bw + ay * bz - az * by,
                        aw * by - ax * bz + ay * bw + az * bx, aw * bz + ax * by - ay * bx + az * bw], -1)


def _qrot(q, v):
    u = q[..., 1:]
    uv = torch.cross(u, v, dim=-1)
    return v + 2.0 * (q[..., :1] * uv + torch.cross(u, uv, dim=-1))


def joint_by_joint(h, q):
    lead = q.shape[:-1]
    qs, ps = [None] * len(Hm._J), [None] * len(Hm._J)
    bq, bp = h.base_rot.double().expand(*lead, 4), h.base_pos.double().expand(*lead, 3)
    for j, (_, parent, *_rest) in enumerate(Hm._J):
        pq = bq if parent < 0 else qs[parent]
        pp = bp if parent < 0 else ps[parent]
        ps[j] = pp + _qrot(pq, h.origins[j].double().expand(*lead, 3))
        axis = h.axes[j].double() / torch.linalg.norm(h.axes[j].double())
        half = q[..., j:j + 1] * 0.5
        qs[j] = _qmul(pq, torch.cat([torch.cos(half), torch.sin(half) * axis], -1))
    pos = torch.stack([ps[j] + _qrot(qs[j], h.cap_off[c].double().expand(*lead, 3))
                       for c, j in enumerate(h.cap_joint)], -2)
    return pos, torch.stack([qs[j] for j in h.cap_joint], -2)


def test_level_batched_kinematics_equal_joint_by_joint():
    h = Hm.SyntheticHand(device="cpu", base_pos=(0.5, 0.2, 0.47), action_scale=0.05)
    gen = torch.Generator().manual_seed(0)
    q = (torch.rand(7, 50, 24, generator=gen, dtype=torch.float64) - 0.5) * 3.0
    pos, rot = h.fk(q.float())
    want_pos, want_rot = joint_by_joint(h, q)
    assert pos.shape == (7, 50, Hm.N_BODIES, 3) and rot.shape == (7, 50, Hm.N_BODIES, 4)
    assert (pos.double() - want_pos).abs().max() < 1e-6
    assert (rot.double() - want_rot).abs().max() < 1e-6
    # gradients of a random projection of every pose wrt the joint angles
    wp = torch.randn(pos.shape, generator=gen, dtype=torch.float64)
    wr = torch.randn(rot.shape, generator=gen, dtype=torch.float64)
    q32 = q.float().requires_grad_(True)
    p32, r32 = h.fk(q32)
    ((p32.double() * wp).sum() + (r32.double() * wr).sum()).backward()
    q64 = q.clone().requires_grad_(True)
    p64, r64 = joint_by_joint(h, q64)
    ((p64 * wp).sum() + (r64 * wr).sum()).backward()
    err = (q32.grad.double() - q64.grad).norm() / q64.grad.norm()
    assert err < 5e-5, float(err)
