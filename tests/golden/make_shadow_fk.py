"""Generate the Shadow-hand kinematics fixtures of this directory from the
reference itself.

Runs DexDeform's own hand kinematics -- mpm/mujoco_parser.py ``prepare``,
mpm/hand.py ``HandSimulator.hand_forward_kinematics`` (:347-381) and
``JointVel_Fk`` (:383-428) with mpm/robots/interface.py's tables -- loaded by
file path from the reference tree.  Their third-party dependencies are not
installed here, so this script stands in small test-only modules for them:
the rotation conversions of pytorch3d 0.7.2 and transforms3d (axangle2mat,
euler2mat) computed with scipy.spatial.transform (an implementation
independent of dexdeform_gb300.shadow_hand), and empty placeholders for the
simulator, shape, progress-bar and config modules that hand.py imports but
the kinematics never use.

Writes, for the right and the left hand:
  shadow_<rh|lh>_model.npz -- the hand model parsed by
      dexdeform_gb300.shadow_hand.parse_mjcf from the reference's MJCF (the
      GPU tests run the real hand from it where the reference tree is absent);
  shadow_<rh|lh>_fk.npz    -- seeded inputs and the reference's outputs.

    python tests/golden/make_shadow_fk.py
"""
import importlib.util
import os
import sys
import types

import numpy as np
import torch
from scipy.spatial.transform import Rotation

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)
REF = os.environ.get("REF_ROOT", "/root/reference")


# ---------------------------------------------------- test-only stand-ins
def _rotvec_to_matrix(v):
    a = v.detach().double().cpu().numpy()
    m = Rotation.from_rotvec(a.reshape(-1, 3)).as_matrix().reshape(a.shape[:-1] + (3, 3))
    return torch.tensor(m, dtype=v.dtype, device=v.device)


def _matrix_to_quaternion(m):
    a = m.detach().double().cpu().numpy()
    q = Rotation.from_matrix(a.reshape(-1, 3, 3)).as_quat()  # x y z w
    q = np.concatenate([q[:, 3:], q[:, :3]], 1).reshape(a.shape[:-2] + (4,))
    return torch.tensor(q, dtype=m.dtype, device=m.device)


def _quaternion_to_matrix(q):
    a = q.detach().double().cpu().numpy()
    x = np.concatenate([a[..., 1:], a[..., :1]], -1).reshape(-1, 4)
    m = Rotation.from_quat(x).as_matrix().reshape(a.shape[:-1] + (3, 3))
    return torch.tensor(m, dtype=q.dtype, device=q.device)


def _install_stubs():
    p3 = types.ModuleType("pytorch3d")
    tr = types.ModuleType("pytorch3d.transforms")
    rc = types.ModuleType("pytorch3d.transforms.rotation_conversions")
    rc.axis_angle_to_matrix = _rotvec_to_matrix
    rc.matrix_to_quaternion = _matrix_to_quaternion
    rc.quaternion_to_matrix = _quaternion_to_matrix
    sys.modules.update({"pytorch3d": p3, "pytorch3d.transforms": tr, "pytorch3d.transforms.rotation_conversions": rc})
    t3 = types.ModuleType("transforms3d")
    ax = types.ModuleType("transforms3d.axangles")
    ax.axangle2mat = lambda axis, angle: Rotation.from_rotvec(
        np.asarray(axis, float) / np.linalg.norm(axis) * angle).as_matrix()
    eu = types.ModuleType("transforms3d.euler")
    eu.euler2mat = lambda ai, aj, ak: Rotation.from_euler("xyz", [ai, aj, ak]).as_matrix()  # static x, y, z
    t3.axangles, t3.euler = ax, eu
    sys.modules.update({"transforms3d": t3, "transforms3d.axangles": ax, "transforms3d.euler": eu})
    tq = types.ModuleType("tqdm")
    tq.tqdm = object
    tools = types.ModuleType("tools")
    tools.Configurable = type("Configurable", (), {"__init__": lambda self, *a, **k: None})
    sys.modules.update({"tqdm": tq, "tools": tools})
    for name in ("mpm", "mpm.robots"):
        sys.modules[name] = types.ModuleType(name)
    cu = types.ModuleType("mpm.cuda_env")
    cu.CudaEnv = type("CudaEnv", (), {})
    sh = types.ModuleType("mpm.shapes")
    sh.Shapes = object

    class _Sim:  # what HandSimulator.__init__ reads of mpm/simulator.py's MPMSimulator
        def __init__(self, n_bodies, dt=1e-4, dx=1 / 64, substeps=20, max_steps=1024, **kw):
            self.n_bodies, self.dt, self.dx, self.substeps, self.max_steps = n_bodies, dt, dx, substeps, max_steps
    sm = types.ModuleType("mpm.simulator")
    sm.MPMSimulator = _Sim
    sys.modules.update({"mpm.cuda_env": cu, "mpm.shapes": sh, "mpm.simulator": sm})


def _load(name, path):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def reference_hand(mode):
    """The reference's HandSimulator for one hand ("rh" or "lh"), its hand
    configuration built as HandEnv.parse_sim_cfg builds it (mpm/hand.py:537-604)."""
    _install_stubs()
    _load("mpm.robots.interface", os.path.join(REF, "mpm", "robots", "interface.py"))
    _load("mpm.mujoco_parser", os.path.join(REF, "mpm", "mujoco_parser.py"))
    hand = _load("mpm.hand", os.path.join(REF, "mpm", "hand.py"))

    class FakeEnv:
        def default_tool_config(self):
            return {}

    cfg = types.SimpleNamespace(mode=mode, scale=1.0, hand_friction=0.9, ctrl_type="vel")
    params = hand.HandEnv.parse_sim_cfg(FakeEnv(), cfg)
    n_bodies = len(params["primitives"])
    sim = hand.HandSimulator(n_bodies, params["hand_cfg"], cfg=cfg, quality=1, device="cpu")
    return sim, params


def main():
    from dexdeform_gb300.shadow_hand import parse_mjcf
    for mode, folder in (("rh", "right_hand"), ("lh", "left_hand")):
        sim, params = reference_hand(mode)
        model = parse_mjcf(os.path.join(REF, "mpm", "assets", "robots", "shadow", folder, "shadow_hand.xml"))
        model.save(os.path.join(HERE, f"shadow_{mode}_model.npz"))
        rng = np.random.default_rng(0 if mode == "rh" else 1)
        S = 4
        lo = np.array([sim.q_lower[0, 0, i].item() for i in range(24)])
        hi = np.array([sim.q_upper[0, 0, i].item() for i in range(24)])
        q = (lo + (hi - lo) * rng.random((S, 1, 24))).astype(np.float32)
        base = np.stack([np.stack([params["hand_cfg"]["root_frame"][0]]) for _ in range(S)]).astype(np.float32)
        base[:, :, :3, 3] += rng.normal(scale=0.05, size=(S, 1, 3)).astype(np.float32)
        pos, rot = sim.hand_forward_kinematics(torch.tensor(base), torch.tensor(q))
        # JointVel_Fk from the default pose: joint velocities with a wrist
        # twist (26 actions), then joint velocities only (20)
        a26 = rng.uniform(-1.2, 1.2, (1, 26)).astype(np.float32)
        p26, r26, (b26, q26) = sim.JointVel_Fk(0, torch.tensor(a26))
        a20 = rng.uniform(-1.2, 1.2, (1, 20)).astype(np.float32)
        p20, r20, (b20, q20) = sim.JointVel_Fk(sim.substeps, torch.tensor(a20))
        np.savez_compressed(
            os.path.join(HERE, f"shadow_{mode}_fk.npz"),
            base=base, q=q, pos=pos.numpy(), rot=rot.numpy(),
            root_frame=np.asarray(params["hand_cfg"]["root_frame"], np.float32),
            q0=sim.joint_rot[0].numpy(), substeps=np.int64(sim.substeps),
            a26=a26, pos26=p26.numpy(), rot26=r26.numpy(), base26=b26.numpy(), q26=q26.numpy(),
            a20=a20, pos20=p20.numpy(), rot20=r20.numpy(), base20=b20.numpy(), q20=q20.numpy(),
            q_lower=sim.q_lower.numpy().reshape(-1), q_upper=sim.q_upper.numpy().reshape(-1),
            action_map=sim.action_map.numpy(), action_scale=sim.torch_action_scale.numpy(),
            types=np.array([0 if p["shape"] == "Box" else 1 for p in params["primitives"]]),
            sizes=np.array([list(p["size"]) + [0.0] * (3 - len(p["size"])) for p in params["primitives"]]))
        print(f"wrote shadow_{mode}_model.npz and shadow_{mode}_fk.npz ({len(params['primitives'])} bodies)")


if __name__ == "__main__":
    main()
