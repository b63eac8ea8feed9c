"""Generate the golden fixtures of this directory from the reference itself.

Runs DexDeform's own mpm/csrc/integrator.cu kernels, compiled for the host by
oracle/build_ref_host.sh (oracle/_ref/libref_host.so), in the reference's
substep schedule (mpm/simulator.py:561-585) on small seeded inputs, and saves
inputs and outputs as compressed .npz files.  The renderer fixture runs the
reference's particle_sdf and render launchers (integrator.cu:1862-1933) with
the counter-based generator of oracle/ref_host/shim/curand_kernel.h.  Needs
the reference tree, so it runs only where that exists; the fixtures it writes
are committed.

    python tests/golden/make_golden.py            # all fixtures
    python tests/golden/make_golden.py render     # only ref_render_64.npz
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))

from dexdeform_gb300 import workloads as W  # noqa: E402
from oracle.oracle import Bodies, CpuMPM, Material, SimParams, ref_available  # noqa: E402
from oracle import oracle as O  # noqa: E402


def env_inputs(env):
    return dict(grid_dim=np.int32(env.grid_dim), dx=np.float64(env.dx), dt=np.float64(env.dt),
                gravity=np.float32(env.gravity), ground_friction=np.float32(env.ground_friction),
                mass=env.mass, vol=env.vol, mu_lam_yield=env.mu_lam_yield, body_tfsr=env.body_tfsr,
                body_args=env.body_args, poses=env.poses)


def sim(env, backend="ref"):
    prm = SimParams(grid_dim=env.grid_dim, dx=env.dx, dt=env.dt, gravity=env.gravity,
                    ground_friction=env.ground_friction)
    return CpuMPM(backend, prm, Material(env.mass, env.vol, env.mu_lam_yield), Bodies(env.body_tfsr, env.body_args))


def rollout_fixture(name, env, steps, keep=(1,)):
    r = sim(env)
    st = env.state()
    out = {f"s0_{k}": st[k] for k in st}
    for t in range(steps):
        st = r.substep(st, env.pose(t), env.pose(t + 1))
        if t + 1 in keep:
            for k in st:
                out[f"s{t + 1}_{k}"] = st[k]
    np.savez_compressed(os.path.join(HERE, name), keep=np.int32(keep), **env_inputs(env), **out)


def grad_fixture(name, env, seed=7):
    r = sim(env)
    st = W.perturb_state(env, seed=seed, v_scale=0.1, c_scale=1.0, f_scale=0.02, f_mode="gaussian")
    nxt = r.substep(st, env.pose(0), env.pose(1))
    rng = np.random.default_rng(seed + 1)
    g_next = {k: rng.normal(size=st[k].shape).astype(np.float32) for k in st}
    g, (bp, br), (nbp, nbr) = r.substep_grad(st, env.pose(0), env.pose(1), nxt["v"], g_next)
    out = {f"in_{k}": st[k] for k in st}
    out.update({f"next_{k}": nxt[k] for k in nxt})
    out.update({f"gnext_{k}": g_next[k] for k in g_next})
    out.update({f"g_{k}": g[k] for k in g})
    out.update(dict(bpos_grad=bp, brot_grad=br, nbpos_grad=nbp, nbrot_grad=nbr))
    np.savez_compressed(os.path.join(HERE, name), **env_inputs(env), **out)


def digest(a):
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest(), np.uint8)


def render_fixture(name="ref_render_64.npz"):
    """Volume bake + path-traced 64 x 64 image of workloads.render_scene(0):
    inputs, the image and depth, and SHA-256 digests of the packed volume,
    sdf and color volume (bit-exact outputs)."""
    sc = W.render_scene(0)
    vol, sdf, colv = O.particle_sdf("ref", sc["x"], sc["color"], sc["bbox_min"], sc["bake"], sc["voxel"], sc["inv_dx"])
    img, dep = O.render("ref", sc, sdf, colv)
    np.savez_compressed(os.path.join(HERE, name), image=img, depth=dep, volume_sha256=digest(vol),
                        sdf_sha256=digest(sdf), color_sha256=digest(colv), sdf_sum=np.float64(sdf.sum()),
                        **{f"in_{k}": np.asarray(v) for k, v in sc.items()})


def main():
    if not ref_available():
        sys.exit("oracle/_ref/libref_host.so missing: run oracle/build_ref_host.sh first")
    render_fixture()
    if sys.argv[1:] == ["render"]:
        return
    # forward: rest start (F = I), 20 substeps, capsules in contact
    rollout_fixture("ref_forward_32.npz", W.tiny_env(0, n=256, grid=32, nb=6, steps=20, dt=1e-4), 20,
                    keep=(1, 5, 20))
    # forward with a box body (type 0) and an ellipsoid object
    env = W.tiny_env(3, n=256, grid=32, nb=4, steps=10, dt=1e-4, shape="ellipsoid")
    env.body_tfsr[0] = (0.0, 0.9, 666.0, 0.0)
    env.body_args[0] = (0.05, 0.01, 0.04, 0.0)
    rollout_fixture("ref_forward_box_32.npz", env, 10, keep=(1, 10))
    # adjoint of one substep from a perturbed (non-rest) state
    grad_fixture("ref_grad_32.npz", W.tiny_env(1, n=256, grid=32, nb=6, steps=2, dt=1e-4))
    env = W.tiny_env(4, n=256, grid=32, nb=4, steps=2, dt=1e-4)
    env.body_tfsr[0] = (0.0, 0.9, 666.0, 0.0)
    env.body_args[0] = (0.05, 0.01, 0.04, 0.0)
    grad_fixture("ref_grad_box_32.npz", env)
    print("wrote", sorted(f for f in os.listdir(HERE) if f.endswith(".npz")))


if __name__ == "__main__":
    main()
