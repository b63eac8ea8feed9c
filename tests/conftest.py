import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


def _ensure(path, script):
    if not os.path.isfile(path):
        subprocess.run(["bash", os.path.join(ROOT, "oracle", script)], check=True, capture_output=True)


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O
    _ensure(O.ORACLE_SO, "build_oracle.sh")
    O.set_svd_mode("reference")
    return O


@pytest.fixture(scope="session")
def native_lib():
    from dexdeform_gb300 import _native as N
    if not N.lib_available():
        from dexdeform_gb300 import build as B
        B.build()
    return N.load()


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def within_spread(got, want, again, bars, factor=4.0):
    """Schedule-equivalence check: every pair (got[i], want[i]) within
    max(bars[i], factor x rel(again[i], want[i])), where `again` repeats the
    run that gave `want` (the spread of two identical runs: float atomics add
    in a different order each time)."""
    for i, (a, b, c, bar) in enumerate(zip(got, want, again, bars)):
        if b is None:
            continue
        n = rel(c, b)
        err = rel(a, b)
        assert err < max(bar, factor * n), (i, err, bar, n)


def golden_env(path):
    """Rebuild the workloads.Env a fixture was generated from."""
    from dexdeform_gb300 import workloads as W
    z = np.load(path)
    st = {k: z[f"s0_{k}"] if f"s0_{k}" in z else z[f"in_{k}"] for k in ("x", "v", "F", "C")}
    env = W.Env(grid_dim=tuple(int(v) for v in z["grid_dim"]), dx=float(z["dx"]), dt=float(z["dt"]),
                gravity=tuple(float(v) for v in z["gravity"]), ground_friction=float(z["ground_friction"]),
                x=st["x"], v=st["v"], F=st["F"], C=st["C"], mass=z["mass"], vol=z["vol"],
                mu_lam_yield=z["mu_lam_yield"], body_tfsr=z["body_tfsr"], body_args=z["body_args"],
                poses=z["poses"])
    return env, z


def oracle_sim(O, env, backend="oracle"):
    prm = O.SimParams(grid_dim=env.grid_dim, dx=env.dx, dt=env.dt, gravity=env.gravity,
                      ground_friction=env.ground_friction)
    return O.CpuMPM(backend, prm, O.Material(env.mass, env.vol, env.mu_lam_yield),
                    O.Bodies(env.body_tfsr, env.body_args))


def oracle_rollout(O, env, steps, mode, state=None, storage="fp32", t0=0):
    """FP64 oracle rollout from substep t0; returns {t: state} for t = 1 ..
    steps (relative to t0) and the starting state under 0.  storage="fp32"
    rounds the state to FP32 between substeps, as the reference stores it
    (mpm/simulator.py:93-96): the dynamics amplify that rounding (e.g. at
    contact and yield thresholds), so an FP64-state rollout measures the
    storage format, not the kernels."""
    O.set_svd_mode(mode)
    try:
        o = oracle_sim(O, env)
        st = state if state is not None else env.state()
        st = {k: np.asarray(v, np.float64) for k, v in st.items()}
        out = {0: st}
        for t in range(steps):
            st = o.substep(st, env.pose(t0 + t), env.pose(t0 + t + 1))
            if storage == "fp32":
                st = {k: v.astype(np.float32).astype(np.float64) for k, v in st.items()}
            out[t + 1] = st
        return out
    finally:
        O.set_svd_mode("reference")


def oracle_chain_adjoint(O, env, states, g_final, mode, t0=0):
    """Chained substep adjoints of the oracle (mpm/simulator.py:573-585 in
    reverse) over the states of oracle_rollout: the gradient of states[0] and
    the body-pose gradients per substep boundary, (T + 1, nb, 3) and
    (T + 1, nb, 4)."""
    O.set_svd_mode(mode)
    try:
        o = oracle_sim(O, env)
        T = len(states) - 1
        g = {k: np.asarray(v, np.float64) for k, v in g_final.items()}
        bp = np.zeros((T + 1, env.nb, 3))
        br = np.zeros((T + 1, env.nb, 4))
        for t in range(T - 1, -1, -1):
            g, (a, b), (c, d) = o.substep_grad(states[t], env.pose(t0 + t), env.pose(t0 + t + 1),
                                               states[t + 1]["v"], g)
            bp[t] += a
            br[t] += b
            bp[t + 1] += c
            br[t + 1] += d
        return g, bp, br
    finally:
        O.set_svd_mode("reference")


gpu = pytest.mark.gpu


def render_fixture(name="ref_render_64.npz"):
    """(scene dict, outputs) of a committed renderer fixture."""
    z = np.load(os.path.join(GOLDEN, name))
    sc = {k[3:]: z[k] for k in z.files if k.startswith("in_")}
    for k in ("voxel", "image"):
        sc[k] = tuple(int(v) for v in sc[k])
    for k in ("inv_dx", "sdf_threshold", "ground"):
        sc[k] = float(sc[k])
    for k in ("bake", "visualize_shape", "max_ray_depth", "spp", "seed"):
        sc[k] = int(sc[k])
    return sc, {k: z[k] for k in z.files if not k.startswith("in_")}


def sha256(a):
    import hashlib
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest(), np.uint8)
