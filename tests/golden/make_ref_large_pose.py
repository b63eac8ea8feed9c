"""Generate tests/golden/ref_large_pose_grad.npz: the body-pose gradients that
the reference's own FP32 adjoint kernels give on the large configuration's
adjoint case of tests/test_gpu_full_size.py.

A body's pose gradient in the reference's contact model sums, over every grid
node the body touches, terms of order 1/dt from the body velocity
(T_next(x) - T_cur(x)) / dt (mpm/csrc/integrator.cu:902-1051).  The pose of
substep t gets them once as the current pose of substep t and once as the next
pose of substep t - 1, with opposite signs, so the row's total is a small
difference of large FP32 sums.  How far FP32 arithmetic lands from the FP64
oracle there is a property of the formula; this fixture records how far the
reference's own FP32 kernels land, as the bar for the GPU's.

It runs DexDeform's mpm/csrc/integrator.cu compiled for the host
(oracle/build_ref_host.sh, backend "ref") over the FP32-stored states of the
FP64 oracle's rollout (the same states the test compares against), chaining
the reference's substep adjoints (mpm/simulator.py:573-585) from the test's
seeded final gradient.  Needs the reference tree, so it runs only where that
exists; the fixture it writes is committed.

    python tests/golden/make_ref_large_pose.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from conftest import oracle_rollout, oracle_sim  # noqa: E402
from dexdeform_gb300 import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402

# the case of tests/test_gpu_full_size.py::test_large_config_adjoint
T, S = 5, 2
STATE_SEED, GRAD_SEED = 8, 4


def case():
    env = W.large_env(0, steps=S * T, sort=False)
    st0 = W.perturb_state(env, seed=STATE_SEED, v_scale=0.1, c_scale=1.0, f_scale=0.02)
    rng = np.random.default_rng(GRAD_SEED)
    g = {"x": rng.normal(size=(env.n, 3)).astype(np.float32), "v": rng.normal(size=(env.n, 3)).astype(np.float32),
         "F": rng.normal(size=(env.n, 3, 3)).astype(np.float32), "C": rng.normal(size=(env.n, 3, 3)).astype(np.float32)}
    return env, st0, g


def main():
    if not O.ref_available():
        raise SystemExit("oracle/_ref/libref_host.so is missing: run oracle/build_ref_host.sh")
    env, st0, g_final = case()
    n_sub = S * T
    states = oracle_rollout(O, env, n_sub, "exact", state=st0)
    ref = oracle_sim(O, env, backend="ref")
    g = {k: np.asarray(v, np.float32) for k, v in g_final.items()}
    bp = np.zeros((n_sub + 1, env.nb, 3))
    br = np.zeros((n_sub + 1, env.nb, 4))
    for t in range(n_sub - 1, -1, -1):
        s = {k: np.asarray(v, np.float32) for k, v in states[t].items()}
        g, (a, b), (c, d) = ref.substep_grad(s, env.pose(t), env.pose(t + 1),
                                             np.asarray(states[t + 1]["v"], np.float32), g)
        bp[t] += a
        br[t] += b
        bp[t + 1] += c
        br[t + 1] += d
    np.savez_compressed(os.path.join(HERE, "ref_large_pose_grad.npz"), pose_position=bp, pose_rotation=br,
                        substeps=np.int64(n_sub), state_seed=np.int64(STATE_SEED), grad_seed=np.int64(GRAD_SEED))
    print("wrote ref_large_pose_grad.npz")


if __name__ == "__main__":
    main()
