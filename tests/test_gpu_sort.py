"""Device-side particle ordering (dexmpm_sort, dexmpm_permute) and the
rollouts that use it.

* The permutation is integer work and must equal, entry for entry, the one
  this file computes in numpy: every env's particles ordered by the 4^3 grid
  block of their stencil base cell, then the cell within the block, then the
  previous index (out-of-grid positions clamped to the nearest cell).
* Permuting is bit-exact, and scatter after gather is the identity.
* A rollout that sorts (at the start of every env step, from the caller's
  sampling order) gives the caller the results of one that never sorts, up to
  the run-to-run ordering of float atomics: the same bars as the other
  schedule-equivalence tests (final state 2e-4, gradients 5e-4).
"""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def cuda(native_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return native_lib


def expected_perm(E, state):
    """numpy restatement of the sort order: perm[i] = old index of the
    particle that goes to i (identity on the padding)."""
    x = state[0:3].cpu().numpy().astype(np.float32)
    perm = np.arange(E.n_particles, dtype=np.int64)
    for e, s in enumerate(E.specs):
        o, n = E.p_off[e], s.n
        inv = np.float32(1.0 / s.dx)
        f = np.floor((x[:, o:o + n] * inv).astype(np.float32) - np.float32(0.5)).astype(np.float64)
        g = np.asarray(s.grid_dim)[:, None]
        c = np.where(f >= 0, np.minimum(f, g - 1), 0).astype(np.int64)
        nby, nbz = s.grid_dim[1] // 4, s.grid_dim[2] // 4
        blk = E.blk_off[e] + ((c[0] >> 2) * nby + (c[1] >> 2)) * nbz + (c[2] >> 2)
        key = (blk << 6) + ((c[0] & 3) << 4) + ((c[1] & 3) << 2) + (c[2] & 3)
        idx = np.arange(o, o + n)
        perm[o:o + n] = idx[np.lexsort((idx, key))]
    return perm


def block_and_cell_sizes(E, state):
    """Largest 4^3-block population, every block's population, largest cell
    population of the sort keys."""
    x = state[0:3].cpu().numpy().astype(np.float32)
    blocks, cells = [], []
    for e, s in enumerate(E.specs):
        o, n = E.p_off[e], s.n
        f = np.floor((x[:, o:o + n] * np.float32(1.0 / s.dx)).astype(np.float32) - np.float32(0.5))
        g = np.asarray(s.grid_dim)[:, None]
        c = np.where(f >= 0, np.minimum(f, g - 1), 0).astype(np.int64)
        blk = ((c[0] >> 2) * (s.grid_dim[1] // 4) + (c[1] >> 2)) * (s.grid_dim[2] // 4) + (c[2] >> 2)
        cell = (c[0] * s.grid_dim[1] + c[1]) * s.grid_dim[2] + c[2]
        bc = np.bincount(blk)
        blocks.append(bc[bc > 0])
        cells.append(np.bincount(cell).max())
    b = np.concatenate(blocks)
    return int(b.max()), b, int(max(cells))


def _engine(envs, **kw):
    from dexdeform_gb300.engine import BatchEngine, EnvSpec
    return BatchEngine([EnvSpec.from_env(e) for e in envs], **kw)


def test_sort_matches_numpy_order_and_permutes_exactly(cuda):
    from dexdeform_gb300 import workloads as W
    envs = W.batch_envs(11, n_envs=5, steps=1, n_lo=300, n_hi=5000, sort=False)
    envs.append(W.make_env(3, 1500, "cube", grid=32, center=(0.5, 0.2, 0.5), extent=0.3, nb=3, steps=1,
                           sort=False))
    # dense clusters: 4^3 blocks of 1,024 - 8,192 particles (staged by a whole
    # CTA), of more than 8,192 (cell by cell), and cells of more than 1,024
    # (insertion sort in place)
    envs.append(W.make_env(4, 6000, "cube", grid=32, center=(0.5, 0.3, 0.5), extent=0.12, nb=1, steps=1,
                           sort=False))
    envs.append(W.make_env(5, 12000, "cube", grid=32, center=(0.41, 0.41, 0.41), extent=0.06, nb=1, steps=1,
                           sort=False))
    envs.append(W.make_env(6, 20000, "cube", grid=32, center=(0.453, 0.453, 0.453), extent=0.07, nb=1, steps=1,
                           sort=False))
    envs[1].x = envs[1].x.copy()
    envs[1].x[7] = (2.0, -0.5, np.nan)   # outside the grid on every axis: clamped, still sorted
    E = _engine(envs)
    s = E.pack_state([e.state() for e in envs])
    sizes = block_and_cell_sizes(E, s)
    assert sizes[0] > 8192 and ((sizes[1] > 1024) & (sizes[1] <= 8192)).any() and sizes[2] > 1024, sizes[::2]
    out = torch.zeros_like(s)
    perm = E.identity_perm(1)[0]
    E.sort(s, out, perm)
    got = perm.cpu().numpy()
    want = expected_perm(E, s)
    assert (got == want).all()
    src = s.cpu().numpy()
    assert np.array_equal(out.cpu().numpy(), src[:, got], equal_nan=True)
    # a second sort of the sorted state keeps it (the scratch was left clean)
    perm2 = E.identity_perm(1)[0]
    out2 = torch.zeros_like(s)
    E.sort(out, out2, perm2)
    assert (perm2.cpu().numpy() == np.arange(E.n_particles)).all()
    assert np.array_equal(out2.cpu().numpy(), out.cpu().numpy(), equal_nan=True)
    # scatter after gather is the identity, also for int32 planes
    back = torch.zeros_like(s)
    E.permute(perm, out, back, inverse=True)
    assert np.array_equal(back.cpu().numpy(), src, equal_nan=True)
    ids = torch.arange(E.n_particles, dtype=torch.int32, device="cuda")[None].repeat(2, 1).contiguous()
    ids_s = torch.zeros_like(ids)
    E.permute(perm, ids, ids_s)
    assert (ids_s.cpu().numpy() == got[None]).all()
    torch.cuda.synchronize()


def test_sorted_order_cuts_scatter_segments(cuda):
    """What the sort is for: after it, a warp's 32 particles share few
    stencil bases (counted on the host from the sorted positions)."""
    from dexdeform_gb300 import workloads as W
    envs = W.batch_envs(0, n_envs=8, steps=1, sort=False)
    E = _engine(envs)
    s = E.pack_state([e.state() for e in envs])
    out = torch.zeros_like(s)
    E.sort(s, out, E.identity_perm(1)[0])

    def mean_bases_per_warp(st):
        x = st[0:3].cpu().numpy()
        n = []
        for e, sp in enumerate(E.specs):
            o = E.p_off[e]
            b = np.floor(x[:, o:o + sp.n] / sp.dx - 0.5).astype(np.int64)
            key = (b[0] * 4096 + b[1]) * 4096 + b[2]
            for w in range(0, sp.n - 31, 32):
                n.append(len(np.unique(key[w:w + 32])))
        return float(np.mean(n))

    # measured on these envs: ~31 distinct bases per warp in sampling order,
    # ~5 after the sort (~3 where an env has ~10 particles per cell)
    before, after = mean_bases_per_warp(s), mean_bases_per_warp(out)
    assert before > 25 and after < 8, (before, after)


def _rollout_pair(envs, T, S, state0_fn, grad=True):
    """Results of rollouts that never sort (twice: the spread of two identical
    runs), sort every env step, or every other one."""
    from dexdeform_gb300.engine import Rollout
    outs = []
    for sort_every in (0, 0, 1, 2):
        E = _engine(envs, grad=grad, grid_slots=2 * T + 2 if grad else 2)
        R = Rollout(E, substeps=T, env_steps=S, sort_every=sort_every)
        R.poses.copy_(torch.tensor(E.pack_poses([e.poses[:, :, :3] for e in envs],
                                                [e.poses[:, :, 3:] for e in envs]), device="cuda")[:S * T + 1])
        s0 = E.pack_state(state0_fn())
        # a per-particle gradient on every field, the same in every variant
        # (a uniform one would hide particles handed back in another order)
        g = torch.randn(s0.shape, device="cuda", generator=torch.Generator(device="cuda").manual_seed(5))
        for _ in range(2):  # eager + capture, then a replay
            fin = R.forward(s0).clone()
            g0 = R.backward(g).clone() if grad else None
        mid = R.state(1).clone() if grad else None
        assert E.error_word() == 0
        outs.append((fin, g0, R.bgrad.clone() if grad else None, mid))
    return outs


def test_sorting_rollout_equals_unsorted(cuda):
    """Forward + backward over 3 env steps, sorting at every env step, every
    other one, or never; inputs in sampling order; results in the caller's
    order agree."""
    from dexdeform_gb300 import workloads as W
    envs = W.batch_envs(5, n_envs=3, steps=30, n_lo=500, n_hi=3000, sort=False)
    outs = _rollout_pair(envs, 10, 3, lambda: [W.perturb_state(e, seed=3, v_scale=0.1, c_scale=1.0, f_scale=0.02)
                                               for e in envs])
    # within max(bar, 4 x the spread of two identical unsorted runs): the
    # per-particle gradient seeds make the float-atomic noise of the adjoint
    # over 30 substeps reach the bar's order
    spread = [rel(a.cpu().numpy(), b.cpu().numpy()) for a, b in zip(outs[0], outs[1])]
    for other in outs[2:]:
        for (a, b), tol, n in zip(zip(outs[0], other), (2e-4, 5e-4, 5e-4, 2e-4), spread):
            assert rel(a.cpu().numpy(), b.cpu().numpy()) < max(tol, 4 * n), (tol, n)


def test_sorting_forward_only_rollout_equals_unsorted(cuda):
    from dexdeform_gb300 import workloads as W
    envs = W.batch_envs(6, n_envs=3, steps=30, n_lo=500, n_hi=3000, sort=False)
    outs = _rollout_pair(envs, 10, 3, lambda: [e.state() for e in envs], grad=False)
    for other in outs[2:]:
        assert rel(other[0].cpu().numpy(), outs[0][0].cpu().numpy()) < 2e-4


def test_env_step_autograd_sorts_and_maps_back(cuda):
    """EnvStep (DiffSim) with and without the sort: same output and the same
    gradients, in the caller's order."""
    from dexdeform_gb300 import workloads as W
    from dexdeform_gb300.engine import EnvSpec, pack_poses
    from dexdeform_gb300.torch_wrapper import DiffSim, env_step
    T = 6
    env = W.tiny_env(4, n=2000, grid=32, nb=5, steps=T, dt=1e-4)
    env.x = env.x[np.random.default_rng(0).permutation(env.n)]  # sampling order
    st = W.perturb_state(env, seed=2, v_scale=0.1, c_scale=1.0, f_scale=0.02)
    poses = torch.tensor(pack_poses(env.poses[:, :, :3], env.poses[:, :, 3:]), device="cuda")
    res = []
    for sort in (False, True):
        sim = DiffSim([EnvSpec.from_env(env)], T, sort=sort)
        s0 = sim.E.pack_state([st]).requires_grad_(True)
        p = poses.clone().requires_grad_(True)
        out = env_step(sim, s0, p)
        w = torch.linspace(-1, 1, out.numel(), device="cuda").reshape(out.shape)
        (out * w).sum().backward()
        res.append((out.detach().clone(), s0.grad.clone(), p.grad.clone()))
        assert sim.E.error_word() == 0
    for (a, b), tol in zip(zip(res[0], res[1]), (2e-5, 5e-4, 5e-4)):
        assert rel(a.cpu().numpy(), b.cpu().numpy()) < tol
