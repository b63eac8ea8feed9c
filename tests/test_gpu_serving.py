"""Serving loop on the GPU: continuous batching with HBM-footprint admission,
resident state, forward and gradient requests overlapping on two streams, and
every result the same alone and in the mix."""
import numpy as np
import pytest

from conftest import rel, within_spread

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def cuda(native_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return native_lib


def _requests(seed, n, T):
    from dexdeform_gb300.serving import poisson_requests
    return poisson_requests(seed=seed, n=n, rate_hz=200.0, n_lo=500, n_hi=4000, h_lo=1, h_hi=3, grad_frac=0.4,
                            substeps=T)


def test_mixed_results_equal_alone(cuda):
    from dexdeform_gb300.serving import Server, latency_stats
    T = 10
    reqs = _requests(0, 8, T)
    assert any(r.grad for r in reqs) and any(not r.grad for r in reqs)
    srv = Server(substeps=T, hbm_budget_bytes=8 * 2 ** 30)
    done = srv.run(reqs)
    assert len(done) == len(reqs)
    assert latency_stats(done)["n"] == len(reqs)
    mixed = {r.rid: r.result for r in done}
    for r in _requests(0, 8, T)[:5]:
        r.arrival = 0.0
        alone = Server(substeps=T, hbm_budget_bytes=8 * 2 ** 30).run([r])[0].result
        for k in alone:
            a, b = alone[k].cpu().numpy(), mixed[r.rid][k].cpu().numpy()
            assert np.isfinite(a).all()
            # states to FP32 rounding; gradients within the run-to-run
            # float-atomic ordering noise of the adjoint (also seen alone vs
            # alone)
            assert rel(b, a) < (1e-5 if k == "state" else 5e-4), (r.rid, k)


def _run(E, envs, T, grad):
    """T substeps forward (and with grad the adjoint of a fixed final
    gradient) of envs on engine E; returns the final state (and the state-0
    and body-pose gradients)."""
    s0 = E.pack_state([_state(e) for e in envs])
    sts = E.new_slots(T + 1)
    sts[0].copy_(s0)
    poses = torch.tensor(E.pack_poses([e.poses[:T + 1, :, :3] for e in envs],
                                      [e.poses[:T + 1, :, 3:] for e in envs]), device="cuda")
    if not grad:
        E.run_substeps(list(sts), poses)
        return (sts[T].clone(),)
    tape = E.new_tape(T)
    E.run_substeps(list(sts), poses, kept=True, tapes=tape)
    g = torch.randn(s0.shape, device="cuda", generator=torch.Generator(device="cuda").manual_seed(6))
    scratch = torch.zeros_like(s0)
    bgrad = torch.zeros_like(poses)
    out = E.run_adjoint(list(sts), g, scratch, poses, bgrad, tapes=tape)
    return sts[T].clone(), out.clone(), bgrad.clone()


def _state(env):
    from dexdeform_gb300 import workloads as W
    return W.perturb_state(env, seed=5, v_scale=0.1, c_scale=1.0, f_scale=0.02)


@pytest.mark.parametrize("grad", [False, True])
def test_relayout_equals_fresh_engine(cuda, grad):
    """An engine re-laid out in place (another number of envs, other grid
    sizes and bodies; a forward slot left in use by the previous layout)
    computes what an engine built for the new envs does, within the bars of
    the other schedule-equivalence tests (the float atomics add in another
    order in each run): states 2e-4, gradients 5e-4."""
    from dexdeform_gb300 import _native as N
    from dexdeform_gb300 import workloads as W
    from dexdeform_gb300.engine import BatchEngine, Capacity, EnvSpec
    T = 8
    A = W.batch_envs(1, n_envs=4, steps=T, n_lo=500, n_hi=3000, sort=False)
    B = W.batch_envs(2, n_envs=3, steps=T, n_lo=500, n_hi=3000, sort=False)
    spec = lambda envs: [EnvSpec.from_env(e) for e in envs]
    cap = Capacity.of(spec(A), 128).union(Capacity.of(spec(B), 128))
    kw = dict(grad=grad, grid_slots=T + 2 if grad else 2, capacity=cap)
    arena = BatchEngine(spec(A), **kw)
    _run(arena, A, T, grad)
    for envs in (B, A[1:3], A):
        arena.relayout(spec(envs))
        got = _run(arena, envs, T, grad)
        fresh = BatchEngine(spec(envs), **kw)
        want, again = _run(fresh, envs, T, grad), _run(fresh, envs, T, grad)
        assert arena.error_word() == 0
        cpu = lambda ts: tuple(t.cpu().numpy() for t in ts)
        within_spread(cpu(got), cpu(want), cpu(again), (2e-4, 5e-4, 5e-4))
    big = W.batch_envs(3, n_envs=6, steps=T, n_lo=500, n_hi=3000, sort=False)
    assert not arena.fits(spec(big))
    with pytest.raises(N.DexError):
        arena.relayout(spec(big))


def test_sorted_rounds_equal_unsorted(cuda):
    """Requests in sampling order: rounds that sort the gathered particles by
    grid cell on the device (the default) return what rounds in the
    requests' own order do, in the requests' order, within the bars of the
    schedule-equivalence tests (states 2e-4, gradients 5e-4)."""
    from dexdeform_gb300.serving import Server
    T = 10
    res = []
    for sort in (False, True):
        reqs = _requests(4, 6, T)
        done = Server(substeps=T, hbm_budget_bytes=8 * 2 ** 30, sort=sort).run(reqs)
        res.append({r.rid: r.result for r in done})
    assert any("grad_state0" in v for v in res[0].values())
    for rid, want in res[0].items():
        for k, a in want.items():
            tol = 2e-4 if k == "state" else 5e-4
            assert rel(res[1][rid][k].cpu().numpy(), a.cpu().numpy()) < tol, (rid, k)


def test_serving_relays_out_instead_of_rebuilding(cuda):
    """Membership changes re-lay the phase's engine out; it is rebuilt only
    when a membership outgrows it."""
    from dexdeform_gb300.serving import Server
    T = 10
    srv = Server(substeps=T, hbm_budget_bytes=8 * 2 ** 30)
    done = srv.run(_requests(3, 12, T))
    assert len(done) == 12
    assert srv.relayouts > 2 * srv.engine_builds
    br = srv.breakdown(1.0)
    assert br["relayouts"] == srv.relayouts


def test_copy_segments_gathers_scatters_and_adds(cuda):
    """dexmpm_copy_segments: blocks of planes of different lengths and
    strides into columns of one buffer and back (copy and add), exactly."""
    from dexdeform_gb300 import _native as N
    from dexdeform_gb300.serving import copy_segments
    gen = torch.Generator(device="cuda").manual_seed(0)
    planes, stride = 5, 1000
    parts = [torch.randn((planes, n), device="cuda", generator=gen) for n in (7, 300, 1, 129)]
    offs = [0, 10, 400, 600]
    buf = torch.zeros((planes, stride), device="cuda")
    copy_segments([(t, t.shape[1], o, t.shape[1]) for t, o in zip(parts, offs)], planes, buf, stride,
                  N.SEGMENTS_GATHER)
    for t, o in zip(parts, offs):
        assert torch.equal(buf[:, o:o + t.shape[1]], t)
    assert float(buf[:, 310:400].abs().sum()) == 0.0
    buf.mul_(2.0)
    back = [torch.zeros_like(t) for t in parts]
    copy_segments([(t, t.shape[1], o, t.shape[1]) for t, o in zip(back, offs)], planes, buf, stride,
                  N.SEGMENTS_SCATTER)
    copy_segments([(t, t.shape[1], o, t.shape[1]) for t, o in zip(parts, offs)], planes, buf, stride,
                  N.SEGMENTS_SCATTER_ADD)
    for t, b, o in zip(parts, back, offs):
        assert torch.equal(b, buf[:, o:o + t.shape[1]]) and torch.allclose(t, 1.5 * b)
    # more segments than one launch carries (512 per launch)
    many = [torch.randn((planes, 3), device="cuda", generator=gen) for _ in range(600)]
    wide = torch.zeros((planes, 3 * 600), device="cuda")
    copy_segments([(t, 3, 3 * i, 3) for i, t in enumerate(many)], planes, wide, 3 * 600, N.SEGMENTS_GATHER)
    assert torch.equal(wide, torch.cat(many, 1))
    # a block that is a row range of a larger tensor (the poses of some substeps)
    poses = torch.randn((30, 3, 8), device="cuda", generator=gen)
    pbuf = torch.zeros((11, 5, 8), device="cuda")
    copy_segments([(poses[12], 3 * 8, 2 * 8, 3 * 8)], 11, pbuf, 5 * 8, N.SEGMENTS_GATHER)
    assert torch.equal(pbuf[:, 2:5], poses[12:23])


def test_admission_respects_budget(cuda):
    from dexdeform_gb300.serving import Server
    T = 10
    reqs = _requests(1, 6, T)
    one = max(r.footprint(T) for r in reqs)
    srv = Server(substeps=T, hbm_budget_bytes=int(one * 1.5))
    peak = []
    orig = srv.step

    def step(now):
        ok = orig(now)
        peak.append(srv.in_use)
        return ok

    srv.step = step
    done = srv.run(reqs)
    assert len(done) == len(reqs)
    assert max(peak) <= srv.budget
    with pytest.raises(ValueError):
        big = _requests(2, 1, T)[0]
        Server(substeps=T, hbm_budget_bytes=1024).submit(big)
