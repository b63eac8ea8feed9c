"""Serving loop on the GPU: continuous batching with HBM-footprint admission,
resident state, forward and gradient requests overlapping on two streams, and
every result the same alone and in the mix."""
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
