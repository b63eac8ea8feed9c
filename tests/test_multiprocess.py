"""The N > 1 host path of bench.py on the CPU: two gloo ranks on 127.0.0.1.
Each rank runs its own replica batch (seeded by its rank; no collective on
the data path), and the whole-job value is the units of all ranks over the
slowest rank's time."""
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, queue):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    envs = bench.build_batch(rank, 3)
    work = sum(e.n for e in envs) * bench.SUBSTEPS * bench.ENV_STEPS
    t_ms = 100.0 * (rank + 1)
    value, t_max = bench.weak_scaling_value(work, t_ms, 5, world)
    queue.put((rank, work, value, t_max, float(envs[0].x[0, 0])))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replicas_and_reductions():
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    (r0, w0, v0, t0, x0), (r1, w1, v1, t1, x1) = res
    assert t0 == t1 == 200.0                      # max over ranks
    assert v0 == v1 == pytest.approx((w0 + w1) * 5 / 0.2)
    assert x0 != x1                               # distinct replica batches


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_reference_arm_prints_the_contract_line(oracle_mod):
    """Rank 0 of the reference arm (bench.py --impl reference) times the CPU
    path on a bounded sample and prints one JSON line with the keys the
    benchmark contract asks for: its own metric, value and unit, impl
    "reference", a cpu_baseline describing the run, and an e2e with no
    host-device copies.  Tiny sizes (2 envs, 1 env step of 2 substeps)."""
    import json
    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--envs", "2", "--substeps", "2", "--env-steps", "1"],
                       capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "particle-substeps/s"
    assert d["steps"] == 1 and d["warmup"] == 0 and d["higher_is_better"] is True and d["ms_per_step"] > 0
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"] and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert "workload" in d["config"]
