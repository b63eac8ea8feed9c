"""The allocation-free entry point, dexmpm_substep_noalloc, through the C ABI.

It exists for callers that cannot call cudaMalloc (an application whose own
pool allocator owns the GPU's memory, a real-time loop that must not block on
an allocation): its scratch is a fixed device array inside the library.  This
test steps one environment twice in a row with it and checks each step against
the existing entry point (dexmpm_substep via BatchEngine), and that the second
call changes the device's free memory by nothing.  It is collected last so that
a failure here leaves every other test already run."""
import ctypes

import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_noalloc_substep_matches_existing_entry_point_twice(native_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from dexdeform_gb300 import _native as N
    from dexdeform_gb300 import workloads as W
    from dexdeform_gb300.engine import BatchEngine, EnvSpec, pack_poses, plan_layout

    env = W.plain_env(0, steps=2)  # 64^3 grid, 5,000 particles, 22 capsules
    spec = EnvSpec.from_env(env)
    poses = torch.tensor(pack_poses(env.poses[:, :, :3], env.poses[:, :, 3:]), device="cuda")

    # existing entry point
    E = BatchEngine([spec])
    s = E.pack_state([env.state()])
    nxt = E.new_slots(1)[0]
    want = []
    for t in range(2):
        E.substep(s, nxt, poses[t], poses[t + 1])
        s, nxt = nxt, s
        want.append(E.unpack_state(s)[0])

    # new entry point: planes of exactly n particles, caller-owned buffers only
    n = env.n
    desc = plan_layout([spec], 128)["envs"][0]
    st = env.state()
    host = np.zeros((24, n), np.float32)
    host[0:3], host[3:6] = st["x"].T, st["v"].T
    host[6:15], host[15:24] = st["F"].reshape(n, 9).T, st["C"].reshape(n, 9).T
    slots = [torch.tensor(host, device="cuda"), torch.zeros((24, n), device="cuda"),
             torch.zeros((24, n), device="cuda")]
    mass = torch.tensor(env.mass, device="cuda")
    vol = torch.tensor(env.vol, device="cuda")
    mly = torch.tensor(np.ascontiguousarray(env.mu_lam_yield.T), device="cuda")
    shapes = torch.tensor(np.concatenate([env.body_tfsr, env.body_args], 1), device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    stream = N.stream_ptr()

    def call(t):
        return native_lib.dexmpm_substep_noalloc(ctypes.byref(desc), N.ptr(slots[t]), N.ptr(slots[t + 1]),
                                                 N.ptr(mass), N.ptr(vol), N.ptr(mly), N.ptr(shapes),
                                                 N.ptr(poses[t]), N.ptr(poses[t + 1]), N.ptr(err), stream)

    assert call(0) == N.OK
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    assert call(1) == N.OK
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before
    assert int(err.item()) == 0

    for t in range(2):
        got = slots[t + 1].cpu().numpy()
        g = {"x": got[0:3].T, "v": got[3:6].T, "F": got[6:15].T.reshape(n, 3, 3), "C": got[15:24].T.reshape(n, 3, 3)}
        for k in ("x", "v", "F", "C"):
            assert rel(g[k], want[t][k]) < 1e-5, (t, k)

    # sizes beyond the array are rejected, not run
    big = plan_layout([EnvSpec.from_env(W.tiny_env(0, n=64, grid=32, nb=1, steps=1))], 128)["envs"][0]
    big.gx = big.gy = big.gz = 68
    assert native_lib.dexmpm_substep_noalloc(ctypes.byref(big), N.ptr(slots[0]), N.ptr(slots[1]), N.ptr(mass),
                                             N.ptr(vol), N.ptr(mly), N.ptr(shapes), N.ptr(poses[0]),
                                             N.ptr(poses[1]), N.ptr(err), stream) == N.ERR_ARG
