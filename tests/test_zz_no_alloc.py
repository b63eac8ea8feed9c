"""The allocation-free entry point, dexmpm_substep_noalloc, through the C ABI.

It exists for callers that cannot call cudaMalloc (an application whose own
pool allocator owns the GPU's memory, a real-time loop that must not block on
an allocation): its scratch is a fixed device array inside the library.  This
test steps one environment twice in a row with it and checks each step against
the existing entry point (dexmpm_substep via BatchEngine), and that the second
call changes the device's free memory by nothing; then a non-cubic grid with no
bodies, and the argument checks.  It is collected last so that
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

    # a second call shape after the first: a non-cubic grid as large as the
    # array allows (128 x 32 x 64 cells), no bodies and null pose pointers;
    # its grid, flags and lists are re-zeroed for the new size
    rng = np.random.default_rng(4)
    n2 = 3000
    x2 = (np.array([1.0, 0.2, 0.5]) + (rng.random((n2, 3)) - 0.5) * 0.2).astype(np.float32)
    env2 = W.Env(grid_dim=(128, 32, 64), dx=1 / 64, dt=5e-5, gravity=(0.0, -30.0, 0.0), ground_friction=0.9,
                 x=x2, v=(rng.normal(size=(n2, 3)) * 0.1).astype(np.float32),
                 F=np.broadcast_to(np.eye(3, dtype=np.float32), (n2, 3, 3)).copy(),
                 C=np.zeros((n2, 3, 3), np.float32), mass=np.full(n2, 1e-6, np.float32),
                 vol=np.full(n2, 1e-6, np.float32), mu_lam_yield=np.tile(np.float32([2083.3, 1388.9, 50.0]), (n2, 1)),
                 body_tfsr=np.zeros((0, 4), np.float32), body_args=np.zeros((0, 4), np.float32),
                 poses=np.zeros((2, 0, 7), np.float32))
    spec2 = EnvSpec.from_env(env2)
    E2 = BatchEngine([spec2])
    dummy = torch.zeros((1, 8), device="cuda")
    a2, b2 = E2.pack_state([env2.state()]), E2.new_slots(1)[0]
    E2.substep(a2, b2, dummy, dummy)
    want2 = E2.unpack_state(b2)[0]
    assert E2.error_word() == 0
    desc2 = plan_layout([spec2], 128)["envs"][0]
    st2 = env2.state()
    h2 = np.zeros((24, n2), np.float32)
    h2[0:3], h2[3:6] = st2["x"].T, st2["v"].T
    h2[6:15], h2[15:24] = st2["F"].reshape(n2, 9).T, st2["C"].reshape(n2, 9).T
    in2, out2 = torch.tensor(h2, device="cuda"), torch.zeros((24, n2), device="cuda")
    m2, v2 = torch.tensor(env2.mass, device="cuda"), torch.tensor(env2.vol, device="cuda")
    mly2 = torch.tensor(np.ascontiguousarray(env2.mu_lam_yield.T), device="cuda")
    null = ctypes.c_void_p(0)
    assert native_lib.dexmpm_substep_noalloc(ctypes.byref(desc2), N.ptr(in2), N.ptr(out2), N.ptr(m2), N.ptr(v2),
                                             N.ptr(mly2), null, null, null, N.ptr(err), stream) == N.OK
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    got2 = out2.cpu().numpy()
    g2 = {"x": got2[0:3].T, "v": got2[3:6].T, "F": got2[6:15].T.reshape(n2, 3, 3),
          "C": got2[15:24].T.reshape(n2, 3, 3)}
    for k in ("x", "v", "F", "C"):
        assert rel(g2[k], want2[k]) < 1e-5, ("non-cubic", k)

    # a null error word and invalid steps are rejected, not run
    assert native_lib.dexmpm_substep_noalloc(ctypes.byref(desc2), N.ptr(in2), N.ptr(out2), N.ptr(m2), N.ptr(v2),
                                             N.ptr(mly2), null, null, null, null, stream) == N.ERR_ARG
    bad = plan_layout([spec2], 128)["envs"][0]
    bad.dx = -bad.dx
    assert native_lib.dexmpm_substep_noalloc(ctypes.byref(bad), N.ptr(in2), N.ptr(out2), N.ptr(m2), N.ptr(v2),
                                             N.ptr(mly2), null, null, null, N.ptr(err), stream) == N.ERR_ARG
    bad = plan_layout([spec2], 128)["envs"][0]
    bad.dt = float("nan")
    assert native_lib.dexmpm_substep_noalloc(ctypes.byref(bad), N.ptr(in2), N.ptr(out2), N.ptr(m2), N.ptr(v2),
                                             N.ptr(mly2), null, null, null, N.ptr(err), stream) == N.ERR_ARG

    # sizes beyond the array are rejected, not run
    big = plan_layout([EnvSpec.from_env(W.tiny_env(0, n=64, grid=32, nb=1, steps=1))], 128)["envs"][0]
    big.gx = big.gy = big.gz = 68
    assert native_lib.dexmpm_substep_noalloc(ctypes.byref(big), N.ptr(slots[0]), N.ptr(slots[1]), N.ptr(mass),
                                             N.ptr(vol), N.ptr(mly), N.ptr(shapes), N.ptr(poses[0]),
                                             N.ptr(poses[1]), N.ptr(err), stream) == N.ERR_ARG
