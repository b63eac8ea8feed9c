"""The CUDA renderer (particle_sdf, render) through libdexmpm.so's C ABI
against the reference's own renderer code (committed fixture, run on the
host with the shared counter-based generator) and the CPU restatement.

The volume bake is compared bit for bit (SHA-256 of the packed volume, the
distance and the color volume).  The images are compared per pixel: the
kernel keeps the reference's unfused float arithmetic, so pixels agree to
the last bit except where cos/sin rounding on the device and on the host
sends a diffuse bounce elsewhere; the bounds allow 1% of such pixels."""
import ctypes

import numpy as np
import pytest

from conftest import render_fixture, sha256

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def cuda(native_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return native_lib


def _t(a, dtype=torch.float32):
    return torch.tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def device_bake(lib, sc):
    from dexdeform_gb300 import _native as N
    nv = int(np.prod(sc["voxel"]))
    vol = torch.full((nv,), (1 << 33) - 1, dtype=torch.int64, device="cuda")
    sdf, tmp = torch.zeros(nv, device="cuda"), torch.zeros(nv, device="cuda")
    colv = torch.zeros((nv, 3), device="cuda")
    x, col = _t(sc["x"]), _t(sc["color"], torch.int32)
    lo, hi = _t(sc["bbox_min"]), _t(sc["bbox_max"])
    g = (ctypes.c_int * 3)(*sc["voxel"])
    assert lib.particle_sdf(N.ptr(vol), N.ptr(x), N.ptr(col), N.ptr(lo), N.ptr(hi), sc["bake"], g, sc["inv_dx"],
                            N.ptr(sdf), N.ptr(colv), N.ptr(tmp), int(x.shape[0]), N.stream_ptr()) == 0
    torch.cuda.synchronize()
    return vol, sdf, colv


def device_render(lib, sc, sdf, colv):
    from dexdeform_gb300 import _native as N
    H, W = sc["image"]
    color, depth = torch.zeros((H * W, 3), device="cuda"), torch.zeros(H * W, device="cuda")
    arrs = [_t(sc[k]) for k in ("bbox_min", "bbox_max", "body_pos", "body_rot", "body_tfsr", "body_args", "cam_rot",
                                "cam_pos", "cam_intr", "light")]
    lo, hi, bp, br, bt, ba, cr, cp, ci, light = arrs
    g = (ctypes.c_int * 3)(*sc["voxel"])
    im = (ctypes.c_int * 3)(H, W, 3)
    rc = lib.render(N.ptr(sdf), N.ptr(lo), N.ptr(hi), N.ptr(colv), N.ptr(bp), N.ptr(br), N.ptr(bt), N.ptr(ba),
                    N.ptr(cr), N.ptr(cp), N.ptr(ci), N.ptr(color), N.ptr(depth), sc["sdf_threshold"], g,
                    int(bp.shape[0]), bool(sc["visualize_shape"]), im, sc["max_ray_depth"], sc["spp"], sc["ground"],
                    sc["seed"], N.ptr(light), N.stream_ptr())
    assert rc == 0
    torch.cuda.synchronize()
    return color.cpu().numpy().reshape(H, W, 3), depth.cpu().numpy().reshape(H, W)


def assert_images_agree(img, dep, ref_img, ref_dep):
    diff = np.abs(img - ref_img).max(-1)
    ddiff = np.abs(dep - ref_dep) / np.maximum(np.abs(ref_dep), 1.0)
    assert np.isfinite(img).all() and np.isfinite(dep).all()
    assert (diff > 1e-6).mean() <= 0.01, (diff > 1e-6).mean()
    assert (ddiff > 1e-6).mean() <= 0.01, (ddiff > 1e-6).mean()
    assert diff.mean() < 1e-3


def test_particle_sdf_is_bit_identical_to_reference(cuda):
    sc, ref = render_fixture()
    vol, sdf, colv = device_bake(cuda, sc)
    assert (sha256(vol.cpu().numpy()) == ref["volume_sha256"]).all()
    assert (sha256(sdf.cpu().numpy()) == ref["sdf_sha256"]).all()
    assert (sha256(colv.cpu().numpy()) == ref["color_sha256"]).all()


def test_render_matches_reference_fixture(cuda):
    sc, ref = render_fixture()
    _, sdf, colv = device_bake(cuda, sc)
    img, dep = device_render(cuda, sc, sdf, colv)
    assert_images_agree(img, dep, ref["image"], ref["depth"])


def test_render_matches_oracle_on_other_scenes(cuda, oracle_mod):
    from dexdeform_gb300 import workloads as W
    for seed, image, spp, depth, vis in ((1, (96, 128), 3, 3, 1), (2, (64, 64), 1, 1, 0)):
        sc = W.render_scene(seed, n=4000, voxel=40, image=image, spp=spp, max_ray_depth=depth)
        sc["visualize_shape"] = vis
        vol, sdf, colv = device_bake(cuda, sc)
        ov, osdf, ocol = oracle_mod.particle_sdf("oracle", sc["x"], sc["color"], sc["bbox_min"], sc["bake"],
                                                 sc["voxel"], sc["inv_dx"])
        assert np.array_equal(vol.cpu().numpy(), ov) and np.array_equal(sdf.cpu().numpy(), osdf)
        img, dep = device_render(cuda, sc, sdf, colv)
        oimg, odep = oracle_mod.render("oracle", sc, osdf, ocol)
        assert_images_agree(img, dep, oimg, odep)


def test_renderer_class_end_to_end(cuda):
    """The drop-in Renderer on the MPMSimulator mirror: bake the simulator's
    particles with their colors and trace its bodies; a fixed seed
    reproduces the image, consecutive renders advance the seed."""
    from dexdeform_gb300 import workloads as W
    from dexdeform_gb300.renderer import Renderer
    from dexdeform_gb300.simulator import MPMSimulator
    env = W.tiny_env(0, n=2000, grid=64, nb=4, steps=2)
    sim = MPMSimulator(env.nb, n_particles=env.n, dx=env.dx, dt=env.dt, grid_size=(1, 1, 1), max_steps=2,
                       substeps=1, gravity=(0, -1, 0), ground_friction=env.ground_friction)
    sim.init_particles(env.vol.astype(np.float64), env.mass.astype(np.float64), env.mu_lam_yield.astype(np.float64))
    sim.init_bodies(env.body_tfsr[:, 0], env.body_tfsr[:, 2], env.body_tfsr[:, 1], env.body_tfsr[:, 3],
                    env.body_args, None)
    st = env.state()
    sim.set_state(0, (st["x"], st["v"], st["F"], st["C"], *list(env.poses[0])))
    sim.set_color(np.full(env.n, 0xC08040, np.int32))
    r = Renderer(voxel_res=(64, 64, 64), image_res=(48, 64), spp=2, inv_dx=128.0)
    r.lookat((0.5, 0.2, 0.5), 0.4, 0.2, 1.5)
    out = r.render(sim, sim.states[0])
    assert out.shape == (48, 64, 4) and np.isfinite(out).all() and r.render_seed == 1
    assert (out[..., 3] > 0).all()
    ground = sim.get_ground_height() * sim.dx
    st0 = sim.states[0]
    nb = sim.n_bodies
    a = r.trace(st0.body_pos.t[:nb], st0.body_rot.t[:nb], sim.body_type_mu_softness_round.t[:nb],
                sim.body_args.t[:nb], ground, seed=5)
    b = r.trace(st0.body_pos.t[:nb], st0.body_rot.t[:nb], sim.body_type_mu_softness_round.t[:nb],
                sim.body_args.t[:nb], ground, seed=5)
    assert np.array_equal(a, b)
