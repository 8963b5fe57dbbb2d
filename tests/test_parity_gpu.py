"""Parity of the CUDA training step against the CPU oracle (GPU only).

Bars (per the engine's contract):
  * integer outputs (radii, tiles hit, per-tile counts, sorted per-tile id
    lists, last-contributor indices): identical to the oracle's float path;
  * image: <= 1e-5 max-abs against the oracle's float path (same decisions);
  * gradients and Adam updates: <= 1e-4 relative L2 against the float path;
    the first step's gradients also against FP64 (after some training FP64
    moves sigma/alpha threshold decisions of a few splats, and its errors are
    printed instead: test_c1_run_sampled_steps, the headline tests).
The FP64 comparison of integer and image outputs is reported and held to a
looser statistical bar: FP64 moves a few threshold decisions.
"""
import numpy as np
import pytest

from msplat_gb300 import engine as E
from msplat_gb300 import synthetic as S

from gpu_helpers import gt_image, rel_l2, run_pair

pytestmark = pytest.mark.gpu

IMG_TOL = 1e-5
GRAD_TOL = 1e-4


@pytest.fixture(scope="module")
def small():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    sc = S.config_small(0)
    cam = sc.train_cams[0]
    gt = gt_image(sc.gt, cam)
    init = S.init_from_gt(sc.gt, 0)
    return sc, cam, gt, init


def _check_forward(eo, r32, n):
    act = r32["radii"] > 0
    assert np.array_equal(eo["radii"], r32["radii"])
    assert np.array_equal(eo["num_tiles_hit"], r32["num_tiles_hit"])
    for k in ("depths", "xys", "conics", "colors", "aabb"):
        assert np.array_equal(eo[k][act], r32[k][act]), k
    assert np.array_equal(eo["tile_counts"], r32["tile_counts"])
    assert eo["num_isect"] == r32["num_isect"]
    assert np.array_equal(eo["gaussian_ids"], r32["gaussian_ids"])
    assert np.array_equal(eo["final_idx"], r32["final_idx"])
    assert np.max(np.abs(eo["out_img"] - r32["out_img"])) <= IMG_TOL
    assert np.max(np.abs(eo["final_Ts"] - r32["final_Ts"])) <= IMG_TOL


def _fp64_report(eo, r64):
    d = np.abs(eo["out_img"] - r64["out_img"])
    return dict(max_abs=float(d.max()), frac_over=float(np.mean(d > IMG_TOL)),
                ids_equal=bool(np.array_equal(eo["gaussian_ids"], r64["gaussian_ids"])),
                radii_mismatch=int(np.sum(eo["radii"] != r64["radii"])))


@pytest.mark.parametrize("raster_mode", [0, 1])
def test_forward_parity(small, raster_mode):
    sc, cam, gt, init = small
    step = E.step_scalars(1, 1, width=cam.width, height=cam.height)
    step["degrees_to_use"] = 3
    eo, res = run_pair(init, cam, gt, step, raster_mode=raster_mode, do_backward=False)
    assert eo["k_max"] == res[32]["k_max"]
    _check_forward(eo, res[32], init.n)
    rep = _fp64_report(eo, res[64])
    print("fp64", rep)
    assert rep["frac_over"] < 2e-3
    assert rep["radii_mismatch"] <= max(2, init.n // 1000)


@pytest.mark.parametrize("raster_mode", [0, 1])
def test_train_step_parity(small, raster_mode):
    sc, cam, gt, init = small
    step = E.step_scalars(1, 1, width=cam.width, height=cam.height)
    step["degrees_to_use"] = 3
    eo, res = run_pair(init, cam, gt, step, raster_mode=raster_mode)
    r32, r64 = res[32], res[64]
    _check_forward(eo, r32, init.n)
    assert abs(eo["loss"] - r32["loss"]) <= 1e-5 * max(1.0, abs(r32["loss"]))
    assert rel_l2(eo["v_rendered"], r32["v_rendered"]) <= 1e-5
    for k in ("v_xy", "v_conic", "v_colors", "v_opacity", "v_mean3d", "v_scale", "v_quat"):
        e32 = rel_l2(eo[k], r32[k])
        e64 = rel_l2(eo[k], r64[k])
        print(k, "rel_l2 fp32", e32, "fp64", e64)
        assert e32 <= GRAD_TOL, k
        assert e64 <= GRAD_TOL, k   # measured 2-4e-6 on GB300
    for k in E.GROUPS:
        before = getattr(init, k).reshape(eo["params"][k].shape)
        upd_e = eo["params"][k] - before
        upd_o = r32["params"][k].reshape(upd_e.shape) - before
        e = rel_l2(upd_e, upd_o)
        print("update", k, e)
        assert e <= GRAD_TOL, k


def test_sgld_parity(small):
    sc, cam, gt, init = small
    step = E.step_scalars(600, 600, width=cam.width, height=cam.height)
    eo, res = run_pair(init, cam, gt, step, do_sgld=True, precs=(32,))
    before = init.means
    e = rel_l2(eo["params"]["means"] - before, res[32]["params"]["means"] - before)
    print("sgld+adam means update rel_l2", e)
    assert e <= GRAD_TOL


@pytest.mark.parametrize("tuning", [dict(tile_order=0, tile_split=1), dict(bwd_pixels=2, tile_order=1),
                                    dict(tile_order=1, tile_split=2)])
def test_edge_cases(small, tuning):
    """Partial edge tiles, splats behind the camera, a NaN colour, a mask:
    with the per-tile sort and one CTA per tile; with the two-pixels-per-
    thread raster backward (second pixels below the image in the bottom
    tiles) and the depth-presorted tile ordering; and with two CTAs per tile
    (bottom halves of the last tile row wholly below the image)."""
    sc, cam0, gt0, init = small
    cam = S.Camera(cam0.cam_to_world, 203, 150, 160.0, 160.0, 101.5, 75.0)
    gt = gt_image(sc.gt, cam)
    g = init.copy()
    g.features_dc[5] = np.nan                 # zombie gate
    g.means[7] = np.array([30.0, 0.0, 0.0])   # far outside / behind
    mask = np.full((cam.height, cam.width), 255, np.uint8)
    mask[40:70, 50:120] = 0
    mask[140:, 190:] = 0                      # across the bottom-right corner
    step = E.step_scalars(700, 700, width=cam.width, height=cam.height)
    eo, res = run_pair(g, cam, gt, step, mask=mask, precs=(32,), tuning=tuning)
    r32 = res[32]
    _check_forward(eo, r32, g.n)
    assert eo["radii"][5] == 0
    assert eo["nan_counts"][7] >= 1
    # loss and dL/dimage on partial edge blocks with a mask (the reference's
    # loss partition of edge tiles)
    assert abs(eo["loss"] - r32["loss"]) <= 1e-5 * max(1.0, abs(r32["loss"]))
    assert rel_l2(eo["v_rendered"], r32["v_rendered"]) <= 1e-5
    for k in ("v_xy", "v_conic", "v_colors", "v_mean3d"):
        assert rel_l2(eo[k], r32[k]) <= GRAD_TOL, k
    for k in E.GROUPS:
        before = getattr(g, k).reshape(eo["params"][k].shape)
        fin = np.isfinite(before)
        upd_e = (eo["params"][k] - before)[fin]
        upd_o = (r32["params"][k].reshape(eo["params"][k].shape) - before)[fin]
        assert rel_l2(upd_e, upd_o) <= GRAD_TOL, k


@pytest.mark.parametrize("raster_mode,tuning", [(0, None), (1, None), (0, dict(bwd_pixels=2))])
def test_needles_and_faint_splats(small, raster_mode, tuning):
    """Warp culling by each splat's reach box at its edges: needle-thin
    Gaussians (scales e^-1.5 by e^-8, random rotations: conics close to
    singular), huge ones, and opacities on both sides of the 1/255 cut.
    Tile lists, last contributors and the image equal the oracle's (which
    tests every pixel), gradients within the usual bar; the backward also in
    its two-pixels-per-thread layout (8x8 warp blocks)."""
    sc, cam, gt, init = small
    rng = np.random.default_rng(7)
    g = init.copy()
    n = g.n
    k = rng.integers(0, 3, n)
    sc3 = np.full((n, 3), -8.0, np.float32)
    sc3[np.arange(n), k] = rng.uniform(-3.0, -1.5, n)
    big = rng.random(n) < 0.01
    sc3[big] = rng.uniform(-1.5, -0.5, (int(big.sum()), 3))
    g.scales[:] = sc3
    cut = np.log(1.0 / 254.0)   # logit of 1/255
    g.opacities[:, 0] = np.where(rng.random(n) < 0.5, cut + rng.normal(0.0, 0.05, n),
                                 rng.uniform(-7.0, 6.0, n)).astype(np.float32)
    step = E.step_scalars(1, 1, width=cam.width, height=cam.height)
    step["degrees_to_use"] = 3
    eo, res = run_pair(g, cam, gt, step, raster_mode=raster_mode, precs=(32,), tuning=tuning)
    r32 = res[32]
    _check_forward(eo, r32, g.n)
    for key in ("v_xy", "v_conic", "v_colors", "v_opacity", "v_mean3d", "v_scale"):
        assert rel_l2(eo[key], r32[key]) <= GRAD_TOL, key


@pytest.mark.parametrize("tuning", [dict(tile_order=0), dict(tile_order=1)])
def test_large_tile_buckets(small, tuning):
    """Every Gaussian of the scene large and a 96x64 view: each of the 24
    tiles holds most of the 16,384 Gaussians, more keys than either tile
    ordering stages in shared memory, and the depth-presorted ordering's
    per-CTA runs reach 1024 keys."""
    sc, cam0, gt0, init = small
    cam = S.Camera(cam0.cam_to_world, 96, 64, 60.0, 60.0, 48.0, 32.0)
    gt = gt_image(sc.gt, cam)
    g = init.copy()
    g.scales[:] = np.float32(0.3)
    g.opacities[:] = np.float32(-4.0)   # faint: the lists stay long behind the front
    step = E.step_scalars(1, 1, width=cam.width, height=cam.height)
    eo, res = run_pair(g, cam, gt, step, precs=(32,), tuning=tuning)
    r32 = res[32]
    assert int(r32["tile_counts"].max()) > 8192
    _check_forward(eo, r32, g.n)
    assert rel_l2(eo["v_rendered"], r32["v_rendered"]) <= 1e-5
    for key in ("v_xy", "v_conic", "v_colors", "v_opacity", "v_mean3d"):
        assert rel_l2(eo[key], r32[key]) <= GRAD_TOL, key


def test_empty_scene(small):
    sc, cam, gt, init = small
    g = S.GaussianSet(*(a[:0].copy() for a in init.arrays()))
    step = E.step_scalars(1, 1, width=cam.width, height=cam.height)
    import torch
    eng = E.Engine(0)
    dg = E.DeviceGaussians(g)
    gt_d = torch.from_numpy(gt).cuda()
    eng.train_step(dg, E.make_args(E.camera_dict(cam), step), gt_d.data_ptr())
    eng.synchronize()
    img = eng.read("out_img", np.float32, cam.width * cam.height * 3)
    assert np.all(img == 0.0)
    assert np.isfinite(eng.loss())
    eng.close()


def test_c1_run_sampled_steps(small):
    """The small configuration as specified: one step, then 100 more (steps
    1-101 over the 8 ring views in turn, the reference's schedules, SGLD on,
    the chunked raster that its 256 tiles select).  Steps 1, 2, 51 and 101
    are checked from the engine's own pre-step parameters and moments against
    the float path (the usual bars) and FP64 (errors printed)."""
    from gpu_helpers import compare_step, engine_step, oracle_from, state_of
    import torch
    sc, cam0, gt0, init = small
    cams = sc.train_cams
    cds = [E.camera_dict(c) for c in cams]
    gts = [gt_image(sc.gt, c) for c in cams]
    gts_d = [torch.from_numpy(g).cuda() for g in gts]
    eng = E.Engine(0)
    dg = E.DeviceGaussians(init)
    sampled = {0, 1, 50, 100}
    for k in range(101):
        v = k % len(cams)
        step = E.step_scalars(1 + k, 1 + k, width=cams[v].width, height=cams[v].height)
        if k in sampled:
            eng.synchronize()
            g, mom = state_of(dg, init)
            eo = engine_step(eng, dg, cds[v], cams[v], step, gts_d[v])
            assert eo["k_max"] > 1   # chunked
            r32 = oracle_from(32, g, mom, cds[v], step, gts[v])
            r64 = oracle_from(64, g, mom, cds[v], step, gts[v])
            compare_step(eo, r32, dict(zip(E.GROUPS, g.arrays())), f"c1 step {1 + k}", r64, fp64_bar=1e-2)
        else:
            eng.train_step(dg, E.make_args(cds[v], step, do_sgld=True), gts_d[v].data_ptr())
    eng.close()
