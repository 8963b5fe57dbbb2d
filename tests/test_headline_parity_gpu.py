"""Parity of the training step at the headline workload (GPU only):
1,000,000 Gaussians (SH degree 3), one 1297x840 view (4,346 tiles, so the
monolithic raster), step 3001 (every SH band, the regularizer and SGLD on) -
exactly bench.py's workload - against the oracle's float path and FP64.

Every launch configuration the autotuner can pick for it is covered: the
depth-presorted tile ordering with two CTAs per tile and one pixel per
thread in the raster backward (the default), one CTA per tile with the
per-tile radix sort, and the two-pixel backward (its pick for the 8-view
batch).

Bars:
  * radii, tiles hit, per-tile counts, sorted per-tile id lists and
    last-contributor indices: identical to the float path;
  * projection outputs of the visible Gaussians: identical;
  * image and final transmittance: <= 1e-5 max-abs against the float path;
  * loss: <= 1e-5 relative; dL/dimage <= 1e-5 relative L2;
  * raster and projection gradients and every parameter update (Adam on six
    groups, regularizer, SGLD): <= 1e-4 relative L2 against the float path;
    against FP64 the error of every output is printed (and held to 1e-3: the
    FP64 run moves a few sigma/alpha threshold decisions).

A 200-step run is also checked at three sampled steps, each step compared
from the engine's own pre-step state (parameters and Adam moments read back
before the step), so the trajectories never have to agree.
"""
import numpy as np
import pytest

from msplat_gb300 import engine as E

from gpu_helpers import compare_step, engine_step, oracle_from, state_of

pytestmark = pytest.mark.gpu

STEP0 = 3001

TUNINGS = {
    "presorted_1px": dict(tile_order=1, bwd_pixels=1, sort_width=512, raster_batch=128, tile_split=2),
    "per_tile_sort": dict(tile_order=0, bwd_pixels=1, sort_width=512, raster_batch=256, tile_split=1),
    "presorted_2px": dict(tile_order=1, bwd_pixels=2, sort_width=512, raster_batch=256, tile_split=1),
}


@pytest.fixture(scope="module")
def headline():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import bench
    sc, model = bench.build_workload()
    cam = sc.train_cams[0]
    cd = E.camera_dict(cam)
    # target: the GT scene rendered by the engine's forward (an input only)
    eng = E.Engine(0)
    gt_dev = E.DeviceGaussians(sc.gt)
    eng.render(gt_dev, E.make_args(cd, {"degrees_to_use": 3}))
    img = eng.read("out_img", np.float32, cam.width * cam.height * 3).reshape(cam.height, cam.width, 3)
    eng.close()
    del gt_dev
    gt = (np.clip(img, 0, 1) * 255 + 0.5).astype(np.uint8)
    return torch, sc, model, cam, cd, gt


@pytest.fixture(scope="module")
def oracle_step(headline):
    torch, sc, model, cam, cd, gt = headline
    step = E.step_scalars(STEP0, STEP0, width=cam.width, height=cam.height)
    zeros = ([np.zeros_like(a) for a in model.arrays()], [np.zeros_like(a) for a in model.arrays()])
    return step, {p: oracle_from(p, model, zeros, cd, step, gt) for p in (32, 64)}


@pytest.mark.parametrize("name", list(TUNINGS))
def test_headline_step(headline, oracle_step, name):
    torch, sc, model, cam, cd, gt = headline
    step, res = oracle_step
    eng = E.Engine(0, model.n)
    eng.set_tuning(**TUNINGS[name])
    dg = E.DeviceGaussians(model)
    gt_d = torch.from_numpy(gt).cuda()
    eo = engine_step(eng, dg, cd, cam, step, gt_d)
    eng.close()
    before = dict(zip(E.GROUPS, model.arrays()))
    print(name, "intersections", eo["num_isect"], "max tile", int(eo["tile_counts"].max()),
          "pairs (oracle)", res[32]["pairs_fwd"], res[32]["pairs_bwd"])
    assert eo["num_isect"] > 5_000_000 and int(eo["tile_counts"].max()) > 4096
    assert eo["k_max"] == 1   # 4346 tiles: the monolithic raster
    compare_step(eo, res[32], before, name, res[64])


def test_headline_run_sampled_steps(headline):
    """200 steps of the bench's run (graph replay, the one-view tuning, the
    eight ring views in turn); steps 0, 99 and 199 are checked against the
    oracle from the engine's own pre-step parameters and moments."""
    torch, sc, model, cam0, cd0, gt0 = headline
    cams = sc.train_cams
    cds = [E.camera_dict(c) for c in cams]
    eng = E.Engine(0, model.n)
    eng.set_tuning(**TUNINGS["presorted_1px"])
    eng.set_graphs(True)
    # targets of all views, rendered by the engine's forward
    gt_dev = E.DeviceGaussians(sc.gt)
    gts = []
    for c, cd in zip(cams, cds):
        eng.render(gt_dev, E.make_args(cd, {"degrees_to_use": 3}))
        img = eng.read("out_img", np.float32, c.width * c.height * 3).reshape(c.height, c.width, 3)
        gts.append((np.clip(img, 0, 1) * 255 + 0.5).astype(np.uint8))
    del gt_dev
    gts_d = [torch.from_numpy(g).cuda() for g in gts]
    dg = E.DeviceGaussians(model)
    sampled = {0, 99, 199}
    checked = 0
    for k in range(200):
        v = k % len(cams)
        step = E.step_scalars(STEP0 + k, STEP0 + k, width=cams[v].width, height=cams[v].height)
        if k in sampled:
            eng.synchronize()
            g, mom = state_of(dg, model)
            eo = engine_step(eng, dg, cds[v], cams[v], step, gts_d[v])
            r32 = oracle_from(32, g, mom, cds[v], step, gts[v])
            r64 = oracle_from(64, g, mom, cds[v], step, gts[v]) if k == 199 else None
            # FP64 after 199 steps of training: FP64 moves the radius, sigma and
            # alpha decisions of more splats as the model sharpens (one flipped
            # radius moves that Gaussian's whole gradient; the state at step 199
            # varies with the order of the float atomics).  The float path is the
            # bit-exact contract; against FP64 the engine is held to the float
            # oracle's own FP64 errors and to sanity bars of 5e-2 (gradients,
            # updates) and 1 % (image values over 1e-5).
            compare_step(eo, r32, dict(zip(E.GROUPS, g.arrays())), f"run step {k}", r64, fp64_bar=5e-2,
                         img_frac_bar=1e-2)
            checked += 1
        else:
            eng.train_step(dg, E.make_args(cds[v], step, do_sgld=True), gts_d[v].data_ptr())
    eng.close()
    assert checked == 3
