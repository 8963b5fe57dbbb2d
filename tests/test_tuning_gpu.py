"""Tunable launch configuration (include/msplat_engine.h MsplatTuning) and
the autotuner.  The sort width, the rasterizers' tile batch and the tile
order (per-tile radix sort or one depth sort per view) must leave every
output of a step bit-identical (tile lists, image; loss, gradients and
updated parameters to float-atomic rounding); the chunk length changes the chunked image only at
float rounding; the autotuner returns a valid configuration and leaves it
set (GPU only)."""
import numpy as np
import pytest

from msplat_gb300 import engine as E
from msplat_gb300 import synthetic as S

from gpu_helpers import gt_image, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene():
    torch = pytest.importorskip("torch")
    sc = S.config_small(6)
    base = sc.train_cams
    cams = [base[1], S.Camera(base[4].cam_to_world, 176, 144, 140.0, 140.0, 88.0, 72.0)]
    gts = [torch.from_numpy(gt_image(sc.gt, c)).cuda() for c in cams]
    return sc, cams, gts, S.init_from_gt(sc.gt, 6)


def _step(init, cams, gts, tuning, views, raster_mode=1):
    eng = E.Engine(0)
    eng.set_tuning(**tuning)
    dg = E.DeviceGaussians(init)
    cams = cams[:views]
    args = [E.make_args(E.camera_dict(c), E.step_scalars(700, 700, width=c.width, height=c.height),
                        raster_mode=raster_mode, do_sgld=True) for c in cams]
    if views == 1:
        eng.train_step(dg, args[0], gts[0].data_ptr())
    else:
        eng.train_step_batch(dg, args, [g.data_ptr() for g in gts[:views]])
    eng.synchronize()
    T = sum(((c.width + 15) // 16) * ((c.height + 15) // 16) for c in cams)
    P = sum(c.width * c.height for c in cams)
    offs = eng.read("tile_offsets", np.uint32, T + 1)
    out = {"offs": offs, "ids": eng.read("isect_ids", np.uint32, int(offs[-1])),
           "img": eng.read("out_img", np.float32, 3 * P), "v_img": eng.read("v_img", np.float32, 3 * P),
           "grad": eng.read("grad", np.float32, 12 * views * init.n), "loss": eng.loss()}
    p, _ = dg.to_numpy()
    out.update({"p_" + k: v for k, v in p.items()})
    st = eng.stats()
    assert st.check_record[0] == 0
    eng.close()
    return out


@pytest.mark.parametrize("views", [1, 2])
def test_sort_width_tile_batch_tile_order_and_split_are_bit_identical(scene, views):
    sc, cams, gts, init = scene
    ref = _step(init, cams, gts, dict(sort_width=512, raster_batch=256, tile_order=0, tile_split=1), views)
    counts = np.diff(ref["offs"].astype(np.int64))
    assert (counts > 0).sum() > 50   # the 256-thread sort class takes the tiles up to 2048 keys
    for tun in (dict(sort_width=256, raster_batch=256, tile_order=0, tile_split=1),
                dict(sort_width=512, raster_batch=128, tile_order=0, tile_split=1),
                dict(sort_width=256, raster_batch=128, tile_order=0, tile_split=1), dict(tile_order=1, tile_split=1),
                dict(tile_order=1, raster_batch=128, tile_split=1), dict(bwd_pixels=2, tile_order=0, tile_split=1),
                dict(tile_order=1, raster_batch=128, bwd_pixels=2, tile_split=1),
                dict(tile_split=2, raster_batch=128, tile_order=0), dict(tile_split=2, raster_batch=256, tile_order=1),
                dict(tile_split=2, raster_batch=128, tile_order=1, bwd_pixels=2)):
        o = _step(init, cams, gts, tun, views)
        for k in ("offs", "ids", "img", "v_img"):
            np.testing.assert_array_equal(o[k], ref[k], err_msg=f"{tun} {k}")
        # the loss (summed over CTAs), the gradients and the parameters: float
        # atomics leave the order of the sums free, so those agree to rounding
        assert abs(o["loss"] - ref["loss"]) <= 1e-6 * abs(ref["loss"])
        assert rel_l2(o["grad"], ref["grad"]) <= 1e-5, tun
        for k in E.GROUPS:
            assert rel_l2(o["p_" + k], ref["p_" + k]) <= 1e-6, (tun, k)


def test_chunk_length(scene):
    """Chunked raster with 256-, 512- and 1024-splat chunks against the
    monolithic raster.  They differ by the chunked algorithm's own rule: each
    chunk stops on its local transmittance (1e-4), so a pixel's few
    contributions behind T = 1e-4 are kept or dropped differently (each below
    1e-4 of the colour); otherwise rounding.  Bounds: 1e-3 per pixel, 1e-5
    mean, gradients 1e-2 relative L2."""
    sc, cams, gts, init = scene
    mono = _step(init, cams, gts, dict(chunk=512), 1, raster_mode=1)
    for ch in (256, 512, 1024):
        o = _step(init, cams, gts, dict(chunk=ch), 1, raster_mode=2)
        d = np.abs(o["img"] - mono["img"])
        eg = rel_l2(o["grad"], mono["grad"])
        print(ch, d.max(), d.mean(), eg)
        assert d.max() <= 1e-3 and d.mean() <= 1e-5, (ch, d.max(), d.mean())
        assert eg <= 1e-2, (ch, eg)


def test_autotune(scene):
    sc, cams, gts, init = scene
    eng = E.Engine(0)
    dg = E.DeviceGaussians(init)
    args = [E.make_args(E.camera_dict(c), E.step_scalars(700, 700, width=c.width, height=c.height)) for c in cams]
    p0, _ = dg.to_numpy()
    cfg, ms = eng.autotune(dg, args, [g.data_ptr() for g in gts], reps=2)
    assert ms > 0
    assert cfg["sort_width"] in (256, 512) and cfg["raster_batch"] in (128, 256)
    assert cfg["chunk"] in (256, 512, 1024) and cfg["raster_mode"] in (0, 1, 2) and cfg["bwd_pixels"] in (1, 2)
    assert cfg["tile_split"] in (1, 2)
    assert eng.tuning() == cfg
    p1, _ = dg.to_numpy()
    for k in E.GROUPS:   # timing runs leave the parameters alone
        np.testing.assert_array_equal(p0[k], p1[k])
    eng.train_step_batch(dg, args, [g.data_ptr() for g in gts])   # and the tuned step trains
    eng.synchronize()
    assert np.isfinite(eng.loss())
    with pytest.raises(RuntimeError):
        eng.set_tuning(sort_width=300)
    eng.close()


@pytest.mark.parametrize("tile_order", [0, 1])
@pytest.mark.parametrize("views", [1, 2])
def test_isect_budget_tile_groups(scene, views, tile_order):
    """A fixed intersection budget smaller than the step's intersections: the
    step runs in tile groups (lists built and rastered group by group, rebuilt
    for the backward) and gives the legacy step's image bit for bit and its
    gradients and update to rounding (float atomics)."""
    sc, cams, gts, init = scene
    ref = _step(init, cams, gts, dict(tile_order=tile_order), views)
    M = int(ref["offs"][-1])
    counts = np.diff(ref["offs"].astype(np.int64))
    slots = max(int(counts.max()), M // 4)

    eng = E.Engine(0)
    eng.set_tuning(tile_order=tile_order)
    eng.set_isect_budget(slots)
    dg = E.DeviceGaussians(init)
    cs = cams[:views]
    args = [E.make_args(E.camera_dict(c), E.step_scalars(700, 700, width=c.width, height=c.height),
                        raster_mode=1, do_sgld=True) for c in cs]
    if views == 1:
        eng.train_step(dg, args[0], gts[0].data_ptr())
    else:
        eng.train_step_batch(dg, args, [g.data_ptr() for g in gts[:views]])
    eng.synchronize()
    st = eng.stats()
    assert st.isect_groups >= 4, st.isect_groups
    assert st.num_intersections == M
    P = sum(c.width * c.height for c in cs)
    np.testing.assert_array_equal(eng.read("out_img", np.float32, 3 * P), ref["img"])
    np.testing.assert_array_equal(eng.read("v_img", np.float32, 3 * P), ref["v_img"])
    assert rel_l2(eng.read("grad", np.float32, 12 * views * init.n), ref["grad"]) <= 1e-5
    p, _ = dg.to_numpy()
    for k in E.GROUPS:
        assert rel_l2(p[k], ref["p_" + k]) <= 1e-6, k
    # a tile larger than the budget is refused (view 0's largest, stepped alone)
    T0 = ((cs[0].width + 15) // 16) * ((cs[0].height + 15) // 16)
    eng.set_isect_budget(int(counts[:T0].max()) - 1)
    with pytest.raises(RuntimeError):
        eng.train_step(dg, args[0], gts[0].data_ptr())
    eng.close()
