"""Heavy tiles: per-tile key counts in every sort class (shared-memory sort
by a 512-thread CTA up to 4096 keys, by a 1024-thread CTA up to 8192, the
global-memory sort above), exact clones (equal depths, ordered by id), and
both raster modes, against the oracle's float path (GPU only)."""
import numpy as np
import pytest

from msplat_gb300 import engine as E
from msplat_gb300 import synthetic as S

from gpu_helpers import gt_image, rel_l2, run_pair

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def heavy():
    a = S.gaussians(4096, seed=7, ball=24000, ball_center=(0.0, 0.0, 0.0), ball_radius=0.12)
    b = S.gaussians(0, seed=8, ball=9000, ball_center=(0.0, 0.5, 0.3), ball_radius=0.1)
    gt = S.GaussianSet(*(np.concatenate([x, y]) for x, y in zip(a.arrays(), b.arrays())))
    cam = S.ring_cameras(8, 256, 256, 205.0)[0]
    img = gt_image(gt, cam)
    init = S.init_from_gt(gt, 0)
    # 400 exact clones of ball Gaussians placed first (lower ids than their originals)
    src = 4096 + np.arange(400) * 37
    init = S.GaussianSet(*(np.concatenate([x[src], x]) for x in init.arrays()))
    return cam, img, init


@pytest.mark.parametrize("raster_mode", [0, 1])
def test_heavy_forward(heavy, raster_mode):
    cam, img, init = heavy
    step = E.step_scalars(1, 1, width=cam.width, height=cam.height)
    step["degrees_to_use"] = 3
    eo, res = run_pair(init, cam, img, step, raster_mode=raster_mode, do_backward=False, precs=(32,))
    r = res[32]
    tc = eo["tile_counts"]
    assert (tc > 8192).sum() >= 3 and ((tc > 4096) & (tc <= 8192)).sum() >= 1
    assert np.array_equal(tc, r["tile_counts"])
    assert np.array_equal(eo["gaussian_ids"], r["gaussian_ids"])
    assert np.array_equal(eo["final_idx"], r["final_idx"])
    assert np.max(np.abs(eo["out_img"] - r["out_img"])) <= 1e-5
    assert np.max(np.abs(eo["final_Ts"] - r["final_Ts"])) <= 1e-5


def test_heavy_train_step(heavy):
    cam, img, init = heavy
    step = E.step_scalars(600, 600, width=cam.width, height=cam.height)
    eo, res = run_pair(init, cam, img, step, raster_mode=0, precs=(32,))
    r = res[32]
    assert np.array_equal(eo["gaussian_ids"], r["gaussian_ids"])
    for k in ("v_xy", "v_conic", "v_colors", "v_opacity", "v_mean3d", "v_scale", "v_quat"):
        assert rel_l2(eo[k], r[k]) <= 1e-4, k
    for k in E.GROUPS:
        before = getattr(init, k).reshape(eo["params"][k].shape)
        assert rel_l2(eo["params"][k] - before, r["params"][k].reshape(before.shape) - before) <= 1e-4, k
