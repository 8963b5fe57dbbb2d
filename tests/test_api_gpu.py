"""The public trainer API (include/msplat_c_api.h, the reference's
core/src/msplat_api.mm and python/msplat/_core.pyi) driven end to end on the
GPU: in-memory dataset, seed initialisation (core/src/model.cpp:81-166), a
training step checked against the oracle, render/evaluate, PLY and .splat
export (core/src/loaders/save_gaussians.cpp), the checkpoint round trip
(model.cpp:698-843) and the render-only viewer."""
import numpy as np
import pytest

from gpu_helpers import gt_image, rel_l2
from msplat_gb300 import api as A
from msplat_gb300 import engine as E
from msplat_gb300 import synthetic as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu

C0 = 0.28209479177387814
BG = (0.6130, 0.0101, 0.3984)


@pytest.fixture(scope="module")
def scene():
    gt = S.gaussians(3000, seed=21, sh_rest_bases=15)
    cams = S.ring_cameras(5, 128, 96, 110.0)
    imgs = [gt_image(gt, c) for c in cams]
    rng = np.random.default_rng(4)
    xyz = (gt.means[:1500] + rng.normal(0.0, 0.02, (1500, 3))).astype(np.float32)
    rgb = rng.integers(0, 256, (1500, 3), dtype=np.uint8)
    return gt, cams, imgs, xyz, rgb


def _config(**kw):
    c = A.TrainingConfig(iterations=1000, cap_max=4000)
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def _seed_quats(n):
    """std::mt19937(42) + uniform_real_distribution<float>(0, 1), three draws per seed."""
    raw = np.random.RandomState(42).randint(0, 2 ** 32, size=3 * n, dtype=np.uint32)
    u01 = np.minimum((raw.astype(np.float64) / 2.0 ** 32).astype(np.float32),
                     np.nextafter(np.float32(1), np.float32(0))).reshape(n, 3)
    u, v, w = (u01[:, k] for k in range(3))
    a = np.sqrt(np.float32(1) - u).astype(np.float64)
    b = np.sqrt(u).astype(np.float64)
    v64, w64 = 2 * np.pi * v.astype(np.float64), 2 * np.pi * w.astype(np.float64)
    return np.stack([a * np.sin(v64), a * np.cos(v64), b * np.sin(w64), b * np.cos(w64)], 1).astype(np.float32)


def test_dataset_split_and_poses(scene):
    gt, cams, imgs, xyz, rgb = scene
    ds = A.Dataset.from_arrays(cams, imgs, xyz, rgb, eval_mode=True, test_every=5)
    assert (ds.num_train, ds.num_test) == (4, 1)            # every 5th camera, from 0, is a test view
    np.testing.assert_array_equal(ds.camera_pose(0), np.asarray(cams[1].cam_to_world, np.float32))
    ds2 = A.Dataset.from_arrays(cams, imgs, xyz, rgb)
    assert (ds2.num_train, ds2.num_test) == (5, 0)


def test_seed_initialisation(scene):
    scipy_spatial = pytest.importorskip("scipy.spatial")
    gt, cams, imgs, xyz, rgb = scene
    ds = A.Dataset.from_arrays(cams, imgs, xyz, rgb)
    t = A.GaussianTrainer(ds, _config())
    assert t.splat_count == 1500 and t.iteration == 0
    means, scales, quats, dc, rest, op = t.get_gaussians()
    np.testing.assert_array_equal(means, xyz)
    d, _ = scipy_spatial.cKDTree(xyz.astype(np.float64)).query(xyz.astype(np.float64), k=4)
    ref_scale = np.log(d[:, 1:].mean(1) * 0.1)
    np.testing.assert_allclose(scales, np.repeat(ref_scale[:, None], 3, 1), rtol=0, atol=2e-5)
    np.testing.assert_allclose(quats, _seed_quats(1500), rtol=0, atol=2e-7)
    np.testing.assert_array_equal(dc, ((rgb / 255.0 - 0.5) / C0).astype(np.float32))
    assert not rest.any()
    np.testing.assert_array_equal(op, np.zeros(1500, np.float32))   # logit(0.5)


def test_first_step_matches_oracle(scene):
    """One camera, so the shuffled camera order cannot differ: the trainer's
    step 1 (SH degree 0, Adam step 1, SGLD on) equals the oracle's."""
    gt, cams, imgs, xyz, rgb = scene
    ds = A.Dataset.from_arrays(cams[:1], imgs[:1], xyz, rgb)
    t = A.GaussianTrainer(ds, _config())
    g0 = S.GaussianSet(*t.get_gaussians())
    s = t.step()
    assert s.iteration == 1 and s.splat_count == 1500
    g1 = t.get_gaussians()
    cam = cams[0]
    step = E.step_scalars(1, 1, width=cam.width, height=cam.height)
    mom = ([np.zeros_like(a) for a in g0.arrays()], [np.zeros_like(a) for a in g0.arrays()])
    ref = g0.copy()
    r = O.train_step(32, ref, E.camera_dict(cam), step, moments=mom, gt=imgs[0], background=BG,
                     do_backward=True, do_optimizer=True, do_sgld=True)
    assert abs(t.last_loss - r["loss"]) <= 1e-5 * abs(r["loss"])
    for k, a, b, a0 in zip(E.GROUPS, g1, ref.arrays(), g0.arrays()):
        upd_e, upd_o = a - a0, b.reshape(a.shape) - a0
        if not upd_o.any():
            assert not upd_e.any(), k
            continue
        assert rel_l2(upd_e, upd_o) <= 1e-4, k


def test_training_render_evaluate(scene):
    gt, cams, imgs, xyz, rgb = scene
    ds = A.Dataset.from_arrays(cams, imgs, xyz, rgb, eval_mode=True, test_every=5)
    # black background, as in the target images
    t = A.GaussianTrainer(ds, _config(sh_degree_interval=1, bg_color=[0.0, 0.0, 0.0]))
    losses = []
    for _ in range(60):
        t.step()
        losses.append(t.last_loss)
    assert np.mean(losses[-8:]) < 0.9 * np.mean(losses[:8]), losses
    m = t.evaluate()
    assert m["num_test"] == 1 and m["num_gaussians"] == t.splat_count
    img = t.render(0, use_test=True)
    assert img.shape == (96, 128, 3)
    ref = imgs[0].astype(np.float32) / 255.0
    assert abs(m["psnr"] - O.psnr(img, ref)) < 1e-3
    assert abs(m["l1"] - O.l1(img, ref)) < 1e-6
    assert abs(m["ssim"] - O.ssim_eval(img, ref)) < 1e-4
    # a pose render is the camera render at the same pose
    pose = ds.camera_pose(2)
    np.testing.assert_array_equal(t.render_from_pose(pose, 2), t.render(2))
    rgba = t.render_to_rgba(pose, 2)
    assert rgba.shape == (96, 128, 4) and (rgba[..., 3] == 255).all()
    exp8 = (np.clip(t.render(2), 0, 1) * np.float32(255)).astype(np.uint8)
    np.testing.assert_array_equal(rgba[..., :3], exp8)


def test_batch_views_step(scene):
    """set_batch_views(4, 1.0) with four training cameras: the first step
    renders each camera once and applies one update from their mean
    gradient, the engine's multi-view step on the same views (any order: the
    mean does not depend on it beyond float rounding), and advances the
    iteration counter by 4; training then still converges."""
    torch = pytest.importorskip("torch")
    gt, cams, imgs, xyz, rgb = scene
    ds = A.Dataset.from_arrays(cams[:4], imgs[:4], xyz, rgb)
    t = A.GaussianTrainer(ds, _config(bg_color=[0.0, 0.0, 0.0]))
    t.set_batch_views(4, 1.0)
    with pytest.raises(ValueError):
        t.set_batch_views(0)
    g0 = S.GaussianSet(*t.get_gaussians())
    s = t.step()
    assert s.iteration == 4
    g1 = t.get_gaussians()
    eng = E.Engine(0)
    dg = E.DeviceGaussians(g0)
    args = [E.make_args(E.camera_dict(c), E.step_scalars(4, 1, width=c.width, height=c.height), do_sgld=True)
            for c in cams[:4]]
    gts = [torch.from_numpy(im).cuda() for im in imgs[:4]]
    eng.train_step_batch(dg, args, [g.data_ptr() for g in gts])
    eng.synchronize()
    ref, _ = dg.to_numpy()
    assert abs(t.last_loss - eng.loss()) <= 1e-5 * abs(eng.loss())
    eng.close()
    for k, a, a0 in zip(E.GROUPS, g1, g0.arrays()):
        upd_t, upd_e = a - a0.reshape(a.shape), ref[k].reshape(a.shape) - a0.reshape(a.shape)
        if not upd_e.any():
            assert not upd_t.any(), k
            continue
        assert rel_l2(upd_t, upd_e) <= 1e-4, k
    losses = [t.last_loss]
    cfg = t.autotune()                         # the launch configuration, timed on the next views
    assert cfg["tile_order"] in (0, 1) and cfg["sort_width"] in (256, 512)
    np.testing.assert_array_equal(t.get_gaussians()[0], g1[0])   # autotuning leaves the model alone
    for _ in range(40):
        t.step()
        losses.append(t.last_loss)
    assert np.mean(losses[-6:]) < 0.9 * np.mean(losses[:6]), losses


def _read_ply(path):
    with open(path, "rb") as f:
        props, n, comment = [], 0, ""
        assert f.readline() == b"ply\n"
        while True:
            line = f.readline().decode().rstrip("\n")
            if line == "end_header":
                break
            if line.startswith("element vertex "):
                n = int(line.split()[-1])
            elif line.startswith("property float "):
                props.append(line.split()[-1])
            elif line.startswith("comment "):
                comment = line
        data = np.frombuffer(f.read(), np.float32).reshape(n, len(props))
    return props, data, comment


def test_export_checkpoint_viewer(scene, tmp_path):
    gt, cams, imgs, xyz, rgb = scene
    ds = A.Dataset.from_arrays(cams[:1], imgs[:1], xyz, rgb)
    t = A.GaussianTrainer(ds, _config(sh_degree_interval=1))
    for _ in range(5):
        t.step()
    means, scales, quats, dc, rest, op = t.get_gaussians()
    n = t.splat_count

    ply = str(tmp_path / "s.ply")
    t.export_ply(ply)
    props, data, comment = _read_ply(ply)
    assert comment == "comment Generated by msplat at iteration 5"
    assert props[:9] == ["x", "y", "z", "nx", "ny", "nz", "f_dc_0", "f_dc_1", "f_dc_2"]
    assert props[9:54] == [f"f_rest_{i}" for i in range(45)]
    assert props[54:] == ["opacity", "scale_0", "scale_1", "scale_2", "rot_0", "rot_1", "rot_2", "rot_3"]
    np.testing.assert_array_equal(data[:, 0:3], means)
    np.testing.assert_array_equal(data[:, 6:9], dc)
    # f_rest is channel-major in the file: f_rest_{c*15+b} = rest[b, c]
    np.testing.assert_array_equal(data[:, 9:54], rest.transpose(0, 2, 1).reshape(n, 45))
    np.testing.assert_array_equal(data[:, 54], op)
    np.testing.assert_array_equal(data[:, 55:58], scales)
    np.testing.assert_array_equal(data[:, 58:62], quats)

    spl = str(tmp_path / "s.splat")
    t.export_splat(spl)
    raw = np.fromfile(spl, np.uint8)
    assert raw.size == 32 * n
    rec = raw.reshape(n, 32)
    pos = rec[:, 0:12].copy().view(np.float32)
    row = {m.tobytes(): i for i, m in enumerate(means)}
    idx = np.array([row[p.tobytes()] for p in pos])
    assert np.array_equal(np.sort(idx), np.arange(n))
    np.testing.assert_allclose(rec[:, 12:24].copy().view(np.float32), np.exp(scales[idx]), rtol=1e-6)
    exp_rgb = np.clip((dc[idx].astype(np.float64) * C0 + 0.5) * 255.0, 0, 255).astype(np.uint8)
    np.testing.assert_array_equal(rec[:, 24:27], exp_rgb)
    sig = (1.0 / (1.0 + np.exp(-op.astype(np.float64))))[idx]
    assert np.abs(rec[:, 27].astype(np.int32) - np.clip(sig * 255, 0, 255).astype(np.int32)).max() <= 1
    exp_q = np.clip(quats[idx] * np.float32(128) + np.float32(128), 0, 255).astype(np.uint8)
    assert np.abs(rec[:, 28:32].astype(np.int32) - exp_q.astype(np.int32)).max() <= 1
    # largest (sum of scales x opacity) first
    key = np.exp(scales[idx].astype(np.float64)).sum(1) * sig
    assert np.all(np.diff(key) <= 1e-6 * key[:-1])

    # the viewer renders the exported PLY like the trainer (same pose, fx = fy)
    cam = cams[0]
    fov_y = float(2 * np.arctan(cam.height / (2 * cam.fy)))
    v = A.Viewer(ply, cam.width, cam.height, fov_y)
    assert v.splat_count == n
    lo, hi = v.bounds()
    np.testing.assert_array_equal(lo, means.min(0))
    np.testing.assert_array_equal(hi, means.max(0))
    A._lib().msplat_viewer_set_background(v.h, *BG)
    pose = np.asarray(cam.cam_to_world, np.float32)
    vi = v.render(pose).astype(np.int32)
    ti = t.render_to_rgba(pose, 0).astype(np.int32)
    assert np.abs(vi - ti).mean() < 0.5 and np.abs(vi - ti).max() <= 8

    ck = str(tmp_path / "s.ckpt")
    t.save_checkpoint(ck)
    t2 = A.GaussianTrainer(ds, _config(sh_degree_interval=1))
    assert t2.load_checkpoint(ck) == 5
    assert t2.iteration == 5 and t2.splat_count == n
    for a, b in zip(t.get_gaussians(), t2.get_gaussians()):
        np.testing.assert_array_equal(a, b)
    # both continue alike (one camera; moments and Adam step restored)
    t.step()
    t2.step()
    for a, b in zip(t.get_gaussians(), t2.get_gaussians()):
        assert rel_l2(a, b) <= 1e-6


def test_set_gaussians_and_errors(scene, tmp_path):
    gt, cams, imgs, xyz, rgb = scene
    ds = A.Dataset.from_arrays(cams[:1], imgs[:1], xyz, rgb)
    t = A.GaussianTrainer(ds, _config())
    t.set_gaussians(gt)
    assert t.splat_count == gt.n
    got = t.get_gaussians()
    for a, b in zip(got, gt.arrays()):
        np.testing.assert_array_equal(a, b.reshape(a.shape))
    assert t.render(0).shape == (96, 128, 3)
    # errors come back as empty results, not crashes
    assert t.render(7).size == 0
    assert t.load_checkpoint(str(tmp_path / "missing.ckpt")) == 0
    with pytest.raises(RuntimeError):
        A.Dataset(str(tmp_path / "no_such_dataset"))
    with pytest.raises(RuntimeError):
        A.Viewer(str(tmp_path / "missing.ply"), 64, 64, 1.0)
