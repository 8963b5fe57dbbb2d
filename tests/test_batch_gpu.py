"""Multi-view training step (msplat_engine_train_step_batch): views of
different sizes go through one launch per stage (the rasterizers: one per run
of consecutive views with the same depth-chunk count, each view's count by the
reference's rule) and give one update from the mean of their gradients.  The batched forward is checked bit for bit against
one-view renders (records, per-tile sorted lists, images); the update against
the oracle's per-view gradients (FP32 path) averaged and pushed through Adam
in numpy with the engine's rules (GPU only)."""
import numpy as np
import pytest

from msplat_gb300 import engine as E
from msplat_gb300 import synthetic as S
from oracle import oracle as O

from gpu_helpers import gt_image, rel_l2

pytestmark = pytest.mark.gpu

C0 = 0.28209479177387814
C1 = 0.4886025119029199
C2 = (1.0925484305920792, -1.0925484305920792, 0.31539156525252005, -1.0925484305920792, 0.5462742152960396)
C3 = (-0.5900435899266435, 2.890611442640554, -0.4570457994644658, 0.3731763325901154, -0.4570457994644658,
      1.445305721320277, -0.5900435899266435)


def _basis(d):
    X, Y, Z = d[:, 0], d[:, 1], d[:, 2]
    xx, yy, zz, xy, yz, xz = X * X, Y * Y, Z * Z, X * Y, Y * Z, X * Z
    return np.stack([-C1 * Y, C1 * Z, -C1 * X, C2[0] * xy, C2[1] * yz, C2[2] * (2 * zz - xx - yy), C2[3] * xz,
                     C2[4] * (xx - yy), C3[0] * Y * (3 * xx - yy), C3[1] * xy * Z, C3[2] * Y * (4 * zz - xx - yy),
                     C3[3] * Z * (2 * zz - 3 * xx - 3 * yy), C3[4] * X * (4 * zz - xx - yy),
                     C3[5] * Z * (xx - yy), C3[6] * X * (xx - 3 * yy)], 1)


def _adam(p, m, v, g, st, bc2, b1=0.9, b2=0.999, eps=1e-8):
    m2 = b1 * m + (1 - b1) * g
    v2 = b2 * v + (1 - b2) * g * g
    return p - st * m2 / (np.sqrt(v2) / bc2 + eps), m2, v2


def _mixed_views(sc):
    base = sc.train_cams
    return [base[0], S.Camera(base[3].cam_to_world, 200, 150, 160.0, 160.0, 100.0, 75.0),
            S.Camera(base[5].cam_to_world, 128, 96, 100.0, 100.0, 64.0, 48.0)]


def _mixed_mode_views(sc):
    """Views whose own raster modes differ under the reference's rule: 130,
    520, 256, 48 and 48 tiles (chunked with K = 71, monolithic, K = 36, then
    two views with K = 192 that share one launch)."""
    base = sc.train_cams
    return [S.Camera(base[3].cam_to_world, 200, 150, 160.0, 160.0, 100.0, 75.0),
            S.Camera(base[1].cam_to_world, 416, 320, 300.0, 300.0, 208.0, 160.0),
            base[0],
            S.Camera(base[5].cam_to_world, 128, 96, 100.0, 100.0, 64.0, 48.0),
            S.Camera(base[6].cam_to_world, 128, 96, 100.0, 100.0, 64.0, 48.0)]


@pytest.mark.parametrize("raster_mode", [1, 2, 0])
def test_batch_forward_matches_single_views(raster_mode):
    """One launch per stage over several views = one-view renders: the
    same radii and records, each view's tile lists equal to its own with the
    record ids offset by view * n (depth ties still ordered by Gaussian), and
    the same image bits.  raster_mode 1: monolithic; 2: 512-splat chunks;
    0: the reference's rule per view (msplat_metal.mm:1204-1224), on views
    of both modes and several chunk counts in one batch."""
    torch = pytest.importorskip("torch")
    sc = S.config_small(4)
    cams = _mixed_views(sc) if raster_mode else _mixed_mode_views(sc)
    init = S.init_from_gt(sc.gt, 4)
    n = init.n
    kw = dict(raster_mode=raster_mode, k_max=3 if raster_mode == 2 else 0, do_optimizer=False)
    gts = [torch.from_numpy(gt_image(sc.gt, c)).cuda() for c in cams]
    eng = E.Engine(0)
    dg = E.DeviceGaussians(init)
    args = [E.make_args(E.camera_dict(c), E.step_scalars(10, 10, width=c.width, height=c.height), **kw)
            for c in cams]
    eng.train_step_batch(dg, args, [g.data_ptr() for g in gts])
    eng.synchronize()
    Ts = [((c.width + 15) // 16) * ((c.height + 15) // 16) for c in cams]
    Ps = [c.width * c.height for c in cams]
    B = len(cams)
    offs = eng.read("tile_offsets", np.uint32, sum(Ts) + 1).astype(np.int64)
    ids = eng.read("isect_ids", np.uint32, int(offs[-1]))
    img = eng.read("out_img", np.float32, 3 * sum(Ps))
    radii = eng.read("radii", np.int32, B * n)
    rec = eng.read("rec", np.float32, B * n * 12)
    st = eng.stats()
    assert st.check_record[0] == 0
    k_batch = st.k_max
    eng.close()
    t0 = p0 = 0
    ks = []
    for v, c in enumerate(cams):
        e1 = E.Engine(0)
        dg1 = E.DeviceGaussians(init)
        e1.render(dg1, E.make_args(E.camera_dict(c), E.step_scalars(10, 10, width=c.width, height=c.height), **kw))
        e1.synchronize()
        ks.append(e1.stats().k_max)
        o1 = e1.read("tile_offsets", np.uint32, Ts[v] + 1).astype(np.int64)
        i1 = e1.read("isect_ids", np.uint32, max(int(o1[-1]), 1))[:int(o1[-1])]
        np.testing.assert_array_equal(e1.read("radii", np.int32, n), radii[v * n:(v + 1) * n])
        np.testing.assert_array_equal(e1.read("rec", np.float32, n * 12), rec[v * n * 12:(v + 1) * n * 12])
        np.testing.assert_array_equal(np.diff(o1), np.diff(offs[t0:t0 + Ts[v] + 1]))
        seg = ids[offs[t0]:offs[t0 + Ts[v]]].astype(np.int64)
        np.testing.assert_array_equal(seg, i1.astype(np.int64) + v * n)
        np.testing.assert_array_equal(e1.read("out_img", np.float32, 3 * Ps[v]), img[3 * p0:3 * (p0 + Ps[v])])
        e1.close()
        t0 += Ts[v]
        p0 += Ps[v]
    assert k_batch == max(ks)
    if raster_mode == 0:
        assert ks == [71, 1, 36, 192, 192], ks


def test_batch_step_matches_oracle_mean_gradient():
    torch = pytest.importorskip("torch")
    sc = S.config_small(2)
    cams = _mixed_mode_views(sc)
    gts = [gt_image(sc.gt, c) for c in cams]
    init = S.init_from_gt(sc.gt, 2)
    B = len(cams)
    rng = np.random.default_rng(0)
    mom = ([rng.uniform(-1e-3, 1e-3, a.shape).astype(np.float32) for a in init.arrays()],
           [rng.uniform(1e-6, 1e-4, a.shape).astype(np.float32) for a in init.arrays()])
    step = 600
    steps = [E.step_scalars(step, step, width=c.width, height=c.height, sh_interval=100) for c in cams]
    nb = {0: 0, 1: 3, 2: 8, 3: 15}[steps[0]["degrees_to_use"]]
    assert nb == 15
    cds = [E.camera_dict(c) for c in cams]
    # SGLD off: deterministic reference; each view's raster mode and chunk
    # count by the reference's rule, in the batch as in the one-view oracle
    args = [E.make_args(cd, st) for cd, st in zip(cds, steps)]
    # engine
    eng = E.Engine(0)
    dg = E.DeviceGaussians(init)
    for k, name in enumerate(E.GROUPS):
        dg.exp_avg[name].copy_(torch.from_numpy(mom[0][k].reshape(dg.exp_avg[name].shape)))
        dg.exp_avg_sq[name].copy_(torch.from_numpy(mom[1][k].reshape(dg.exp_avg_sq[name].shape)))
    gt_d = [torch.from_numpy(g).cuda() for g in gts]
    eng.train_step_batch(dg, args, [t.data_ptr() for t in gt_d])
    eng.synchronize()
    loss_e = eng.loss()
    params, _ = dg.to_numpy()
    eng.close()
    # reference: per-view oracle gradients (loss scaled by 1/B), summed
    n = init.n
    acc = {k: np.zeros(a.shape, np.float64) for k, a in zip(E.GROUPS, init.arrays())}
    vis = np.zeros(n, bool)
    losses = []
    for cd, st, gt in zip(cds, steps, gts):
        st = dict(st)
        st["loss_inv_n"] = st["loss_inv_n"] / B
        r = O.train_step(32, init.copy(), cd, st, gt=gt, do_backward=True, do_optimizer=False, want_ids=False)
        losses.append(r["loss"])            # the loss value is not scaled by loss_inv_n
        v = r["radii"] > 0
        vis |= v
        acc["means"] += np.where(v[:, None], r["v_mean3d"], 0)
        acc["scales"] += np.where(v[:, None], r["v_scale"], 0)
        acc["quats"] += np.where(v[:, None], r["v_quat"], 0)
        acc["opacities"] += np.where(v, r["v_opacity"], 0).reshape(acc["opacities"].shape)
        d = init.means.astype(np.float64) - np.asarray(cd["cam_pos"], np.float64)
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        vc = np.where(v[:, None], r["v_colors"], 0.0)
        acc["features_dc"] += C0 * vc
        acc["features_rest"][:, :nb] += (_basis(d)[:, :, None] * vc[:, None, :])[:, :nb]
    assert abs(loss_e - np.mean(losses)) <= 1e-4 * abs(np.mean(losses))
    s0 = steps[0]
    # regularizer (step >= 500), as the engine's Adam adds it
    sig = 1 / (1 + np.exp(-init.opacities.astype(np.float64)))
    acc["opacities"] += s0["op_reg"] * sig * (1 - sig) / n
    acc["scales"] += s0["sc_reg"] * np.exp(np.clip(init.scales.astype(np.float64), -15, 15)) / n / 3
    gidx = {"means": 0, "scales": 1, "quats": 2, "features_dc": 3, "features_rest": 4, "opacities": 5}
    for k, a in zip(E.GROUPS, init.arrays()):
        gi = gidx[k]
        p, m, v = a.astype(np.float64), mom[0][gi].astype(np.float64), mom[1][gi].astype(np.float64)
        p2, _, _ = _adam(p, m, v, acc[k], s0["step_size"][gi], s0["bc2_sqrt"][gi])
        if k in ("features_dc", "features_rest"):   # SH: Gaussians visible in some view, bands in use
            keep = np.broadcast_to(vis.reshape((-1,) + (1,) * (a.ndim - 1)), a.shape)
            p2 = np.where(keep, p2, p)
        # the parameters are float32: compare updates after rounding the reference's to float32
        upd_e = params[k].reshape(a.shape).astype(np.float64) - a
        upd_r = p2.astype(np.float32).astype(np.float64) - a
        e = rel_l2(upd_e, upd_r)
        print(k, e)
        assert e <= 1e-4, (k, e)


def test_batch_graph_replay_matches_eager():
    torch = pytest.importorskip("torch")
    sc = S.config_small(3)
    cams = [sc.train_cams[0], S.Camera(sc.train_cams[2].cam_to_world, 160, 120, 130.0, 130.0, 80.0, 60.0)]
    gts = [torch.from_numpy(gt_image(sc.gt, c)).cuda() for c in cams]
    init = S.init_from_gt(sc.gt, 3)

    def run(graphs):
        eng = E.Engine(0)
        eng.set_graphs(graphs)
        dg = E.DeviceGaussians(init)
        for k in range(5):
            args = [E.make_args(E.camera_dict(c), E.step_scalars(600 + k, 600 + k, width=c.width, height=c.height),
                                do_sgld=True) for c in cams]
            eng.train_step_batch(dg, args, [g.data_ptr() for g in gts])
        eng.synchronize()
        p, _ = dg.to_numpy()
        l = eng.loss()
        eng.close()
        return p, l

    pe, le = run(False)
    pg, lg = run(True)
    assert abs(le - lg) <= 1e-5 * abs(le)
    for k in E.GROUPS:
        base = getattr(init, k).reshape(pe[k].shape)
        assert rel_l2(pg[k] - base, pe[k] - base) <= 1e-4, k


def test_batch_loss_with_masks_matches_single_views():
    """The loss stage of a multi-view step with per-view masks (two masked
    views, one without; masks reaching the image borders) against one-view
    steps of the same views: each view's dL/dimage (scaled by 1/B in the
    batch) and loss.  The one-view loss stage is the one the parity tests
    hold to the oracle."""
    torch = pytest.importorskip("torch")
    sc = S.config_small(5)
    cams = _mixed_views(sc)
    gts = [torch.from_numpy(gt_image(sc.gt, c)).cuda() for c in cams]
    init = S.init_from_gt(sc.gt, 5)
    rng = np.random.default_rng(5)
    masks = []
    for k, c in enumerate(cams):
        if k == 1:
            masks.append(None)
            continue
        m = np.full((c.height, c.width), 255, np.uint8)
        m[rng.random((c.height, c.width)) < 0.1] = 0
        m[:7, :] = 0
        m[:, -9:] = 0
        masks.append(torch.from_numpy(m).cuda())
    B = len(cams)
    args = [E.make_args(E.camera_dict(c), E.step_scalars(10, 10, width=c.width, height=c.height), raster_mode=1)
            for c in cams]
    eng = E.Engine(0)
    dg = E.DeviceGaussians(init)
    eng.train_step_batch(dg, args, [g.data_ptr() for g in gts], [m.data_ptr() if m is not None else None for m in masks])
    eng.synchronize()
    P = [c.width * c.height for c in cams]
    v_batch = eng.read("v_img", np.float32, 3 * sum(P))
    loss_batch = eng.loss()
    eng.close()
    off, losses = 0, []
    for k, c in enumerate(cams):
        e1 = E.Engine(0)
        d1 = E.DeviceGaussians(init)
        e1.train_step(d1, args[k], gts[k].data_ptr(), masks[k].data_ptr() if masks[k] is not None else None)
        e1.synchronize()
        v1 = e1.read("v_img", np.float32, 3 * P[k])
        losses.append(e1.loss())
        e1.close()
        vb = v_batch[off:off + 3 * P[k]].astype(np.float64) * B
        off += 3 * P[k]
        assert rel_l2(vb, v1) <= 1e-6, k
    assert abs(loss_batch - np.mean(losses)) <= 1e-6 * abs(np.mean(losses))
