"""The CPU oracle checked against the reference's own known answers (CPU only).

* Eq. 9 relocation: the invariants of the reference's tests/test_relocation.cpp
  (centre alpha, integral of composite alpha, N == 1 no-op, no over-shrink),
  restated here for the oracle's or_compute_relocation.
* The deterministic exp shared with the engine: within 2 ulp of exp.
* FP64 gradients of the transcribed step against central finite differences
  on a small scene (the only pin available for the rasterizer/projection VJPs,
  which the reference's tests do not cover).
"""
import math

import numpy as np
import pytest

from msplat_gb300 import synthetic as S
from oracle import oracle as O


@pytest.mark.parametrize("o", [0.05, 0.1, 0.5, 0.9, 0.998])
@pytest.mark.parametrize("n", [1, 2, 3, 5, 12, 51])
def test_relocation_eq9(o, n):
    on, sn = O.compute_relocation(np.float32(o), np.ones(3, np.float32), n)
    sn = float(sn[0])
    centre = 1.0 - (1.0 - on) ** n
    assert abs(centre - np.float32(o)) <= 1e-5
    x = np.arange(-20.0, 20.0, 0.0005)
    a = on * np.exp(-x * x / (2.0 * sn * sn))
    integral = np.sum(1.0 - (1.0 - a) ** n) * 0.0005
    want = float(np.float32(o)) * math.sqrt(2 * math.pi)
    assert abs(integral / want - 1.0) <= 2e-3
    if n == 1:
        assert abs(sn - 1.0) <= 1e-6 and abs(on - np.float32(o)) <= 1e-6
    else:
        assert sn > math.sqrt(1.0 / n)


def test_relocation_clamps_n():
    a = O.compute_relocation(0.5, np.ones(3, np.float32), 51)
    b = O.compute_relocation(0.5, np.ones(3, np.float32), 200)
    assert a[0] == b[0] and np.array_equal(a[1], b[1])
    c = O.compute_relocation(0.5, np.ones(3, np.float32), 0)
    assert c[0] == np.float32(0.5)


def test_det_expf_accuracy():
    xs = np.concatenate([np.linspace(-87.0, 88.0, 20001), np.linspace(-6.0, 0.0, 5001),
                         np.linspace(-15.0, 15.0, 3001)]).astype(np.float32)
    got = O.det_expf(xs).astype(np.float64)
    ref = np.exp(xs.astype(np.float64))
    ulp = np.spacing(ref.astype(np.float32)).astype(np.float64)
    err = np.abs(got - ref) / ulp
    assert err.max() <= 2.0, float(err.max())
    assert O.det_expf([-100.0])[0] == 0.0 and np.isinf(O.det_expf([100.0])[0])


def _tiny_case(seed=3, n=48, w=40, h=36):
    gt_scene = S.gaussians(n, seed, sh_rest_bases=15)
    gt_scene.scales[:] = -2.5
    gt_scene.means *= 0.6
    cam = S.ring_cameras(1, w, h, 45.0)[0]
    vm, pm, cp = O.prepare_cam(cam.cam_to_world, w, h, cam.fx, cam.fy)
    cd = dict(viewmat=vm, projmat=pm, cam_pos=cp, fx=cam.fx, fy=cam.fy, cx=cam.cx, cy=cam.cy, width=w, height=h)
    r = O.train_step(64, gt_scene.copy(), cd, {"degrees_to_use": 0}, do_backward=False, do_optimizer=False,
                     background=(0.2, 0.1, 0.3), want_ids=False)
    gt = (np.clip(r["out_img"], 0, 1) * 255 + 0.5).astype(np.uint8)
    g = S.init_from_gt(gt_scene, seed, jitter=0.03, log_scale=-2.5, opacity=0.3)
    return g, cd, gt


# L1 only: the per-pixel loss is sum_c |x - gt| / 3, whose image gradient the
# kernel scales by loss_inv_n, so loss_inv_n = 1/3 makes v_rendered the exact
# derivative of loss_sum.  SH degree 0 (the reference does not differentiate
# the view direction) and no alpha/sigma cutoffs (they make the loss
# discontinuous; they only mask terms of the VJP).
FD_STEP = {"degrees_to_use": 0, "loss_inv_n": 1.0 / 3.0}


def _loss_sum(g, cd, gt):
    r = O.train_step(64, g.copy(), cd, FD_STEP, gt=gt, ssim_weight=0.0, do_backward=False, do_optimizer=False,
                     background=(0.2, 0.1, 0.3), raster_mode=1, want_ids=False, no_cutoff=True)
    return r["loss"] * (cd["width"] * cd["height"])


def test_fp64_gradients_finite_differences():
    """Rasterizer + projection VJPs (means, log-scales, quaternion on the
    tangent space, opacity logit, DC colour) against central differences."""
    g, cd, gt = _tiny_case()
    r = O.train_step(64, g.copy(), cd, FD_STEP, gt=gt, ssim_weight=0.0, do_backward=True, do_optimizer=False,
                     background=(0.2, 0.1, 0.3), raster_mode=1, want_ids=False, no_cutoff=True)
    vis = np.nonzero(r["radii"] > 0)[0][:10]
    assert len(vis) >= 6
    h = 1e-4
    fd_all, an_all = [], []

    def fd(mutate):
        gp, gm = g.copy(), g.copy()
        mutate(gp, +h)
        mutate(gm, -h)
        return (_loss_sum(gp, cd, gt) - _loss_sum(gm, cd, gt)) / (2 * h)

    pm = np.asarray(cd["projmat"], np.float64).reshape(4, 4)
    for i in vis:
        # The reference's project_pix_vjp (.metal:1252-1270) maps v_proj back
        # through rows 0-2 of the projection only, so the dependence of the
        # pixel centre on the homogeneous w (row 3) is dropped.  The engine
        # keeps that; the exact gradient is the oracle's plus the w-row term
        # -(v_ndc.x * hx + v_ndc.y * hy) * rw^2 * P[3, :3].
        p = np.append(g.means[i].astype(np.float64), 1.0)
        hx, hy, hw = pm[0] @ p, pm[1] @ p, pm[3] @ p
        rw = 1.0 / (hw + 1e-6)
        vnx = 0.5 * cd["width"] * r["v_xy"][i, 0]
        vny = 0.5 * cd["height"] * r["v_xy"][i, 1]
        corr = pm[3, :3] * (-(vnx * hx + vny * hy)) * rw * rw
        for c in range(3):
            fd_all.append(fd(lambda G, d: G.means[i].__setitem__(c, G.means[i][c] + d)))
            an_all.append(r["v_mean3d"][i, c] + corr[c])
            fd_all.append(fd(lambda G, d: G.scales[i].__setitem__(c, G.scales[i][c] + d)))
            an_all.append(r["v_scale"][i, c])
            fd_all.append(fd(lambda G, d: G.features_dc[i].__setitem__(c, G.features_dc[i][c] + d)))
            an_all.append(r["v_colors"][i, c] * 0.28209479177387814)
        fd_all.append(fd(lambda G, d: G.opacities[i].__setitem__(0, G.opacities[i][0] + d)))
        an_all.append(r["v_opacity"][i])
        # quaternion: the reference's gradient ignores the normalisation, so
        # compare its tangent-space projection with differences along the sphere
        q = g.quats[i].astype(np.float64)
        qn = q / np.linalg.norm(q)
        vq = r["v_quat"][i].astype(np.float64)
        proj = (vq - qn * np.dot(qn, vq)) / np.linalg.norm(q)
        t = proj / (np.linalg.norm(proj) + 1e-30)
        fd_all.append(fd(lambda G, d: G.quats[i].__setitem__(slice(None), (q + d * t).astype(np.float32))))
        an_all.append(np.dot(proj, t))
    fd_all = np.array(fd_all)
    an_all = np.array(an_all)
    err = np.linalg.norm(fd_all - an_all) / np.linalg.norm(fd_all)
    assert err < 2e-2, err


def test_fp32_mirror_close_to_fp64():
    sc = S.config_small(0)
    cam = sc.train_cams[1]
    vm, pm, cp = O.prepare_cam(cam.cam_to_world, cam.width, cam.height, cam.fx, cam.fy)
    cd = dict(viewmat=vm, projmat=pm, cam_pos=cp, fx=cam.fx, fy=cam.fy, cx=cam.cx, cy=cam.cy,
              width=cam.width, height=cam.height)
    r32 = O.train_step(32, sc.gt.copy(), cd, {"degrees_to_use": 3}, do_backward=False, do_optimizer=False)
    r64 = O.train_step(64, sc.gt.copy(), cd, {"degrees_to_use": 3}, do_backward=False, do_optimizer=False)
    assert np.mean(r32["radii"] == r64["radii"]) > 0.999
    d = np.abs(r32["out_img"] - r64["out_img"])
    assert np.mean(d > 1e-5) < 2e-3
    assert r32["k_max"] == 36   # 256 tiles < 400: chunked, K = ceil(6 * 48N / T / 512)


def test_eval_metrics():
    rng = np.random.default_rng(0)
    a = rng.random((20, 24, 3)).astype(np.float32)
    b = np.clip(a + rng.normal(0, 0.05, a.shape), 0, 1).astype(np.float32)
    mse = np.mean((a.astype(np.float64) - b) ** 2)
    assert abs(O.psnr(a, b) - 10 * np.log10(1 / mse)) < 1e-4
    assert abs(O.l1(a, b) - np.mean(np.abs(a - b))) < 1e-6
    assert abs(O.ssim_eval(a, a) - 1.0) < 1e-6
    assert 0.0 < O.ssim_eval(a, b) < 1.0


def test_mlp_oracle_gradients_finite_differences():
    """The MLP restatement's analytic gradient (float64, no rounding) against
    central differences of its own loss."""
    from oracle import mlp_oracle as M
    rng = np.random.default_rng(4)
    X = np.zeros((40, 32))
    X[:, :M.N_IN] = rng.normal(0, 1, (40, M.N_IN))
    T = rng.normal(0, 0.5, (40, 2))
    P = M.init_params(1).astype(np.float64)
    P[M.OFF["b1"][0]:M.OFF["b1"][0] + 64] = rng.normal(0, 0.1, 64)
    loss, g = M.loss_and_grad(X, T, P, rounding=False)
    idx = rng.choice(np.nonzero(g)[0], 60, replace=False)
    h = 1e-6
    fd = []
    for i in idx:
        Pp, Pm = P.copy(), P.copy()
        Pp[i] += h
        Pm[i] -= h
        fd.append((M.loss_and_grad(X, T, Pp, False)[0] - M.loss_and_grad(X, T, Pm, False)[0]) / (2 * h))
    fd = np.array(fd)
    assert np.linalg.norm(fd - g[idx]) / np.linalg.norm(fd) < 1e-6


def test_mlp_oracle_bf16_rounding():
    from oracle import mlp_oracle as M
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 0.0, 65504.0], np.float32)
    r = M.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125   # ties to even; 1 + 1.5 ulp rounds up
    assert abs(r[3] + 3.140625) < 1e-6 and r[4] == 0.0


def _fd_scene(n=512, seed=3, size=64):
    """The autograd test's scene: 512 Gaussians at a 64x64 view, opacity 0.73
    (alpha below the 0.999 clamp), dim colours (no saturate clamp)."""
    gt = S.gaussians(n, seed=seed)
    g = S.init_from_gt(gt, seed)
    g.opacities[:] = 1.0
    rng = np.random.default_rng(11)
    g.features_dc[:] = rng.uniform(-0.5, 0.3, g.features_dc.shape).astype(np.float32)
    g.features_rest *= np.float32(0.1)
    g.scales += rng.normal(0.0, 0.3, g.scales.shape).astype(np.float32)   # anisotropic: the rotation matters
    cam = S.ring_cameras(4, size, size, 51.25 * size / 64)[1]
    vm, pm, cp = O.prepare_cam(cam.cam_to_world, cam.width, cam.height, cam.fx, cam.fy)
    cd = dict(viewmat=vm, projmat=pm, cam_pos=cp, fx=cam.fx, fy=cam.fy, cx=cam.cx, cy=cam.cy, width=size,
              height=size)
    w = rng.normal(0.0, 1.0, (size, size, 3)).astype(np.float32)
    return g, cd, w


def _tile_rects(o, cd):
    f = np.float32
    tx, ty = (cd["width"] + 15) // 16, (cd["height"] + 15) // 16

    def conv(v, hi):
        return np.clip(np.trunc(np.clip(np.where(np.isfinite(v), v, 0), -2e9, 2e9)).astype(np.int64), 0, hi)
    cx, cy = o["xys"][:, 0] / f(16), o["xys"][:, 1] / f(16)
    rx, ry = o["aabb"][:, 0] / f(16), o["aabb"][:, 1] / f(16)
    return np.stack([conv(cx - rx, tx), conv(cy - ry, ty), conv(cx + rx + f(1), tx), conv(cy + ry + f(1), ty),
                     o["radii"] > 0], 1)


@pytest.mark.parametrize("group", ["means", "scales", "quats", "features_dc", "features_rest", "opacities"])
def test_fp64_gradients_directional_fd(group):
    """The FP64 analytic gradient of L = sum(W * image) (no sigma/alpha
    cutoffs) against central differences along random directions that move
    every visible Gaussian at once, three directions per parameter group.
    Gaussians whose tile rectangle or place in a depth-sorted list changes
    between the two evaluations are held still (the rendered image jumps
    there).  Relative error <= 1e-6.  Means: SH degree 0 (the reference does
    not differentiate the view direction) and the homogeneous w-row term the
    reference's pixel VJP leaves out added in closed form (.metal:1252-1270);
    quaternions: directions tangent to the unit sphere (the reference's
    gradient ignores the normalisation)."""
    from gpu_helpers import C0, sh_basis
    g, cd, w = _fd_scene()
    deg = 0 if group == "means" else 3
    eps = 1e-5 if group == "means" else 1e-4
    bg = (0.1, 0.2, 0.3)

    def run(gg, backward):
        return O.train_step(64, gg, cd, {"degrees_to_use": deg}, gt=None, v_img=w, background=bg,
                            do_backward=backward, do_optimizer=False, want_ids=not backward, no_cutoff=True)
    r = run(g.copy(), True)
    o0 = run(g.copy(), False)
    vis = r["radii"] > 0
    assert vis.sum() > 400
    if group == "means":
        pm = np.asarray(cd["projmat"], np.float64).reshape(4, 4)
        p = np.concatenate([g.means.astype(np.float64), np.ones((g.n, 1))], 1)
        rw = 1.0 / (p @ pm[3] + 1e-6)
        vnx = 0.5 * cd["width"] * r["v_xy"][:, 0].astype(np.float64)
        vny = 0.5 * cd["height"] * r["v_xy"][:, 1].astype(np.float64)
        corr = pm[3, :3][None, :] * (-(vnx * (p @ pm[0]) + vny * (p @ pm[1])) * rw * rw)[:, None]
        grad = r["v_mean3d"] + corr
    elif group == "scales":
        grad = r["v_scale"]
    elif group == "quats":
        q = g.quats.astype(np.float64)
        qn = q / np.linalg.norm(q, axis=1, keepdims=True)
        vq = r["v_quat"].astype(np.float64)
        grad = (vq - qn * np.sum(qn * vq, 1, keepdims=True)) / np.linalg.norm(q, axis=1, keepdims=True)
    elif group == "opacities":
        grad = r["v_opacity"][:, None]
    else:
        d = g.means.astype(np.float64) - np.asarray(cd["cam_pos"], np.float64)
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        grad = C0 * r["v_colors"] if group == "features_dc" else sh_basis(d)[:, :, None] * r["v_colors"][:, None, :]
    grad = np.where(vis.reshape((-1,) + (1,) * (grad.ndim - 1)), grad, 0.0)
    rects0 = _tile_rects(o0, cd)
    rng = np.random.default_rng({"means": 1, "scales": 2, "quats": 3, "features_dc": 4, "features_rest": 5,
                                 "opacities": 6}[group])
    base = getattr(g, group).astype(np.float64)
    for trial in range(3):
        v = rng.normal(size=base.shape)
        if group == "quats":
            v -= qn * np.sum(qn * v, 1, keepdims=True)
        v[~vis] = 0
        for _ in range(6):
            gp, gm = g.copy(), g.copy()
            getattr(gp, group)[...] = (base + eps * v).astype(np.float32)
            getattr(gm, group)[...] = (base - eps * v).astype(np.float32)
            op, om = run(gp.copy(), False), run(gm.copy(), False)
            still = np.zeros(g.n, bool)
            for oo in (op, om):
                still |= np.any(_tile_rects(oo, cd) != rects0, 1)
                for t in range(o0["tile_bins"].shape[0]):
                    a = o0["gaussian_ids"][o0["tile_bins"][t, 0]:o0["tile_bins"][t, 1]]
                    b = oo["gaussian_ids"][oo["tile_bins"][t, 0]:oo["tile_bins"][t, 1]]
                    if not np.array_equal(a, b):
                        m = min(len(a), len(b))
                        k = np.flatnonzero(a[:m] != b[:m])
                        first = int(k[0]) if len(k) else m
                        still[a[first:]] = True
                        still[b[first:]] = True
            if not (still & np.any(v.reshape(g.n, -1) != 0, 1)).any():
                break
            v[still] = 0
        moved = int(np.any(v.reshape(g.n, -1) != 0, 1).sum())
        assert moved > 250, moved
        dth = getattr(gp, group).astype(np.float64) - getattr(gm, group).astype(np.float64)
        fd = op["img_dot_v"] - om["img_dot_v"]
        an = float(np.sum(grad * dth))
        err = abs(fd - an) / abs(fd)
        print(group, trial, "moved", moved, "fd", fd, "analytic", an, "rel", err)
        assert err <= 1e-6, (group, trial, err)
