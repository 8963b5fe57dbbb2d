"""The torch.autograd binding (msplat_gb300.autograd.rasterize) on a
512-Gaussian 64x64 view (GPU only).

The chain of checks: the engine's gradients equal the oracle's analytic
gradients (float path within 1e-4, FP64 within 1e-5) for an arbitrary image
gradient; the oracle's FP64 analytic gradient without the sigma/alpha
cutoffs equals central differences of its forward along directions that
move every visible Gaussian at once within 1e-6
(tests/test_oracle.py::test_fp64_gradients_directional_fd, CPU).  The last
test here compares the engine (with the cutoffs) with differences of the
cutoff-free forward per Gaussian: what separates them is the part of the
gradient the reference's cutoffs drop."""
import numpy as np
import pytest

from msplat_gb300 import engine as E
from msplat_gb300 import synthetic as S
from oracle import oracle as O

from gpu_helpers import rel_l2, sh_grads

pytestmark = pytest.mark.gpu

@pytest.fixture(scope="module")
def scene():
    torch = pytest.importorskip("torch")
    gt = S.gaussians(512, seed=3)
    init = S.init_from_gt(gt, 3)
    # opacity 0.73: alpha stays below the 0.999 clamp, and the alpha < 1/255
    # cutoff (which the differences below do not apply) falls at sigma 5.2,
    # close to the sigma cutoff, so little of the gradient lies beyond them
    init.opacities[:] = 1.0
    rng = np.random.default_rng(11)
    # dim colours: no pixel reaches the saturate clamp (not differentiated)
    init.features_dc[:] = rng.uniform(-0.5, 0.3, init.features_dc.shape).astype(np.float32)
    init.features_rest *= np.float32(0.1)
    cam = S.ring_cameras(4, 64, 64, 51.25)[1]
    cd = E.camera_dict(cam)
    W = rng.normal(0.0, 1.0, (64, 64, 3)).astype(np.float32)
    return torch, init, cd, W


def _engine_grads(torch, g, cd, W, deg=3, bg=(0.1, 0.2, 0.3)):
    from msplat_gb300.autograd import rasterize
    ts = [torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda().requires_grad_(True) for a in g.arrays()]
    img = rasterize(*ts, camera=cd, background=bg, sh_degree=deg)
    loss = (img * torch.from_numpy(W).cuda()).sum()
    loss.backward()
    return img.detach().cpu().numpy(), [t.grad.detach().cpu().numpy() for t in ts]


def _oracle(prec, g, cd, W, deg=3, bg=(0.1, 0.2, 0.3), no_cutoff=False):
    return O.train_step(prec, g.copy(), cd, {"degrees_to_use": deg}, gt=None, v_img=W, background=bg,
                        do_backward=True, do_optimizer=False, want_ids=False, no_cutoff=no_cutoff)


def test_autograd_matches_oracle(scene):
    torch, g, cd, W = scene
    img, (gm, gs, gq, gdc, grest, gop) = _engine_grads(torch, g, cd, W)
    for prec, tol in ((32, 1e-4), (64, 1e-5)):   # measured ~4e-7 and ~2e-6 on GB300
        r = _oracle(prec, g, cd, W)
        if prec == 32:
            assert np.max(np.abs(img - r["out_img"])) <= 1e-5
        vis = r["radii"] > 0
        assert vis.sum() > 300
        v_dc, v_rest = sh_grads(g, cd, r)
        pairs = [("means", gm, np.where(vis[:, None], r["v_mean3d"], 0)),
                 ("scales", gs, np.where(vis[:, None], r["v_scale"], 0)),
                 ("quats", gq, np.where(vis[:, None], r["v_quat"], 0)),
                 ("opacities", gop.reshape(-1), np.where(vis, r["v_opacity"], 0)),
                 ("features_dc", gdc, v_dc), ("features_rest", grest, v_rest)]
        for name, a, b in pairs:
            e = rel_l2(a, b)
            print(prec, name, e)
            assert e <= tol, (prec, name, e)


def test_autograd_finite_differences(scene):
    """Per-Gaussian central differences of L = sum(W * image) through the
    oracle's FP64 forward (h = 1e-4; the sigma and alpha cutoffs are off
    there, so no difference straddles a jump), against the binding's
    gradients.  Means get the closed-form term of the homogeneous w row the
    reference's pixel VJP leaves out; quaternions are compared along the
    sphere."""
    torch, g, cd, W = scene
    img, (gm, gs, gq, gdc, grest, gop) = _engine_grads(torch, g, cd, W)
    assert img.max() < 1.0 and img.min() > 0.0
    r = _oracle(64, g, cd, W)
    bg = (0.1, 0.2, 0.3)
    h = 1e-4

    def L(gg):
        o = O.train_step(64, gg, cd, {"degrees_to_use": 3}, gt=None, background=bg, do_backward=False,
                         do_optimizer=False, want_ids=False, no_cutoff=True)
        return float(np.sum(o["out_img"].astype(np.float64) * W))

    def fd(mutate):
        gp, gmn = g.copy(), g.copy()
        mutate(gp, +h)
        mutate(gmn, -h)
        return (L(gp) - L(gmn)) / (2 * h)

    pm = np.asarray(cd["projmat"], np.float64).reshape(4, 4)
    vis = np.nonzero(r["radii"] > 0)[0]
    rng = np.random.default_rng(5)
    pick = rng.choice(vis, 6, replace=False)
    fd_all, an_all = [], []
    for i in pick:
        p = np.append(g.means[i].astype(np.float64), 1.0)
        hx, hy, hw = pm[0] @ p, pm[1] @ p, pm[3] @ p
        rw = 1.0 / (hw + 1e-6)
        vnx, vny = 0.5 * cd["width"] * r["v_xy"][i, 0], 0.5 * cd["height"] * r["v_xy"][i, 1]
        corr = pm[3, :3] * (-(vnx * hx + vny * hy)) * rw * rw
        for c in range(3):
            fd_all.append(fd(lambda G, d: G.means[i].__setitem__(c, G.means[i][c] + d)))
            an_all.append(gm[i, c] + corr[c])
            fd_all.append(fd(lambda G, d: G.scales[i].__setitem__(c, G.scales[i][c] + d)))
            an_all.append(gs[i, c])
            fd_all.append(fd(lambda G, d: G.features_dc[i].__setitem__(c, G.features_dc[i][c] + d)))
            an_all.append(gdc[i, c])
        for b, c in ((0, 0), (4, 1), (11, 2)):
            fd_all.append(fd(lambda G, d: G.features_rest[i, b].__setitem__(c, G.features_rest[i, b, c] + d)))
            an_all.append(grest[i, b, c])
        fd_all.append(fd(lambda G, d: G.opacities.reshape(-1).__setitem__(i, G.opacities.reshape(-1)[i] + d)))
        an_all.append(gop.reshape(-1)[i])
        q = g.quats[i].astype(np.float64)
        qn = q / np.linalg.norm(q)
        vq = gq[i].astype(np.float64)
        proj = (vq - qn * np.dot(qn, vq)) / np.linalg.norm(q)
        t = proj / (np.linalg.norm(proj) + 1e-30)
        fd_all.append(fd(lambda G, d: G.quats[i].__setitem__(slice(None), (q + d * t).astype(np.float32))))
        an_all.append(np.dot(proj, t))
    fd_all, an_all = np.array(fd_all), np.array(an_all)
    err = np.linalg.norm(fd_all - an_all) / np.linalg.norm(fd_all)
    print("fd rel err", err)
    assert err < 3e-2, err
