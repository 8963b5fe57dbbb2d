"""The oracle pinned to the reference's own source (CPU).

oracle/ref_build.py compiles the reference's Metal code unchanged as host C++
(oracle/_ref, built from the reference tree): the per-Gaussian helpers and
the bodies of project_and_sh_forward_kernel, project_and_sh_backward_kernel
(with its fused SH Adam), fused_adam_kernel, sgld_noise_gen/sgld_noise_kernel,
mcmc_reg_grad_kernel, count_intersections_kernel and
scatter_intersections_kernel, and - threadgroups run on host threads - the
tile scan and per-tile bitonic sort + pack, the monolithic and chunked
forward rasterizers with the merge, the three SSIM +
L1 kernels and the monolithic and chunked backward rasterizers (the chunked
one where it is defined: see oracle/ref_build.py).

Per-Gaussian stages, bit for bit against the oracle's float path: projection
(centres, depths, radii, conics, tiles hit, colours, extents), the tile
rectangles, sort keys and active test that order every per-tile list, the
SSIM window, and, from the same rasterizer gradients, the projection VJPs,
the SH Adam, regularizer, Adam and SGLD updates of every parameter and moment.
Pixel stages: per-tile lists, image, final transmittance, last contributors
and dL/dimage bit for bit (monolithic, and chunked with the reference's K
rule), the loss within 1e-6; the rasterizer gradients within 1e-6 (the
reference sums them with atomics) and the whole step's updates within 1e-5,
after the monolithic backward and, on a view where it is defined, the
chunked one.  exp() is the same function on both sides (the oracle's
det_expf; Metal's exp has no published bits).

Two parts:
  * live, on 100,000 random Gaussians (with culled, degenerate, non-finite and
    extreme ones) and small views with several splat batches per tile, partial
    edge tiles, a mask and a background, where the reference tree exists (the
    build container);
  * against the committed vectors tests/golden/ref_vectors.npz and
    ref_pixel_vectors.npz, made by tests/golden/make_ref_vectors.py from the
    same library, everywhere.
"""
import ctypes
import hashlib
import os

import numpy as np
import pytest

from msplat_gb300 import synthetic as S
from msplat_gb300.schedule import GROUPS, step_scalars
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_vectors.npz")
FWD_KEYS = ("xys", "depths", "radii", "conics", "num_tiles_hit", "colors", "aabb")


def ring_camera(width=1297, height=840, fx=1000.0, k=1):
    cam = S.ring_cameras(8, width, height, fx)[k]
    vm, pm, cp = O.prepare_cam(cam.cam_to_world, cam.width, cam.height, cam.fx, cam.fy)
    return dict(viewmat=vm, projmat=pm, cam_pos=cp, fx=cam.fx, fy=cam.fy, cx=cam.cx, cy=cam.cy, width=cam.width,
                height=cam.height)


def random_inputs(n, seed):
    """Gaussians in and around the view (plus extreme, culled, degenerate and
    non-finite ones), random Adam moments and rasterizer gradients."""
    rng = np.random.default_rng(seed)
    g = S.gaussians(n, seed)
    g.means *= np.float32(1.5)
    k = rng.permutation(n)
    g.scales[k[:n // 100]] = rng.uniform(-1.0, 1.0, (n // 100, 3)).astype(np.float32)       # huge
    g.scales[k[n // 100:n // 50]] = np.float32(-14.0)                                       # tiny (det cut)
    g.scales[k[n // 50:n // 50 + 4]] = np.float32(-20.0)                                    # below the clamp
    g.quats[k[200:210]] = 0.0                                                               # epsilon floor
    g.means[k[300:310]] = np.array([3.0, 0.0, 0.5], np.float32)                             # at the camera
    g.features_dc[k[400]] = np.nan                                                          # zombie gate
    g.features_rest[k[401], 3, 1] = np.inf
    g.opacities[:, 0] = rng.normal(0.0, 3.0, n).astype(np.float32)
    mom = ([np.abs(rng.normal(0, 1e-3, a.shape)).astype(np.float32) * (rng.random(a.shape) < 0.8) for a in g.arrays()],
           [np.abs(rng.normal(0, 1e-6, a.shape)).astype(np.float32) * (rng.random(a.shape) < 0.8) for a in g.arrays()])
    rg = np.concatenate([rng.normal(0, 1e-4, (n, 2)), rng.normal(0, 1e-3, (n, 3)), rng.normal(0, 1e-3, (n, 3)),
                         rng.normal(0, 1e-3, (n, 1))], axis=1).astype(np.float32)
    rg[k[500], 5] = np.nan          # SH Adam gate
    rg[k[501], 0] = np.inf          # Adam gate on the means
    return g, mom, rg


def oracle_run(g, mom, rg, cam, step):
    g = g.copy()
    mom = ([a.copy() for a in mom[0]], [a.copy() for a in mom[1]])
    r = O.train_step(32, g, cam, step, moments=mom, raster_grads=rg, do_backward=True, do_optimizer=True,
                     do_sgld=True, want_ids=True)
    return r, g, mom


def ref_run(g, mom, rg, cam, step):
    from oracle import ref as R
    g = g.copy()
    mom = ([a.copy() for a in mom[0]], [a.copy() for a in mom[1]])
    fwd = R.project_fwd(g, cam, step["degrees_to_use"])
    bwd = R.step_after_raster(g, mom, cam, step, rg, fwd)
    return fwd, bwd, g, mom


def _same(a, b):
    return np.array_equal(np.asarray(a), np.asarray(b), equal_nan=True)


def compare(r, g_o, mom_o, fwd, bwd, g_r, mom_r):
    act = fwd["radii"] > 0
    assert act.sum() > 0.3 * act.size
    assert _same(r["radii"], fwd["radii"]) and _same(r["num_tiles_hit"], fwd["num_tiles_hit"])
    for k in ("xys", "depths", "conics", "colors", "aabb"):
        assert _same(r[k][act], fwd[k][act]), k
    assert _same(r["nan_counts"][7:13], fwd["nan_counts"][7:13])
    for k in ("v_mean3d", "v_scale", "v_quat"):
        assert _same(np.where(act[:, None], r[k], 0), bwd[k]), k
    for name, a, b in zip(GROUPS, g_o.arrays(), g_r.arrays()):
        assert _same(a, b), name
    for m in range(2):
        for name, a, b in zip(GROUPS, mom_o[m], mom_r[m]):
            assert _same(a, b), (m, name)


needs_reference = pytest.mark.skipif(not __import__("oracle.ref", fromlist=["available"]).available(),
                                     reason="the reference tree is not present (the GPU box)")


@pytest.fixture(scope="module")
def ref_lib():
    from oracle import ref as R
    R.lib()
    R.set_expf(ctypes.cast(O.lib().or_det_expf, ctypes.c_void_p).value)
    return R


@needs_reference
@pytest.mark.parametrize("step_no,deg", [(1, 0), (1500, 1), (2500, 2), (3001, 3)])
def test_live_per_gaussian_stages(ref_lib, step_no, deg):
    cam = ring_camera()
    g, mom, rg = random_inputs(100_000, 11 + step_no)
    step = step_scalars(step_no, step_no, width=cam["width"], height=cam["height"])
    assert step["degrees_to_use"] == deg
    r, g_o, mom_o = oracle_run(g, mom, rg, cam, step)
    fwd, bwd, g_r, mom_r = ref_run(g, mom, rg, cam, step)
    compare(r, g_o, mom_o, fwd, bwd, g_r, mom_r)


@needs_reference
def test_live_tile_lists(ref_lib):
    """Per-tile lists from the reference's get_tile_bbox, gaussian_is_active and
    make_sort_key (ascending keys) equal the oracle's lists."""
    cam = ring_camera(320, 208, 260.0)
    g, mom, rg = random_inputs(20_000, 5)
    step = step_scalars(3001, 3001, width=cam["width"], height=cam["height"])
    r = O.train_step(32, g.copy(), cam, step, do_backward=False, do_optimizer=False, want_ids=True)
    fwd = ref_lib.project_fwd(g, cam, 3)
    rect = ref_lib.tile_rects(fwd["xys"], fwd["aabb"], cam["width"], cam["height"])
    act, keys = ref_lib.sort_keys(fwd["radii"], fwd["depths"])
    tx, ty = (cam["width"] + 15) // 16, (cam["height"] + 15) // 16
    lists = [[] for _ in range(tx * ty)]
    for i in np.flatnonzero(act):
        x0, y0, x1, y1 = rect[i]
        for y in range(y0, y1):
            for x in range(x0, x1):
                lists[y * tx + x].append(i)
    ids = np.concatenate([np.array(sorted(L, key=lambda i: int(keys[i])), np.int64) for L in lists if L])
    assert ids.size == r["num_isect"] > 10_000
    assert np.array_equal(ids, r["gaussian_ids"])
    assert np.array_equal([len(L) for L in lists], r["tile_counts"])


@needs_reference
def test_live_ssim_window(ref_lib):
    assert np.array_equal(ref_lib.gauss_1d(), O.gauss_1d())


def test_golden_vectors():
    """The oracle against the reference library's outputs stored in
    tests/golden/ref_vectors.npz (no reference tree needed)."""
    z = np.load(GOLDEN)
    cam = {k[4:]: z[k] for k in z.files if k.startswith("cam_")}
    for k in ("fx", "fy", "cx", "cy"):
        cam[k] = float(cam[k])
    for k in ("width", "height"):
        cam[k] = int(cam[k])
    g = S.GaussianSet(*(z["in_" + k] for k in GROUPS))
    mom = ([z["in_m_" + k] for k in GROUPS], [z["in_v_" + k] for k in GROUPS])
    step = step_scalars(int(z["step"]), int(z["step"]), width=cam["width"], height=cam["height"])
    r, g_o, mom_o = oracle_run(g, mom, z["in_raster_grads"], cam, step)
    fwd = {k: z["fwd_" + k] for k in FWD_KEYS + ("nan_counts",)}
    bwd = {k: z["bwd_" + k] for k in ("v_mean3d", "v_scale", "v_quat")}
    g_r = S.GaussianSet(*(z["out_" + k] for k in GROUPS))
    mom_r = ([z["out_m_" + k] for k in GROUPS], [z["out_v_" + k] for k in GROUPS])
    compare(r, g_o, mom_o, fwd, bwd, g_r, mom_r)
    assert np.array_equal(O.gauss_1d(), z["gauss_1d"])


PIXEL_CASES = {
    # width, height, Gaussians, seed, mask, background, raster mode (1: monolithic, 0: the
    # reference's rule, which takes the chunked rasterizer below 400 tiles)
    "plain": (48, 32, 300, 3, False, (0.0, 0.0, 0.0), 1),
    "ragged_mask_bg": (50, 34, 350, 4, True, (0.25, 0.5, 0.75), 1),
    "chunked": (40, 32, 1800, 5, True, (0.1, 0.2, 0.3), 0),
}


def pixel_case(name):
    """A small view (several 64-splat batches per tile), its target and
    optional mask; the Gaussians include a NaN colour (zombie gate)."""
    W, H, n, seed, with_mask, bg, _ = PIXEL_CASES[name]
    cam = ring_camera(W, H, 0.8 * W, k=2)
    g = S.gaussians(n, seed)
    g.features_dc[7] = np.nan
    rng = np.random.default_rng(seed)
    gt = rng.integers(0, 256, (H, W, 3), dtype=np.uint8)
    mask = None
    if with_mask:
        mask = np.full((H, W), 255, np.uint8)
        mask[5:15, 10:30] = 0
        mask[H - 6:, W - 9:] = 0
    return cam, g, gt, mask, bg


def chunked_backward_case():
    """One 16x16 tile under 560 Gaussians: 520 wide, faint ones (screen
    sigma about 50 px, opacity 0.0055-0.009) that reach every pixel with
    alpha >= 1/255, so every pixel has a contributor in each chunk (where the
    reference's chunked backward is defined), and 40 small ones; three
    chunks of 512 splats (the last empty), final transmittance 0.002-0.03,
    so the second chunk's splats carry gradient."""
    W = H = 16
    cam = ring_camera(W, H, 0.8 * W, k=2)
    rng = np.random.default_rng(11)
    nb, ns = 520, 40
    g = S.gaussians(nb + ns, 11)
    g.means[:nb] = rng.uniform(-0.3, 0.3, (nb, 3)).astype(np.float32)
    g.scales[:nb] = rng.uniform(2.3, 2.6, (nb, 3)).astype(np.float32)
    op = rng.uniform(0.0055, 0.009, nb)
    g.opacities[:nb, 0] = np.log(op / (1 - op)).astype(np.float32)
    g.features_dc[:nb] = rng.uniform(-1.0, 1.0, (nb, 3)).astype(np.float32)
    g.scales[nb:] = rng.normal(-1.8, 0.2, (ns, 3)).astype(np.float32)
    g.opacities[nb:, 0] = rng.normal(-1.0, 0.5, ns).astype(np.float32)
    gt = np.random.default_rng(12).integers(0, 256, (H, W, 3), dtype=np.uint8)
    return cam, g, gt


def dense_tile_case():
    """One 16x16 tile under 2200 small Gaussians: more than 2048 keys, so the
    reference sorts the tile with its device-memory bitonic network (4096
    padded keys); monolithic raster, transmittance down to the 1e-4 stop."""
    W = H = 16
    cam = ring_camera(W, H, 0.8 * W, k=2)
    rng = np.random.default_rng(21)
    n = 2200
    g = S.gaussians(n, 21)
    g.means[:] = rng.uniform(-0.25, 0.25, (n, 3)).astype(np.float32)
    g.scales[:] = rng.normal(-1.2, 0.3, (n, 3)).astype(np.float32)
    g.opacities[:, 0] = rng.normal(-2.5, 1.0, n).astype(np.float32)
    gt = rng.integers(0, 256, (H, W, 3), dtype=np.uint8)
    return cam, g, gt


def check_pixel_path(r, o, backward=True):
    """The oracle's float path (r) against the reference kernels' pixel stages
    (o); the rasterizer gradients only when the reference's backward ran."""
    assert r["num_isect"] == o["num_isect"]
    assert np.array_equal(r["gaussian_ids"], o["gaussian_ids"])
    assert np.array_equal(r["tile_bins"], o["tile_bins"])
    for k in ("out_img", "final_Ts", "final_idx", "v_rendered"):
        assert np.array_equal(r[k], o[k]), k
    assert abs(r["loss"] - o["loss"]) <= 1e-6 * abs(r["loss"])
    for k in ("v_xy", "v_conic", "v_colors", "v_opacity") if backward else ():
        e = np.linalg.norm((r[k] - o[k]).ravel()) / np.linalg.norm(o[k].ravel())
        assert e <= 1e-6, (k, e)


@needs_reference
@pytest.mark.parametrize("name", list(PIXEL_CASES))
def test_live_pixel_path(ref_lib, name):
    """Tile lists, forward rasterizer, SSIM + L1 loss and backward rasterizer
    of the reference (threadgroups on host threads) against the oracle's
    float path: lists, image, transmittance, last contributors and dL/dimage
    identical, loss within 1e-6, rasterizer gradients within 1e-6 (the
    reference adds them with atomics in no fixed order); then the whole
    step's updates from the reference's per-Gaussian kernels within 1e-5."""
    cam, g, gt, mask, bg = pixel_case(name)
    step = step_scalars(3001, 3001, width=cam["width"], height=cam["height"])
    mom = ([np.zeros_like(a) for a in g.arrays()], [np.zeros_like(a) for a in g.arrays()])
    g_o = g.copy()
    mom_o = ([a.copy() for a in mom[0]], [a.copy() for a in mom[1]])
    mode = PIXEL_CASES[name][-1]
    r = O.train_step(32, g_o, cam, step, moments=mom_o, gt=gt, mask=mask, background=bg, raster_mode=mode,
                     do_sgld=True)
    fwd = ref_lib.project_fwd(g, cam, 3)
    o = ref_lib.raster_step(fwd, g.opacities, cam, gt=gt, mask=mask, background=bg,
                            loss_inv_n=step["loss_inv_n"], k_max=r["k_max"])
    assert int(np.diff(o["tile_bins"], axis=1).max()) > (512 if mode == 0 else 128)
    assert (r["k_max"] > 2) == (mode == 0)
    # the chunked backward runs where it is defined (oracle/ref_build.py)
    assert o["backward_ran"] or mode != 1
    check_pixel_path(r, o, backward=o["backward_ran"])
    if o["backward_ran"]:
        check_step_updates(ref_lib, g, g_o, mom, cam, step, o, fwd)


def check_step_updates(ref_lib, g, g_o, mom, cam, step, o, fwd):
    """The whole step's updates from the reference's per-Gaussian kernels,
    fed with its rasterizer gradients, against the oracle's (g_o): within
    1e-5 relative of each group's update."""
    g_r = g.copy()
    ref_lib.step_after_raster(g_r, mom, cam, step, o["raster_grads"], fwd)
    for name_, a, b, before in zip(GROUPS, g_o.arrays(), g_r.arrays(), g.arrays()):
        fin = np.isfinite(before)
        e = np.linalg.norm((a - b)[fin]) / max(np.linalg.norm((b - before)[fin]), 1e-30)
        assert e <= 1e-5, (name_, e)


@needs_reference
def test_live_chunked_backward(ref_lib):
    """The reference's chunked backward (compute_chunk_prefix_suffix_kernel,
    then rasterize_backward_chunked_kernel per chunk, threadgroups on host
    threads) on a view where it is defined, against the oracle's chunked
    float path: lists, image, transmittance, last contributors and dL/dimage
    identical, rasterizer gradients within 1e-6 (atomics), every splat of
    the second chunk with gradient; then the step's updates within 1e-5."""
    cam, g, gt = chunked_backward_case()
    step = step_scalars(3001, 3001, width=cam["width"], height=cam["height"])
    mom = ([np.zeros_like(a) for a in g.arrays()], [np.zeros_like(a) for a in g.arrays()])
    g_o = g.copy()
    mom_o = ([a.copy() for a in mom[0]], [a.copy() for a in mom[1]])
    r = O.train_step(32, g_o, cam, step, moments=mom_o, gt=gt, raster_mode=0, k_max=3, do_sgld=True)
    assert r["k_max"] == 3
    fwd = ref_lib.project_fwd(g, cam, 3)
    o = ref_lib.raster_step(fwd, g.opacities, cam, gt=gt, loss_inv_n=step["loss_inv_n"], k_max=3)
    assert o["backward_ran"]
    assert int(np.diff(o["tile_bins"], axis=1).max()) > 512
    check_pixel_path(r, o, backward=True)
    late = o["gaussian_ids"][512:]
    assert late.size > 0 and np.count_nonzero(o["v_opacity"][late]) == late.size
    check_step_updates(ref_lib, g, g_o, mom, cam, step, o, fwd)


def test_golden_pixel_vectors():
    """The oracle's pixel stages against the reference kernels' outputs stored
    in tests/golden/ref_pixel_vectors.npz (no reference tree needed)."""
    z = np.load(os.path.join(os.path.dirname(GOLDEN), "ref_pixel_vectors.npz"))
    for name in PIXEL_CASES:
        cam, g, gt, mask, bg = pixel_case(name)
        step = step_scalars(3001, 3001, width=cam["width"], height=cam["height"])
        r = O.train_step(32, g.copy(), cam, step, gt=gt, mask=mask, background=bg,
                         raster_mode=PIXEL_CASES[name][-1], do_optimizer=False)
        o = {k[len(name) + 1:]: z[k] for k in z.files if k.startswith(name + "/")}
        o["num_isect"] = int(o["num_isect"])
        o["loss"] = float(o["loss"])
        check_pixel_path(r, o, backward="v_xy" in o)


@needs_reference
def test_live_dense_tile(ref_lib):
    """A tile of more than 2048 keys (the reference's device-memory bitonic
    sort) through the reference's pixel stages against the oracle's float
    path: lists, image, transmittance, last contributors and dL/dimage
    identical, rasterizer gradients within 1e-6."""
    cam, g, gt = dense_tile_case()
    step = step_scalars(3001, 3001, width=cam["width"], height=cam["height"])
    r = O.train_step(32, g.copy(), cam, step, gt=gt, raster_mode=1, do_optimizer=False)
    o = ref_lib.raster_step(ref_lib.project_fwd(g, cam, 3), g.opacities, cam, gt=gt, loss_inv_n=step["loss_inv_n"])
    assert int(np.diff(o["tile_bins"], axis=1).max()) > 2048 and o["backward_ran"]
    assert float(o["final_Ts"].min()) < 1.01e-4
    check_pixel_path(r, o, backward=True)


def test_golden_dense_tile():
    """The oracle on dense_tile_case() against the reference kernels' outputs
    stored in tests/golden/ref_pixel_vectors.npz (no reference tree needed)."""
    z = np.load(os.path.join(os.path.dirname(GOLDEN), "ref_pixel_vectors.npz"))
    cam, g, gt = dense_tile_case()
    step = step_scalars(3001, 3001, width=cam["width"], height=cam["height"])
    r = O.train_step(32, g.copy(), cam, step, gt=gt, raster_mode=1, do_optimizer=False)
    o = {k[len("dense/"):]: z[k] for k in z.files if k.startswith("dense/")}
    o["num_isect"] = int(o["num_isect"])
    o["loss"] = float(o["loss"])
    assert int(np.diff(o["tile_bins"], axis=1).max()) > 2048
    check_pixel_path(r, o, backward=True)


def test_golden_chunked_backward():
    """The oracle's chunked forward and backward against the reference
    kernels' outputs on chunked_backward_case(), stored in
    tests/golden/ref_pixel_vectors.npz (no reference tree needed)."""
    z = np.load(os.path.join(os.path.dirname(GOLDEN), "ref_pixel_vectors.npz"))
    cam, g, gt = chunked_backward_case()
    step = step_scalars(3001, 3001, width=cam["width"], height=cam["height"])
    r = O.train_step(32, g.copy(), cam, step, gt=gt, raster_mode=0, k_max=3, do_optimizer=False)
    o = {k[len("chunked_bwd/"):]: z[k] for k in z.files if k.startswith("chunked_bwd/")}
    o["num_isect"] = int(o["num_isect"])
    o["loss"] = float(o["loss"])
    check_pixel_path(r, o, backward=True)


# ---- MCMC host code (model.cpp:311-660, compiled against oracle/model_shim.h) ----

def mcmc_state(n, cap, seed, dead=True):
    """cap rows, the first n in use.  With dead: 8 % faded (sigmoid(opacity)
    in (0.0005, 0.005)), 1 % with one non-finite parameter (mean, scale,
    quaternion, DC or rest coefficient), 1 % outside a cull radius of 3; the
    rest alive.  Random Adam moments; rows past n zero."""
    rng = np.random.default_rng(seed)
    g = S.gaussians(cap, seed)
    g.opacities[:, 0] = np.maximum(rng.normal(0.5, 1.0, cap), -5.0).astype(np.float32)
    if dead:
        k = rng.permutation(n)
        nf, nn, nc = n * 8 // 100, n // 100, n // 100
        op = rng.uniform(0.0005, 0.005, nf)
        g.opacities[k[:nf], 0] = np.log(op / (1 - op)).astype(np.float32)
        bad = k[nf:nf + nn]
        g.means[bad[0::5], 1] = np.nan
        g.scales[bad[1::5], 2] = np.inf
        g.quats[bad[2::5], 0] = np.nan
        g.features_dc[bad[3::5], 0] = -np.inf
        g.features_rest[bad[4::5], 7, 2] = np.nan
        far = k[nf + nn:nf + nn + nc]
        g.means[far] *= np.float32(4.0) / np.maximum(np.linalg.norm(g.means[far], axis=1, keepdims=True), 1e-3)
    for a in g.arrays():
        a[n:] = 0
    mom = ([np.abs(rng.normal(0, 1e-3, a.shape)).astype(np.float32) for a in g.arrays()],
           [np.abs(rng.normal(0, 1e-6, a.shape)).astype(np.float32) for a in g.arrays()])
    return g, mom


def _copy_state(g, mom):
    return g.copy(), ([a.copy() for a in mom[0]], [a.copy() for a in mom[1]])


def _state_digest(g, mom):
    h = hashlib.sha256()
    for a in list(g.arrays()) + list(mom[0]) + list(mom[1]):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def mcmc_pairs(g0, g_r, n, n_new, dead):
    """The (dst, src) moves of a pass, recovered from its output: a dead row
    or a new row holds a copy of its source's mean, and sources keep their
    means, so each copied mean names one row of the input."""
    rows = np.flatnonzero(~dead) if dead is not None else np.arange(n)
    key = {g0.means[i].tobytes(): i for i in rows}
    assert len(key) == rows.size
    dst = np.concatenate([np.flatnonzero(dead) if dead is not None else np.zeros(0, np.int64),
                          np.arange(n, n_new)]).astype(np.int32)
    src = np.array([key[g_r.means[d].tobytes()] for d in dst], np.int32)
    return dst, src


MCMC_CASES = {
    # rows in use, rows, seed, with dead rows: relocation only (no room to grow), growth only
    "relocate": (2000, 2000, 5, True),
    "grow": (2000, 2400, 6, False),
}


@needs_reference
@pytest.mark.parametrize("name", list(MCMC_CASES))
def test_live_mcmc_host_code(ref_lib, name):
    """The reference's Model::mcmcAfterTrain pass at step 600 (classification
    of faded, non-finite and culled Gaussians, relocation with Eq. 9 and the
    copies, growth by 5 % toward the cap, moments zeroed) against the
    oracle's restatement given the reference's own draws: the dead rows are
    the oracle's (or_mcmc_dead_mask), alive rows keep their means, and every
    parameter and moment after or_mcmc_apply is bit-identical."""
    n, cap, seed, with_dead = MCMC_CASES[name]
    g0, m0 = mcmc_state(n, cap, seed, with_dead)
    g_r, m_r = _copy_state(g0, m0)
    n_new, rc = ref_lib.mcmc_after_train(g_r, m_r, n, 600, 30000, 3.0, 0)
    dead, cnt = O.mcmc_dead_mask(S.GaussianSet(*(a[:n] for a in g0.arrays())), 3.0)
    if with_dead:
        assert cnt == n // 10 and n_new == n and rc == 1
        assert np.array_equal(g_r.means[:n][~dead], g0.means[:n][~dead])
    else:
        assert cnt == 0 and n_new == int(np.float32(1.05) * np.float32(n)) and rc == 1
    dst, src = mcmc_pairs(g0, g_r, n, n_new, dead if with_dead else None)
    g_o, m_o = _copy_state(g0, m0)
    O.mcmc_apply(g_o, m_o, dst, src)
    for k, a, b in zip(GROUPS, g_o.arrays(), g_r.arrays()):
        assert a.tobytes() == b.tobytes(), k
    for k, a, b in zip(GROUPS * 2, m_o[0] + m_o[1], m_r[0] + m_r[1]):
        assert a.tobytes() == b.tobytes(), k
    # the pass is a no-op before step 500, off the 100-step cadence and in the last 16.7 %
    for step in (400, 650, 25000):
        g_n, m_n = _copy_state(g0, m0)
        assert ref_lib.mcmc_after_train(g_n, m_n, n, step, 30000, 3.0, 0) == (n, 0)
        assert _state_digest(g_n, m_n) == _state_digest(g0, m0)


def test_golden_mcmc_host_code():
    """The oracle's MCMC restatement against tests/golden/ref_mcmc_vectors.npz
    (the reference pass's moves and a SHA-256 of its output state, written
    by tests/golden/make_ref_vectors.py): the same moves applied by
    or_mcmc_apply give the same bytes (no reference tree needed)."""
    z = np.load(os.path.join(os.path.dirname(GOLDEN), "ref_mcmc_vectors.npz"))
    for name, (n, cap, seed, with_dead) in MCMC_CASES.items():
        g0, m0 = mcmc_state(n, cap, seed, with_dead)
        if with_dead:
            dead, _ = O.mcmc_dead_mask(S.GaussianSet(*(a[:n] for a in g0.arrays())), 3.0)
            assert np.array_equal(np.flatnonzero(dead), z[name + "/dst"][:int(dead.sum())])
        O.mcmc_apply(g0, m0, z[name + "/dst"], z[name + "/src"])
        assert _state_digest(g0, m0) == str(z[name + "/sha256"])


# ---- camera setup and evaluation metrics (model.cpp:33-49, 845-889; ssim.cpp:26-123) ----

@needs_reference
def test_live_prepare_cam(ref_lib):
    """The reference's Model::prepareCam against the oracle's prepare_cam and
    the engine library's msplat_prepare_camera: view and projection-view
    matrices and camera centre bit for bit over random poses, sizes and focal
    lengths; its SH degree and degrees-to-use bands as the step schedule's."""
    from msplat_gb300 import engine as E
    from msplat_gb300.schedule import step_scalars
    rng = np.random.default_rng(3)
    cams = S.ring_cameras(8, 640, 480, 500.0, seed=3, jitter=1.0)
    for k in range(64):
        c = cams[k % 8]
        c2w = np.asarray(c.cam_to_world, np.float32).copy()
        c2w[:3, 3] += rng.normal(0, 0.5, 3).astype(np.float32)
        w, h = int(rng.integers(16, 2000)), int(rng.integers(16, 2000))
        fx, fy = float(rng.uniform(100, 3000)), float(rng.uniform(100, 3000))
        cx, cy = w / 2.0, h / 2.0
        step = int(rng.integers(0, 30000))
        vm, pvm, cp, ints = ref_lib.prepare_cam(c2w, w, h, fx, fy, cx, cy, step)
        for got in (O.prepare_cam(c2w, w, h, np.float32(fx), np.float32(fy)),
                    E.prepare_cam(c2w, w, h, np.float32(fx), np.float32(fy))):
            assert np.array_equal(np.asarray(got[0]).ravel(), vm)
            assert np.array_equal(np.asarray(got[1]).ravel(), pvm)
            assert np.array_equal(np.asarray(got[2]).ravel(), cp)
        assert ints == (w, h, 3, step_scalars(step, max(step, 1))["degrees_to_use"], (w + 15) // 16, (h + 15) // 16)


@needs_reference
def test_live_eval_metrics(ref_lib):
    """The reference's psnr, l1_loss and ssim_eval against the oracle's and
    the engine library's host metrics (msplat_psnr, msplat_l1,
    msplat_ssim_eval, which the trainer's evaluate uses) on random images of
    odd sizes: identical floats."""
    import ctypes as C
    from msplat_gb300 import build
    lib = C.CDLL(build.build())
    fp = C.POINTER(C.c_float)
    lib.msplat_psnr.restype = lib.msplat_l1.restype = lib.msplat_ssim_eval.restype = C.c_float
    lib.msplat_psnr.argtypes = lib.msplat_l1.argtypes = [fp, fp, C.c_longlong]
    lib.msplat_ssim_eval.argtypes = [fp, fp, C.c_int, C.c_int]
    rng = np.random.default_rng(9)
    for h, w in ((17, 23), (64, 48), (101, 7), (5, 130)):
        gt = rng.random((h, w, 3), dtype=np.float32)
        img = np.clip(gt + rng.normal(0, 0.05, gt.shape), 0, 1).astype(np.float32)
        ref = ref_lib.metrics(img, gt)
        mine = (float(O.psnr(img, gt)), float(O.l1(img, gt)), float(O.ssim_eval(img, gt)))
        pi, pg = img.ctypes.data_as(fp), gt.ctypes.data_as(fp)
        eng = (float(lib.msplat_psnr(pi, pg, img.size)), float(lib.msplat_l1(pi, pg, img.size)),
               float(lib.msplat_ssim_eval(pi, pg, h, w)))
        assert np.float32(mine[0]) == np.float32(ref[0]) and np.float32(eng[0]) == np.float32(ref[0])
        assert np.float32(mine[1]) == np.float32(ref[1]) and np.float32(eng[1]) == np.float32(ref[1])
        assert np.float32(mine[2]) == np.float32(ref[2]) and np.float32(eng[2]) == np.float32(ref[2])


# ---- dataset ingestion (loaders/load_colmap.cpp, load_ply.cpp, input_data.cpp:115-169) ----

def write_colmap_scene(root, seed, ply_points=False):
    """A COLMAP binary dataset: 12 views from two cameras (PINHOLE and
    SIMPLE_PINHOLE) written in shuffled order with unsorted names, small PNG
    images, and 200 points with tracks (points3D.bin), or as a binary PLY
    (points3D.ply) with ply_points; returns nothing (files only)."""
    import struct
    from test_dataset_io import _pose, _w2c, _write_ply_points, write_png
    rng = np.random.default_rng(seed)
    sp = root / "sparse" / "0"
    os.makedirs(sp)
    os.makedirs(root / "images")
    with open(sp / "cameras.bin", "wb") as f:
        f.write(struct.pack("<Q", 2))
        f.write(struct.pack("<IiQQ", 1, 1, 32, 24) + struct.pack("<4d", 29.5, 31.25, 16.0, 12.0))
        f.write(struct.pack("<IiQQ", 2, 0, 40, 20) + struct.pack("<3d", 27.0, 20.0, 10.0))
    names = [f"v{int(k):03d}_{int(rng.integers(1000))}.png" for k in rng.permutation(12)]
    with open(sp / "images.bin", "wb") as f:
        f.write(struct.pack("<Q", 12))
        for k, name in enumerate(names):
            a = rng.uniform(0, 2 * np.pi)
            eye = (rng.uniform(3, 6) * np.cos(a), rng.uniform(3, 6) * np.sin(a), rng.uniform(-1, 2))
            q, t = _w2c(_pose(eye))
            cam = 1 + (k % 2)
            f.write(struct.pack("<I4d3dI", k + 1, *q, *t, cam) + name.encode() + b"\0")
            f.write(struct.pack("<Q", 1) + struct.pack("<ddQ", 1.0, 2.0, 7))
            w, h = (32, 24) if cam == 1 else (40, 20)
            img = rng.integers(0, 256, (h, w, 3), dtype=np.uint8)
            write_png(root / "images" / name, [img[y].tobytes() for y in range(h)], 2, 8)
    xyz = rng.normal(0, 1.5, (200, 3))
    rgb = rng.integers(0, 256, (200, 3), dtype=np.uint8)
    if ply_points:
        _write_ply_points(sp / "points3D.ply", xyz.astype(np.float32), rgb)
        return
    with open(sp / "points3D.bin", "wb") as f:
        f.write(struct.pack("<Q", 200))
        for i in range(200):
            f.write(struct.pack("<Q3d3Bd", i, *xyz[i], *rgb[i], 0.5))
            f.write(struct.pack("<Q", 2) + struct.pack("<IIII", 1, 0, 2, 0))


@needs_reference
@pytest.mark.parametrize("seed,ply_points", [(1, False), (2, False), (3, True)])
def test_live_colmap_loader(ref_lib, tmp_path, seed, ply_points):
    """The reference's COLMAP binary loader with its point readers
    (points3D.bin, or points3D.ply) and autoScaleAndCenter against the
    library's msplat_dataset_create: the same cameras in the same order
    (sorted by file name), identical intrinsics and sizes, camera-to-world
    poses and centred, scaled points bit for bit."""
    import ctypes as C
    from msplat_gb300 import api as A
    write_colmap_scene(tmp_path, seed, ply_points)
    cams, (xyz, rgb), _ = ref_lib.load_colmap(tmp_path)
    assert [c["name"] for c in cams] == sorted(c["name"] for c in cams)
    ds = A.Dataset(str(tmp_path))
    L = A._lib()
    assert ds.num_train == len(cams) == 12
    for i, c in enumerate(cams):
        intr, size, c2w = np.zeros(4, np.float32), np.zeros(2, np.int32), np.zeros(16, np.float32)
        img = np.zeros((c["size"][1], c["size"][0], 3), np.uint8)
        assert L.msplat_dataset_camera(ds.h, i, 0, intr.ctypes.data_as(C.POINTER(C.c_float)),
                                       size.ctypes.data_as(C.POINTER(C.c_int)),
                                       c2w.ctypes.data_as(C.POINTER(C.c_float)),
                                       img.ctypes.data_as(C.POINTER(C.c_uint8))) == 0
        assert tuple(size) == c["size"]
        assert np.array_equal(intr, c["intr"]) and not c["dist"].any()
        assert np.array_equal(c2w, c["c2w"].ravel()), (i, c2w - c["c2w"].ravel())
    pts, cols = np.zeros_like(xyz), np.zeros_like(rgb)
    assert L.msplat_dataset_points(ds.h, pts.ctypes.data_as(C.POINTER(C.c_float)),
                                   cols.ctypes.data_as(C.POINTER(C.c_uint8))) == len(xyz)
    assert np.array_equal(pts, xyz) and np.array_equal(cols, rgb)


# ---- Gaussian PLY / .splat files (loaders/save_gaussians.cpp:8-231) ----

def file_gaussians(n, seed):
    """n Gaussians with extreme values and a few non-finite rows (which the
    writers drop), in the layouts of the C API."""
    rng = np.random.default_rng(seed)
    g = S.gaussians(n, seed)
    arrs = [g.means * np.float32(3.0), g.scales, g.quats, g.features_dc, g.features_rest, g.opacities[:, 0].copy()]
    arrs[1][::17] = rng.uniform(-12, 3, (len(arrs[1][::17]), 3)).astype(np.float32)
    arrs[5][::13] = rng.normal(0, 8, len(arrs[5][::13])).astype(np.float32)
    arrs[2][5] = 0.0
    arrs[0][7, 1] = np.nan
    arrs[4][11, 3, 2] = np.inf
    arrs[5][19] = -np.inf
    arrs[3][23, 0] = np.nan
    return [np.ascontiguousarray(a, np.float32) for a in arrs]


@needs_reference
@pytest.mark.parametrize("keep_crs", [False, True])
def test_live_gaussian_files(ref_lib, tmp_path, keep_crs):
    """The library's PLY and .splat writers (msplat_write_ply /
    msplat_write_splat, the trainer's export code) against the reference's
    saveGaussianPly / saveGaussianSplat: byte-identical files, non-finite
    Gaussians dropped, with and without the dataset-frame mapping; and its
    PLY reader (msplat_read_ply) against loadGaussianPly: identical arrays
    and iteration."""
    from msplat_gb300 import api as A
    arrs = file_gaussians(500, 4)
    crs = dict(keep_crs=keep_crs, scale=0.37, translation=(1.5, -2.25, 0.125)) if keep_crs else {}
    for splat in (False, True):
        mine, ref = tmp_path / f"mine{int(splat)}", tmp_path / f"ref{int(splat)}"
        if splat:
            A.write_splat(str(mine), arrs, **crs)
        else:
            A.write_ply(str(mine), arrs, step=7000, **crs)
        ref_lib.save_gaussians(ref, arrs, splat=splat, step=7000, **crs)
        assert mine.read_bytes() == ref.read_bytes()
    got, step = A.read_ply(str(tmp_path / "ref0"), **crs)
    want, step_r = ref_lib.load_gaussians(tmp_path / "ref0", **crs)
    assert step == step_r == 7000 and got[0].shape[0] == 496
    for a, b in zip(got, want):
        assert a.tobytes() == b.tobytes()


@needs_reference
def test_live_checkpoint_files(ref_lib, tmp_path):
    """The library's checkpoint writer (msplat_write_checkpoint, the
    trainer's save code) against the reference's Model::saveCheckpoint:
    byte-identical files; and each side's reader on the other's file
    (msplat_read_checkpoint with its validation, Model::loadCheckpoint):
    the same iteration, Adam step, learning rates, parameters and moments."""
    from msplat_gb300 import api as A
    rng = np.random.default_rng(8)
    n = 257
    params = file_gaussians(n, 8)
    params[0][7, 1] = 1.0          # a checkpoint keeps every Gaussian, finite or not; keep these finite
    params[4][11, 3, 2] = 0.5
    params[5][19] = -3.0
    params[3][23, 0] = 0.25
    ea = [np.abs(rng.normal(0, 1e-3, a.shape)).astype(np.float32) for a in params]
    eas = [np.abs(rng.normal(0, 1e-6, a.shape)).astype(np.float32) for a in params]
    lr = np.array([1.3e-4, 5e-3, 1e-3, 2.5e-3, 1.25e-4, 5e-2], np.float32)
    mine, ref = tmp_path / "mine.ckpt", tmp_path / "ref.ckpt"
    A.write_checkpoint(str(mine), 4321, params, ea, eas, 4321, lr)
    ref_lib.save_checkpoint(ref, 4321, params, ea, eas, 4321, lr)
    assert mine.read_bytes() == ref.read_bytes()
    for got in (A.read_checkpoint(str(ref)), ref_lib.load_checkpoint(mine)):
        it, steps, lrs, p, m1, m2 = got
        assert (it, steps) == (4321, 4321)
        assert np.array_equal(lrs, np.concatenate([lr, np.float32([0.00016, 0.0000016])]))
        for a, b in zip(p + m1 + m2, params + ea + eas):
            assert a.tobytes() == np.ascontiguousarray(b, np.float32).reshape(a.shape).tobytes()


def _compare_dataset(ref_lib, root, fmt, n):
    """The reference's loader (fmt) and the library's msplat_dataset_create
    on one directory: the same n cameras in the same order, identical sizes,
    intrinsics and camera-to-world poses, the same centred, scaled points."""
    import ctypes as C
    from msplat_gb300 import api as A
    cams, (xyz, rgb), _ = ref_lib.load_colmap(root, fmt)
    ds = A.Dataset(str(root))
    L = A._lib()
    assert ds.num_train == len(cams) == n
    for i, c in enumerate(cams):
        intr, size, c2w = np.zeros(4, np.float32), np.zeros(2, np.int32), np.zeros(16, np.float32)
        img = np.zeros((c["size"][1], c["size"][0], 3), np.uint8)
        assert L.msplat_dataset_camera(ds.h, i, 0, intr.ctypes.data_as(C.POINTER(C.c_float)),
                                       size.ctypes.data_as(C.POINTER(C.c_int)),
                                       c2w.ctypes.data_as(C.POINTER(C.c_float)),
                                       img.ctypes.data_as(C.POINTER(C.c_uint8))) == 0
        assert tuple(size) == c["size"], i
        assert np.array_equal(intr, c["intr"]), (i, intr, c["intr"])
        assert np.array_equal(c2w, c["c2w"].ravel()), (i, c2w - c["c2w"].ravel())
    pts, cols = np.zeros_like(xyz), np.zeros_like(rgb)
    assert L.msplat_dataset_points(ds.h, pts.ctypes.data_as(C.POINTER(C.c_float)),
                                   cols.ctypes.data_as(C.POINTER(C.c_uint8))) == len(xyz)
    assert np.array_equal(pts, xyz) and np.array_equal(cols, rgb)


def _write_image(path, w, h, rng):
    from test_dataset_io import write_png
    img = rng.integers(0, 256, (h, w, 3), dtype=np.uint8)
    write_png(path, [img[y].tobytes() for y in range(h)], 2, 8)


@needs_reference
def test_live_nerfstudio_loader(ref_lib, tmp_path):
    """The reference's loadNerfstudio (nlohmann's calls answered by
    oracle/json_shim.h) against the library's loader on a transforms.json
    with global intrinsics, per-frame overrides, frames listed unsorted,
    file paths with and without extensions and long decimal poses."""
    import json
    from test_dataset_io import _pose, _write_ply_points
    rng = np.random.default_rng(5)
    os.makedirs(tmp_path / "images")
    frames = []
    for k in rng.permutation(9):
        a = rng.uniform(0, 2 * np.pi)
        eye = (rng.uniform(3, 6) * np.cos(a), rng.uniform(3, 6) * np.sin(a), rng.uniform(-1, 2))
        fr = {"file_path": f"images/v{k}" + (".png" if k % 2 else ""),
              "transform_matrix": [[float(v) for v in row] for row in _pose(eye)]}
        w, h = 32, 24
        if k % 3 == 0:
            fr.update({"w": 40, "h": 20, "fl_x": 27.123456789, "fl_y": 21.5, "cx": 20.25, "cy": 10})
            w, h = 40, 20
        _write_image(tmp_path / "images" / f"v{k}.png", w, h, rng)
        frames.append(fr)
    json.dump({"w": 32, "h": 24, "fl_x": 30.0, "fl_y": 31.7, "cx": 16.0, "cy": 12.0, "frames": frames,
               "ply_file_path": "points.ply"}, open(tmp_path / "transforms.json", "w"))
    _write_ply_points(tmp_path / "points.ply", rng.normal(0, 1.3, (80, 3)).astype(np.float32),
                      rng.integers(0, 256, (80, 3), dtype=np.uint8))
    _compare_dataset(ref_lib, tmp_path, "nerfstudio", 9)


@needs_reference
@pytest.mark.parametrize("layout", [1, 2])
def test_live_polycam_loader(ref_lib, tmp_path, layout):
    """The reference's loadPolycam against the library's loader: layout 1
    (one JSON per keyframe with R_ij, t_2j and intrinsics, cx/cy defaulted
    on some) and layout 2 (one cameras.json of frames with 4x4 matrices)."""
    import json
    from test_dataset_io import _pose, _write_ply_points
    rng = np.random.default_rng(6 + layout)
    poses = []
    for k in range(7):
        a = rng.uniform(0, 2 * np.pi)
        poses.append(_pose((rng.uniform(3, 6) * np.cos(a), rng.uniform(3, 6) * np.sin(a), rng.uniform(-1, 2))))
    if layout == 1:
        kd, idir = tmp_path / "keyframes" / "corrected_cameras", tmp_path / "keyframes" / "corrected_images"
        os.makedirs(kd)
        os.makedirs(idir)
        for k, c2w in enumerate(poses):
            R, t = c2w[:3, :3].copy(), c2w[:3, 3].copy()
            R[1:] *= -1
            t[1:] *= -1
            d = {"width": 32, "height": 24, "fx": 30.0 + k / 7.0, "fy": 29.5}
            if k % 2:
                d.update({"cx": 15.75, "cy": 12.5})
            d.update({"t_20": float(t[0]), "t_21": float(t[1]), "t_22": float(t[2])})
            d.update({f"R_{a}{b}": float(R[a, b]) for a in range(3) for b in range(3)})
            json.dump(d, open(kd / f"{k:03d}.json", "w"))
            _write_image(idir / f"{k:03d}.png", 32, 24, rng)
        ply = tmp_path / "keyframes" / "point_cloud.ply"
    else:
        os.makedirs(tmp_path / "images")
        frames = []
        for k, c2w in enumerate(poses):
            frames.append({"width": 32, "height": 24, "fx": 30.0, "fy": 30.0 + k, "cx": 16.0, "cy": 12.0,
                           "transform_matrix": [[float(v) for v in row] for row in c2w],
                           "file_path": f"images/p{k}.png"})
            _write_image(tmp_path / "images" / f"p{k}.png", 32, 24, rng)
        json.dump({"frames": frames}, open(tmp_path / "cameras.json", "w"))
        ply = tmp_path / "point_cloud.ply"
    _write_ply_points(ply, rng.normal(0, 1.3, (60, 3)).astype(np.float32), rng.integers(0, 256, (60, 3), dtype=np.uint8))
    _compare_dataset(ref_lib, tmp_path, "polycam", 7)


# ---- seed initialisation (model.cpp:80-254, kdtree_tensor.hpp) ----

SEED_CASES = {
    # points, cap, options: defaults; seed decimation (points above 75 % of the cap);
    # decimation off (truncation to the cap); other opacity and scale multiplier, SH degree 1
    "default": (1500, 100_000, {}, 3),
    "decimated": (1500, 1800, {}, 3),
    "truncated": (1500, 1200, {"seed_decimation": False}, 3),
    "options": (900, 100_000, {"init_opacity": 0.1, "init_scale_mult": 1.0}, 1),
}


@needs_reference
@pytest.mark.parametrize("name", list(SEED_CASES))
def test_live_seed_initialisation(ref_lib, name):
    """The reference's Model::Model and setupOptimizers (its nanoflann
    k-nearest query answered by a brute-force stand-in with nanoflann's
    metric) against the library's seed initialisation (msplat_seed_gaussians,
    the trainer's own code, with its grid search): identical Gaussians in use
    (KNN scales, mt19937 quaternions, DC from colours, opacity logits,
    decimation or truncation), duplicate points included."""
    from msplat_gb300 import api as A
    n, cap, opts, deg = SEED_CASES[name]
    rng = np.random.default_rng(len(name))
    xyz = rng.normal(0, 2.0, (n, 3)).astype(np.float32)
    xyz[10:14] = xyz[3]                              # duplicates: distance 0 counts
    xyz[50:60] *= np.float32(40.0)                   # far-out points: sparse neighbourhoods
    rgb = rng.integers(0, 256, (n, 3), dtype=np.uint8)
    o = A.TrainerOptions(**opts)
    mine = A.seed_gaussians(xyz, rgb, sh_degree=deg, cap_max=cap, options=o)
    ref = ref_lib.seed_model(xyz, rgb, sh_degree=deg, cap_max=cap, init_opacity=o.init_opacity,
                             init_scale_mult=o.init_scale_mult, decimate=o.seed_decimation)
    want_rows = {"default": n, "decimated": cap // 2, "truncated": cap, "options": n}[name]
    assert mine[0].shape[0] == ref[0].shape[0] == want_rows
    for k, a, b in zip(GROUPS, mine, ref):
        assert a.tobytes() == b.reshape(a.shape).tobytes(), (k, np.abs(a - b.reshape(a.shape)).max())


@needs_reference
def test_live_resize_area(ref_lib):
    """The reference's resizeArea (loaders/image_io.cpp:115-161) against the
    library's (msplat_image_resize: the dataset's --downscale-factor and the
    training masks' resize): identical floats for downscales by integer and
    fractional factors and for upscales."""
    import ctypes as C
    from msplat_gb300 import build
    lib = C.CDLL(build.build())
    fp = C.POINTER(C.c_float)
    lib.msplat_image_resize.argtypes = [fp, C.c_int, C.c_int, C.c_int, C.c_int, fp]
    L = ref_lib.lib()
    L.ref_resize_area.argtypes = [fp, C.c_int, C.c_int, C.c_int, C.c_int, fp]
    rng = np.random.default_rng(13)
    img = (rng.integers(0, 256, (37, 53, 3)) / np.float32(255.0)).astype(np.float32)
    for dw, dh in ((26, 18), (17, 12), (53, 37), (20, 30), (106, 74), (7, 5)):
        a = np.zeros((dh, dw, 3), np.float32)
        b = np.zeros_like(a)
        assert lib.msplat_image_resize(img.ctypes.data_as(fp), 53, 37, dw, dh, a.ctypes.data_as(fp)) == 0
        L.ref_resize_area(img.ctypes.data_as(fp), 53, 37, dw, dh, b.ctypes.data_as(fp))
        assert a.tobytes() == b.tobytes(), (dw, dh, np.abs(a - b).max())


@needs_reference
def test_live_camera_selection(ref_lib, tmp_path):
    """The reference's InputData::getCameras (--val: mt19937(42) pick or
    file-name match) and splitTrainTest (--eval) against the library's
    msplat_dataset_hold_out and eval split, on 11 cameras."""
    import ctypes as C
    import json
    from msplat_gb300 import api as A
    from test_dataset_io import _pose, _write_ply_points
    rng = np.random.default_rng(2)
    os.makedirs(tmp_path / "images")
    frames = []
    n = 11
    for k in range(n):
        _write_image(tmp_path / "images" / f"cam{k:02d}.png", 16, 12, rng)
        a = 2 * np.pi * k / n
        frames.append({"file_path": f"images/cam{k:02d}.png", "transform_matrix": _pose((4 * np.cos(a), 4 * np.sin(a), 1.0)).tolist()})
    json.dump({"w": 16, "h": 12, "fl_x": 15.0, "fl_y": 15.0, "cx": 8.0, "cy": 6.0, "frames": frames,
               "ply_file_path": "p.ply"}, open(tmp_path / "transforms.json", "w"))
    _write_ply_points(tmp_path / "p.ply", rng.normal(0, 1, (20, 3)).astype(np.float32),
                      rng.integers(0, 256, (20, 3), dtype=np.uint8))
    paths = [str(tmp_path / "images" / f"cam{k:02d}.png").encode() for k in range(n)]
    L = ref_lib.lib()
    arr = (C.c_char_p * n)(*paths)
    for pick in ("random", "cam07", "no_such_name"):
        want = L.ref_val_camera(n, arr, 1, pick.encode())
        assert A.Dataset(str(tmp_path)).hold_out(pick) == want
    for every in (1, 3, 8):
        test = np.zeros(n, np.int32)
        L.ref_split_train_test(n, every, test.ctypes.data_as(C.POINTER(C.c_int)))
        ds = A.Dataset(str(tmp_path), eval_mode=True, test_every=every)
        assert (ds.num_test, ds.num_train) == (int(test.sum()), n - int(test.sum()))
        full = A.Dataset(str(tmp_path))
        imgs = [full.camera(i)["image"].tobytes() for i in range(n)]
        got = sorted(imgs.index(ds.camera(i, use_test=True)["image"].tobytes()) for i in range(ds.num_test))
        assert got == list(np.flatnonzero(test))


@needs_reference
def test_live_mask_loading(ref_lib, tmp_path):
    """The reference's Camera::loadMask (its image decoding replaced by an
    8-bit PGM reader; both sides then see the same pixels) against the
    library's --mask-dir loading: the same lookup (appended, then swapped
    name), area resize to the camera, > 0.5 threshold and all-white rule,
    masks and contributing counts identical."""
    import ctypes as C
    from msplat_gb300 import api as A
    write_colmap_scene(tmp_path, 9)
    md = tmp_path / "masks"
    os.makedirs(md)
    rng = np.random.default_rng(9)
    cams, _, _ = ref_lib.load_colmap(tmp_path)

    def pgm(path, m):
        path.write_bytes(b"P5 %d %d 255\n" % (m.shape[1], m.shape[0]) + m.tobytes())

    for i, c in enumerate(cams):
        w, h = c["size"]
        name = c["name"]
        kind = i % 4
        if kind == 0:       # same size, appended name
            pgm(md / (name + ".png"), (rng.random((h, w)) > 0.3).astype(np.uint8) * 255)
        elif kind == 1:     # other size, swapped name
            pgm(md / (name.rsplit(".", 1)[0] + ".png"), rng.integers(0, 256, (h // 2 + 3, w // 3 + 1), dtype=np.uint8))
        elif kind == 2:     # all white
            pgm(md / (name + ".png"), np.full((h, w), 255, np.uint8))
    ds = A.Dataset(str(tmp_path), mask_dir=str(md))
    L = ref_lib.lib()
    L.ref_load_mask.restype = C.c_longlong
    for i, c in enumerate(cams):
        w, h = c["size"]
        ref = np.zeros((h, w), np.uint8)
        n = L.ref_load_mask(str(md).encode(), c["name"].encode(), w, h, ref.ctypes.data_as(C.POINTER(C.c_uint8)))
        mine = ds.mask(i)
        if n < 0:
            assert mine is None, i
        else:
            assert mine is not None and np.array_equal(mine, ref) and int((mine > 0).sum()) == n, i
