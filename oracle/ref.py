"""ctypes front end of oracle/_ref/libmsplat_ref.so — TEST INFRASTRUCTURE ONLY.

The library is the reference's own Metal source for the per-Gaussian stages
(projection + SH, projection backward + SH Adam, Adam, SGLD, regularizer,
tile rectangle, sort key, active test, SSIM window) and the pixel stages
(count, tile scan, scatter, per-tile sort + pack, monolithic and chunked
rasterizers forward and backward, SSIM + L1 loss), and its host code on the
path (camera setup, the MCMC relocation and growth pass, evaluation
metrics), compiled as host C++ by oracle/ref_build.py from the reference
tree (threadgroups on host threads).  It exists only where the
reference tree does (the build container); the GPU machine never has it.  Only
tests/ and tests/golden/make_ref_vectors.py use it, to pin the oracle.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libmsplat_ref.so")
REFERENCE = os.environ.get("MSPLAT_REFERENCE", "/root/reference")

FP = C.POINTER(C.c_float)
IP = C.POINTER(C.c_int)
UP = C.POINTER(C.c_uint32)
_lib = None


def available() -> bool:
    return os.path.exists(os.path.join(REFERENCE, "core", "metal", "msplat_metal.metal"))


def lib():
    """Build (from the reference tree) and load the library."""
    global _lib
    if _lib is None:
        from oracle import ref_build
        ref_build.build(REFERENCE, quiet=True)
        _lib = C.CDLL(LIB_PATH)
    return _lib


def _p(a, t=FP):
    return None if a is None else a.ctypes.data_as(t)


def set_expf(fn_ptr):
    """exp() of the compiled source: a C function pointer float(float), or None for libm."""
    L = lib()
    L.ref_set_expf.argtypes = [C.c_void_p]
    L.ref_set_expf(fn_ptr)


def project_fwd(g, cam, degrees_to_use, clip=0.01):
    """Projection + SH colour (project_and_sh_forward_kernel); outputs of culled
    Gaussians stay zero."""
    n = g.n
    o = {"xys": np.zeros((n, 2), np.float32), "depths": np.zeros(n, np.float32), "radii": np.zeros(n, np.int32),
         "conics": np.zeros((n, 3), np.float32), "num_tiles_hit": np.zeros(n, np.int32),
         "colors": np.zeros((n, 3), np.float32), "aabb": np.zeros((n, 2), np.float32),
         "nan_counts": np.zeros(16, np.uint32), "backward_ran": np.zeros(1, np.int32)}
    deg = {0: 0, 3: 1, 8: 2, 15: 3}[g.features_rest.shape[1]]
    cp = np.asarray(cam["cam_pos"], np.float32)
    vm = np.ascontiguousarray(cam["viewmat"], np.float32).ravel()
    pm = np.ascontiguousarray(cam["projmat"], np.float32).ravel()
    lib().ref_project_fwd(
        n, _p(g.means), _p(g.scales), _p(g.quats), _p(vm), _p(pm), C.c_float(cam["fx"]), C.c_float(cam["fy"]),
        C.c_float(cam["cx"]), C.c_float(cam["cy"]), int(cam["width"]), int(cam["height"]), C.c_float(clip), deg,
        int(degrees_to_use), _p(cp), _p(g.features_dc), _p(g.features_rest), _p(o["xys"]), _p(o["depths"]),
        _p(o["radii"], IP), _p(o["conics"]), _p(o["num_tiles_hit"], IP), _p(o["colors"]), _p(o["aabb"]),
        _p(o["nan_counts"], UP))
    return o


def step_after_raster(g, mom, cam, step, raster_grads, fwd, do_sgld=True):
    """The reference's per-Gaussian work after the rasterizer backward, in the
    host's order (core/src/model.cpp:901-975): projection backward with the
    fused SH Adam, regularizer gradient, Adam on means/scales/quats/opacity,
    SGLD.  g and mom (exp_avg[6], exp_avg_sq[6]) are updated in place.
    raster_grads: [N, 9] (v_xy 2, v_conic 3, v_colors 3, v_opacity 1)."""
    L = lib()
    n = g.n
    rg = np.ascontiguousarray(raster_grads, np.float32).reshape(n, 9)
    v_xy = np.ascontiguousarray(rg[:, 0:2])
    v_conic = np.ascontiguousarray(rg[:, 2:5])
    v_col = np.ascontiguousarray(rg[:, 5:8])
    v_op = np.ascontiguousarray(rg[:, 8])
    v_mean = np.zeros((n, 3), np.float32)
    v_scale = np.zeros((n, 3), np.float32)
    v_quat = np.zeros((n, 4), np.float32)
    nan = np.zeros(16, np.uint32)
    deg = {0: 0, 3: 1, 8: 2, 15: 3}[g.features_rest.shape[1]]
    cp = np.asarray(cam["cam_pos"], np.float32)
    vm = np.ascontiguousarray(cam["viewmat"], np.float32).ravel()
    pm = np.ascontiguousarray(cam["projmat"], np.float32).ravel()
    ss, bc = step["step_size"], step["bc2_sqrt"]
    f = C.c_float
    ea, eas = mom
    L.ref_project_bwd(
        n, _p(g.means), _p(g.scales), _p(g.quats), _p(vm), _p(pm), f(cam["fx"]), f(cam["fy"]), f(cam["cx"]),
        f(cam["cy"]), int(cam["width"]), int(cam["height"]), _p(fwd["radii"], IP), _p(fwd["conics"]), _p(v_xy), None,
        _p(v_conic), _p(v_col), deg, int(step["degrees_to_use"]), _p(cp), _p(v_mean), _p(v_scale), _p(v_quat),
        _p(g.features_dc), _p(g.features_rest), _p(ea[3]), _p(eas[3]), _p(ea[4]), _p(eas[4]), f(ss[3]), f(bc[3]),
        f(ss[4]), f(bc[4]), f(step["beta1"]), f(step["beta2"]), f(step["eps"]), _p(nan, UP))
    v_op_total = v_op.copy()
    v_scale_total = v_scale.copy()
    if step.get("op_reg", 0.0) > 0.0 or step.get("sc_reg", 0.0) > 0.0:
        L.ref_reg_grad(n, _p(g.opacities), _p(g.scales), _p(v_op_total), _p(v_scale_total), f(step["op_reg"]),
                       f(step["sc_reg"]), _p(fwd["radii"], IP), f(step.get("invis_scale", 1.0)), _p(eas[3]))
    for grp, grad in ((0, v_mean), (1, v_scale_total), (2, v_quat), (5, v_op_total)):
        p = [g.means, g.scales, g.quats, None, None, g.opacities][grp]
        L.ref_adam(p.size, _p(p), _p(np.ascontiguousarray(grad)), _p(ea[grp]), _p(eas[grp]), f(ss[grp]),
                   f(step["beta1"]), f(step["beta2"]), f(bc[grp]), f(step["eps"]), grp, _p(nan, UP))
    noise = np.zeros((n, 3), np.float32)
    if do_sgld:
        L.ref_sgld(n, _p(g.means), _p(g.scales), _p(g.quats), _p(g.opacities), C.c_uint32(int(step["seed"])),
                   f(step["noise_lr"]), f(step["xyz_lr"]), f(step["max_disp"]), _p(noise))
    return {"v_mean3d": v_mean, "v_scale": v_scale, "v_quat": v_quat, "nan_counts": nan, "noise": noise}


def tile_rects(xys, aabb, width, height):
    n = xys.shape[0]
    r = np.zeros((n, 4), np.int32)
    lib().ref_tile_rect(n, _p(np.ascontiguousarray(xys, np.float32)), _p(np.ascontiguousarray(aabb, np.float32)),
                        int(width), int(height), _p(r, IP))
    return r


def sort_keys(radii, depths):
    n = radii.shape[0]
    act = np.zeros(n, np.uint8)
    keys = np.zeros(n, np.uint64)
    lib().ref_sort_keys(n, _p(np.ascontiguousarray(radii, np.int32), IP), _p(np.ascontiguousarray(depths, np.float32)),
                        act.ctypes.data_as(C.POINTER(C.c_uint8)), keys.ctypes.data_as(C.POINTER(C.c_uint64)))
    return act.astype(bool), keys


def gauss_1d():
    w = np.zeros(11, np.float32)
    lib().ref_gauss_1d(_p(w))
    return w


def raster_step(fwd, opacities, cam, gt=None, mask=None, v_img=None, background=(0.0, 0.0, 0.0), ssim_weight=0.2,
                loss_inv_n=None, ids_capacity=None, k_max=1, chunk_size=512):
    """The pixel stages of one step of one view from the reference's kernels
    (count, tile scan, scatter, per-tile sort + pack, forward raster, SSIM +
    L1 loss, backward raster): lists, image, final transmittance and last
    contributors, loss sum, dL/dimage and the per-Gaussian rasterizer
    gradients.  gt (uint8 [H,W,3]) runs the loss; otherwise v_img is the image
    gradient.  k_max > 1: the chunked rasterizers with k_max chunks of
    chunk_size splats (the caller applies the reference's K rule); the
    chunked backward runs only where it is defined (every 8x8 threadgroup's
    lanes all leave or all stay at its early exit in each chunk), and
    "backward_ran" says whether the gradients were computed."""
    W, H = int(cam["width"]), int(cam["height"])
    n = fwd["radii"].shape[0]
    T = ((W + 15) // 16) * ((H + 15) // 16)
    cap = int(ids_capacity or max(1, 64 * n))
    o = {"tile_bins": np.zeros((T, 2), np.int32), "gaussian_ids": np.zeros(cap, np.int32),
         "out_img": np.zeros((H, W, 3), np.float32), "final_Ts": np.zeros((H, W), np.float32),
         "final_idx": np.zeros((H, W), np.int32), "loss_sum": np.zeros(1, np.float32),
         "v_rendered": np.zeros((H, W, 3), np.float32) if v_img is None else np.ascontiguousarray(v_img, np.float32).copy(),
         "v_xy": np.zeros((n, 2), np.float32), "v_conic": np.zeros((n, 3), np.float32),
         "v_colors": np.zeros((n, 3), np.float32), "v_opacity": np.zeros(n, np.float32),
         "nan_counts": np.zeros(16, np.uint32), "backward_ran": np.zeros(1, np.int32)}
    bg = np.asarray(background, np.float32)
    gt = None if gt is None else np.ascontiguousarray(gt, np.uint8)
    mask = None if mask is None else np.ascontiguousarray(mask, np.uint8)
    u8 = C.POINTER(C.c_uint8)
    L = lib()
    L.ref_raster_step.restype = C.c_longlong
    m = L.ref_raster_step(
        n, _p(fwd["xys"]), _p(fwd["depths"]), _p(fwd["radii"], IP), _p(fwd["conics"]), _p(fwd["colors"]),
        _p(fwd["aabb"]), _p(np.ascontiguousarray(opacities, np.float32).reshape(-1)), W, H, _p(bg),
        None if gt is None else gt.ctypes.data_as(u8), None if mask is None else mask.ctypes.data_as(u8),
        C.c_float(ssim_weight), C.c_float(loss_inv_n if loss_inv_n is not None else 1.0 / (3.0 * W * H)),
        _p(o["tile_bins"], IP), _p(o["gaussian_ids"], IP), C.c_longlong(cap), _p(o["out_img"]), _p(o["final_Ts"]),
        _p(o["final_idx"], IP), _p(o["loss_sum"]), _p(o["v_rendered"]), _p(o["v_xy"]), _p(o["v_conic"]),
        _p(o["v_colors"]), _p(o["v_opacity"]), _p(o["nan_counts"], UP), int(k_max), int(chunk_size),
        _p(o["backward_ran"], IP))
    if m < 0:
        raise RuntimeError("more intersections than ids_capacity")
    o["num_isect"] = int(m)
    o["backward_ran"] = bool(o["backward_ran"][0])
    o["gaussian_ids"] = o["gaussian_ids"][:m].copy()
    o["loss"] = float(o["loss_sum"][0]) / (W * H)
    o["raster_grads"] = np.concatenate([o["v_xy"], o["v_conic"], o["v_colors"], o["v_opacity"][:, None]], axis=1)
    return o


def mcmc_after_train(g, moments, num_active, step, max_steps, cull_radius, reloc_count=0):
    """One pass of the reference's Model::mcmcAfterTrain (model.cpp:497-660,
    compiled unchanged) over g (a GaussianSet of cap rows, the first
    num_active in use) and moments (exp_avg[6], exp_avg_sq[6], the same
    shapes), both updated in place: dead Gaussians relocated onto alive ones
    and growth toward the cap, with the reference's own draws
    (std::discrete_distribution over mt19937).  Returns (num_active,
    reloc_count) after the pass."""
    L = lib()
    arrays = g.arrays()
    for a in list(arrays) + list(moments[0]) + list(moments[1]):
        assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]
    cap = arrays[0].shape[0]
    strides = np.array([a.size // a.shape[0] for a in arrays], np.int32)
    ea = (FP * 6)(*[_p(a) for a in moments[0]])
    eas = (FP * 6)(*[_p(a) for a in moments[1]])
    rc = C.c_int(int(reloc_count))
    L.ref_mcmc_after_train.restype = C.c_int
    n = L.ref_mcmc_after_train(cap, int(num_active), int(strides[4]), *[_p(a) for a in arrays], ea, eas,
                               _p(strides, IP), int(step), int(max_steps), C.c_float(cull_radius), C.byref(rc))
    return int(n), int(rc.value)


def prepare_cam(c2w, width, height, fx, fy, cx, cy, step=0, sh_degree=3, sh_interval=1000, rest_bases=15):
    """The reference's Model::prepareCam (model.cpp:845-889, compiled
    unchanged): view matrix, projection-view matrix, camera centre and
    (width, height, SH degree, degrees to use, tiles across, tiles down)."""
    L = lib()
    c2w = np.ascontiguousarray(c2w, np.float32).reshape(16)
    vm, pvm, cp = np.zeros(16, np.float32), np.zeros(16, np.float32), np.zeros(3, np.float32)
    ints = np.zeros(6, np.int32)
    L.ref_prepare_cam(_p(c2w), int(width), int(height), C.c_float(fx), C.c_float(fy), C.c_float(cx),
                      C.c_float(cy), int(step), int(sh_degree), int(sh_interval), int(rest_bases), _p(vm), _p(pvm),
                      _p(cp), _p(ints, IP))
    return vm, pvm, cp, tuple(int(v) for v in ints)


def metrics(img, gt):
    """The reference's evaluation metrics (psnr, l1_loss: model.cpp:33-49;
    ssim_eval: ssim.cpp:61-123, window 11, sigma 1.5) of two [H, W, 3]
    float32 images."""
    L = lib()
    img = np.ascontiguousarray(img, np.float32)
    gt = np.ascontiguousarray(gt, np.float32)
    h, w = img.shape[:2]
    out = []
    for name in ("ref_psnr", "ref_l1", "ref_ssim_eval"):
        f = getattr(L, name)
        f.restype = C.c_float
        out.append(float(np.float32(f(_p(img), _p(gt), h, w))))
    return tuple(out)


def load_colmap(root, fmt="colmap"):
    """The reference's loaders::loadColmap (load_colmap.cpp), or with fmt
    "nerfstudio" / "polycam" loadNerfstudio / loadPolycam (compiled
    unchanged) of a dataset directory: a list of cameras (dicts with c2w
    [4,4], intr (fx, fy, cx, cy), size (w, h), dist (k1, k2, k3, p1, p2),
    name) in its order, the point cloud (xyz, rgb) after its centring and
    scaling, and (scale, translation)."""
    L = lib()
    L.ref_dataset_load.restype = C.c_void_p
    h = L.ref_dataset_load(str(root).encode(), {"colmap": 0, "nerfstudio": 1, "polycam": 2}[fmt])
    if not h:
        raise RuntimeError(f"the reference's loader rejected {root}")
    h = C.c_void_p(h)
    try:
        cams = []
        for i in range(L.ref_colmap_num_cameras(h)):
            c2w, intr = np.zeros(16, np.float32), np.zeros(4, np.float32)
            size, dist = np.zeros(2, np.int32), np.zeros(5, np.float32)
            name = C.create_string_buffer(512)
            L.ref_colmap_camera(h, i, _p(c2w), _p(intr), _p(size, IP), _p(dist), name, 512)
            cams.append(dict(c2w=c2w.reshape(4, 4), intr=intr, size=tuple(int(v) for v in size), dist=dist,
                             name=name.value.decode()))
        L.ref_colmap_points.restype = C.c_longlong
        n = L.ref_colmap_points(h, None, None)
        xyz, rgb = np.zeros((n, 3), np.float32), np.zeros((n, 3), np.uint8)
        L.ref_colmap_points(h, _p(xyz), rgb.ctypes.data_as(C.POINTER(C.c_uint8)))
        scale, tr = C.c_float(), np.zeros(3, np.float32)
        L.ref_colmap_transform(h, C.byref(scale), _p(tr))
        return cams, (xyz, rgb), (float(scale.value), tr)
    finally:
        L.ref_colmap_free(h)


def save_gaussians(path, arrays, splat=False, step=0, keep_crs=False, scale=1.0, translation=(0.0, 0.0, 0.0)):
    """The reference's saveGaussianPly, or saveGaussianSplat with splat
    (save_gaussians.cpp:10-139, compiled unchanged), of host arrays (means,
    scales, quats, features_dc, features_rest [n, R, 3], opacities)."""
    L = lib()
    a = [np.ascontiguousarray(x, np.float32) for x in arrays]
    n = a[0].shape[0]
    rest = a[4].reshape(n, -1, 3).shape[1]
    t = np.asarray(translation, np.float32)
    L.ref_save_gaussians(str(path).encode(), int(splat), n, rest, *[_p(x) for x in a], int(step), int(keep_crs),
                         C.c_float(scale), _p(t))


def load_gaussians(path, keep_crs=False, scale=1.0, translation=(0.0, 0.0, 0.0)):
    """The reference's loadGaussianPly (save_gaussians.cpp:141-231):
    ([means, scales, quats, features_dc, features_rest [n, R, 3],
    opacities], iteration)."""
    L = lib()
    t = np.asarray(translation, np.float32)
    L.ref_load_gaussians.restype = C.c_void_p
    h = L.ref_load_gaussians(str(path).encode(), C.c_float(scale), _p(t), int(keep_crs))
    if not h:
        raise RuntimeError(f"the reference's loader rejected {path}")
    h = C.c_void_p(h)
    try:
        info = np.zeros(3, np.int32)
        L.ref_loaded_info(h, _p(info, IP))
        n, rest, step = (int(v) for v in info)
        arrs = [np.zeros(s, np.float32) for s in ((n, 3), (n, 3), (n, 4), (n, 3), (n, rest, 3), (n,))]
        L.ref_loaded_arrays(h, *[_p(x) for x in arrs])
        return arrs, step
    finally:
        L.ref_loaded_free(h)


def save_checkpoint(path, step, params, exp_avg, exp_avg_sq, adam_steps, adam_lr, means_lr=(0.00016, 0.0000016),
                    sh_degree=3):
    """The reference's Model::saveCheckpoint (model.cpp:725-764, compiled
    unchanged) of a model in host arrays (six groups each of parameters and
    Adam moments in the C API's layouts)."""
    L = lib()
    n = int(np.asarray(params[0]).shape[0])
    keep = [[np.ascontiguousarray(a, np.float32) for a in grp] for grp in (params, exp_avg, exp_avg_sq)]
    ptrs = [(FP * 6)(*[_p(a) for a in grp]) for grp in keep]
    lr = np.asarray(adam_lr, np.float32)
    L.ref_save_checkpoint(str(path).encode(), int(step), n, int(sh_degree), int(adam_steps), _p(lr),
                          C.c_float(means_lr[0]), C.c_float(means_lr[1]), *ptrs)


def load_checkpoint(path):
    """The reference's Model::loadCheckpoint (model.cpp:766-843): (step, Adam
    step, learning rates [8], params [6], exp_avg [6], exp_avg_sq [6])."""
    L = lib()
    L.ref_load_checkpoint.restype = C.c_void_p
    h = L.ref_load_checkpoint(str(path).encode())
    if not h:
        raise RuntimeError(f"the reference's loader rejected {path}")
    h = C.c_void_p(h)
    try:
        ints, lr = np.zeros(4, np.int32), np.zeros(8, np.float32)
        L.ref_checkpoint_state(h, _p(ints, IP), _p(lr))
        step, n, adam_steps, rest = (int(v) for v in ints)
        shapes = [(n, 3), (n, 3), (n, 4), (n, 3), (n, rest, 3), (n,)]
        grps = [[np.zeros(s, np.float32) for s in shapes] for _ in range(3)]
        L.ref_checkpoint_arrays(h, *[(FP * 6)(*[_p(a) for a in g]) for g in grps])
        return step, adam_steps, lr, grps[0], grps[1], grps[2]
    finally:
        L.ref_checkpoint_free(h)


def seed_model(xyz, rgb, sh_degree=3, cap_max=1_000_000, init_opacity=0.5, init_scale_mult=0.1, decimate=True):
    """The reference's seed initialisation (Model::Model and
    setupOptimizers, model.cpp:80-254, compiled unchanged; its k-nearest
    query answered by oracle/nanoflann_shim.h): the Gaussians in use
    [means, scales, quats, features_dc, features_rest, opacities]."""
    L = lib()
    xyz = np.ascontiguousarray(xyz, np.float32)
    rgb = np.ascontiguousarray(rgb, np.uint8)
    n = xyz.shape[0]
    rest = (sh_degree + 1) ** 2 - 1
    arrs = [np.zeros(s, np.float32) for s in ((n, 3), (n, 3), (n, 4), (n, 3), (n, rest, 3), (n,))]
    L.ref_seed_model.restype = C.c_int
    rows = L.ref_seed_model(n, _p(xyz), rgb.ctypes.data_as(C.POINTER(C.c_uint8)), int(sh_degree), int(cap_max),
                            C.c_float(init_opacity), C.c_float(init_scale_mult), int(decimate), *[_p(a) for a in arrs])
    return [a[:rows] for a in arrs]
