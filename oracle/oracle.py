"""ctypes front end of the CPU oracle — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import
this module.  The oracle restates the msplat training step (see
msplat_oracle.h for what it follows and how far it is pinned).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmsplat_oracle.so")
_lock = threading.Lock()
_lib = None

FP = C.POINTER(C.c_float)
IP = C.POINTER(C.c_int)
U8P = C.POINTER(C.c_uint8)


class OrStepIn(C.Structure):
    _fields_ = [
        ("num_points", C.c_int), ("rest_bases", C.c_int), ("width", C.c_int), ("height", C.c_int),
        ("viewmat", C.c_float * 16), ("projmat", C.c_float * 16),
        ("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float),
        ("cam_pos", C.c_float * 3), ("background", C.c_float * 3),
        ("clip_thresh", C.c_float), ("degrees_to_use", C.c_int),
        ("means", FP), ("scales", FP), ("quats", FP), ("features_dc", FP), ("features_rest", FP),
        ("opacities", FP),
        ("exp_avg", FP * 6), ("exp_avg_sq", FP * 6),
        ("step_size", C.c_float * 6), ("bc2_sqrt", C.c_float * 6),
        ("beta1", C.c_float), ("beta2", C.c_float), ("eps", C.c_float),
        ("op_reg", C.c_float), ("sc_reg", C.c_float), ("invis_scale", C.c_float),
        ("gt", U8P), ("mask", U8P), ("ssim_weight", C.c_float), ("loss_inv_n", C.c_float),
        ("raster_mode", C.c_int), ("k_max", C.c_int), ("isect_capacity", C.c_longlong),
        ("do_sgld", C.c_int), ("seed", C.c_uint32), ("noise_lr", C.c_float), ("xyz_lr", C.c_float),
        ("max_disp", C.c_float),
        ("do_backward", C.c_int), ("do_optimizer", C.c_int), ("no_cutoff", C.c_int),
        ("v_img_in", FP),
        ("tile_row_lo", C.c_int), ("tile_row_hi", C.c_int),
        ("raster_grads_in", FP),
    ]


class OrStepOut(C.Structure):
    _fields_ = [
        ("xys", FP), ("depths", FP), ("conics", FP), ("colors", FP), ("aabb", FP),
        ("radii", IP), ("num_tiles_hit", IP),
        ("tile_counts", IP), ("tile_bins", IP), ("gaussian_ids", IP),
        ("ids_capacity", C.c_longlong), ("num_isect", C.c_longlong),
        ("out_img", FP), ("final_Ts", FP), ("final_idx", IP),
        ("loss", C.c_double), ("v_rendered", FP),
        ("v_xy", FP), ("v_conic", FP), ("v_colors", FP), ("v_opacity", FP),
        ("v_mean3d", FP), ("v_scale", FP), ("v_quat", FP),
        ("nan_counts", C.c_uint32 * 16), ("k_max_used", C.c_int),
        ("pairs_fwd", C.c_longlong), ("pairs_bwd", C.c_longlong), ("img_dot_v", C.c_double),
    ]


def build(force: bool = False) -> str:
    """Compile the oracle (make) if the library is missing or stale."""
    src = [os.path.join(HERE, f) for f in ("msplat_oracle.cpp", "msplat_oracle.h")]
    stale = not os.path.exists(LIB_PATH) or any(os.path.getmtime(s) > os.path.getmtime(LIB_PATH) for s in src)
    if force or stale:
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(LIB_PATH)
            L.or_train_step.argtypes = [C.c_int, C.POINTER(OrStepIn), C.POINTER(OrStepOut)]
            L.or_train_step.restype = C.c_int
            L.or_det_expf.argtypes = [C.c_float]
            L.or_det_expf.restype = C.c_float
            L.or_gauss_1d.argtypes = [FP]
            L.or_compute_relocation.argtypes = [C.c_float, FP, C.c_int, FP, FP]
            L.or_prepare_cam.argtypes = [FP, C.c_int, C.c_int, C.c_float, C.c_float, FP, FP, FP]
            for n in ("or_psnr", "or_l1"):
                getattr(L, n).argtypes = [FP, FP, C.c_longlong]
                getattr(L, n).restype = C.c_double
            L.or_ssim_eval.argtypes = [FP, FP, C.c_int, C.c_int]
            L.or_ssim_eval.restype = C.c_double
            L.or_mcmc_dead_mask.argtypes = [C.c_int, C.c_int, FP, FP, FP, FP, FP, FP, C.c_float, U8P]
            L.or_mcmc_dead_mask.restype = C.c_int
            L.or_mcmc_apply.argtypes = [C.c_int, IP, IP, C.c_int, FP, FP, FP, FP, FP, FP,
                                        C.POINTER(FP), C.POINTER(FP), IP]
            L.or_num_threads.restype = C.c_int
            _lib = L
    return _lib


def _fp(a):
    return a.ctypes.data_as(FP)


def det_expf(x):
    L = lib()
    return np.array([L.or_det_expf(float(v)) for v in np.asarray(x, np.float32).ravel()], np.float32)


def gauss_1d():
    w = np.zeros(11, np.float32)
    lib().or_gauss_1d(_fp(w))
    return w


def compute_relocation(o_old: float, s_old, n: int):
    s_old = np.ascontiguousarray(s_old, np.float32)
    o_new = np.zeros(1, np.float32)
    s_new = np.zeros(3, np.float32)
    lib().or_compute_relocation(C.c_float(o_old), _fp(s_old), n, _fp(o_new), _fp(s_new))
    return float(o_new[0]), s_new


def prepare_cam(c2w, width, height, fx, fy):
    c2w = np.ascontiguousarray(c2w, np.float32).reshape(16)
    vm = np.zeros(16, np.float32)
    pm = np.zeros(16, np.float32)
    cp = np.zeros(3, np.float32)
    lib().or_prepare_cam(_fp(c2w), width, height, fx, fy, _fp(vm), _fp(pm), _fp(cp))
    return vm, pm, cp


def psnr(img, gt):
    img = np.ascontiguousarray(img, np.float32); gt = np.ascontiguousarray(gt, np.float32)
    return lib().or_psnr(_fp(img), _fp(gt), img.size)


def l1(img, gt):
    img = np.ascontiguousarray(img, np.float32); gt = np.ascontiguousarray(gt, np.float32)
    return lib().or_l1(_fp(img), _fp(gt), img.size)


def ssim_eval(img, gt):
    img = np.ascontiguousarray(img, np.float32); gt = np.ascontiguousarray(gt, np.float32)
    return lib().or_ssim_eval(_fp(img), _fp(gt), img.shape[0], img.shape[1])


def num_threads() -> int:
    return lib().or_num_threads()


def train_step(prec: int, g, cam, step, *, moments=None, gt=None, mask=None, background=(0.0, 0.0, 0.0),
               ssim_weight=0.2, do_backward=True, do_optimizer=True, do_sgld=False, raster_mode=0, k_max=0,
               isect_capacity=0, want_ids=True, no_cutoff=False, v_img=None, tile_rows=None, ids_capacity=0,
               raster_grads=None):
    """Run one oracle step.

    g        : GaussianSet, UPDATED IN PLACE when do_optimizer / do_sgld.
    cam      : dict with viewmat, projmat, fx, fy, cx, cy, cam_pos, width, height.
    step     : dict of the per-step scalars (degrees_to_use, step_size[6],
               bc2_sqrt[6], beta1, beta2, eps, op_reg, sc_reg, invis_scale,
               loss_inv_n, seed, noise_lr, xyz_lr, max_disp).
    moments  : (exp_avg[6], exp_avg_sq[6]) float32 arrays, updated in place.
    tile_rows: (lo, hi) or None: only tiles in rows [lo, hi) get lists and
               are rasterized (forward and backward); the rest stay empty.
    ids_capacity: slots of the returned id lists (0: the larger of 48 N and
               isect_capacity).
    raster_grads: [N, 9] float32 or None: per-Gaussian rasterizer gradients
               (v_xy, v_conic, v_colors, v_opacity) used in place of the
               raster backward.
    Returns a dict of numpy outputs.
    """
    L = lib()
    N = g.n
    W, H = int(cam["width"]), int(cam["height"])
    T = ((W + 15) // 16) * ((H + 15) // 16)
    P = W * H
    ins = OrStepIn()
    ins.num_points, ins.rest_bases, ins.width, ins.height = N, g.features_rest.shape[1], W, H
    ins.viewmat[:] = [float(v) for v in np.asarray(cam["viewmat"], np.float32).ravel()]
    ins.projmat[:] = [float(v) for v in np.asarray(cam["projmat"], np.float32).ravel()]
    ins.fx, ins.fy, ins.cx, ins.cy = cam["fx"], cam["fy"], cam["cx"], cam["cy"]
    ins.cam_pos[:] = [float(v) for v in cam["cam_pos"]]
    ins.background[:] = [float(v) for v in background]
    ins.clip_thresh = 0.01
    ins.degrees_to_use = int(step.get("degrees_to_use", 3))
    for name in ("means", "scales", "quats", "features_dc", "features_rest", "opacities"):
        a = getattr(g, name)
        assert a.dtype == np.float32 and a.flags.c_contiguous
        setattr(ins, name, _fp(a))
    if moments is None:
        moments = ([np.zeros_like(a) for a in g.arrays()], [np.zeros_like(a) for a in g.arrays()])
    for k in range(6):
        ins.exp_avg[k] = _fp(moments[0][k])
        ins.exp_avg_sq[k] = _fp(moments[1][k])
    ins.step_size[:] = [float(v) for v in step.get("step_size", [0.0] * 6)]
    ins.bc2_sqrt[:] = [float(v) for v in step.get("bc2_sqrt", [1.0] * 6)]
    ins.beta1, ins.beta2, ins.eps = step.get("beta1", 0.9), step.get("beta2", 0.999), step.get("eps", 1e-8)
    ins.op_reg, ins.sc_reg = step.get("op_reg", 0.0), step.get("sc_reg", 0.0)
    ins.invis_scale = step.get("invis_scale", 1.0)
    keep = []
    if gt is not None:
        gt = np.ascontiguousarray(gt, np.uint8)
        keep.append(gt)
        ins.gt = gt.ctypes.data_as(U8P)
    if mask is not None:
        mask = np.ascontiguousarray(mask, np.uint8)
        keep.append(mask)
        ins.mask = mask.ctypes.data_as(U8P)
    ins.ssim_weight = ssim_weight
    ins.loss_inv_n = step.get("loss_inv_n", 1.0 / (3.0 * P))
    ins.raster_mode, ins.k_max, ins.isect_capacity = raster_mode, k_max, isect_capacity
    ins.do_sgld, ins.seed = int(do_sgld), int(step.get("seed", 0)) & 0xFFFFFFFF
    ins.noise_lr, ins.xyz_lr, ins.max_disp = step.get("noise_lr", 5e5), step.get("xyz_lr", 1.6e-4), step.get("max_disp", 0.05)
    ins.do_backward, ins.do_optimizer = int(do_backward), int(do_optimizer)
    ins.no_cutoff = int(no_cutoff)
    if v_img is not None:
        v_img = np.ascontiguousarray(v_img, np.float32)
        keep.append(v_img)
        ins.v_img_in = _fp(v_img)
    if raster_grads is not None:
        raster_grads = np.ascontiguousarray(raster_grads, np.float32).reshape(N, 9)
        keep.append(raster_grads)
        ins.raster_grads_in = _fp(raster_grads)
    if tile_rows is not None:
        ins.tile_row_lo, ins.tile_row_hi = int(tile_rows[0]), int(tile_rows[1])

    o = {
        "xys": np.zeros((N, 2), np.float32), "depths": np.zeros(N, np.float32), "conics": np.zeros((N, 3), np.float32),
        "colors": np.zeros((N, 3), np.float32), "aabb": np.zeros((N, 2), np.float32),
        "radii": np.zeros(N, np.int32), "num_tiles_hit": np.zeros(N, np.int32),
        "tile_counts": np.zeros(T, np.int32), "tile_bins": np.zeros((T, 2), np.int32),
        "out_img": np.zeros((H, W, 3), np.float32), "final_Ts": np.zeros((H, W), np.float32),
        "final_idx": np.zeros((H, W), np.int32), "v_rendered": np.zeros((H, W, 3), np.float32),
        "v_xy": np.zeros((N, 2), np.float32), "v_conic": np.zeros((N, 3), np.float32),
        "v_colors": np.zeros((N, 3), np.float32), "v_opacity": np.zeros(N, np.float32),
        "v_mean3d": np.zeros((N, 3), np.float32), "v_scale": np.zeros((N, 3), np.float32),
        "v_quat": np.zeros((N, 4), np.float32),
    }
    out = OrStepOut()
    for k, a in o.items():
        setattr(out, k, a.ctypes.data_as(IP if a.dtype == np.int32 else FP))
    ids = None
    if want_ids:
        cap = int(ids_capacity) if ids_capacity > 0 else max(1, 48 * N, int(isect_capacity))
        ids = np.zeros(cap, np.int32)
        out.gaussian_ids = ids.ctypes.data_as(IP)
        out.ids_capacity = cap
    rc = L.or_train_step(prec, C.byref(ins), C.byref(out))
    if rc != 0:
        raise RuntimeError(f"or_train_step failed: {rc}")
    M = int(out.num_isect)
    o["num_isect"] = M
    if ids is not None:
        o["gaussian_ids"] = ids[:M].copy()
    o["loss"] = float(out.loss)
    o["nan_counts"] = np.array(out.nan_counts[:], np.uint32)
    o["k_max"] = int(out.k_max_used)
    o["pairs_fwd"], o["pairs_bwd"] = int(out.pairs_fwd), int(out.pairs_bwd)
    o["img_dot_v"] = float(out.img_dot_v)
    o["moments"] = moments
    return o


def mcmc_dead_mask(g, cull_radius: float):
    d = np.zeros(g.n, np.uint8)
    cnt = lib().or_mcmc_dead_mask(g.n, g.features_rest.shape[1] * 3, _fp(g.means), _fp(g.scales), _fp(g.quats),
                                  _fp(g.features_dc), _fp(g.features_rest), _fp(g.opacities), cull_radius,
                                  d.ctypes.data_as(U8P))
    return d.astype(bool), cnt


def mcmc_apply(g, moments, dst, src):
    """Apply a relocation with given (dst, src) pairs; g/moments are full-capacity arrays (in place)."""
    dst = np.ascontiguousarray(dst, np.int32)
    src = np.ascontiguousarray(src, np.int32)
    ea = (FP * 6)(*[_fp(a) for a in moments[0]])
    eas = (FP * 6)(*[_fp(a) for a in moments[1]])
    strides = np.array([a.size // a.shape[0] for a in g.arrays()], np.int32)
    lib().or_mcmc_apply(len(dst), dst.ctypes.data_as(IP), src.ctypes.data_as(IP), g.features_rest.shape[1] * 3,
                        _fp(g.means), _fp(g.scales), _fp(g.quats), _fp(g.features_dc), _fp(g.features_rest),
                        _fp(g.opacities), ea, eas, strides.ctypes.data_as(IP))
