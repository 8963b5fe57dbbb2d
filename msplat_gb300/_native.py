"""ctypes view of the engine's C ABI (include/msplat_engine.h).

The shared library is built in-tree by msplat_gb300.build; loading fails
loudly when it is missing — there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libmsplat_gb300.so")
_lock = threading.Lock()
_lib = None

FP = C.POINTER(C.c_float)


class MsplatGaussians(C.Structure):
    _fields_ = [("num_points", C.c_int), ("rest_bases", C.c_int),
                ("means", C.c_void_p), ("scales", C.c_void_p), ("quats", C.c_void_p),
                ("features_dc", C.c_void_p), ("features_rest", C.c_void_p), ("opacities", C.c_void_p)]


class MsplatAdamState(C.Structure):
    _fields_ = [("exp_avg", C.c_void_p * 6), ("exp_avg_sq", C.c_void_p * 6)]


class MsplatStepArgs(C.Structure):
    _fields_ = [("viewmat", C.c_float * 16), ("projmat", C.c_float * 16),
                ("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float),
                ("width", C.c_int), ("height", C.c_int),
                ("cam_pos", C.c_float * 3), ("background", C.c_float * 3),
                ("clip_thresh", C.c_float), ("degrees_to_use", C.c_int),
                ("ssim_weight", C.c_float), ("loss_inv_n", C.c_float),
                ("step_size", C.c_float * 6), ("bc2_sqrt", C.c_float * 6),
                ("beta1", C.c_float), ("beta2", C.c_float), ("eps", C.c_float),
                ("op_reg", C.c_float), ("sc_reg", C.c_float), ("invis_scale", C.c_float),
                ("raster_mode", C.c_int), ("k_max", C.c_int), ("do_optimizer", C.c_int), ("do_sgld", C.c_int),
                ("seed", C.c_uint32), ("noise_lr", C.c_float), ("xyz_lr", C.c_float), ("max_disp", C.c_float)]


STAGES = ("project", "tiles", "raster_fwd", "loss", "raster_bwd", "project_bwd", "adam", "sgld")


class MsplatEngineStats(C.Structure):
    _fields_ = [("num_intersections", C.c_longlong), ("max_tile_count", C.c_int), ("k_max", C.c_int),
                ("num_tiles", C.c_int), ("nan_counts", C.c_uint32 * 16), ("stage_ms", C.c_float * len(STAGES)),
                ("timed_steps", C.c_longlong), ("launches", C.c_longlong), ("check_record", C.c_uint32 * 3),
                ("isect_groups", C.c_int)]


class MsplatMcmcStats(C.Structure):
    _fields_ = [("num_dead", C.c_int), ("num_culled", C.c_int), ("num_nonfinite", C.c_int),
                ("num_relocated", C.c_int), ("num_grown", C.c_int), ("num_active", C.c_int)]


class MsplatGradients(C.Structure):
    _fields_ = [("v_means", C.c_void_p), ("v_scales", C.c_void_p), ("v_quats", C.c_void_p),
                ("v_features_dc", C.c_void_p), ("v_features_rest", C.c_void_p), ("v_opacities", C.c_void_p)]


class MsplatTuning(C.Structure):
    """include/msplat_engine.h MsplatTuning"""
    _fields_ = [("sort_width", C.c_int), ("raster_batch", C.c_int), ("chunk", C.c_int), ("raster_mode", C.c_int),
                ("tile_order", C.c_int), ("bwd_pixels", C.c_int), ("tile_split", C.c_int)]


def lib(build_if_missing: bool = True):
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            if not build_if_missing:
                raise RuntimeError(f"msplat_gb300 native library missing: {LIB_PATH}")
            from . import build as _b
            _b.build()
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        L.msplat_engine_create.argtypes = [C.c_int, C.c_int]
        L.msplat_engine_create.restype = vp
        L.msplat_engine_destroy.argtypes = [vp]
        L.msplat_engine_last_error.argtypes = [vp]
        L.msplat_engine_last_error.restype = C.c_char_p
        L.msplat_engine_train_step.argtypes = [vp, C.POINTER(MsplatGaussians), C.POINTER(MsplatAdamState),
                                               C.POINTER(MsplatStepArgs), vp, vp]
        L.msplat_engine_train_step_host.argtypes = [vp, C.POINTER(MsplatGaussians), C.POINTER(MsplatAdamState),
                                                    C.POINTER(MsplatStepArgs), vp, vp]
        L.msplat_engine_render.argtypes = [vp, C.POINTER(MsplatGaussians), C.POINTER(MsplatStepArgs)]
        L.msplat_engine_synchronize.argtypes = [vp]
        L.msplat_engine_loss.argtypes = [vp, FP]
        L.msplat_engine_loss_async.argtypes = [vp, vp]
        L.msplat_engine_stats.argtypes = [vp, C.POINTER(MsplatEngineStats)]
        L.msplat_engine_set_timing.argtypes = [vp, C.c_int]
        L.msplat_engine_buffer.argtypes = [vp, C.c_char_p, C.POINTER(C.c_void_p)]
        L.msplat_engine_buffer.restype = C.c_longlong
        L.msplat_engine_read.argtypes = [vp, C.c_char_p, vp, C.c_longlong]
        L.msplat_engine_mcmc.argtypes = [vp, C.POINTER(MsplatGaussians), C.POINTER(MsplatAdamState), C.c_int,
                                         C.c_float, C.POINTER(C.c_int), C.POINTER(MsplatMcmcStats)]
        L.msplat_engine_marker.argtypes = [vp, C.c_int]
        L.msplat_engine_set_graphs.argtypes = [vp, C.c_int]
        L.msplat_engine_train_step_batch.argtypes = [vp, C.POINTER(MsplatGaussians), C.POINTER(MsplatAdamState),
                                                     C.POINTER(MsplatStepArgs), C.c_int, C.POINTER(vp),
                                                     C.POINTER(vp)]
        L.msplat_engine_backward.argtypes = [vp, C.POINTER(MsplatGaussians), C.POINTER(MsplatStepArgs), vp,
                                             C.POINTER(MsplatGradients)]
        L.msplat_engine_set_isect_budget.argtypes = [vp, C.c_longlong]
        L.msplat_engine_set_tuning.argtypes = [vp, C.POINTER(MsplatTuning)]
        L.msplat_engine_get_tuning.argtypes = [vp, C.POINTER(MsplatTuning)]
        L.msplat_engine_autotune.argtypes = [vp, C.POINTER(MsplatGaussians), C.POINTER(MsplatStepArgs), C.c_int,
                                             C.POINTER(vp), C.POINTER(vp), C.c_int, C.POINTER(MsplatTuning), FP]
        L.msplat_engine_marker_elapsed.argtypes = [vp, FP]
        L.msplat_engine_stream.argtypes = [vp]
        L.msplat_engine_stream.restype = vp
        _lib = L
        return L
