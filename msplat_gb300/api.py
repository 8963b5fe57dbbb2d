"""Python surface of msplat's trainer (the reference's python/msplat/_core.pyi:
TrainingConfig, Dataset, GaussianTrainer, sync, cleanup) over the public C API
of libmsplat_gb300.so.  No torch; images come back as numpy arrays."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _native as N


class _MsplatConfig(C.Structure):
    _fields_ = [("iterations", C.c_int), ("shDegree", C.c_int), ("shDegreeInterval", C.c_int),
                ("ssimWeight", C.c_float), ("capMax", C.c_int), ("noiseLr", C.c_float), ("opacityReg", C.c_float),
                ("scaleReg", C.c_float), ("cullRadius", C.c_float), ("keepCrs", C.c_bool),
                ("downscaleFactor", C.c_float), ("bgColor", C.c_float * 3)]


class _TrainerOptions(C.Structure):
    _fields_ = [("initOpacity", C.c_float), ("initScaleMult", C.c_float), ("seedDecimation", C.c_int),
                ("positionLrMaxSteps", C.c_int), ("regVisibilityDuty", C.c_float)]


class _Stats(C.Structure):
    _fields_ = [("iteration", C.c_int), ("splatCount", C.c_int), ("msPerStep", C.c_float)]


class _Eval(C.Structure):
    _fields_ = [("psnr", C.c_float), ("ssim", C.c_float), ("l1", C.c_float), ("numTest", C.c_int),
                ("numGaussians", C.c_int)]


class _Pixels(C.Structure):
    _fields_ = [("data", C.POINTER(C.c_float)), ("width", C.c_int), ("height", C.c_int)]


_bound = False


def _lib():
    global _bound
    L = N.lib()
    if _bound:
        return L
    vp, cp, fp = C.c_void_p, C.c_char_p, C.POINTER(C.c_float)
    L.msplat_dataset_create.argtypes = [cp, C.c_float, C.c_bool, C.c_int]
    L.msplat_dataset_create.restype = vp
    L.msplat_dataset_create_ex.argtypes = [cp, C.c_float, C.c_bool, C.c_int, cp]
    L.msplat_dataset_create_ex.restype = vp
    L.msplat_dataset_camera.argtypes = [vp, C.c_int, C.c_int, fp, C.POINTER(C.c_int), fp, C.POINTER(C.c_uint8)]
    L.msplat_dataset_points.argtypes = [vp, fp, C.POINTER(C.c_uint8)]
    L.msplat_trainer_load_ply.argtypes = [vp, cp]
    L.msplat_trainer_set_learned_relocation.argtypes = [vp, C.c_int]
    L.msplat_trainer_set_learned_prune.argtypes = [vp, C.c_float]
    L.msplat_trainer_learned_stats.argtypes = [vp, fp, C.POINTER(C.c_int)]
    L.msplat_trainer_learned_eval.argtypes = [vp, fp]
    L.msplat_trainer_set_batch_views.argtypes = [vp, C.c_int, C.c_float]
    L.msplat_trainer_set_isect_budget.argtypes = [vp, C.c_float]
    L.msplat_trainer_autotune.argtypes = [vp, vp]
    L.msplat_dataset_create_from_memory.argtypes = [C.c_int, fp, fp, C.POINTER(C.c_int), C.POINTER(vp),
                                                    C.POINTER(vp), C.c_int, fp, C.POINTER(C.c_uint8), C.c_bool,
                                                    C.c_int, C.c_bool]
    L.msplat_dataset_create_from_memory.restype = vp
    L.msplat_dataset_destroy.argtypes = [vp]
    L.msplat_dataset_num_train.argtypes = [vp]
    L.msplat_dataset_num_test.argtypes = [vp]
    L.msplat_dataset_camera_pose.argtypes = [vp, C.c_int, fp]
    L.msplat_trainer_create.argtypes = [vp, _MsplatConfig]
    L.msplat_trainer_create.restype = vp
    L.msplat_trainer_create_ex.argtypes = [vp, _MsplatConfig, C.POINTER(_TrainerOptions)]
    L.msplat_trainer_create_ex.restype = vp
    L.msplat_default_trainer_options.argtypes = [C.POINTER(_TrainerOptions)]
    L.msplat_seed_gaussians.argtypes = [C.c_int, fp, C.POINTER(C.c_uint8), C.c_int, C.c_int,
                                        C.POINTER(_TrainerOptions), fp, fp, fp, fp, fp, fp]
    L.msplat_trainer_destroy.argtypes = [vp]
    L.msplat_trainer_step.argtypes = [vp]
    L.msplat_trainer_step.restype = _Stats
    L.msplat_trainer_train.argtypes = [vp]
    L.msplat_trainer_evaluate.argtypes = [vp]
    L.msplat_trainer_evaluate.restype = _Eval
    L.msplat_trainer_render.argtypes = [vp, C.c_int, C.c_bool]
    L.msplat_trainer_render.restype = _Pixels
    L.msplat_trainer_render_pose.argtypes = [vp, fp, C.c_int]
    L.msplat_trainer_render_pose.restype = _Pixels
    L.msplat_trainer_render_pose_to_buffer.argtypes = [vp, fp, C.c_int, C.POINTER(C.c_uint8),
                                                       C.POINTER(C.c_int), C.POINTER(C.c_int)]
    for n in ("export_ply", "export_splat", "save_checkpoint"):
        getattr(L, f"msplat_trainer_{n}").argtypes = [vp, cp]
    L.msplat_trainer_load_checkpoint.argtypes = [vp, cp]
    L.msplat_trainer_splat_count.argtypes = [vp]
    L.msplat_trainer_iteration.argtypes = [vp]
    L.msplat_trainer_set_gaussians.argtypes = [vp, C.c_int, C.c_int, fp, fp, fp, fp, fp, fp]
    L.msplat_trainer_get_gaussians.argtypes = [vp, fp, fp, fp, fp, fp, fp]
    L.msplat_trainer_last_loss.argtypes = [vp]
    L.msplat_trainer_last_loss.restype = C.c_float
    L.msplat_trainer_engine.argtypes = [vp]
    L.msplat_trainer_engine.restype = vp
    L.msplat_trainer_mcmc_stats.argtypes = [vp, C.POINTER(N.MsplatMcmcStats)]
    hg = [C.c_int, C.c_int, fp, fp, fp, fp, fp, fp]
    L.msplat_write_ply.argtypes = [cp] + hg + [C.c_int, C.c_int, C.c_float, fp]
    L.msplat_write_splat.argtypes = [cp] + hg + [C.c_int, C.c_float, fp]
    L.msplat_ply_info.argtypes = [cp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.msplat_read_ply.argtypes = [cp, C.c_int, C.c_float, fp, fp, fp, fp, fp, fp, fp]
    fpp = C.POINTER(fp)
    L.msplat_write_checkpoint.argtypes = [cp, C.c_int, C.c_int, C.c_int, C.c_int, fp, C.c_float, C.c_float,
                                          fpp, fpp, fpp]
    L.msplat_read_checkpoint.argtypes = [cp, fp, fp, C.POINTER(C.c_int), fpp, fpp, fpp]
    L.msplat_checkpoint_info.argtypes = [cp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.msplat_dataset_create_masked.argtypes = [cp, C.c_float, C.c_bool, C.c_int, cp, cp]
    L.msplat_dataset_create_masked.restype = vp
    L.msplat_dataset_mask.argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_uint8)]
    L.msplat_dataset_hold_out.argtypes = [vp, cp]
    L.msplat_dataset_camera_file.argtypes = [vp, C.c_int, C.c_int, C.c_char_p, C.c_int]
    L.msplat_dataset_transform.argtypes = [vp, fp, fp]
    L.msplat_dataset_mask.restype = C.c_longlong
    L.msplat_viewer_create.argtypes = [cp, C.c_int, C.c_int, C.c_float]
    L.msplat_viewer_create.restype = vp
    L.msplat_viewer_render.argtypes = [vp, fp, C.POINTER(C.c_uint8)]
    L.msplat_viewer_splat_count.argtypes = [vp]
    L.msplat_viewer_get_size.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.msplat_viewer_bounds.argtypes = [vp, fp, fp]
    L.msplat_viewer_density_center.argtypes = [vp, fp]
    L.msplat_viewer_render_buffer.argtypes = [vp, fp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.msplat_viewer_render_buffer.restype = vp
    L.msplat_viewer_set_background.argtypes = [vp, C.c_float, C.c_float, C.c_float]
    L.msplat_viewer_resize.argtypes = [vp, C.c_int, C.c_int]
    L.msplat_viewer_set_fov.argtypes = [vp, C.c_float]
    L.msplat_viewer_destroy.argtypes = [vp]
    _bound = True
    return L


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


@dataclass
class TrainingConfig:
    """Defaults of the reference (core/include/msplat_c_api.h:32-47); the
    densification knobs of the stale python binding are accepted and ignored,
    as the reference's MCMC core ignores them."""
    iterations: int = 30000
    sh_degree: int = 3
    sh_degree_interval: int = 1000
    ssim_weight: float = 0.2
    cap_max: int = 1_000_000
    noise_lr: float = 5e5
    opacity_reg: float = 0.01
    scale_reg: float = 0.01
    cull_radius: float = 3.0
    keep_crs: bool = False
    downscale_factor: float = 1.0
    bg_color: list = field(default_factory=lambda: [0.6130, 0.0101, 0.3984])
    num_downscales: int = 2
    resolution_schedule: int = 3000
    refine_every: int = 100
    warmup_length: int = 500
    reset_alpha_every: int = 30
    densify_grad_thresh: float = 0.0002
    densify_size_thresh: float = 0.01
    stop_screen_size_at: int = 4000
    split_screen_size: float = 0.05
    output: str = "splat.ply"
    save_every: int = -1

    def native(self) -> _MsplatConfig:
        c = _MsplatConfig()
        c.iterations, c.shDegree, c.shDegreeInterval = self.iterations, self.sh_degree, self.sh_degree_interval
        c.ssimWeight, c.capMax, c.noiseLr = self.ssim_weight, self.cap_max, self.noise_lr
        c.opacityReg, c.scaleReg, c.cullRadius = self.opacity_reg, self.scale_reg, self.cull_radius
        c.keepCrs, c.downscaleFactor = self.keep_crs, self.downscale_factor
        c.bgColor[:] = [float(v) for v in self.bg_color]
        return c


@dataclass
class TrainingStats:
    iteration: int
    splat_count: int
    ms_per_step: float


class Dataset:
    def __init__(self, path: str | None = None, downscale_factor: float = 1.0, eval_mode: bool = False,
                 test_every: int = 8, colmap_image_path: str | None = None, mask_dir: str | None = None,
                 _handle=None):
        L = _lib()
        if _handle is not None:
            self.h = _handle
        elif mask_dir:
            self.h = L.msplat_dataset_create_masked(path.encode(), downscale_factor, eval_mode, test_every,
                                                    colmap_image_path.encode() if colmap_image_path else None,
                                                    mask_dir.encode())
        else:
            self.h = L.msplat_dataset_create_ex(path.encode(), downscale_factor, eval_mode, test_every,
                                                colmap_image_path.encode() if colmap_image_path else None)
        if not self.h:
            raise RuntimeError(f"could not load dataset {path!r}")

    @classmethod
    def from_arrays(cls, cameras, images, points_xyz, points_rgb, eval_mode=False, test_every=8, normalize=False,
                    masks=None):
        """cameras: list of synthetic.Camera (cam_to_world, width, height, fx, fy, cx, cy)."""
        L = _lib()
        n = len(cameras)
        c2w = np.ascontiguousarray(np.stack([np.asarray(c.cam_to_world, np.float32).reshape(16) for c in cameras]))
        intr = np.ascontiguousarray(np.array([[c.fx, c.fy, c.cx, c.cy] for c in cameras], np.float32))
        sizes = np.ascontiguousarray(np.array([[c.width, c.height] for c in cameras], np.int32))
        imgs = [np.ascontiguousarray(im, np.uint8) for im in images]
        ptrs = (C.c_void_p * n)(*[im.ctypes.data for im in imgs])
        mptrs = None
        if masks is not None:
            ms = [np.ascontiguousarray(m, np.uint8) if m is not None else None for m in masks]
            mptrs = (C.c_void_p * n)(*[m.ctypes.data if m is not None else None for m in ms])
        xyz = np.ascontiguousarray(points_xyz, np.float32)
        rgb = np.ascontiguousarray(points_rgb, np.uint8)
        h = L.msplat_dataset_create_from_memory(n, _fp(c2w), _fp(intr), sizes.ctypes.data_as(C.POINTER(C.c_int)),
                                                ptrs, mptrs, xyz.shape[0], _fp(xyz),
                                                rgb.ctypes.data_as(C.POINTER(C.c_uint8)), eval_mode, test_every,
                                                normalize)
        if not h:
            raise RuntimeError("could not build a dataset from the arrays (empty image size or missing points?)")
        return cls(_handle=h)

    def camera_file(self, i: int, use_test: bool = False) -> str:
        """Camera i's image file ("" for in-memory datasets)."""
        L = _lib()
        n = L.msplat_dataset_camera_file(self.h, i, int(use_test), None, 0)
        if n < 0:
            raise IndexError(i)
        buf = C.create_string_buffer(n + 1)
        L.msplat_dataset_camera_file(self.h, i, int(use_test), buf, n + 1)
        return buf.value.decode()

    @property
    def transform(self):
        """(scale, translation): dataset-frame positions are x / scale + translation."""
        sc, t = np.zeros(1, np.float32), np.zeros(3, np.float32)
        _lib().msplat_dataset_transform(self.h, _fp(sc), _fp(t))
        return float(sc[0]), t

    def hold_out(self, val_image: str = "random") -> int:
        """Withholds one training camera for validation (the reference CLI's
        --val / --val-image): it becomes test camera 0.  Returns its former
        training index."""
        i = _lib().msplat_dataset_hold_out(self.h, val_image.encode())
        if i < 0:
            raise RuntimeError("cannot hold out a validation camera (eval mode, or no cameras)")
        return i

    def mask(self, i: int, use_test: bool = False):
        """Camera i's training mask (uint8 [H, W], 255 = contributes), or None."""
        L = _lib()
        n = L.msplat_dataset_mask(self.h, i, int(use_test), None)
        if n == -2:
            raise IndexError(i)
        if n < 0:
            return None
        size = np.zeros(2, np.int32)
        L.msplat_dataset_camera(self.h, i, int(use_test), None, size.ctypes.data_as(C.POINTER(C.c_int)), None, None)
        m = np.zeros((size[1], size[0]), np.uint8)
        L.msplat_dataset_mask(self.h, i, int(use_test), m.ctypes.data_as(C.POINTER(C.c_uint8)))
        return m

    @property
    def num_train(self) -> int:
        return _lib().msplat_dataset_num_train(self.h)

    @property
    def num_test(self) -> int:
        return _lib().msplat_dataset_num_test(self.h)

    def camera(self, index: int, use_test: bool = False) -> dict:
        """Intrinsics, size, pose and the 8-bit image of a training (or test) view."""
        L = _lib()
        intr = np.zeros(4, np.float32)
        size = np.zeros(2, np.int32)
        c2w = np.zeros(16, np.float32)
        if L.msplat_dataset_camera(self.h, index, int(use_test), _fp(intr), size.ctypes.data_as(C.POINTER(C.c_int)),
                                   _fp(c2w), None) != 0:
            raise IndexError(index)
        img = np.zeros((int(size[1]), int(size[0]), 3), np.uint8)
        L.msplat_dataset_camera(self.h, index, int(use_test), None, None, None,
                                img.ctypes.data_as(C.POINTER(C.c_uint8)))
        return {"fx": float(intr[0]), "fy": float(intr[1]), "cx": float(intr[2]), "cy": float(intr[3]),
                "width": int(size[0]), "height": int(size[1]), "cam_to_world": c2w.reshape(4, 4), "image": img}

    def camera_pose(self, index: int) -> np.ndarray:
        out = np.zeros(16, np.float32)
        _lib().msplat_dataset_camera_pose(self.h, index, _fp(out))
        return out.reshape(4, 4)

    def __del__(self):
        if getattr(self, "h", None):
            _lib().msplat_dataset_destroy(self.h)
            self.h = None


def _take(px: _Pixels) -> np.ndarray:
    if not px.data:
        return np.zeros((0, 0, 3), np.float32)
    n = px.width * px.height * 3
    out = np.ctypeslib.as_array(px.data, shape=(n,)).copy().reshape(px.height, px.width, 3)
    C.CDLL(None).free(C.cast(px.data, C.c_void_p))
    return out


@dataclass
class TrainerOptions:
    """Options the reference's CLI sets on its model (seed opacity and scale,
    seed decimation, the means learning-rate decay length, the regularizer's
    visibility duty); the defaults are the reference's."""
    init_opacity: float = 0.5
    init_scale_mult: float = 0.1
    seed_decimation: bool = True
    position_lr_max_steps: int = 30000
    reg_visibility_duty: float = 1.0

    def native(self) -> _TrainerOptions:
        return _TrainerOptions(self.init_opacity, self.init_scale_mult, int(self.seed_decimation),
                               self.position_lr_max_steps, self.reg_visibility_duty)


def seed_gaussians(points_xyz, points_rgb, sh_degree: int = 3, cap_max: int = 1_000_000,
                   options: TrainerOptions | None = None):
    """The trainer's seed initialisation on the host: Gaussians [means,
    scales, quats, features_dc, features_rest, opacities] from a point
    cloud, after seed decimation or truncation to the cap."""
    xyz = np.ascontiguousarray(points_xyz, np.float32)
    rgb = np.ascontiguousarray(points_rgb, np.uint8)
    n = xyz.shape[0]
    rest = (sh_degree + 1) ** 2 - 1
    shapes = [(n, 3), (n, 3), (n, 4), (n, 3), (n, rest, 3), (n,)]
    arrs = [np.zeros(s, np.float32) for s in shapes]
    opt = (options or TrainerOptions()).native()
    rows = _lib().msplat_seed_gaussians(n, _fp(xyz), rgb.ctypes.data_as(C.POINTER(C.c_uint8)), int(sh_degree),
                                        int(cap_max), C.byref(opt), *[_fp(a) for a in arrs])
    if rows < 0:
        raise RuntimeError("invalid seed arguments")
    return [a[:rows] for a in arrs]


class GaussianTrainer:
    def __init__(self, dataset: Dataset, config: TrainingConfig, options: TrainerOptions | None = None):
        self.dataset = dataset   # the dataset must outlive the trainer
        self.config = config
        if options is None:
            self.h = _lib().msplat_trainer_create(dataset.h, config.native())
        else:
            self.h = _lib().msplat_trainer_create_ex(dataset.h, config.native(), C.byref(options.native()))
        if not self.h:
            raise RuntimeError("could not create trainer")

    def step(self) -> TrainingStats:
        s = _lib().msplat_trainer_step(self.h)
        return TrainingStats(s.iteration, s.splatCount, s.msPerStep)

    def train(self, callback=None, callback_every: int = 100):
        while self.iteration < self.config.iterations:
            s = self.step()
            if callback and s.iteration % callback_every == 0:
                callback(s)

    def evaluate(self) -> dict:
        m = _lib().msplat_trainer_evaluate(self.h)
        return {"psnr": m.psnr, "ssim": m.ssim, "l1": m.l1, "num_test": m.numTest, "num_gaussians": m.numGaussians}

    def render(self, cam_idx: int, use_test: bool = False) -> np.ndarray:
        return _take(_lib().msplat_trainer_render(self.h, cam_idx, use_test))

    def render_from_pose(self, cam_to_world, ref_cam_idx: int = 0) -> np.ndarray:
        m = np.ascontiguousarray(cam_to_world, np.float32).reshape(16)
        return _take(_lib().msplat_trainer_render_pose(self.h, _fp(m), ref_cam_idx))

    def render_to_rgba(self, cam_to_world, ref_cam_idx: int = 0) -> np.ndarray:
        L = _lib()
        m = np.ascontiguousarray(cam_to_world, np.float32).reshape(16)
        w, h = C.c_int(), C.c_int()
        L.msplat_trainer_render_pose_to_buffer(self.h, _fp(m), ref_cam_idx, None, C.byref(w), C.byref(h))
        out = np.zeros((h.value, w.value, 4), np.uint8)
        L.msplat_trainer_render_pose_to_buffer(self.h, _fp(m), ref_cam_idx,
                                               out.ctypes.data_as(C.POINTER(C.c_uint8)), C.byref(w), C.byref(h))
        return out

    def export_ply(self, path: str):
        _lib().msplat_trainer_export_ply(self.h, path.encode())

    def export_splat(self, path: str):
        _lib().msplat_trainer_export_splat(self.h, path.encode())

    def set_learned_relocation(self, enabled: bool = True):
        """Weight MCMC source draws by the online-trained proposal MLP (see msplat_gb300.h)."""
        if _lib().msplat_trainer_set_learned_relocation(self.h, int(enabled)) != 0:
            raise RuntimeError("could not switch the learned relocation proposal")

    def set_learned_prune(self, forecast_opacity: float):
        """The learned proposal's forecast-pruning threshold: Gaussians whose forecast
        opacity one window ahead is at most this are relocated with the dead ones
        (0: off; default 0.02)."""
        if _lib().msplat_trainer_set_learned_prune(self.h, float(forecast_opacity)) != 0:
            raise RuntimeError("could not set forecast pruning")

    def set_batch_views(self, num_views: int, lr_scale: float = 0.0):
        """Render `num_views` cameras per step and update from their mean gradient,
        learning rates times lr_scale (0: num_views ** 0.75); iterations count views."""
        if _lib().msplat_trainer_set_batch_views(self.h, int(num_views), float(lr_scale)) != 0:
            raise ValueError(f"invalid number of views per step: {num_views}")

    def set_isect_budget(self, bytes_per_gaussian: float):
        """Fixed intersection buffers (bytes per Gaussian of the cap; 0 = legacy), tile groups beyond."""
        if _lib().msplat_trainer_set_isect_budget(self.h, float(bytes_per_gaussian)) != 0:
            raise ValueError(f"invalid intersection budget: {bytes_per_gaussian}")

    def autotune(self) -> dict:
        """Time the engine's launch configurations on the next training views and keep the fastest."""
        from ._native import MsplatTuning
        t = MsplatTuning()
        if _lib().msplat_trainer_autotune(self.h, C.cast(C.byref(t), C.c_void_p)) != 0:
            raise RuntimeError("autotune failed")
        return {k: getattr(t, k) for k, _ in MsplatTuning._fields_}

    def learned_stats(self) -> dict:
        loss = (C.c_float * 1)()
        rounds = C.c_int()
        on = _lib().msplat_trainer_learned_stats(self.h, loss, C.byref(rounds))
        return {"enabled": on == 1, "last_loss": float(loss[0]), "rounds": rounds.value}

    def learned_eval(self) -> dict:
        """Held-out mean squared errors of the proposal's forecasts against the
        persistence forecasts, averaged over the rounds evaluated."""
        m = (C.c_float * 4)()
        rounds = _lib().msplat_trainer_learned_eval(self.h, m)
        return {"rounds_evaluated": rounds, "mse_opacity": m[0], "mse_opacity_persistence": m[1], "mse_activity": m[2],
                "mse_activity_persistence": m[3]}

    def mcmc_stats(self) -> dict:
        """Counts of the last MCMC relocation round and the rounds run so far."""
        st = N.MsplatMcmcStats()
        rounds = _lib().msplat_trainer_mcmc_stats(self.h, C.byref(st))
        d = {k: getattr(st, k) for k, _ in N.MsplatMcmcStats._fields_}
        d["rounds"] = rounds
        return d

    def engine_nan_counts(self) -> np.ndarray:
        """The engine's non-finite telemetry counters (grad_nan_counts slots)."""
        s = N.MsplatEngineStats()
        _lib().msplat_engine_stats(_lib().msplat_trainer_engine(self.h), C.byref(s))
        return np.array(s.nan_counts[:], np.uint32)

    def load_ply(self, path: str) -> int:
        """Replace the Gaussians with a trained PLY (fresh optimizer); returns its iteration."""
        rc = _lib().msplat_trainer_load_ply(self.h, path.encode())
        if rc < 0:
            raise RuntimeError(f"could not load {path!r}")
        return rc

    def save_checkpoint(self, path: str):
        _lib().msplat_trainer_save_checkpoint(self.h, path.encode())

    def load_checkpoint(self, path: str) -> int:
        return _lib().msplat_trainer_load_checkpoint(self.h, path.encode())

    def set_gaussians(self, g):
        L = _lib()
        arrs = [np.ascontiguousarray(a, np.float32) for a in g.arrays()]
        rc = L.msplat_trainer_set_gaussians(self.h, arrs[0].shape[0], arrs[4].shape[1], *[_fp(a) for a in arrs])
        if rc != 0:
            raise RuntimeError("set_gaussians failed")

    def get_gaussians(self, rest_bases: int = 15):
        n = self.splat_count
        shapes = [(n, 3), (n, 3), (n, 4), (n, 3), (n, rest_bases, 3), (n,)]
        arrs = [np.zeros(s, np.float32) for s in shapes]
        _lib().msplat_trainer_get_gaussians(self.h, *[_fp(a) for a in arrs])
        return arrs

    @property
    def last_loss(self) -> float:
        return float(_lib().msplat_trainer_last_loss(self.h))

    @property
    def splat_count(self) -> int:
        return _lib().msplat_trainer_splat_count(self.h)

    @property
    def iteration(self) -> int:
        return _lib().msplat_trainer_iteration(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            _lib().msplat_trainer_destroy(self.h)
            self.h = None


class Viewer:
    def __init__(self, ply_path: str, width: int, height: int, fov_y: float):
        self.h = _lib().msplat_viewer_create(ply_path.encode(), width, height, fov_y)
        if not self.h:
            raise RuntimeError(f"could not load {ply_path!r}")

    def render(self, cam_to_world) -> np.ndarray:
        L = _lib()
        w, h = C.c_int(), C.c_int()
        L.msplat_viewer_get_size(self.h, C.byref(w), C.byref(h))
        out = np.zeros((h.value, w.value, 4), np.uint8)
        m = np.ascontiguousarray(cam_to_world, np.float32).reshape(16)
        L.msplat_viewer_render(self.h, _fp(m), out.ctypes.data_as(C.POINTER(C.c_uint8)))
        return out

    @property
    def splat_count(self) -> int:
        return _lib().msplat_viewer_splat_count(self.h)

    def bounds(self):
        lo, hi = np.zeros(3, np.float32), np.zeros(3, np.float32)
        _lib().msplat_viewer_bounds(self.h, _fp(lo), _fp(hi))
        return lo, hi

    def density_center(self):
        c = np.zeros(3, np.float32)
        _lib().msplat_viewer_density_center(self.h, _fp(c))
        return c

    def __del__(self):
        if getattr(self, "h", None):
            _lib().msplat_viewer_destroy(self.h)
            self.h = None


def _host_arrays(gaussians):
    """(means, scales, quats, features_dc, features_rest [n, R, 3], opacities)
    as contiguous float32 arrays, and the rest bases R."""
    arrs = [np.ascontiguousarray(a, np.float32) for a in gaussians]
    n = arrs[0].shape[0]
    rest = arrs[4].reshape(n, -1, 3).shape[1] if arrs[4].size else 0
    return arrs, n, rest


def write_ply(path: str, gaussians, step: int = 0, keep_crs: bool = False, scale: float = 1.0,
              translation=(0.0, 0.0, 0.0)) -> None:
    """Writes Gaussians held on the host (the arrays get_gaussians returns,
    or a GaussianSet's arrays) as the trainer's PLY export does."""
    arrs, n, rest = _host_arrays(gaussians)
    t = np.asarray(translation, np.float32)
    if _lib().msplat_write_ply(path.encode(), n, rest, *[_fp(a) for a in arrs], int(step), int(keep_crs),
                               float(scale), _fp(t)) != 0:
        raise RuntimeError(f"could not write {path}")


def write_splat(path: str, gaussians, keep_crs: bool = False, scale: float = 1.0,
                translation=(0.0, 0.0, 0.0)) -> None:
    """Writes Gaussians held on the host as the trainer's .splat export does."""
    arrs, n, rest = _host_arrays(gaussians)
    t = np.asarray(translation, np.float32)
    if _lib().msplat_write_splat(path.encode(), n, rest, *[_fp(a) for a in arrs], int(keep_crs), float(scale),
                                 _fp(t)) != 0:
        raise RuntimeError(f"could not write {path}")


def read_ply(path: str, keep_crs: bool = False, scale: float = 1.0, translation=(0.0, 0.0, 0.0)):
    """A Gaussian PLY as the trainer loads it: ([means, scales, quats,
    features_dc, features_rest [n, R, 3], opacities], iteration)."""
    L = _lib()
    n, rest, step = C.c_int(), C.c_int(), C.c_int()
    if L.msplat_ply_info(path.encode(), C.byref(n), C.byref(rest), C.byref(step)) != 0:
        raise RuntimeError(f"could not read {path}")
    n = n.value
    shapes = [(n, 3), (n, 3), (n, 4), (n, 3), (n, rest.value, 3), (n,)]
    arrs = [np.zeros(s, np.float32) for s in shapes]
    t = np.asarray(translation, np.float32)
    if L.msplat_read_ply(path.encode(), int(keep_crs), float(scale), _fp(t), *[_fp(a) for a in arrs]) != 0:
        raise RuntimeError(f"could not read {path}")
    return arrs, step.value


def write_checkpoint(path: str, iteration: int, params, exp_avg, exp_avg_sq, adam_steps: int, adam_lr,
                     means_lr=(0.00016, 0.0000016), sh_degree: int = 3) -> None:
    """Writes a checkpoint (the trainer's format and code) of a model held on
    the host: six groups each of parameters and Adam moments (the arrays
    get_gaussians returns), the six learning rates and the Adam step."""
    grps = [[np.ascontiguousarray(a, np.float32) for a in g] for g in (params, exp_avg, exp_avg_sq)]
    ptrs = [(C.POINTER(C.c_float) * 6)(*[_fp(a) for a in g]) for g in grps]
    lr = np.asarray(adam_lr, np.float32)
    if _lib().msplat_write_checkpoint(path.encode(), int(iteration), grps[0][0].shape[0], int(sh_degree),
                                      int(adam_steps), _fp(lr), float(means_lr[0]), float(means_lr[1]),
                                      *ptrs) != 0:
        raise RuntimeError(f"could not write {path}")


def read_checkpoint(path: str):
    """A checkpoint read and validated as the trainer loads it: (iteration,
    Adam step, learning rates [8] (six groups, means init, means final),
    params [6], exp_avg [6], exp_avg_sq [6])."""
    L = _lib()
    n, deg, it = C.c_int(), C.c_int(), C.c_int()
    if L.msplat_checkpoint_info(path.encode(), C.byref(n), C.byref(deg), C.byref(it)) != 0:
        raise RuntimeError(f"could not read {path}")
    n, rest = n.value, (deg.value + 1) ** 2 - 1
    shapes = [(n, 3), (n, 3), (n, 4), (n, 3), (n, rest, 3), (n,)]
    grps = [[np.zeros(s, np.float32) for s in shapes] for _ in range(3)]
    lr, mlr, steps = np.zeros(6, np.float32), np.zeros(2, np.float32), C.c_int()
    ptrs = [(C.POINTER(C.c_float) * 6)(*[_fp(a) for a in g]) for g in grps]
    if L.msplat_read_checkpoint(path.encode(), _fp(lr), _fp(mlr), C.byref(steps), *ptrs) != 0:
        raise RuntimeError(f"could not read {path}")
    return it.value, steps.value, np.concatenate([lr, mlr]), grps[0], grps[1], grps[2]


def sync():
    N.lib().msplat_sync()


def cleanup():
    N.lib().msplat_cleanup()
