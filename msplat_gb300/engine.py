"""Python handle on the CUDA training engine (include/msplat_engine.h).

Device buffers are torch CUDA tensors (PyTorch is used here for device memory
only); every computation runs in the engine's own kernels.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _native as N
from .schedule import BETA1, BETA2, EPS, GROUPS, LR_INIT, step_scalars  # noqa: F401


def prepare_cam(c2w, width: int, height: int, fx: float, fy: float):
    """World->camera and projection*view matrices and camera position
    (core/src/model.cpp:845-889), computed by the library."""
    L = N.lib()
    c2w = np.ascontiguousarray(c2w, np.float32).reshape(16)
    vm = np.zeros(16, np.float32)
    pm = np.zeros(16, np.float32)
    cp = np.zeros(3, np.float32)
    L.msplat_prepare_camera(c2w.ctypes.data_as(N.FP), width, height, C.c_float(fx), C.c_float(fy),
                            vm.ctypes.data_as(N.FP), pm.ctypes.data_as(N.FP), cp.ctypes.data_as(N.FP))
    return vm, pm, cp


def make_args(cam: dict, step: dict, background=(0.0, 0.0, 0.0), ssim_weight=0.2, raster_mode=0, k_max=0,
              do_optimizer=True, do_sgld=False) -> N.MsplatStepArgs:
    a = N.MsplatStepArgs()
    a.viewmat[:] = [float(v) for v in np.asarray(cam["viewmat"], np.float32).ravel()]
    a.projmat[:] = [float(v) for v in np.asarray(cam["projmat"], np.float32).ravel()]
    a.fx, a.fy, a.cx, a.cy = cam["fx"], cam["fy"], cam["cx"], cam["cy"]
    a.width, a.height = int(cam["width"]), int(cam["height"])
    a.cam_pos[:] = [float(v) for v in cam["cam_pos"]]
    a.background[:] = [float(v) for v in background]
    a.clip_thresh = 0.01
    a.degrees_to_use = int(step.get("degrees_to_use", 3))
    a.ssim_weight = ssim_weight
    a.loss_inv_n = step.get("loss_inv_n", 1.0 / (3.0 * a.width * a.height))
    a.step_size[:] = [float(v) for v in step.get("step_size", [0.0] * 6)]
    a.bc2_sqrt[:] = [float(v) for v in step.get("bc2_sqrt", [1.0] * 6)]
    a.beta1, a.beta2, a.eps = step.get("beta1", BETA1), step.get("beta2", BETA2), step.get("eps", EPS)
    a.op_reg, a.sc_reg, a.invis_scale = step.get("op_reg", 0.0), step.get("sc_reg", 0.0), step.get("invis_scale", 1.0)
    a.raster_mode, a.k_max = raster_mode, k_max
    a.do_optimizer, a.do_sgld = int(do_optimizer), int(do_sgld)
    a.seed = int(step.get("seed", 0)) & 0xFFFFFFFF
    a.noise_lr, a.xyz_lr, a.max_disp = step.get("noise_lr", 5e5), step.get("xyz_lr", 1.6e-4), step.get("max_disp", 0.05)
    return a


def camera_dict(cam) -> dict:
    """synthetic.Camera -> the dict the step helpers use."""
    vm, pm, cp = prepare_cam(cam.cam_to_world, cam.width, cam.height, cam.fx, cam.fy)
    return dict(viewmat=vm, projmat=pm, cam_pos=cp, fx=cam.fx, fy=cam.fy, cx=cam.cx, cy=cam.cy,
                width=cam.width, height=cam.height)


class DeviceGaussians:
    """Parameters and Adam moments as CUDA tensors (reference layouts).

    With `cap` the tensors hold `cap` rows (the MCMC budget, Model::cap_max)
    of which the first `active` are live; MCMC growth raises `active`."""

    def __init__(self, g, device="cuda", cap: int | None = None):
        import torch
        self.torch = torch
        cap = g.n if cap is None else int(cap)
        if cap < g.n:
            raise ValueError("cap below the number of Gaussians")
        self.params = {}
        for k, a in zip(GROUPS, g.arrays()):
            t = torch.zeros((cap,) + a.shape[1:], dtype=torch.float32, device=device)
            t[:g.n] = torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(device)
            self.params[k] = t
        self.exp_avg = {k: torch.zeros_like(v) for k, v in self.params.items()}
        self.exp_avg_sq = {k: torch.zeros_like(v) for k, v in self.params.items()}
        self.rest_bases = int(g.features_rest.shape[1])
        self.active = g.n

    @property
    def n(self):
        return self.active

    @property
    def cap(self):
        return int(self.params["means"].shape[0])

    def native(self):
        p = self.params
        g = N.MsplatGaussians(self.n, self.rest_bases, p["means"].data_ptr(), p["scales"].data_ptr(),
                              p["quats"].data_ptr(), p["features_dc"].data_ptr(), p["features_rest"].data_ptr(),
                              p["opacities"].data_ptr())
        st = N.MsplatAdamState()
        for i, k in enumerate(GROUPS):
            st.exp_avg[i] = self.exp_avg[k].data_ptr()
            st.exp_avg_sq[i] = self.exp_avg_sq[k].data_ptr()
        return g, st

    def to_numpy(self, rows: int | None = None):
        r = self.n if rows is None else rows
        return {k: v[:r].detach().cpu().numpy() for k, v in self.params.items()}, \
               ({k: v[:r].cpu().numpy() for k, v in self.exp_avg.items()},
                {k: v[:r].cpu().numpy() for k, v in self.exp_avg_sq.items()})


class Engine:
    """One CUDA engine (stream + device arena)."""

    def __init__(self, device: int = 0, max_points: int = 0):
        self.L = N.lib()
        self.h = self.L.msplat_engine_create(device, max_points)
        if not self.h:
            raise RuntimeError("msplat_engine_create failed")

    def close(self):
        if self.h:
            self.L.msplat_engine_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(f"msplat engine error {rc}: {self.L.msplat_engine_last_error(self.h).decode()}")

    def train_step(self, dg: DeviceGaussians, args: N.MsplatStepArgs, gt_ptr: int, mask_ptr: int | None = None):
        g, st = dg.native()
        self._check(self.L.msplat_engine_train_step(self.h, C.byref(g), C.byref(st), C.byref(args), gt_ptr,
                                                    mask_ptr or None))

    def train_step_batch(self, dg: DeviceGaussians, args: list, gt_ptrs: list, mask_ptrs: list | None = None):
        """One optimizer update from the mean gradient of several views (any sizes)."""
        g, st = dg.native()
        n = len(args)
        arr = (N.MsplatStepArgs * n)(*args)
        gts = (C.c_void_p * n)(*gt_ptrs)
        masks = (C.c_void_p * n)(*(mask_ptrs or [None] * n)) if mask_ptrs else None
        self._check(self.L.msplat_engine_train_step_batch(self.h, C.byref(g), C.byref(st), arr, n, gts, masks))

    def train_step_host(self, dg: DeviceGaussians, args: N.MsplatStepArgs, gt_host_ptr: int,
                        mask_host_ptr: int | None = None):
        g, st = dg.native()
        self._check(self.L.msplat_engine_train_step_host(self.h, C.byref(g), C.byref(st), C.byref(args), gt_host_ptr,
                                                         mask_host_ptr or None))

    def render(self, dg: DeviceGaussians, args: N.MsplatStepArgs):
        g, _ = dg.native()
        self._check(self.L.msplat_engine_render(self.h, C.byref(g), C.byref(args)))

    def backward(self, g: N.MsplatGaussians, args: N.MsplatStepArgs, v_img_ptr: int, grads: N.MsplatGradients):
        """dL/d(parameters) for dL/d(image) at v_img_ptr (device float [H,W,3]); the
        forward of (g, args) is recomputed.  Gradients go to the pointers in grads."""
        self._check(self.L.msplat_engine_backward(self.h, C.byref(g), C.byref(args), v_img_ptr, C.byref(grads)))

    def render_raw(self, g: N.MsplatGaussians, args: N.MsplatStepArgs):
        self._check(self.L.msplat_engine_render(self.h, C.byref(g), C.byref(args)))

    def mcmc(self, dg: DeviceGaussians, cull_radius: float, relocation_count: int):
        """One relocation + growth round on the device; returns (stats, new relocation_count)."""
        g, st = dg.native()
        rc = C.c_int(relocation_count)
        out = N.MsplatMcmcStats()
        self._check(self.L.msplat_engine_mcmc(self.h, C.byref(g), C.byref(st), dg.cap, cull_radius, C.byref(rc),
                                              C.byref(out)))
        dg.active = out.num_active
        return out, rc.value

    def synchronize(self):
        self._check(self.L.msplat_engine_synchronize(self.h))

    def loss(self) -> float:
        v = C.c_float()
        self._check(self.L.msplat_engine_loss(self.h, C.byref(v)))
        return float(v.value)

    def stats(self) -> N.MsplatEngineStats:
        s = N.MsplatEngineStats()
        self._check(self.L.msplat_engine_stats(self.h, C.byref(s)))
        return s

    def set_timing(self, on: bool):
        self._check(self.L.msplat_engine_set_timing(self.h, int(on)))

    def loss_async(self, dst_ptr: int):
        """Enqueue the copy of the last step's loss sums (one float per view) to
        page-locked host memory at dst_ptr; valid after synchronize()."""
        self._check(self.L.msplat_engine_loss_async(self.h, C.c_void_p(dst_ptr)))

    def set_graphs(self, on: bool):
        """Capture repeated steps into CUDA graphs and replay them."""
        self._check(self.L.msplat_engine_set_graphs(self.h, int(on)))

    def set_isect_budget(self, slots: int):
        """Fixed intersection buffers of `slots` slots (0: legacy); larger views in tile groups."""
        self._check(self.L.msplat_engine_set_isect_budget(self.h, int(slots)))

    TUNING_FIELDS = ("sort_width", "raster_batch", "chunk", "raster_mode", "tile_order", "bwd_pixels", "tile_split")

    def set_tuning(self, **kw):
        """Change fields of the launch configuration (see MsplatTuning)."""
        t = N.MsplatTuning()
        self._check(self.L.msplat_engine_get_tuning(self.h, C.byref(t)))
        for k, v in kw.items():
            if k not in self.TUNING_FIELDS:
                raise KeyError(k)
            setattr(t, k, int(v))
        self._check(self.L.msplat_engine_set_tuning(self.h, C.byref(t)))

    def tuning(self) -> dict:
        t = N.MsplatTuning()
        self._check(self.L.msplat_engine_get_tuning(self.h, C.byref(t)))
        return {k: getattr(t, k) for k in self.TUNING_FIELDS}

    def autotune(self, dg: "DeviceGaussians", args: list, gt_ptrs: list, mask_ptrs: list | None = None,
                 reps: int = 3):
        """Time the candidate launch configurations on these views and keep the
        fastest; returns (configuration dict, step ms)."""
        g, _ = dg.native()
        n = len(args)
        arr = (N.MsplatStepArgs * n)(*args)
        gts = (C.c_void_p * n)(*gt_ptrs)
        masks = (C.c_void_p * n)(*(mask_ptrs or [None] * n))
        t = N.MsplatTuning()
        ms = C.c_float()
        self._check(self.L.msplat_engine_autotune(self.h, C.byref(g), arr, n, gts, masks, int(reps), C.byref(t),
                                                  C.byref(ms)))
        return {k: getattr(t, k) for k in self.TUNING_FIELDS}, float(ms.value)

    def buffer(self, name: str):
        p = C.c_void_p()
        n = self.L.msplat_engine_buffer(self.h, name.encode(), C.byref(p))
        return (p.value, n) if n >= 0 else (None, -1)

    def read(self, name: str, dtype, count: int) -> np.ndarray:
        out = np.zeros(count, dtype)
        self._check(self.L.msplat_engine_read(self.h, name.encode(), out.ctypes.data, out.nbytes))
        return out

    def marker(self, which: int):
        self._check(self.L.msplat_engine_marker(self.h, which))

    def marker_elapsed(self) -> float:
        v = C.c_float()
        self._check(self.L.msplat_engine_marker_elapsed(self.h, C.byref(v)))
        return float(v.value)

    def stream(self) -> int:
        return self.L.msplat_engine_stream(self.h)
