"""Differentiable rasterization for PyTorch: projection + tile sort +
rasterizer as one torch.autograd.Function over the engine's kernels.

    image = rasterize(means, scales, quats, features_dc, features_rest,
                      opacities, camera, background=(0, 0, 0), sh_degree=3)

Inputs are float32 CUDA tensors in the reference layouts (means [N,3],
log-scales [N,3], quaternions [N,4] (w,x,y,z), features_dc [N,3],
features_rest [N,R,3], opacity logits [N] or [N,1]).  `camera` is a dict
with viewmat/projmat/cam_pos/fx/fy/cx/cy/width/height (engine.camera_dict).
The output is the composited image [H,W,3] (clamped to [0,1], as the
reference renders it).

Backward recomputes the forward (projection, covariance, tile lists and
transmittance) instead of keeping it, then runs the same VJPs as the
training step (rasterize_backward_kernel and project_and_sh_backward_kernel,
msplat_metal.metal:931-1135, 1860-2042), including their quirks: the
saturate clamp is not differentiated, an alpha clamped to 0.999 gets no
gradient, the pixel-centre VJP uses projection rows 0-2 only, and the
quaternion gradient ignores the normalisation.  No torch fallback exists:
the CUDA library must be present.
"""
from __future__ import annotations

import threading

import numpy as np
import torch

from . import _native as N
from . import engine as E

_engines: dict = {}
_elock = threading.Lock()


def _engine(device: int) -> E.Engine:
    with _elock:
        eng = _engines.get(device)
        if eng is None:
            eng = E.Engine(device)
            _engines[device] = eng
        return eng


def _check(t: torch.Tensor, name: str, shape_tail) -> torch.Tensor:
    if not t.is_cuda or t.dtype != torch.float32:
        raise TypeError(f"{name} must be a float32 CUDA tensor")
    if tuple(t.shape[1:]) != tuple(shape_tail):
        raise ValueError(f"{name} has shape {tuple(t.shape)}, expected [N, {', '.join(map(str, shape_tail))}]")
    return t.contiguous()


def _gaussians(means, scales, quats, dc, rest, opac) -> N.MsplatGaussians:
    n = means.shape[0]
    return N.MsplatGaussians(n, int(rest.shape[1]), means.data_ptr(), scales.data_ptr(), quats.data_ptr(),
                             dc.data_ptr(), rest.data_ptr() if rest.numel() else None, opac.data_ptr())


class RasterizeGaussians(torch.autograd.Function):
    @staticmethod
    def forward(ctx, means, scales, quats, features_dc, features_rest, opacities, camera, background, sh_degree):
        dev = means.device.index if means.device.index is not None else torch.cuda.current_device()
        n = means.shape[0]
        means = _check(means, "means", (3,))
        scales = _check(scales, "scales", (3,))
        quats = _check(quats, "quats", (4,))
        features_dc = _check(features_dc, "features_dc", (3,))
        if features_rest.dim() != 3 or features_rest.shape[0] != n or features_rest.shape[2] != 3:
            raise ValueError("features_rest must be [N, R, 3]")
        features_rest = _check(features_rest, "features_rest", tuple(features_rest.shape[1:]))
        op_shape = opacities.shape
        opacities = opacities.reshape(n).contiguous()
        if not opacities.is_cuda or opacities.dtype != torch.float32:
            raise TypeError("opacities must be a float32 CUDA tensor")
        eng = _engine(dev)
        args = E.make_args(camera, {"degrees_to_use": int(sh_degree)}, background=background, do_optimizer=False)
        g = _gaussians(means, scales, quats, features_dc, features_rest, opacities)
        torch.cuda.synchronize(dev)   # inputs written on torch's stream; the engine has its own
        with torch.cuda.device(dev):
            eng.render_raw(g, args)
            h, w = int(camera["height"]), int(camera["width"])
            img = torch.empty((h, w, 3), dtype=torch.float32, device=means.device)
            # device-to-device copy of the composited image (waits for the engine)
            rc = eng.L.msplat_engine_read(eng.h, b"out_img", img.data_ptr(), h * w * 3 * 4)
            if rc != 0:
                raise RuntimeError("reading the rendered image failed")
        ctx.save_for_backward(means, scales, quats, features_dc, features_rest, opacities)
        ctx.camera, ctx.background, ctx.sh_degree, ctx.op_shape = camera, background, sh_degree, op_shape
        return img

    @staticmethod
    def backward(ctx, v_img):
        means, scales, quats, dc, rest, opac = ctx.saved_tensors
        dev = means.device.index if means.device.index is not None else torch.cuda.current_device()
        eng = _engine(dev)
        v_img = v_img.contiguous().float()
        grads = [torch.empty_like(t) for t in (means, scales, quats, dc, rest, opac)]
        out = N.MsplatGradients(grads[0].data_ptr(), grads[1].data_ptr(), grads[2].data_ptr(), grads[3].data_ptr(),
                                grads[4].data_ptr() if rest.numel() else None, grads[5].data_ptr())
        args = E.make_args(ctx.camera, {"degrees_to_use": int(ctx.sh_degree)}, background=ctx.background,
                           do_optimizer=False)
        g = _gaussians(means, scales, quats, dc, rest, opac)
        torch.cuda.synchronize(dev)
        with torch.cuda.device(dev):
            eng.backward(g, args, v_img.data_ptr(), out)
            eng.synchronize()
        return (grads[0], grads[1], grads[2], grads[3], grads[4], grads[5].reshape(ctx.op_shape), None, None, None)


def rasterize(means, scales, quats, features_dc, features_rest, opacities, camera, background=(0.0, 0.0, 0.0),
              sh_degree: int = 3) -> torch.Tensor:
    return RasterizeGaussians.apply(means, scales, quats, features_dc, features_rest, opacities, camera,
                                    tuple(float(b) for b in background), sh_degree)
