"""Shared pieces of the GPU parity tests: run one step on the engine and on
the oracle from the same inputs and collect comparable outputs."""
from __future__ import annotations

import numpy as np

from msplat_gb300 import engine as E
from msplat_gb300 import synthetic as S
from oracle import oracle as O


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    d = np.linalg.norm(a - b)
    n = np.linalg.norm(b)
    return float(d / n) if n > 0 else float(d)


def gt_image(scene_gt, cam, background=(0.0, 0.0, 0.0)):
    """Target image rendered by the oracle (FP64), quantised to uint8."""
    c = E.camera_dict(cam)
    r = O.train_step(64, scene_gt.copy(), c, {"degrees_to_use": 3}, do_backward=False, do_optimizer=False,
                     background=background, want_ids=False)
    return (np.clip(r["out_img"], 0.0, 1.0) * 255.0 + 0.5).astype(np.uint8)


def engine_outputs(eng, n, W, H, with_grads=True):
    T = ((W + 15) // 16) * ((H + 15) // 16)
    P = W * H
    o = {}
    rec = eng.read("rec", np.float32, n * 12).reshape(n, 12)
    o["xys"], o["opac"], o["conics"], o["colors"] = rec[:, 0:2], rec[:, 2], rec[:, 4:7], rec[:, 8:11]
    o["depths"] = eng.read("depths", np.float32, n)
    o["radii"] = eng.read("radii", np.int32, n)
    o["aabb"] = eng.read("aabb", np.float32, 2 * n).reshape(n, 2)
    o["num_tiles_hit"] = eng.read("tiles_hit", np.int32, n)
    o["tile_counts"] = eng.read("tile_counts", np.uint32, T).astype(np.int64)
    offs = eng.read("tile_offsets", np.uint32, T + 1).astype(np.int64)
    o["tile_offsets"] = offs
    M = int(offs[-1])
    o["num_isect"] = M
    o["gaussian_ids"] = eng.read("isect_ids", np.int32, max(M, 1))[:M].copy()
    o["out_img"] = eng.read("out_img", np.float32, P * 3).reshape(H, W, 3)
    o["final_Ts"] = eng.read("final_T", np.float32, P).reshape(H, W)
    o["final_idx"] = eng.read("final_idx", np.int32, P).reshape(H, W)
    if with_grads:
        o["v_rendered"] = eng.read("v_img", np.float32, P * 3).reshape(H, W, 3)
        gr = eng.read("grad", np.float32, n * 12).reshape(n, 12)
        o["v_xy"], o["v_opacity"], o["v_conic"], o["v_colors"] = gr[:, 0:2], gr[:, 2], gr[:, 4:7], gr[:, 8:11]
        o["v_mean3d"] = eng.read("v_mean", np.float32, n * 3).reshape(n, 3)
        o["v_scale"] = eng.read("v_scale", np.float32, n * 3).reshape(n, 3)
        o["v_quat"] = eng.read("v_quat", np.float32, n * 4).reshape(n, 4)
    return o


def run_pair(init: S.GaussianSet, cam, gt, step: dict, *, raster_mode=0, k_max=0, do_sgld=False, mask=None,
             background=(0.0, 0.0, 0.0), precs=(32, 64), do_backward=True, tuning=None):
    """One step on the engine and on the oracle (each precision in `precs`).
    tuning: engine launch configuration fields (MsplatTuning) set first.
    Returns (engine outputs + updated params, {prec: oracle outputs + params})."""
    import torch
    cd = E.camera_dict(cam)
    W, H = cam.width, cam.height
    eng = E.Engine(0)
    if tuning:
        eng.set_tuning(**tuning)
    dg = E.DeviceGaussians(init)
    args = E.make_args(cd, step, background=background, raster_mode=raster_mode, k_max=k_max, do_sgld=do_sgld)
    if do_backward:
        gt_d = torch.from_numpy(np.ascontiguousarray(gt)).cuda()
        mask_d = torch.from_numpy(np.ascontiguousarray(mask)).cuda() if mask is not None else None
        eng.train_step(dg, args, gt_d.data_ptr(), mask_d.data_ptr() if mask_d is not None else None)
    else:
        eng.render(dg, args)
    eng.synchronize()
    eo = engine_outputs(eng, init.n, W, H, with_grads=do_backward)
    if do_backward:
        eo["loss"] = eng.loss()
    st = eng.stats()
    rec = list(st.check_record)
    assert rec[0] == 0, f"checked build: bound {rec[0]} failed at index {rec[1] | (rec[2] << 32)}"
    eo["k_max"] = st.k_max
    eo["nan_counts"] = np.array(st.nan_counts[:], np.uint32)
    params, moments = dg.to_numpy()
    eo["params"] = params
    eo["moments"] = moments
    eng.close()
    res = {}
    for prec in precs:
        g = init.copy()
        mom = ([np.zeros_like(a) for a in g.arrays()], [np.zeros_like(a) for a in g.arrays()])
        r = O.train_step(prec, g, cd, step, moments=mom, gt=gt if do_backward else None, mask=mask,
                         background=background, do_backward=do_backward, do_optimizer=do_backward,
                         do_sgld=do_sgld, raster_mode=raster_mode, k_max=k_max)
        r["params"] = dict(zip(E.GROUPS, g.arrays()))
        r["params"]["opacities"] = r["params"]["opacities"].reshape(-1)
        res[prec] = r
    return eo, res
