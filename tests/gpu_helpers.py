"""Shared pieces of the GPU parity tests: run one step on the engine and on
the oracle from the same inputs and collect comparable outputs."""
from __future__ import annotations

import numpy as np

from msplat_gb300 import engine as E
from msplat_gb300 import synthetic as S
from oracle import oracle as O


C0 = 0.28209479177387814
C1 = 0.4886025119029199
C2 = (1.0925484305920792, -1.0925484305920792, 0.31539156525252005, -1.0925484305920792, 0.5462742152960396)
C3 = (-0.5900435899266435, 2.890611442640554, -0.4570457994644658, 0.3731763325901154, -0.4570457994644658,
      1.445305721320277, -0.5900435899266435)


def sh_basis(d):
    """Real SH basis without the constant term, bands 1-3 (15 values), for unit directions d [N,3]."""
    X, Y, Z = d[:, 0], d[:, 1], d[:, 2]
    xx, yy, zz, xy, yz, xz = X * X, Y * Y, Z * Z, X * Y, Y * Z, X * Z
    return np.stack([-C1 * Y, C1 * Z, -C1 * X,
                     C2[0] * xy, C2[1] * yz, C2[2] * (2 * zz - xx - yy), C2[3] * xz, C2[4] * (xx - yy),
                     C3[0] * Y * (3 * xx - yy), C3[1] * xy * Z, C3[2] * Y * (4 * zz - xx - yy),
                     C3[3] * Z * (2 * zz - 3 * xx - 3 * yy), C3[4] * X * (4 * zz - xx - yy), C3[5] * Z * (xx - yy),
                     C3[6] * X * (xx - 3 * yy)], axis=1)


def sh_grads(g, cd, r, deg=3):
    """dL/d(features_dc) and dL/d(features_rest) from the oracle's colour
    gradient (the SH chain the projection backward applies)."""
    d = g.means.astype(np.float64) - np.asarray(cd["cam_pos"], np.float64)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    vis = (r["radii"] > 0)[:, None]
    vc = np.where(vis, r["v_colors"], 0.0)
    v_dc = C0 * vc
    nb = {0: 0, 1: 3, 2: 8, 3: 15}[deg]
    basis = sh_basis(d)
    v_rest = np.zeros(g.features_rest.shape)
    v_rest[:, :nb, :] = basis[:, :nb, None] * vc[:, None, :]
    return v_dc, v_rest


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


IMG_TOL = 1e-5
GRAD_TOL = 1e-4
FP64_BAR = 1e-3
GRADS = ("v_xy", "v_conic", "v_colors", "v_opacity", "v_mean3d", "v_scale", "v_quat")


def state_of(dg, like):
    """The engine's parameters and Adam moments as a GaussianSet and moment
    lists shaped like `like` (read back after a synchronize)."""
    params, moments = dg.to_numpy()
    shapes = [a.shape for a in like.arrays()]
    g = S.GaussianSet(*(np.ascontiguousarray(params[n].reshape(sh)) for n, sh in zip(E.GROUPS, shapes)))
    mom = tuple([np.ascontiguousarray(m[n].reshape(sh)) for n, sh in zip(E.GROUPS, shapes)] for m in moments)
    return g, mom


def oracle_from(prec, g, moments, cd, step, gt, do_sgld=True, raster_mode=0):
    """One oracle step from a copy of (g, moments); returns its outputs and the
    updated parameters."""
    g = g.copy()
    mom = ([a.copy() for a in moments[0]], [a.copy() for a in moments[1]])
    r = O.train_step(prec, g, cd, step, moments=mom, gt=gt, do_sgld=do_sgld, raster_mode=raster_mode)
    r["params"] = dict(zip(E.GROUPS, g.arrays()))
    return r


def engine_step(eng, dg, cd, cam, step, gt_d, do_sgld=True, raster_mode=0):
    """One engine training step; its outputs, statistics and updated state."""
    eng.train_step(dg, E.make_args(cd, step, do_sgld=do_sgld, raster_mode=raster_mode), gt_d.data_ptr())
    eng.synchronize()
    eo = engine_outputs(eng, dg.n, cam.width, cam.height)
    eo["loss"] = eng.loss()
    st = eng.stats()
    eo["k_max"] = st.k_max
    eo["check"] = list(st.check_record)
    eo["params"], eo["moments"] = dg.to_numpy()
    return eo


def step_errors(eo, r, before):
    """Errors of the engine's step outputs against one oracle run."""
    e = {"image_max_abs": float(np.max(np.abs(eo["out_img"] - r["out_img"]))),
         "final_T_max_abs": float(np.max(np.abs(eo["final_Ts"] - r["final_Ts"]))),
         "loss_rel": abs(eo["loss"] - r["loss"]) / max(abs(r["loss"]), 1e-30),
         "v_rendered": rel_l2(eo["v_rendered"], r["v_rendered"])}
    for k in GRADS:
        e[k] = rel_l2(eo[k], r[k])
    for k in E.GROUPS:
        b = before[k].reshape(eo["params"][k].shape)
        e["update_" + k] = rel_l2(eo["params"][k] - b, r["params"][k].reshape(b.shape) - b)
    return e


def compare_step(eo, r32, before, label, r64=None, fp64_bar=FP64_BAR, img_frac_bar=2e-3):
    """One step's parity bars: integer outputs, lists, last contributors and
    visible projection outputs identical to the float path; image and final
    transmittance within 1e-5 max-abs; loss within 1e-5 relative; dL/dimage,
    the rasterizer and projection gradients and every parameter update within
    1e-4 relative L2.  Every error is printed first.  Against FP64 (r64) the
    errors are printed and returned, and held to fp64_bar (gradients,
    updates: 1e-3 by default), to img_frac_bar (0.2 % by default) of image
    values over 1e-5, and to the float oracle's own FP64 errors (gradients
    and updates plus 2e-4, the image fraction plus 1e-4: the engine follows
    the float arithmetic within 1e-4, so it may not stray further from FP64
    than that arithmetic does)."""
    act = r32["radii"] > 0
    e32 = step_errors(eo, r32, before)
    print(label, "float-path errors:", {k: float("%.3g" % v) for k, v in e32.items()})
    rep = {}
    if r64 is not None:
        rep = step_errors(eo, r64, before)
        d = np.abs(eo["out_img"] - r64["out_img"])
        rep["image_frac_over_1e-5"] = float(np.mean(d > IMG_TOL))
        rep["lists_equal"] = bool(np.array_equal(eo["gaussian_ids"], r64["gaussian_ids"]))
        rep["radii_mismatch"] = int(np.sum(eo["radii"] != r64["radii"]))
        print(label, "FP64 errors:", {k: (float("%.3g" % v) if isinstance(v, float) else v) for k, v in rep.items()})
        own = step_errors(r32, r64, before)
        own["image_frac_over_1e-5"] = float(np.mean(np.abs(r32["out_img"] - r64["out_img"]) > IMG_TOL))
        print(label, "float oracle's FP64 errors:", {k: float("%.3g" % v) for k, v in own.items()})
    assert eo["check"][0] == 0
    assert eo["k_max"] == r32["k_max"], (label, eo["k_max"], r32["k_max"])
    assert np.array_equal(eo["radii"], r32["radii"]), label
    assert np.array_equal(eo["num_tiles_hit"], r32["num_tiles_hit"]), label
    for k in ("depths", "xys", "conics", "colors", "aabb"):
        assert np.array_equal(eo[k][act], r32[k][act]), (label, k)
    assert np.array_equal(eo["tile_counts"], r32["tile_counts"]), label
    assert eo["num_isect"] == r32["num_isect"], label
    assert np.array_equal(eo["gaussian_ids"], r32["gaussian_ids"]), label
    assert np.array_equal(eo["final_idx"], r32["final_idx"]), label
    assert e32["image_max_abs"] <= IMG_TOL and e32["final_T_max_abs"] <= IMG_TOL, label
    assert e32["loss_rel"] <= 1e-5, label
    for k, v in e32.items():
        if k not in ("image_max_abs", "final_T_max_abs", "loss_rel"):
            assert v <= GRAD_TOL, (label, k, v)
    if r64 is not None:
        assert rep["image_frac_over_1e-5"] < img_frac_bar, (label, rep["image_frac_over_1e-5"])
        assert rep["image_frac_over_1e-5"] <= own["image_frac_over_1e-5"] + 1e-4, label
        for k in list(GRADS) + ["update_" + g for g in E.GROUPS]:
            assert rep[k] <= fp64_bar, (label, k, rep[k])
            assert rep[k] <= own[k] + 2e-4, (label, k, rep[k], own[k])
    return rep
