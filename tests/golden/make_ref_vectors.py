#!/usr/bin/env python3
"""Writes tests/golden/ref_vectors.npz: inputs and outputs of the reference's
own per-Gaussian Metal code (projection + SH, projection backward + SH Adam,
regularizer, Adam, SGLD), compiled as host C++ by oracle/ref_build.py from the
reference tree, on 512 random Gaussians at step 3001; and
tests/golden/ref_pixel_vectors.npz: the outputs of its pixel stages (tile
lists, forward rasterizers, SSIM + L1 loss, monolithic and chunked backward
rasterizers) on the small views of tests/test_ref_pin.py (their inputs are
regenerated from seeds); and tests/golden/ref_mcmc_vectors.npz: the moves
and a SHA-256 of the output state of the reference's MCMC host pass
(model.cpp:311-660) on the states of tests/test_ref_pin.py —
the vectors tests/test_ref_pin.py holds the oracle to where the reference
tree is absent.  Needs the reference tree (default /root/reference,
or MSPLAT_REFERENCE).

Usage: python tests/golden/make_ref_vectors.py
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from msplat_gb300 import synthetic as S  # noqa: E402
from msplat_gb300.schedule import GROUPS, step_scalars  # noqa: E402
from oracle import oracle as O, ref as R  # noqa: E402
from test_ref_pin import (FWD_KEYS, MCMC_CASES, PIXEL_CASES, _copy_state, _state_digest,  # noqa: E402
                          chunked_backward_case, dense_tile_case, mcmc_pairs, mcmc_state, pixel_case,
                          random_inputs, ref_run, ring_camera)


def main():
    R.lib()
    R.set_expf(ctypes.cast(O.lib().or_det_expf, ctypes.c_void_p).value)
    cam = ring_camera(640, 416, 500.0, k=3)
    g, mom, rg = random_inputs(512, 7)
    step = 3001
    st = step_scalars(step, step, width=cam["width"], height=cam["height"])
    fwd, bwd, g_r, mom_r = ref_run(g, mom, rg, cam, st)
    out = {"step": np.int64(step), "in_raster_grads": rg, "gauss_1d": R.gauss_1d()}
    for k, v in cam.items():
        out["cam_" + k] = np.asarray(v)
    for k, a, b in zip(GROUPS, g.arrays(), g_r.arrays()):
        out["in_" + k], out["out_" + k] = a, b
    for k, a, b, c, d in zip(GROUPS, mom[0], mom[1], mom_r[0], mom_r[1]):
        out["in_m_" + k], out["in_v_" + k], out["out_m_" + k], out["out_v_" + k] = a, b, c, d
    for k in FWD_KEYS + ("nan_counts",):
        out["fwd_" + k] = fwd[k]
    for k in ("v_mean3d", "v_scale", "v_quat"):
        out["bwd_" + k] = bwd[k]
    path = os.path.join(HERE, "ref_vectors.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")

    # the pixel stages (tile lists, rasterizers, loss) of small views
    pix = {}
    for name in PIXEL_CASES:
        cam, g, gt, mask, bg = pixel_case(name)
        st = step_scalars(3001, 3001, width=cam["width"], height=cam["height"])
        fwd = R.project_fwd(g, cam, 3)
        k = O.train_step(32, g.copy(), cam, st, gt=gt, mask=mask, background=bg, raster_mode=PIXEL_CASES[name][-1],
                         do_backward=False, do_optimizer=False, want_ids=False)["k_max"]
        o = R.raster_step(fwd, g.opacities, cam, gt=gt, mask=mask, background=bg, loss_inv_n=st["loss_inv_n"],
                          k_max=k)
        keys = ["num_isect", "gaussian_ids", "tile_bins", "out_img", "final_Ts", "final_idx", "loss", "v_rendered"]
        if o["backward_ran"]:   # the chunked backward runs only where it is defined
            keys += ["v_xy", "v_conic", "v_colors", "v_opacity"]
        for k in keys:
            pix[f"{name}/{k}"] = np.asarray(o[k])
    # the chunked backward, on a view where it is defined
    cam, g, gt = chunked_backward_case()
    st = step_scalars(3001, 3001, width=cam["width"], height=cam["height"])
    o = R.raster_step(R.project_fwd(g, cam, 3), g.opacities, cam, gt=gt, loss_inv_n=st["loss_inv_n"], k_max=3)
    assert o["backward_ran"]
    for k in ["num_isect", "gaussian_ids", "tile_bins", "out_img", "final_Ts", "final_idx", "loss", "v_rendered",
              "v_xy", "v_conic", "v_colors", "v_opacity"]:
        pix[f"chunked_bwd/{k}"] = np.asarray(o[k])
    # a tile of more than 2048 keys (the device-memory bitonic sort)
    cam, g, gt = dense_tile_case()
    st = step_scalars(3001, 3001, width=cam["width"], height=cam["height"])
    o = R.raster_step(R.project_fwd(g, cam, 3), g.opacities, cam, gt=gt, loss_inv_n=st["loss_inv_n"])
    for k in ["num_isect", "gaussian_ids", "tile_bins", "out_img", "final_Ts", "final_idx", "loss", "v_rendered",
              "v_xy", "v_conic", "v_colors", "v_opacity"]:
        pix[f"dense/{k}"] = np.asarray(o[k])
    path = os.path.join(HERE, "ref_pixel_vectors.npz")
    np.savez_compressed(path, **pix)
    print(path, os.path.getsize(path), "bytes")

    # the MCMC host code: each case's moves and a digest of the output state
    mc = {}
    for name, (n, cap, seed, with_dead) in MCMC_CASES.items():
        g0, m0 = mcmc_state(n, cap, seed, with_dead)
        g_r, m_r = _copy_state(g0, m0)
        n_new, _ = R.mcmc_after_train(g_r, m_r, n, 600, 30000, 3.0, 0)
        dead = None
        if with_dead:
            dead, _ = O.mcmc_dead_mask(S.GaussianSet(*(a[:n] for a in g0.arrays())), 3.0)
        dst, src = mcmc_pairs(g0, g_r, n, n_new, dead)
        mc[name + "/dst"], mc[name + "/src"] = dst, src
        mc[name + "/sha256"] = np.array(_state_digest(g_r, m_r))
    path = os.path.join(HERE, "ref_mcmc_vectors.npz")
    np.savez_compressed(path, **mc)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
