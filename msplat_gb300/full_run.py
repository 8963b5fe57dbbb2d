"""The full-scale training run through the public trainer API.

    python -m msplat_gb300.full_run [--iters 7000] [--seed 0] [--init 100000] [--learned] [--batch-views B]

Scene (synthetic.config_full): 1,000,000 ground-truth Gaussians plus a
200,000-Gaussian ground plane; 160 ring/elevation-jittered training views and
20 held-out views at 1297x840, targets rendered by the engine's forward pass.
Training starts from `--init` random points (uniform in the unit ball,
random colours) through msplat_dataset_create_from_memory and the
reference's trainer (msplat_trainer_step: its camera order, learning-rate
schedule, SH degree raised every 1000 iterations, MCMC relocation and 5 %
growth every 100 steps up to the 1,000,000 cap).  Reported: wall-clock
iterations/s over the whole run (MCMC rounds included), the Gaussian count,
held-out PSNR / SSIM / L1 over the 20 views (msplat_trainer_evaluate, the
reference's Trainer::evaluate), per-stage milliseconds over a few eager
steps at the end, and the trained model's rasterization load on the last
of those views: intersections, tile list lengths and the (pixel, splat)
pairs the backward walks, with the raster backward's FP32 rate.  Prints one
JSON line.  --profile-step adds one more eager step inside a profiler range
(cudaProfilerStart/Stop), for `ncu --profile-from-start off`.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import sys
import time

import numpy as np


def build(seed=0, n_init=100_000):
    """Cameras (every 9th a held-out view), their targets, and seed points."""
    from . import engine as E
    from . import synthetic as S
    sc = S.config_full(seed, n_train=160, n_test=20)
    cams = []
    train = list(sc.train_cams)
    for k in range(20):
        cams.append(sc.test_cams[k])
        cams.extend(train[8 * k:8 * k + 8])
    eng = E.Engine(0)
    dg = E.DeviceGaussians(sc.gt)
    imgs = []
    for c in cams:
        eng.render(dg, E.make_args(E.camera_dict(c), {"degrees_to_use": 3}))
        img = eng.read("out_img", np.float32, c.width * c.height * 3).reshape(c.height, c.width, 3)
        imgs.append((np.clip(img, 0, 1) * 255 + 0.5).astype(np.uint8))
    eng.close()
    del dg
    rng = np.random.default_rng(seed + 101)
    d = rng.normal(size=(n_init, 3))
    xyz = (d / np.linalg.norm(d, axis=1, keepdims=True) * rng.random((n_init, 1)) ** (1 / 3)).astype(np.float32)
    rgb = rng.integers(0, 256, (n_init, 3), dtype=np.uint8)
    return cams, imgs, xyz, rgb


def time_to(psnr_curve, target):
    """Wall clock at which a (iteration, wall s, dB) curve first reaches
    `target` dB, interpolated linearly between the two evaluations around
    the crossing (the first evaluation's time when it is already there);
    None when it never does."""
    prev = None
    for _, w, p in psnr_curve:
        if p >= target:
            if prev is None:
                return w
            return prev[0] + (w - prev[0]) * (target - prev[1]) / (p - prev[1])
        prev = (w, p)
    return None


def held_out_psnr(t, test_imgs):
    """Mean over the held-out views of 10 log10(1 / MSE) against the uint8
    targets / 255 (the reference's Trainer::evaluate PSNR)."""
    vals = []
    for i, gt in enumerate(test_imgs):
        img = t.render(i, True).astype(np.float64)
        mse = float(np.mean((img - gt.astype(np.float64) / 255.0) ** 2))
        vals.append(10.0 * np.log10(1.0 / max(mse, 1e-20)))
    return float(np.mean(vals))


def run(iters=7000, seed=0, n_init=100_000, cap=1_000_000, timing_steps=20, profile_step=False, learned=False,
        eval_every=0, prune=None, batch=1):
    """eval_every > 0: held-out PSNR every that many iterations (outside the
    timed wall clock) in `psnr_curve` as (iteration, wall s, dB)."""
    from . import api as A
    from . import _native as N
    cams, imgs, xyz, rgb = build(seed, n_init)
    ds = A.Dataset.from_arrays(cams, imgs, xyz, rgb, eval_mode=True, test_every=9)
    assert ds.num_train == 160 and ds.num_test == 20
    test_imgs = imgs[0::9][:20] if eval_every > 0 else []   # every 9th view is held out
    del imgs
    t = A.GaussianTrainer(ds, A.TrainingConfig(iterations=iters, cap_max=cap, bg_color=[0.0, 0.0, 0.0]))
    if learned:
        t.set_learned_relocation(True)
        if prune is not None:
            t.set_learned_prune(prune)
    if batch > 1:   # views per optimizer step (iterations count views), learning rates x batch ** 0.75
        t.set_batch_views(batch)
    curve, psnr_curve = [], []
    A.sync()
    t0 = time.perf_counter()
    paused = 0.0
    while t.iteration < iters:
        t.step()
        if t.iteration % 1000 == 0:
            A.sync()
            curve.append((t.iteration, time.perf_counter() - t0 - paused, t.splat_count))
        if eval_every > 0 and t.iteration % eval_every == 0:
            A.sync()
            p0 = time.perf_counter()
            psnr_curve.append((t.iteration, p0 - t0 - paused, held_out_psnr(t, test_imgs)))
            paused += time.perf_counter() - p0
    A.sync()
    wall = time.perf_counter() - t0 - paused
    ev = t.evaluate()
    # per-stage times: a few more steps with CUDA events between the stages
    L = A._lib()
    e = L.msplat_trainer_engine(t.h)
    L.msplat_engine_set_timing(e, 1)
    for _ in range(timing_steps):
        t.step()
    A.sync()
    st = N.MsplatEngineStats()
    L.msplat_engine_stats(e, ctypes.byref(st))
    L.msplat_engine_set_timing(e, 0)
    stage_ms = {name: st.stage_ms[i] / max(1, st.timed_steps) for i, name in enumerate(N.STAGES)}
    load = raster_load(L, e, cams[1].width, cams[1].height, stage_ms["raster_bwd"])
    if profile_step:
        import torch
        torch.cuda.profiler.start()
        t.step()
        A.sync()
        torch.cuda.profiler.stop()
    return {"workload": f"{iters} iterations from {n_init:,} random points, MCMC to the {cap:,} cap, 160 train + "
                        "20 held-out views at 1297x840 (synthetic 1M + 200k GT scene), public trainer API",
            "iters_per_s": iters / wall, "wall_s": wall, "final_gaussians": t.splat_count,
            "held_out_psnr": ev["psnr"], "held_out_ssim": ev["ssim"], "held_out_l1": ev["l1"],
            "num_test": ev["num_test"], "curve": curve, "stage_ms_at_end": stage_ms, "trained_view": load,
            "mcmc_rounds": t.mcmc_stats()["rounds"], "learned": bool(learned), "batch_views": batch,
            "psnr_curve": psnr_curve}


def raster_load(L, e, W, H, bwd_ms):
    """Tile lists and backward (pixel, splat) pairs of the engine's last step
    (a W x H view): per pixel inside the image, from min(last contributor,
    tile end - 1) down to the tile's first splat, the walk of the
    reference's rasterize_backward_kernel (msplat_metal.metal:931-1135);
    the FP32 rate counts 60 flops per pair."""
    tx = (W + 15) // 16
    T = tx * ((H + 15) // 16)
    offs = np.zeros(T + 1, np.uint32)
    fidx = np.zeros(W * H, np.int32)
    L.msplat_engine_read(e, b"tile_offsets", offs.ctypes.data, offs.nbytes)
    L.msplat_engine_read(e, b"final_idx", fidx.ctypes.data, fidx.nbytes)
    offs = offs.astype(np.int64)
    counts = np.diff(offs)
    y, x = np.mgrid[0:H, 0:W]
    tile = (y // 16) * tx + (x // 16)
    s, end = offs[tile], offs[tile + 1]
    pairs = int(np.maximum(0, np.minimum(end - 1, fidx.reshape(H, W).astype(np.int64)) - s + 1).sum())
    return {"width": W, "height": H, "intersections": int(offs[-1]), "max_tile": int(counts.max()),
            "mean_tile": float(counts.mean()), "pairs_bwd": pairs, "pairs_per_intersection": pairs / max(1, int(offs[-1])),
            "raster_bwd_tflops_fp32": pairs * 60 / (bwd_ms * 1e-3) / 1e12}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--iters", type=int, default=7000)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--init", type=int, default=100_000)
    ap.add_argument("--learned", action="store_true", help="with the learned relocation proposal")
    ap.add_argument("--batch-views", type=int, default=1, help="views per optimizer step")
    ap.add_argument("--profile-step", action="store_true",
                    help="one more eager step inside cudaProfilerStart/Stop (ncu --profile-from-start off)")
    a = ap.parse_args(argv)
    print(json.dumps(run(a.iters, a.seed, a.init, profile_step=a.profile_step, learned=a.learned,
                         batch=a.batch_views)), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
