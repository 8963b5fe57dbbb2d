"""Command-line training driver: `python -m msplat_gb300.cli <dataset> [options]`.

The options and the run follow the reference's `msplat` CLI (cli/msplat.mm)
and `msplat-train` (python/msplat/cli.py): load a COLMAP / Nerfstudio /
Polycam dataset, train with MCMC densification to --num-iters, optionally
resume from a trained PLY, save every N steps, stop early when the held-out
PSNR stops improving (two consecutive 5000-step gates below --early-stop dB,
from step 10000, needs --eval), export PLY or .splat, evaluate PSNR / SSIM /
L1 on the held-out views and write their renders.  Everything runs through
the library's C API; no training math lives here.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import struct
import sys
import time
import zlib

import numpy as np

from . import api as A


def _write_png(path: str, rgb: np.ndarray):
    """8-bit RGB PNG (filter 0 rows, zlib) for the evaluation renders."""
    img = np.clip(np.round(rgb * 255.0), 0, 255).astype(np.uint8) if rgb.dtype != np.uint8 else rgb
    h, w, _ = img.shape
    raw = b"".join(b"\x00" + img[y].tobytes() for y in range(h))

    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF)

    data = (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0)) +
            chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b""))
    with open(path, "wb") as f:
        f.write(data)


def _psnr(img: np.ndarray, gt_u8: np.ndarray) -> float:
    mse = float(np.mean((img.astype(np.float64) - gt_u8.astype(np.float64) / 255.0) ** 2))
    return 10.0 * math.log10(1.0 / max(mse, 1e-12))


def parse(argv=None):
    p = argparse.ArgumentParser(prog="msplat", description="Train 3D Gaussian Splatting on a dataset (GB300).")
    p.add_argument("input", help="dataset (COLMAP, Nerfstudio, Polycam)")
    p.add_argument("-o", "--output", default="splat.ply", help="output scene (.ply or .splat)")
    p.add_argument("-s", "--save-every", type=int, default=-1, help="save every N steps (-1 to disable)")
    p.add_argument("--resume", default="", help="resume training from a PLY file")
    p.add_argument("--val", action="store_true", help="withhold a camera for validation")
    p.add_argument("--val-image", default="random", help="validation image (file name substring, or random)")
    p.add_argument("--val-render", default="", help="directory for the validation camera's render every 10 steps")
    p.add_argument("--eval", action="store_true", help="evaluate on held-out test views")
    p.add_argument("--test-every", type=int, default=8, help="hold out every Nth image for eval")
    p.add_argument("--eval-render", default="", help="directory for each eval view's render and ground truth (PNG)")
    p.add_argument("-n", "--num-iters", type=int, default=30000, help="number of iterations")
    p.add_argument("-d", "--downscale-factor", type=float, default=1.0, help="image downscale factor")
    p.add_argument("--sh-degree", type=int, default=3, help="max spherical harmonics degree")
    p.add_argument("--sh-degree-interval", type=int, default=1000, help="increase SH degree every N steps")
    p.add_argument("--ssim-weight", type=float, default=0.2, help="SSIM loss weight (0 = L1 only)")
    p.add_argument("--cap-max", type=int, default=1_000_000, help="maximum Gaussian budget")
    p.add_argument("--noise-lr", type=float, default=5e5, help="SGLD noise learning rate")
    p.add_argument("--opacity-reg", type=float, default=0.01, help="opacity regularization weight")
    p.add_argument("--scale-reg", type=float, default=0.01, help="scale regularization weight")
    p.add_argument("--cull-radius", type=float, default=3.0, help="cull splats with |mean| > r (0 = off)")
    p.add_argument("--keep-crs", action="store_true", help="export in the input coordinate system")
    p.add_argument("--bg-color", type=float, nargs=3, default=[0.6130, 0.0101, 0.3984], help="background RGB (0-1)")
    p.add_argument("--colmap-image-path", default="", help="override the COLMAP image directory")
    p.add_argument("--mask-dir", default="",
                   help="training masks: <dir>/<image name>.png (or the name's extension swapped); "
                        "white = train, black = ignore (COLMAP datasets)")
    p.add_argument("--early-stop", type=float, default=0.0,
                   help="stop when test-subset PSNR improves less than this (dB) over 5000 steps (needs --eval)")
    p.add_argument("--reg-visibility-duty", type=float, default=1.0,
                   help="scale of the opacity/scale regularizer for Gaussians not seen in a step (1 = full)")
    p.add_argument("--no-seed-decimation", action="store_true",
                   help="keep every seed point (no 50%% subsample above 75%% of --cap-max)")
    p.add_argument("--position-lr-max-steps", type=int, default=30000,
                   help="steps over which the position learning rate decays")
    p.add_argument("--init-opacity", type=float, default=0.5, help="seed opacity at init")
    p.add_argument("--init-scale", type=float, default=0.1, help="seed scale multiplier on the kNN spacing")
    p.add_argument("--log-every", type=int, default=100, help="print progress every N steps")
    p.add_argument("--batch-views", type=int, default=1,
                   help="cameras per optimizer step (mean gradient; iterations count views; 1 = one camera per step)")
    p.add_argument("--batch-lr-scale", type=float, default=0.0,
                   help="learning-rate factor of multi-view steps (0 = batch views ** 0.75)")
    p.add_argument("--isect-budget", type=float, default=0.0,
                   help="fixed intersection buffers in bytes per Gaussian of --cap-max (the reference's "
                        "MSPLAT_ISECT_BUDGET, e.g. 1000); larger views are rastered in tile groups; 0 = legacy")
    p.add_argument("--autotune", action="store_true",
                   help="time the engine's launch configurations on the first training views and keep the fastest")
    p.add_argument("--learned-relocation", action="store_true",
                   help="online-trained proposal MLP: weights MCMC relocation sources and relocates the "
                        "Gaussians it forecasts to fade")
    p.add_argument("--learned-prune", type=float, default=None,
                   help="forecast-pruning threshold of the learned proposal (forecast opacity; 0 = off; "
                        "default 0.02)")
    a = p.parse_args(argv)
    a.downscale_factor = max(a.downscale_factor, 1.0)
    return a


def save_cameras(path: str, ds: A.Dataset, keep_crs: bool, test_every: int = 0, held: int = -1) -> None:
    """cameras.json as the reference writes it next to the scene
    (InputData::saveCameras, core/src/input_data.cpp:209-240): every camera
    in the loader's order with its image file name, size, intrinsics,
    rotation (OpenCV axes: the pose's columns 1 and 2 negated back) and
    position (in the dataset's own frame with keep_crs).  test_every: the
    eval split the dataset was made with; held: the --val camera's index."""
    n = ds.num_train + ds.num_test
    order = []
    if test_every > 0:
        t = r = 0
        for i in range(n):
            if i % test_every == 0:
                order.append((True, t)); t += 1
            else:
                order.append((False, r)); r += 1
    else:
        order = [(False, i) for i in range(ds.num_train)]
        if held >= 0:
            order.insert(held, (True, 0))
    scale, tr = ds.transform
    out = []
    for use_test, i in order:
        c = ds.camera(i, use_test)
        m = np.asarray(c["cam_to_world"], np.float32).reshape(4, 4)
        R = m[:3, :3].copy()
        R[:, 1:] *= np.float32(-1.0)
        T = m[:3, 3].copy()
        if keep_crs:
            T = T / np.float32(scale) + tr
        fx, fy, cx, cy = (float(np.float32(c[k])) for k in ("fx", "fy", "cx", "cy"))
        out.append({"file_path": os.path.basename(ds.camera_file(i, use_test)), "width": int(c["width"]),
                    "height": int(c["height"]), "fx": fx, "fy": fy, "cx": cx, "cy": cy,
                    "rotation": [[float(v) for v in row] for row in R], "translation": [float(v) for v in T]})
    with open(path, "w") as f:
        json.dump(out, f, indent=2, sort_keys=True)


def _save(trainer: A.GaussianTrainer, path: str):
    if path.endswith(".splat"):
        trainer.export_splat(path)
    else:
        trainer.export_ply(path)


def main(argv=None) -> int:
    a = parse(argv)
    t0 = time.time()
    ds = A.Dataset(a.input, downscale_factor=a.downscale_factor, eval_mode=a.eval, test_every=a.test_every,
                   colmap_image_path=a.colmap_image_path or None, mask_dir=a.mask_dir or None)
    print(f"Loaded {ds.num_train} train cameras" + (f", {ds.num_test} test cameras" if a.eval else "") +
          f" in {time.time() - t0:.1f} s", flush=True)
    # validation camera (the reference CLI: --val-render implies --val; eval mode splits instead)
    val = (a.val or bool(a.val_render)) and not a.eval
    held = -1
    if val:
        held = ds.hold_out(a.val_image)
        if a.val_render:
            os.makedirs(a.val_render, exist_ok=True)
    cfg = A.TrainingConfig(iterations=a.num_iters, sh_degree=a.sh_degree, sh_degree_interval=a.sh_degree_interval,
                           ssim_weight=a.ssim_weight, cap_max=a.cap_max, noise_lr=a.noise_lr,
                           opacity_reg=a.opacity_reg, scale_reg=a.scale_reg, cull_radius=a.cull_radius,
                           keep_crs=a.keep_crs, downscale_factor=a.downscale_factor, bg_color=list(a.bg_color),
                           output=a.output, save_every=a.save_every)
    opts = A.TrainerOptions(init_opacity=a.init_opacity, init_scale_mult=a.init_scale,
                            seed_decimation=not a.no_seed_decimation,
                            position_lr_max_steps=a.position_lr_max_steps,
                            reg_visibility_duty=a.reg_visibility_duty)
    trainer = A.GaussianTrainer(ds, cfg, opts if opts != A.TrainerOptions() else None)
    if a.batch_views > 1:
        trainer.set_batch_views(a.batch_views, a.batch_lr_scale)
    if a.learned_relocation:
        trainer.set_learned_relocation(True)
        if a.learned_prune is not None:
            trainer.set_learned_prune(a.learned_prune)
    if a.isect_budget > 0:
        trainer.set_isect_budget(a.isect_budget)
    if a.autotune:
        print(f"Launch configuration: {trainer.autotune()}", flush=True)
    if a.resume:
        step0 = trainer.load_ply(a.resume)
        print(f"Resumed from {a.resume} at step {step0}", flush=True)
    if ds.num_train == 0 and trainer.iteration < a.num_iters:
        print("No training views (--test-every 1) but training steps were requested", file=sys.stderr)
        return 1
    last_gate, misses, stopped = -1e9, 0, 0
    t_start = time.time()

    def crossed(prev, cur, period):   # a period boundary in (prev, cur]: steps may advance by several views
        return period > 0 and cur // period > prev // period

    while trainer.iteration < a.num_iters:
        prev = trainer.iteration
        s = trainer.step()
        step = s.iteration
        if crossed(prev, step, a.log_every):
            el = time.time() - t_start
            print(f"step={step:>6}  splats={s.splat_count:>9,}  loss={trainer.last_loss:.5f}  "
                  f"ms={s.ms_per_step:.2f}  elapsed={el:.1f}s", flush=True)
        if crossed(prev, step, a.save_every):
            root, ext = os.path.splitext(a.output)
            _save(trainer, f"{root}_{step}{ext or '.ply'}")
        if val and a.val_render and crossed(prev, step, 10):
            _write_png(os.path.join(a.val_render, f"{step}.png"), trainer.render(0, use_test=True))
        if (a.early_stop > 0 and a.eval and ds.num_test > 0 and step >= 10000 and crossed(prev, step, 5000) and
                step < a.num_iters):
            n_sub = min(30, ds.num_test)
            stride = max(1, ds.num_test // n_sub)
            vals = [_psnr(trainer.render(i, use_test=True), ds.camera(i, use_test=True)["image"])
                    for i in range(0, ds.num_test, stride)][:n_sub]
            gate = float(np.mean(vals))
            msg = f"[early-stop] step={step} subset_psnr={gate:.4f}"
            if last_gate > -1e8:
                msg += f" delta={gate - last_gate:.4f}"
            print(msg, flush=True)
            if last_gate > -1e8 and gate - last_gate < a.early_stop:
                misses += 1
                if misses >= 2:
                    print(f"early-stop: two gates below {a.early_stop} dB per 5000 steps; stopping at step {step}")
                    stopped = step
            else:
                misses = 0
            last_gate = gate
            if stopped:
                break
    save_cameras(os.path.join(os.path.dirname(a.output) or ".", "cameras.json"), ds, a.keep_crs,
                 a.test_every if a.eval else 0, held)
    _save(trainer, a.output)
    print(f"Saved {a.output} ({trainer.splat_count:,} Gaussians, {time.time() - t_start:.1f} s of training)")
    if a.eval and ds.num_test > 0:
        m = trainer.evaluate()
        print(f"\n=== Evaluation ({m['num_test']} test views) ===")
        print(f"  PSNR:  {m['psnr']:.4f}")
        print(f"  SSIM:  {m['ssim']:.4f}")
        print(f"  L1:    {m['l1']:.4f}")
        print(f"  Gaussians: {m['num_gaussians']:,}")
        if a.eval_render:
            os.makedirs(a.eval_render, exist_ok=True)
            for i in range(ds.num_test):
                _write_png(os.path.join(a.eval_render, f"test_{i:04d}.png"), trainer.render(i, use_test=True))
                _write_png(os.path.join(a.eval_render, f"test_{i:04d}_gt.png"), ds.camera(i, use_test=True)["image"])
    A.cleanup()
    return 0


if __name__ == "__main__":
    sys.exit(main())
