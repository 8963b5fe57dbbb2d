"""Time-to-PSNR of the learned relocation proposal against plain
opacity-weighted MCMC relocation, on the small synthetic scene.

    python -m msplat_gb300.relocation_ab [--iters 6000] [--seed 0] [--arms plain,learned,batch4x3_learned]

Scene: 16,384 ground-truth Gaussians (synthetic.config_small), 8 training
views at 256x256 and 4 held-out views between them, targets rendered by the
engine.  Both arms start from the same seed points (jittered ground-truth
means, colours from the ground truth) and the same configuration (MCMC cap
32,768, black background); the learned arm switches the proposal on.
Held-out PSNR is measured every `--eval-every` steps outside the timed
training time.  Time-to-PSNR: the training wall-clock at which each arm
first reaches the plain arm's final PSNR minus 0.1 dB.  Optional arms
`batchB[xS][_learned]` train with B views per optimizer step (the mean
gradient of B cameras, one update, learning rates x S, default
`--batch-lr-scale` or B ** 0.75); iterations count views, so every arm sees
the same number of views.  Prints one JSON
line.
"""
from __future__ import annotations

import argparse
import json
import math
import sys
import time

import numpy as np


def _scene(seed):
    from . import engine as E
    from . import synthetic as S
    sc = S.config_small(seed)
    test = S.ring_cameras(4, 256, 256, 205.0, phase=np.pi / 8, height_z=0.8)
    eng = E.Engine(0)
    dg = E.DeviceGaussians(sc.gt)
    imgs = []
    for c in list(sc.train_cams) + list(test):
        eng.render(dg, E.make_args(E.camera_dict(c), {"degrees_to_use": 3}))
        img = eng.read("out_img", np.float32, 256 * 256 * 3).reshape(256, 256, 3)
        imgs.append((np.clip(img, 0, 1) * 255 + 0.5).astype(np.uint8))
    eng.close()
    rng = np.random.default_rng(seed + 1)
    xyz = (sc.gt.means + rng.normal(0, 0.05, sc.gt.means.shape)).astype(np.float32)
    col = np.clip((sc.gt.features_dc * 0.28209479177387814 + 0.5) * 255.0, 0, 255).astype(np.uint8)
    return list(sc.train_cams) + list(test), imgs, xyz, col


def run_arm(cams, imgs, xyz, col, learned, iters, eval_every, batch=1, lr_scale=0.0):
    import torch
    from . import api as A
    # the last 4 views are held out: train on the first 8, evaluate the others by pose
    ds = A.Dataset.from_arrays(cams[:8], imgs[:8], xyz, col)
    cfg = A.TrainingConfig(iterations=iters, cap_max=32768, bg_color=[0.0, 0.0, 0.0])
    t = A.GaussianTrainer(ds, cfg)
    if learned:
        t.set_learned_relocation(True)
    if batch > 1:
        t.set_batch_views(batch, lr_scale)

    def held_out_psnr():
        vals = []
        for c, gt in zip(cams[8:], imgs[8:]):
            img = t.render_from_pose(np.asarray(c.cam_to_world, np.float32), 0)
            mse = float(np.mean((img.astype(np.float64) - gt.astype(np.float64) / 255.0) ** 2))
            vals.append(10 * math.log10(1.0 / max(mse, 1e-12)))
        return float(np.mean(vals))

    curve = []
    train_s = 0.0
    torch.cuda.synchronize()
    while t.iteration < iters:
        t0 = time.perf_counter()
        stop = min(iters, t.iteration + eval_every)   # iterations count views
        while t.iteration < stop:
            t.step()
        A.sync()
        train_s += time.perf_counter() - t0
        curve.append((t.iteration, train_s, held_out_psnr()))
    out = {"curve": curve, "final_psnr": curve[-1][2], "train_s": train_s, "splats": t.splat_count}
    if learned:
        out["proposal"] = t.learned_stats()
    return out


def time_to(curve, target):
    for step, s, p in curve:
        if p >= target:
            return step, s
    return None, None


def _arm_spec(name, default_lr=0.0):
    """'plain' | 'learned' | 'batch<B>[x<lr scale>][_learned]' -> (learned, B, lr scale)"""
    learned = name.endswith("learned")
    base = name[:-len("_learned")] if name.endswith("_learned") else name
    if base.startswith("batch"):
        spec = base[len("batch"):]
        if "x" in spec:
            b, lr = spec.split("x", 1)
            return learned, int(b), float(lr)
        return learned, int(spec), default_lr
    if base in ("plain", "learned"):
        return learned, 1, 0.0
    raise ValueError(f"unknown arm {name!r}")


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--iters", type=int, default=6000)
    ap.add_argument("--eval-every", type=int, default=250)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--arms", default="plain,learned", help="comma-separated; the first is the target's source")
    ap.add_argument("--batch-lr-scale", type=float, default=0.0, help="learning-rate factor of batch arms (0: B ** 0.75)")
    a = ap.parse_args(argv)
    names = [x.strip() for x in a.arms.split(",") if x.strip()]
    if "plain" not in names:
        names.insert(0, "plain")
    names.remove("plain")
    names.insert(0, "plain")
    cams, imgs, xyz, col = _scene(a.seed)
    runs = {}
    for nm in names:
        learned, b, lr = _arm_spec(nm, a.batch_lr_scale)
        runs[nm] = run_arm(cams, imgs, xyz, col, learned, a.iters, a.eval_every, batch=b, lr_scale=lr)
    plain = runs["plain"]
    target = plain["final_psnr"] - 0.1
    ps, pt = time_to(plain["curve"], target)
    res = {"workload": "learned vs plain MCMC relocation, 16,384-Gaussian synthetic scene, 8 train + 4 held-out "
                       "views at 256x256, cap 32,768", "iters": a.iters, "target_psnr": target}
    for nm, r in runs.items():
        st, tt = time_to(r["curve"], target)
        res[nm] = {"final_psnr": r["final_psnr"], "train_s": r["train_s"], "time_to_target_s": tt,
                   "step_to_target": st, "splats": r["splats"]}
        if "proposal" in r:
            res[nm]["proposal"] = r["proposal"]
        if nm != "plain":
            res[nm]["time_ratio"] = (tt / pt) if (tt is not None and pt) else None
    if "learned" in runs:
        res["time_ratio"] = res["learned"]["time_ratio"]
    res["curves"] = {nm: r["curve"] for nm, r in runs.items()}
    print(json.dumps(res), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
