"""Time-to-PSNR of the learned relocation proposal against plain
opacity-weighted MCMC relocation, on the small synthetic scene.

    python -m msplat_gb300.relocation_ab [--iters 6000] [--seeds 0,1,2,3,4]
        [--arms plain,learned,batch4x3,batch4x3_learned]

Scene: 16,384 ground-truth Gaussians (synthetic.config_small), 8 training
views at 256x256 and 4 held-out views between them, targets rendered by the
engine.  Both arms start from the same seed points (jittered ground-truth
means, colours from the ground truth) and the same configuration (MCMC cap
32,768, black background); the learned arm switches the proposal on (source
weighting and forecast pruning; `learned_noprune`: source weighting only).
Held-out PSNR is measured every `--eval-every` steps outside the timed
training time.  Reported per arm against its plain counterpart (`plain` for
the one-view arms, the same batch arm without `_learned` for a batched
learned arm): the held-out PSNR at the fixed iteration count (the gain per
seed: mean, sd and seeds won), and time-to-PSNR, the training wall-clock at
which the arm first reaches its counterpart's final PSNR minus 0.1 dB, per
seed and as mean and sd over seeds.  Optional arms
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


def _scene(seed, init="jitter", n_init=4096):
    """Targets of the small synthetic scene and the seed points: the ground
    truth's means jittered (init="jitter"), or n_init points uniform in the
    unit ball with random colours (init="random": most die early, so MCMC
    relocation and growth do much of the work)."""
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
    if init == "random":
        d = rng.normal(size=(n_init, 3))
        xyz = (d / np.linalg.norm(d, axis=1, keepdims=True) * rng.random((n_init, 1)) ** (1 / 3)).astype(np.float32)
        col = rng.integers(0, 256, (n_init, 3), dtype=np.uint8)
    else:
        xyz = (sc.gt.means + rng.normal(0, 0.05, sc.gt.means.shape)).astype(np.float32)
        col = np.clip((sc.gt.features_dc * 0.28209479177387814 + 0.5) * 255.0, 0, 255).astype(np.uint8)
    return list(sc.train_cams) + list(test), imgs, xyz, col


def run_arm(cams, imgs, xyz, col, learned, iters, eval_every, batch=1, lr_scale=0.0, prune=None):
    import torch
    from . import api as A
    # the last 4 views are held out: train on the first 8, evaluate the others by pose
    ds = A.Dataset.from_arrays(cams[:8], imgs[:8], xyz, col)
    cfg = A.TrainingConfig(iterations=iters, cap_max=32768, bg_color=[0.0, 0.0, 0.0])
    t = A.GaussianTrainer(ds, cfg)
    if learned:
        t.set_learned_relocation(True)
        if prune is not None:
            t.set_learned_prune(prune)
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
        out["proposal"].update(t.learned_eval())
    return out


def time_to(curve, target):
    for step, s, p in curve:
        if p >= target:
            return step, s
    return None, None


def _arm_spec(name, default_lr=0.0):
    """'plain' | 'learned' | 'learned_noprune' | 'batch<B>[x<lr scale>][_learned]' -> (learned, B, lr scale)"""
    if name == "learned_noprune":
        return True, 1, 0.0
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


def compare(cams, imgs, xyz, col, names, iters, eval_every, batch_lr_scale=0.0):
    """Runs every arm on one scene.  The target of each arm is the final PSNR
    of its plain counterpart minus 0.1 dB: `plain` for the one-view arms,
    `batch<B>...` without `_learned` for the batched learned arms."""
    runs = {}
    for nm in names:
        learned, b, lr = _arm_spec(nm, batch_lr_scale)
        runs[nm] = run_arm(cams, imgs, xyz, col, learned, iters, eval_every, batch=b, lr_scale=lr,
                           prune=0.0 if nm == "learned_noprune" else None)
    res = {}
    for nm, r in runs.items():
        base = nm[:-len("_learned")] if nm.endswith("_learned") else nm
        if base in ("learned", "learned_noprune"):
            base = "plain"
        ref = runs.get(base, runs["plain"])
        target = ref["final_psnr"] - 0.1
        _, t_ref = time_to(ref["curve"], target)
        st, tt = time_to(r["curve"], target)
        res[nm] = {"final_psnr": r["final_psnr"], "train_s": r["train_s"], "time_to_target_s": tt,
                   "step_to_target": st, "splats": r["splats"], "vs": base, "target_psnr": target,
                   "time_ratio": (tt / t_ref) if (tt is not None and t_ref) else None,
                   # area under the held-out PSNR curve per evaluation (a deterministic proxy)
                   "mean_psnr": float(np.mean([p for _, _, p in r["curve"]])),
                   "curve": r["curve"]}
        if "proposal" in r:
            res[nm]["proposal"] = r["proposal"]
    return res


def summarize(per_seed, names):
    """mean and sd over seeds of each arm's time ratio, final and mean PSNR,
    and its held-out PSNR at the fixed iteration count against its plain
    counterpart's (the gain per seed: mean, sd, seeds won)."""
    out = {}
    for nm in names:
        rows = [ps[nm] for ps in per_seed]
        ratios = [r["time_ratio"] for r in rows if r["time_ratio"] is not None]
        gains = [ps[nm]["final_psnr"] - ps[ps[nm]["vs"]]["final_psnr"] for ps in per_seed if ps[nm]["vs"] in ps]
        out[nm] = {"vs": rows[0]["vs"], "seeds": len(rows), "reached": len(ratios),
                   "time_ratio_mean": float(np.mean(ratios)) if ratios else None,
                   "time_ratio_sd": float(np.std(ratios, ddof=1)) if len(ratios) > 1 else None,
                   "final_psnr_mean": float(np.mean([r["final_psnr"] for r in rows])),
                   "mean_psnr_mean": float(np.mean([r["mean_psnr"] for r in rows])),
                   "final_psnr_gain_mean": float(np.mean(gains)) if gains else None,
                   "final_psnr_gain_sd": float(np.std(gains, ddof=1)) if len(gains) > 1 else None,
                   "final_psnr_wins": int(sum(g > 0 for g in gains))}
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--iters", type=int, default=6000)
    ap.add_argument("--eval-every", type=int, default=250)
    ap.add_argument("--seeds", default="0", help="comma-separated scene seeds")
    ap.add_argument("--arms", default="plain,learned", help="comma-separated arm names")
    ap.add_argument("--batch-lr-scale", type=float, default=0.0, help="learning-rate factor of batch arms (0: B ** 0.75)")
    ap.add_argument("--curves", action="store_true", help="include the PSNR curves")
    ap.add_argument("--init", default="jitter", choices=["jitter", "random"],
                    help="seed points: jittered ground truth, or random points in the unit ball")
    ap.add_argument("--n-init", type=int, default=4096, help="random seed points (--init random)")
    a = ap.parse_args(argv)
    names = [x.strip() for x in a.arms.split(",") if x.strip()]
    if "plain" in names:
        names.remove("plain")
    names.insert(0, "plain")
    seeds = [int(x) for x in a.seeds.split(",") if x.strip()]
    per_seed = []
    for sd in seeds:
        cams, imgs, xyz, col = _scene(sd, a.init, a.n_init)
        per_seed.append(compare(cams, imgs, xyz, col, names, a.iters, a.eval_every, a.batch_lr_scale))
    res = {"workload": "learned vs plain MCMC relocation, 16,384-Gaussian synthetic scene, 8 train + 4 held-out "
                       "views at 256x256, cap 32,768", "iters": a.iters, "seeds": seeds,
           "init": a.init, "summary": summarize(per_seed, names)}
    if not a.curves:
        for ps in per_seed:
            for r in ps.values():
                r.pop("curve", None)
    res["per_seed"] = per_seed
    print(json.dumps(res), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
