#!/usr/bin/env python3
"""Training-step benchmark of the msplat GB300 engine.

Workload (one step = one training iteration, Model::fullIteration):
  1,000,000 Gaussians (SH degree 3), one 1297x840 view per step, L1+0.2*SSIM
  loss, backward, fused SH Adam, regularizer + Adam, SGLD, on a synthetic
  scene: 1M GT Gaussians + 200k ground-plane Gaussians (synthetic.config_full),
  ring/elevation-jittered cameras, targets rendered from the GT scene by the
  engine's forward pass.  The trained model is a 1M subset of the GT scene
  with jittered means (the steady state of a run at its 1M cap), training
  steps 3001.. (all SH bands active, regularizer and SGLD on).

Arms:
  default            the CUDA engine.  `value` = iterations/s with the targets
                     resident in HBM; `e2e` = the same through the C ABI with
                     the target image copied from pinned host memory each step
                     and the loss read back.
  --impl reference   the reference's own implementation cannot run here
                     (Metal only), so the arm times the CPU restatement of it
                     (oracle/, FP64, OpenMP on all host cores) on the same
                     workload, one full iteration per step.

Also reported:
  batched        the multi-view step on the same model, 8 views of mixed sizes
                 per step (2 each of 1297x840, 979x546, 648x420 and 2594x1680,
                 same camera poses, focal length scaled with the width), one
                 launch per stage over all views, as a captured graph;
  e2e_trainer    iterations/s through the reference's public trainer API
                 (msplat_trainer_step), the model resumed at iteration 3001
                 from a checkpoint, MCMC rounds inside the timed region;
  time_to_psnr   learned vs plain relocation (and learned + batched vs plain
                 + batched) on the small scene over five seeds: held-out
                 PSNR at the fixed iteration count and time to PSNR;
  full_run       the full configuration trained from 100k random points to
                 the 1M cap over 7000 iterations, with held-out PSNR / SSIM;
                 full_run_learned and full_run_learned_batched the same with
                 the learned relocation proposal, alone and with 4 views per
                 step: held-out PSNR gain and time to the plain run's final
                 PSNR - 0.1 dB;
  roofline.fp32  the rasterizer backward's FP32-pipe fraction from the
                 (pixel, splat) pairs the reference's algorithm walks.

Under torchrun (N > 1) every rank trains its own replica on its own GPU
("replicas only": the step has no cross-GPU exchange).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "train iters/s & ms/step at 1M splats 1297×840 vs CPU oracle; learned vs plain time-to-PSNR"
N_MODEL = 1_000_000
VIEWS = 8

# Algorithmic bytes per unit (per Gaussian / intersection / pixel) of each
# stage, SH degree 3: what the stage must read and write at minimum.
STAGE_BYTES = {
    "project": dict(g=284),                      # params 232 B in, projection 52 B out
    "tiles": dict(g=52, i=20),                   # count/scatter; key write 8, key read 8, id write 4 per intersection
    "raster_fwd": dict(i=40, p=20),              # id 4 + record gather 36 per intersection
    "loss": dict(p=27),
    "raster_bwd": dict(i=80, p=20),              # id 4 + record gather 40 + gradient read-modify-write 36
    "project_bwd": dict(g=1284),                 # incl. SH Adam on 48 coefficients
    "adam": dict(g=368),                         # 4 groups (308) + regularizer (60)
    "sgld": dict(g=80),
}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    from msplat_gb300 import replicas
    return replicas.dist_env()


def build_workload(seed=0, n_model=N_MODEL, views=VIEWS):
    import numpy as np
    from msplat_gb300 import synthetic as S
    sc = S.config_full(seed, n_train=views, n_test=0)
    rng = np.random.default_rng(seed + 5)
    sel = np.sort(rng.choice(sc.gt.n, n_model, replace=False))
    model = S.GaussianSet(*(np.ascontiguousarray(a[sel]) for a in sc.gt.arrays()))
    model.means += rng.normal(0.0, 0.01, model.means.shape).astype(np.float32)
    return sc, model


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()

    def summary(self):
        self.f.flush()
        rows = []
        try:
            with open(self.f.name) as fh:
                for line in fh:
                    parts = [x.strip() for x in line.split(",")]
                    if len(parts) >= 9:
                        rows.append(parts)
        except OSError:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def oracle_camera(cam):
    """Camera dict of a synthetic camera, matrices from the oracle's
    prepare_cam (Model::prepareCam, core/src/model.cpp:845-889): the CPU arms
    never load the engine library."""
    from oracle import oracle as O
    vm, pm, cp = O.prepare_cam(cam.cam_to_world, cam.width, cam.height, cam.fx, cam.fy)
    return dict(viewmat=vm, projmat=pm, cam_pos=cp, fx=cam.fx, fy=cam.fy, cx=cam.cx, cy=cam.cy,
                width=cam.width, height=cam.height)


def cpu_baseline(model, cam, gt, steps=4):
    """FP64 oracle (OpenMP, all host cores) timed on full iterations of the workload."""
    import numpy as np
    from msplat_gb300.schedule import step_scalars
    from oracle import oracle as O
    cd = oracle_camera(cam)
    g = model.copy()
    mom = ([np.zeros_like(a) for a in g.arrays()], [np.zeros_like(a) for a in g.arrays()])
    times = []
    for k in range(steps):
        st = step_scalars(3001 + k, 3001 + k, width=cam.width, height=cam.height)
        t0 = time.perf_counter()
        O.train_step(64, g, cd, st, moments=mom, gt=gt, do_sgld=True, want_ids=False)
        times.append(time.perf_counter() - t0)
    sec = statistics.median(times[1:] if len(times) > 2 else times)
    return {"value": 1.0 / sec, "unit": "iters/s", "cores": O.num_threads(), "kind": "port",
            "sample": f"{len(times)} full FP64 iterations of the workload (1M Gaussians, 1297x840, view 0), "
                      f"median {sec:.2f} s/iter"}


def run_reference(args):
    """--impl reference: the CPU restatement of the reference step (oracle).

    Camera matrices, step scalars, scene and targets all come from the oracle
    and pure-Python helpers: the engine library is never loaded by this arm."""
    import numpy as np
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from msplat_gb300.schedule import step_scalars
    from oracle import oracle as O
    sc, model = build_workload()
    cam = sc.train_cams[0]
    cd = oracle_camera(cam)
    ref = O.train_step(64, sc.gt.copy(), cd, {"degrees_to_use": 3}, do_backward=False, do_optimizer=False,
                       want_ids=False)
    gt = (np.clip(ref["out_img"], 0, 1) * 255 + 0.5).astype(np.uint8)
    g = model.copy()
    mom = ([np.zeros_like(a) for a in g.arrays()], [np.zeros_like(a) for a in g.arrays()])

    def step(k):
        st = step_scalars(3001 + k, 3001 + k, width=cam.width, height=cam.height)
        O.train_step(64, g, cd, st, moments=mom, gt=gt, do_sgld=True, want_ids=False)

    for k in range(args.warmup):
        step(k)
    t0 = time.perf_counter()
    for k in range(args.steps):
        step(args.warmup + k)
    sec = (time.perf_counter() - t0) / max(1, args.steps)
    v = 1.0 / sec
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": "iters/s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": config_dict(args),
           "cpu_baseline": {"value": v, "unit": "iters/s", "cores": O.num_threads(), "kind": "port",
                            "sample": "full FP64 iterations of the workload (the reference is Metal-only: "
                                      "unavailable on this box; its CPU restatement is timed)"},
           "e2e": {"value": v, "unit": "iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    loaded = loaded_libraries()
    if loaded is not None:
        out["libraries_loaded"] = loaded
        if any("libmsplat_gb300" in x for x in loaded):
            raise RuntimeError("the reference arm loaded the engine library")
    print(json.dumps(out), flush=True)
    return 0


def loaded_libraries():
    """This project's shared libraries mapped into the process (Linux), or None."""
    try:
        with open("/proc/self/maps") as f:
            paths = {line.split()[-1] for line in f if line.rstrip().endswith(".so")}
    except OSError:
        return None
    return sorted(os.path.relpath(p, ROOT) for p in paths if p.startswith(ROOT))


def sm_max_mhz():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["sm_max_mhz"])
    except (OSError, KeyError, ValueError):
        return 2070.0


def backward_pairs(eng, cd):
    """(pixel, splat) pairs the reference's backward walks for the engine's
    last step of view cd: per pixel inside the image, from min(last
    contributor, tile end - 1) down to the tile's first splat."""
    import numpy as np
    W, H = cd["width"], cd["height"]
    tx = (W + 15) // 16
    T = tx * ((H + 15) // 16)
    offs = eng.read("tile_offsets", np.uint32, T + 1).astype(np.int64)
    fidx = eng.read("final_idx", np.int32, W * H).reshape(H, W).astype(np.int64)
    y, x = np.mgrid[0:H, 0:W]
    t = (y // 16) * tx + (x // 16)
    s, e = offs[t], offs[t + 1]
    return int(np.maximum(0, np.minimum(e - 1, fidx) - s + 1).sum())


def write_checkpoint(path, model, step, adam_steps):
    """A checkpoint in the reference's format (core/src/model.cpp:698-843) of
    the model with zeroed Adam moments at the given iteration: how the public
    trainer resumes a run (msplat_trainer_load_checkpoint)."""
    import struct
    import numpy as np
    from msplat_gb300.schedule import LR_INIT
    n = model.n
    with open(path, "wb") as f:
        f.write(struct.pack("<6I", 0x4C50534D, 1, step, n, 3, adam_steps))
        f.write(np.asarray(LR_INIT, np.float32).tobytes() + struct.pack("<2f", 0.00016, 0.0000016))
        arrays = list(model.arrays())
        for block in (arrays, [np.zeros_like(a) for a in arrays], [np.zeros_like(a) for a in arrays]):
            for g, a in enumerate(block):
                shape = [n, 15, 3] if g == 4 else ([n, 1] if g == 5 else [n, a.shape[1]])
                data = np.ascontiguousarray(a, np.float32).tobytes()
                f.write(struct.pack("<I", len(shape)) + struct.pack(f"<{len(shape)}q", *shape))
                f.write(struct.pack("<Q", len(data)) + data)


def run_trainer_e2e(sc, model, gts_host, steps):
    """Iterations/s of msplat_trainer_step, the reference's public API, at the
    headline workload: the 1M model resumed at iteration 3001 from a
    checkpoint, the bench's 8 views in the trainer's own shuffled order, its
    learning-rate schedule and MCMC relocation every 100 steps (rounds fall
    in the timed region), wall clock from the first step to the device's
    completion of the last."""
    import time
    import numpy as np
    from msplat_gb300 import api as A
    imgs = [g.numpy() for g in gts_host]
    ds = A.Dataset.from_arrays(sc.train_cams, imgs, model.means[:4096], np.zeros((4096, 3), np.uint8))
    t = A.GaussianTrainer(ds, A.TrainingConfig(iterations=30000, cap_max=model.n, bg_color=[0.0, 0.0, 0.0]))
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "resume.ckpt")
        write_checkpoint(path, model, 3000, 3000)
        assert t.load_checkpoint(path) == 3000
    for _ in range(5):          # warm-up: uploads, graph capture of each camera
        t.step()
    A.sync()
    rounds0 = t.mcmc_stats()["rounds"]
    t0 = time.perf_counter()
    for _ in range(steps):
        t.step()
    A.sync()
    sec = time.perf_counter() - t0
    return {"value": steps / sec, "unit": "iters/s", "steps": steps, "api": "msplat_trainer_step",
            "mcmc_rounds_timed": t.mcmc_stats()["rounds"] - rounds0, "gaussians": t.splat_count,
            "workload": "1M Gaussians resumed at iteration 3001 (checkpoint), 8 views at 1297x840, MCMC every "
                        "100 steps, the trainer's camera order and schedules"}


BATCH_SIZES = [(1297, 840), (979, 546), (648, 420), (2594, 1680)] * 2


def batched_cameras(sc):
    """The batched workload's 8 views: ring poses 0..7, sizes BATCH_SIZES."""
    from msplat_gb300 import synthetic as S
    out = []
    for k, (w, h) in enumerate(BATCH_SIZES):
        c = sc.train_cams[k % len(sc.train_cams)]
        f = c.fx * w / c.width
        out.append(S.Camera(c.cam_to_world, w, h, f, f, 0.5 * w, 0.5 * h))
    return out


def run_batched(eng, E, sc, dg, warmup, steps, step_base):
    """Multi-view steps of the batched workload; returns its JSON object."""
    import numpy as np
    import torch
    cams = [E.camera_dict(c) for c in batched_cameras(sc)]
    gt_dev = E.DeviceGaussians(sc.gt)
    gts = []
    for cd in cams:
        eng.render(gt_dev, E.make_args(cd, {"degrees_to_use": 3}))
        img = eng.read("out_img", np.float32, cd["width"] * cd["height"] * 3)
        gts.append(torch.from_numpy((np.clip(img, 0, 1) * 255 + 0.5).astype(np.uint8)).cuda())
    del gt_dev
    ptrs = [g.data_ptr() for g in gts]

    def one(k):
        args = [E.make_args(cd, E.step_scalars(step_base + k, step_base + k, width=cd["width"], height=cd["height"]),
                            do_sgld=True) for cd in cams]
        eng.train_step_batch(dg, args, ptrs)

    # the launch configuration: tuned on this workload (CUDA events, whole
    # steps without updates), then the timed steps replay the tuned graph
    eng.set_tuning(sort_width=512, raster_batch=128, chunk=512, raster_mode=0, tile_order=1, bwd_pixels=1,
                   tile_split=2)   # the defaults
    untuned = eng.tuning()
    args0 = [E.make_args(cd, E.step_scalars(step_base, step_base, width=cd["width"], height=cd["height"]))
             for cd in cams]
    tuned, tuned_ms = eng.autotune(dg, args0, ptrs, reps=3)
    for k in range(warmup):
        one(k)
    eng.synchronize()
    l0 = eng.stats().launches
    eng.marker(0)
    for k in range(steps):
        one(warmup + k)
    eng.marker(1)
    ms = eng.marker_elapsed() / steps
    launches = (eng.stats().launches - l0) / steps
    # per-stage times from eager steps with events between the stages (an
    # NVTX range names them for profilers: ncu --nvtx --nvtx-include batched_steps/)
    eng.set_timing(True)
    nvtx = getattr(torch.cuda, "nvtx", None)
    if nvtx is not None:
        try:
            nvtx.range_push("batched_steps")
        except Exception:   # a build without NVTX: no range
            nvtx = None
    for k in range(5):
        one(warmup + steps + k)
    eng.synchronize()
    if nvtx is not None:
        nvtx.range_pop()
    st = eng.stats()
    eng.set_timing(False)
    stage_ms = {name: st.stage_ms[i] / max(1, st.timed_steps) for i, name in enumerate(E.N.STAGES)}
    px = sum(w * h for w, h in BATCH_SIZES)
    return {"workload": "8 views per step: 2 each of 1297x840, 979x546, 648x420, 2594x1680 "
                        f"({px / 1e6:.2f} Mpx), {dg.n / 1e6:g}M Gaussians, one launch per stage, CUDA graph",
            "views_per_step": len(cams), "ms_per_step": ms, "iters_per_s": 1e3 / ms,
            "views_per_s": len(cams) * 1e3 / ms, "mpx_per_s": px / 1e6 * 1e3 / ms,
            "launches_per_step": launches, "loss": eng.loss(), "stage_ms": stage_ms,
            "num_intersections": int(st.num_intersections), "tuning": tuned, "untuned": untuned,
            "autotune_step_ms": tuned_ms}


def config_dict(args):
    n = getattr(args, "gaussians", N_MODEL)
    return {"workload": f"{n / 1e6:g}M Gaussians (SH deg 3) training step at 1297x840, synthetic 1M+200k GT scene",
            "n_gaussians": n, "width": 1297, "height": 840, "views": VIEWS, "sh_degree": 3,
            "raster": "monolithic (4346 tiles >= 400)", "l2": "working set > L2 (params+moments 0.7 GB/step)",
            "seed": 0}


def run_engine(args):
    import numpy as np
    import torch
    from msplat_gb300 import engine as E

    from msplat_gb300 import replicas as R
    ws, rank, local = dist_env()
    R.init(ws)
    torch.cuda.set_device(local)
    n_model = args.gaussians
    sc, model = build_workload(n_model=n_model)
    eng = E.Engine(local, n_model)
    cams = [E.camera_dict(c) for c in sc.train_cams]

    # targets: the GT scene rendered by the engine (forward path, parity-tested)
    gt_dev = E.DeviceGaussians(sc.gt)
    gts_host, gts_dev = [], []
    for cd in cams:
        eng.render(gt_dev, E.make_args(cd, {"degrees_to_use": 3}))
        img = eng.read("out_img", np.float32, cd["width"] * cd["height"] * 3).reshape(cd["height"], cd["width"], 3)
        u8 = (np.clip(img, 0, 1) * 255 + 0.5).astype(np.uint8)
        gts_host.append(torch.from_numpy(u8).pin_memory())
        gts_dev.append(torch.from_numpy(u8).cuda())
    del gt_dev
    torch.cuda.synchronize()

    dg = E.DeviceGaussians(model)
    step_base = 3001

    def one(k, host):
        cd = cams[k % len(cams)]
        st = E.step_scalars(step_base + k, step_base + k, width=cd["width"], height=cd["height"])
        a = E.make_args(cd, st, do_sgld=True)
        if host:
            eng.train_step_host(dg, a, gts_host[k % len(cams)].data_ptr())
        else:
            eng.train_step(dg, a, gts_dev[k % len(cams)].data_ptr())

    def barrier():
        R.barrier(ws)

    def max_over_ranks(x):
        return R.max_over_ranks(ws, x)

    # launch configuration: the autotuner times whole steps of this workload
    # (no updates) over its candidates and keeps the fastest
    tuned, tuned_ms = None, None
    if args.tuning:   # a fixed configuration, e.g. "tile_order=1,sort_width=512"
        eng.set_tuning(**{k: int(v) for k, v in (kv.split("=") for kv in args.tuning.split(","))})
        tuned = eng.tuning()
    elif not args.no_autotune:
        cd0 = cams[0]
        a0 = E.make_args(cd0, E.step_scalars(step_base, step_base, width=cd0["width"], height=cd0["height"]))
        tuned, tuned_ms = eng.autotune(dg, [a0], [gts_dev[0].data_ptr()], reps=5)

    # the step runs as a captured CUDA graph: the first step of this shape
    # runs eagerly, the second is captured, later ones replay it
    eng.set_graphs(True)
    for k in range(args.warmup):
        one(k, False)
    eng.synchronize()

    # kernel-only: targets resident in HBM
    launches0 = eng.stats().launches
    with Clocks(local) as clk:
        barrier()
        torch.cuda.synchronize()
        eng.synchronize()
        eng.marker(0)
        for k in range(args.steps):
            one(args.warmup + k, False)
        eng.marker(1)
        dev_ms = eng.marker_elapsed()
        eng.synchronize()
        barrier()
    launches = eng.stats().launches - launches0
    dev_ms = max_over_ranks(dev_ms)
    ms_step = dev_ms / args.steps
    value = R.job_rate(ws, args.steps, dev_ms / 1e3)

    # end to end through the C ABI, every step: the pinned host image in
    # (uploaded on the engine's copy stream, overlapping the step before) and
    # the loss out (copied to pinned host memory in stream order); the clock
    # stops once the last loss is on the host
    loss_host = torch.zeros(args.steps, dtype=torch.float32).pin_memory()
    # the same workload as the device-fed run: the model restarts from its
    # initial state (its per-step cost grows as it trains) and takes the same
    # steps; the warm-up gives each of the two upload buffers its eager step
    # and its graph capture before the clock starts
    dg = E.DeviceGaussians(model)
    for k in range(args.warmup):          # the device-fed run's warm-up steps (W >= 3), host-fed
        one(k, True)
    barrier()
    eng.synchronize()
    t0 = time.perf_counter()
    for k in range(args.steps):
        one(args.warmup + k, True)
        eng.loss_async(loss_host.data_ptr() + 4 * k)
    eng.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    if not bool(torch.isfinite(loss_host).all()):
        raise RuntimeError("non-finite loss in the end-to-end run")
    e2e = {"value": R.job_rate(ws, args.steps, e2e_s), "unit": "iters/s",
           "h2d_bytes_per_step": int(gts_host[0].numel()), "d2h_bytes_per_step": 4}
    # the same through the reference's public trainer API (msplat_trainer_step)
    e2e_trainer = None
    if not args.no_trainer:
        try:
            e2e_trainer = run_trainer_e2e(sc, model, gts_host, max(300, args.steps))
        except Exception as ex:   # reported, never fatal to the throughput line
            e2e_trainer = {"error": str(ex)[:200]}

    # per-stage times: CUDA events between the stages of eager steps (events
    # inside a step need it launched kernel by kernel)
    eng.set_timing(True)
    pair_counts = []
    for k in range(min(args.steps, 20)):
        step_k = args.warmup + 2 * args.steps + k
        one(step_k, False)
        eng.synchronize()
        pair_counts.append(backward_pairs(eng, cams[step_k % len(cams)]))
    eng.synchronize()
    st = eng.stats()
    eng.set_timing(False)

    # roofline of the dominant stage (CUDA events on the engine's stream)
    stage_ms = {name: st.stage_ms[i] / max(1, st.timed_steps) for i, name in enumerate(E.N.STAGES)}
    units = {"g": n_model, "i": float(st.num_intersections), "p": 1297 * 840}
    dom = max(stage_ms, key=stage_ms.get)
    alg = sum(units[u] * b for u, b in STAGE_BYTES[dom].items())
    peak, kind = measured_peaks()
    achieved = alg / (stage_ms[dom] / 1e3) / 1e9
    traffic = None
    tf = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tf):
        try:
            traffic = json.load(open(tf)).get(dom)
        except (OSError, ValueError):
            traffic = None
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_kind": kind, "traffic": traffic,
                "algorithmic_bytes": alg, "ms": stage_ms[dom]}
    # the rasterizer backward is bound by its FP32 issue, not by HBM: its
    # FP32-pipe fraction from the (pixel, splat) pairs the reference's
    # algorithm walks (from each pixel's last contributor down to its tile's
    # first splat, rasterize_backward_kernel) x 60 FP32 operations
    try:
        pairs = float(np.mean(pair_counts))
        props = torch.cuda.get_device_properties(local)
        fp32_peak = props.multi_processor_count * 128 * 2 * sm_max_mhz() * 1e6 / 1e12
        flops = 60.0 * pairs / (stage_ms["raster_bwd"] / 1e3) / 1e12
        roofline["fp32"] = {"kernel": "raster_bwd", "pairs": pairs, "flops_per_pair": 60,
                            "achieved": flops, "peak": fp32_peak, "unit": "TFLOP/s", "frac": flops / fp32_peak,
                            "peak_kind": "nominal: SMs x 128 FP32 lanes x 2 x max SM clock"}
    except Exception as ex:   # reported, never fatal to the throughput line
        roofline["fp32"] = {"error": str(ex)[:200]}
    # the whole step against HBM: the algorithmic bytes of one iteration
    # (2140 B per Gaussian, 128 B per intersection, 67 B per pixel: the
    # per-unit figures of the workload's byte model without the 76 B per
    # intersection of the reference's pack, which this design does not do)
    # over the graph-replayed step time
    step_bytes = 2140.0 * units["g"] + 128.0 * units["i"] + 67.0 * units["p"]
    roofline["step"] = {"algorithmic_bytes": step_bytes, "ms": ms_step,
                        "achieved": step_bytes / (ms_step / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                        "frac": step_bytes / (ms_step / 1e3) / 1e9 / peak}

    batched = None
    if not args.no_batched:
        try:
            batched = run_batched(eng, E, sc, dg, 3, max(5, args.steps // 4), step_base + 100000)
            batched["single_view_mpx_per_s"] = value / ws * 1297 * 840 / 1e6
        except Exception as ex:   # reported, never fatal to the throughput line
            batched = {"error": str(ex)[:200]}

    out = {"metric": METRIC, "value": value, "unit": "iters/s", "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config_dict(args),
           "roofline": roofline, "stage_ms": stage_ms, "num_intersections": int(st.num_intersections),
           "max_tile_count": int(st.max_tile_count), "gpu_launches": int(launches), "e2e": e2e,
           "e2e_trainer": e2e_trainer,
           "cuda_graph": True, "tuning": tuned, "autotune_step_ms": tuned_ms, "batched": batched,
           "clocks": clk.summary()}
    if rank == 0 and not args.no_time_to_psnr:
        # the metric's second half: learned vs plain relocation, held-out PSNR
        # at the fixed iteration count and time to PSNR (small synthetic
        # scene, five seeds; msplat_gb300.relocation_ab): learned against
        # plain, and learned + batched against plain + batched
        try:
            from msplat_gb300 import relocation_ab as AB
            arms = ["plain", "learned", "batch4x3", "batch4x3_learned"]
            per_seed = []
            for sd in (0, 1, 2, 3, 4):
                cams_ab, imgs_ab, xyz_ab, col_ab = AB._scene(sd)
                per_seed.append(AB.compare(cams_ab, imgs_ab, xyz_ab, col_ab, arms, 6000, 250))
            summ = AB.summarize(per_seed, arms)
            out["time_to_psnr"] = {
                "workload": "16,384-Gaussian synthetic scene, 8 train + 4 held-out views at 256x256, MCMC cap "
                            "32,768, 6000 iterations (views), seeds 0-4; each arm against its plain "
                            "counterpart: held-out PSNR at 6000 iterations, and time to the counterpart's final "
                            "held-out PSNR - 0.1 dB (batch4x3: 4 views per step, one launch per stage, learning "
                            "rates x 3)",
                "summary": summ,
                "psnr_gain_at_fixed_iterations_db": summ["learned"]["final_psnr_gain_mean"],
                "psnr_gain_learned_batched_vs_plain_batched_db": summ["batch4x3_learned"]["final_psnr_gain_mean"],
                "ratio": summ["learned"]["time_ratio_mean"],
                "ratio_learned_batched_vs_plain_batched": summ["batch4x3_learned"]["time_ratio_mean"],
                "per_seed": [{k: {"time_ratio": v["time_ratio"], "final_psnr": v["final_psnr"],
                                  "time_to_target_s": v["time_to_target_s"]} for k, v in ps.items()}
                             for ps in per_seed],
                "proposal_forecast_mse": [ps["learned"].get("proposal") for ps in per_seed]}
        except Exception as ex:   # reported, never fatal to the throughput line
            out["time_to_psnr"] = {"error": str(ex)[:200]}
    if rank == 0 and not args.no_full_run:
        try:
            from msplat_gb300 import full_run
            eng.close()
            out["full_run"] = full_run.run(eval_every=500)
            fr = out["full_run"]
            # the same configuration with the learned relocation proposal, and
            # with the proposal and 4 views per step (the learned + batched
            # form): held-out PSNR at the fixed iteration count against the
            # plain run's, and the wall clock at which each run first reaches
            # the plain run's final held-out PSNR - 0.1 dB (PSNR every 500
            # iterations outside the timed clock, the crossing interpolated
            # linearly between two evaluations)
            target = fr["held_out_psnr"] - 0.1
            tp = full_run.time_to(fr["psnr_curve"], target)
            for key, kw in (("full_run_learned", dict(learned=True)),
                            ("full_run_learned_batched", dict(learned=True, batch=4))):
                r = full_run.run(eval_every=500, **kw)
                o = {k: r[k] for k in ("iters_per_s", "wall_s", "final_gaussians", "held_out_psnr", "held_out_ssim",
                                       "held_out_l1", "curve", "psnr_curve", "mcmc_rounds", "batch_views")}
                o["psnr_gain_vs_plain_db"] = r["held_out_psnr"] - fr["held_out_psnr"]
                tr = full_run.time_to(r["psnr_curve"], target)
                o["time_to_target"] = {"target_db": target, "plain_s": tp, "run_s": tr,
                                       "ratio": (tr / tp) if (tp and tr) else None}
                out[key] = o
        except Exception as ex:   # reported, never fatal to the throughput line
            out.setdefault("full_run", {"error": str(ex)[:200]})
            out["full_run_learned"] = {"error": str(ex)[:200]}
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(model, sc.train_cams[0], gts_host[0].numpy(), steps=args.cpu_steps)
    if rank == 0:
        print(json.dumps(out), flush=True)
    eng.close()
    R.finish(ws)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=4)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-time-to-psnr", action="store_true",
                    help="skip the learned-vs-plain relocation time-to-PSNR runs")
    ap.add_argument("--no-batched", action="store_true", help="skip the multi-view (8 views per step) measurement")
    ap.add_argument("--no-trainer", action="store_true", help="skip the public-API (msplat_trainer_step) measurement")
    ap.add_argument("--no-full-run", action="store_true",
                    help="skip the full configuration's run: 7000 iterations from 100k random points to the 1M cap, "
                         "held-out PSNR/SSIM over 20 views (msplat_gb300.full_run)")
    ap.add_argument("--no-autotune", action="store_true", help="time the default launch configuration")
    ap.add_argument("--tuning", default="", help="fixed launch configuration instead of the autotuner, "
                                                 "e.g. tile_order=1,sort_width=512")
    ap.add_argument("--gaussians", type=int, default=N_MODEL,
                    help="trained Gaussians (default 1M; smaller only for profiling captures)")
    args = ap.parse_args()
    if args.warmup < 3:
        log("warmup raised to 3")
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_engine(args)


if __name__ == "__main__":
    sys.exit(main())
