"""Deterministic synthetic scenes and camera rigs.

The reference trains on captured datasets (mipnerf360 and similar); none is
available here, so the training workloads use seeded synthetic scenes with the
shapes and value distributions of the benchmark configurations:

* Gaussians: means uniform in the unit ball, log-scales N(-4.5, 0.5) per axis,
  quaternions = normalised N(0, I4) stored (w, x, y, z), opacity logits N(1, 1),
  SH degree 3 with DC uniform in [-1.7, 1.7] and higher bands N(0, 0.05).
* Optional ground plane: z ~ N(-1, 0.02), flat scales.
* Optional dense ball near the camera path (heavy tiles).
* Cameras: a ring of radius 3 at height 0.5 looking at the origin, world up +z,
  written as camera-to-world matrices in the reference's OpenGL convention
  (columns right, up, back; core/src/model.cpp:857-866 flips columns 1 and 2).

All arrays are float32 and C-contiguous, in the reference's layouts
(core/include/model.hpp:65-70): means [N,3], scales [N,3] (log), quats [N,4],
features_dc [N,3], features_rest [N,15,3], opacities [N,1] (logit).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

SH_C0 = 0.28209479177387814


@dataclass
class GaussianSet:
    means: np.ndarray
    scales: np.ndarray
    quats: np.ndarray
    features_dc: np.ndarray
    features_rest: np.ndarray
    opacities: np.ndarray

    @property
    def n(self) -> int:
        return int(self.means.shape[0])

    def copy(self) -> "GaussianSet":
        return GaussianSet(*(a.copy() for a in self.arrays()))

    def arrays(self):
        return (self.means, self.scales, self.quats, self.features_dc, self.features_rest, self.opacities)


@dataclass
class Camera:
    cam_to_world: np.ndarray  # 4x4 row-major, OpenGL axes
    width: int
    height: int
    fx: float
    fy: float
    cx: float
    cy: float


@dataclass
class Scene:
    gt: GaussianSet
    train_cams: list = field(default_factory=list)
    test_cams: list = field(default_factory=list)


def _unit_ball(rng, n, radius=1.0, center=(0.0, 0.0, 0.0)):
    v = rng.standard_normal((n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True) + 1e-12
    r = rng.random(n) ** (1.0 / 3.0) * radius
    return (v * r[:, None] + np.asarray(center)[None, :]).astype(np.float32)


def _quats(rng, n):
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True) + 1e-12
    return q.astype(np.float32)


def gaussians(n: int, seed: int, sh_rest_bases: int = 15, ground: int = 0, ball: int = 0,
              ball_center=(2.2, 0.0, 0.45), ball_radius: float = 0.1) -> GaussianSet:
    """GT scene of n Gaussians plus `ground` plane and `ball` heavy-tile Gaussians."""
    rng = np.random.default_rng(seed)
    means = _unit_ball(rng, n)
    scales = rng.normal(-4.5, 0.5, (n, 3)).astype(np.float32)
    quats = _quats(rng, n)
    dc = rng.uniform(-1.7, 1.7, (n, 3)).astype(np.float32)
    rest = rng.normal(0.0, 0.05, (n, sh_rest_bases, 3)).astype(np.float32)
    op = rng.normal(1.0, 1.0, (n, 1)).astype(np.float32)
    parts = [(means, scales, quats, dc, rest, op)]
    if ground:
        g_means = np.stack([rng.uniform(-1.5, 1.5, ground), rng.uniform(-1.5, 1.5, ground),
                            rng.normal(-1.0, 0.02, ground)], axis=1).astype(np.float32)
        g_scales = np.stack([rng.normal(-4.0, 0.3, ground), rng.normal(-4.0, 0.3, ground),
                             np.full(ground, -7.0)], axis=1).astype(np.float32)
        g_quats = np.tile(np.array([[1, 0, 0, 0]], np.float32), (ground, 1))
        parts.append((g_means, g_scales, g_quats, rng.uniform(-1.7, 1.7, (ground, 3)).astype(np.float32),
                      rng.normal(0, 0.05, (ground, sh_rest_bases, 3)).astype(np.float32),
                      rng.normal(1.0, 1.0, (ground, 1)).astype(np.float32)))
    if ball:
        parts.append((_unit_ball(rng, ball, ball_radius, ball_center),
                      rng.normal(-6.0, 0.5, (ball, 3)).astype(np.float32), _quats(rng, ball),
                      rng.uniform(-1.7, 1.7, (ball, 3)).astype(np.float32),
                      rng.normal(0, 0.05, (ball, sh_rest_bases, 3)).astype(np.float32),
                      rng.normal(1.0, 1.0, (ball, 1)).astype(np.float32)))
    cat = [np.ascontiguousarray(np.concatenate([p[k] for p in parts], axis=0)) for k in range(6)]
    return GaussianSet(*cat)


def look_at_c2w(eye, target=(0.0, 0.0, 0.0), up=(0.0, 0.0, 1.0)) -> np.ndarray:
    """Camera-to-world (OpenGL: x right, y up, camera looks down -z)."""
    eye = np.asarray(eye, np.float64)
    f = np.asarray(target, np.float64) - eye
    f /= np.linalg.norm(f)
    r = np.cross(f, np.asarray(up, np.float64))
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    m = np.eye(4)
    m[:3, 0], m[:3, 1], m[:3, 2], m[:3, 3] = r, u, -f, eye
    return m.astype(np.float32)


def ring_cameras(count: int, width: int, height: int, fx: float, fy: float | None = None,
                 radius: float = 3.0, height_z: float = 0.5, seed: int | None = None,
                 jitter: float = 0.0, phase: float = 0.0) -> list:
    fy = fx if fy is None else fy
    rng = np.random.default_rng(seed) if seed is not None else None
    cams = []
    for i in range(count):
        a = phase + 2.0 * math.pi * i / count
        r, z = radius, height_z
        if rng is not None and jitter > 0:
            a += rng.uniform(-jitter, jitter) * 2.0 * math.pi / count
            r *= 1.0 + rng.uniform(-0.1, 0.1) * jitter
            z += rng.uniform(-0.3, 0.3) * jitter
        eye = (r * math.cos(a), r * math.sin(a), z)
        cams.append(Camera(look_at_c2w(eye), width, height, float(fx), float(fy), width / 2.0, height / 2.0))
    return cams


def init_from_gt(gt: GaussianSet, seed: int, n: int | None = None, jitter: float = 0.05,
                 log_scale: float = -4.0, opacity: float = 0.5) -> GaussianSet:
    """Training start: jittered GT means, isotropic scale, random SH, logit(opacity)."""
    rng = np.random.default_rng(seed + 1000003)
    n = gt.n if n is None else n
    idx = np.arange(n) % gt.n
    means = (gt.means[idx] + rng.normal(0.0, jitter, (n, 3))).astype(np.float32)
    scales = np.full((n, 3), log_scale, np.float32)
    quats = _quats(rng, n)
    dc = rng.uniform(-1.7, 1.7, (n, 3)).astype(np.float32)
    rest = rng.normal(0.0, 0.05, (n, gt.features_rest.shape[1], 3)).astype(np.float32)
    op = np.full((n, 1), math.log(opacity / (1.0 - opacity)), np.float32)
    return GaussianSet(np.ascontiguousarray(means), scales, quats, dc, rest, op)


def random_points_init(n: int, seed: int, sh_rest_bases: int = 15, radius: float = 1.2,
                       log_scale: float = -4.0) -> GaussianSet:
    """Training start from random points (the 100k-seed workload)."""
    rng = np.random.default_rng(seed + 2000003)
    means = _unit_ball(rng, n, radius)
    scales = np.full((n, 3), log_scale, np.float32)
    return GaussianSet(means, scales, _quats(rng, n), rng.uniform(-1.7, 1.7, (n, 3)).astype(np.float32),
                       np.zeros((n, sh_rest_bases, 3), np.float32), np.zeros((n, 1), np.float32))


# Benchmark configurations --------------------------------------------------

def config_small(seed: int = 0) -> Scene:
    """16,384 GT Gaussians, 8 ring cameras at 256x256, fx = fy = 205."""
    gt = gaussians(16384, seed)
    return Scene(gt, ring_cameras(8, 256, 256, 205.0), [])


def config_full(seed: int = 0, n: int = 1_000_000, ground: int = 200_000, n_train: int = 160,
                n_test: int = 20) -> Scene:
    """1M GT Gaussians + 200k ground plane; ring views at 1297x840."""
    gt = gaussians(n, seed, ground=ground)
    w, h = 1297, 840
    fx = 0.5 * w / math.tan(0.5 * math.radians(60.0))
    train = ring_cameras(n_train, w, h, fx, seed=seed + 11, jitter=1.0)
    test = ring_cameras(n_test, w, h, fx, seed=seed + 13, jitter=1.0, phase=math.pi / max(n_test, 1))
    return Scene(gt, train, test)


def config_heavy(seed: int = 0, n: int = 3_000_000, n_views: int = 40, ball_frac: float = 0.3,
                 width: int = 4946, height: int = 3286) -> Scene:
    """Heavy-tile stress: n GT Gaussians, ball_frac of them in a 0.1-radius ball
    0.8 in front of the first ring camera (on the camera path), n_views ring
    views at 4946x3286 with a 60-degree horizontal field of view."""
    ball = int(ball_frac * n)
    gt = gaussians(n - ball, seed, ball=ball, ball_center=(2.2, 0.0, 0.45), ball_radius=0.1)
    fx = 0.5 * width / math.tan(0.5 * math.radians(60.0))
    return Scene(gt, ring_cameras(n_views, width, height, fx), [])

