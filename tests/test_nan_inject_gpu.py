"""Host-side NaN injection through the public trainer (GPU only).

MSPLAT_NAN_INJECT=<step> poisons features_dc of 100 Gaussians at the end of
that step's MCMC round (core/src/model.cpp:638-659).  What must follow, as in
the reference: the poisoned Gaussians are gated out of every later step by the
projection's zombie gate (the non-finite telemetry counts them, the image and
loss stay finite), and the next MCMC round classifies every one of them as
dead (non-finite) and relocates them, so no non-finite parameter is left.
"""
import numpy as np
import pytest

from gpu_helpers import gt_image
from msplat_gb300 import api as A
from msplat_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

INJECT = 600


def test_nan_injection_is_contained_and_relocated(monkeypatch):
    gt = S.gaussians(3000, seed=21, sh_rest_bases=15)
    cams = S.ring_cameras(5, 128, 96, 110.0)
    imgs = [gt_image(gt, c) for c in cams]
    rng = np.random.default_rng(4)
    xyz = (gt.means[:1500] + rng.normal(0.0, 0.02, (1500, 3))).astype(np.float32)
    rgb = rng.integers(0, 256, (1500, 3), dtype=np.uint8)
    ds = A.Dataset.from_arrays(cams, imgs, xyz, rgb)
    monkeypatch.setenv("MSPLAT_NAN_INJECT", str(INJECT))   # read when the trainer is created
    t = A.GaussianTrainer(ds, A.TrainingConfig(iterations=2000, cap_max=4000))
    while t.iteration < INJECT:
        t.step()
    assert t.mcmc_stats()["rounds"] == 2                    # steps 500 and 600
    dc = t.get_gaussians()[3]
    poisoned = int((~np.isfinite(dc)).any(axis=1).sum())
    assert 90 <= poisoned <= 100                            # 100 draws with repeats
    gate0 = t.engine_nan_counts()[7]
    for _ in range(10):
        t.step()
        assert np.isfinite(t.last_loss)
    assert t.engine_nan_counts()[7] > gate0                  # the projection gate caught them
    while t.iteration < INJECT + 100:
        t.step()
    st = t.mcmc_stats()
    assert st["rounds"] == 3
    assert st["num_nonfinite"] == poisoned, st
    assert st["num_dead"] >= poisoned
    arrs = t.get_gaussians()
    assert all(np.isfinite(a).all() for a in arrs)
    img = t.render(0)
    assert np.isfinite(img).all()
