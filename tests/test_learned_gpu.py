"""What the trained relocation network gains over the rule without it (GPU).

The learned proposal's MLP forecasts, for a Gaussian, its opacity and its
activity (log mean |dL/d centre| while visible) one training window (500
steps) ahead.  The plain MCMC rule uses the Gaussian's current opacity, i.e.
the persistence forecast.  At every training round after the first the
trainer checks the MLP on the round's new labels before training on them
(held out), against persistence.  On the small synthetic scene the network
must beat persistence on both outputs: activity by at least 2x in mean
squared error, opacity at all.  (Time to held-out PSNR against plain
relocation, over seeds, is measured by msplat_gb300.relocation_ab.)
"""
import pytest

pytestmark = pytest.mark.gpu


def test_learned_forecasts_beat_persistence():
    from msplat_gb300 import relocation_ab as AB
    cams, imgs, xyz, col = AB._scene(0)
    r = AB.run_arm(cams, imgs, xyz, col, True, 4000, 1000)
    p = r["proposal"]
    print("learned proposal", p)
    assert p["enabled"] and p["rounds"] >= 6 and p["rounds_evaluated"] >= 5, p
    assert p["mse_activity"] <= 0.5 * p["mse_activity_persistence"], p
    assert p["mse_opacity"] < p["mse_opacity_persistence"], p
