"""The per-step scalars of the training step (msplat_gb300.schedule), on the
host: the SH degree bands, the regularizer gate, Adam's bias corrections with
float betas raised in double (core/src/model.cpp:901-975) and the SGLD
displacement cap."""
import numpy as np

from msplat_gb300.schedule import BETA1, BETA2, LR_INIT, step_scalars


def test_sh_degree_bands():
    for step, deg in [(0, 0), (999, 0), (1000, 1), (2999, 2), (3000, 3), (9000, 3)]:
        assert step_scalars(step, max(step, 1))["degrees_to_use"] == deg
    assert step_scalars(5000, 5000, sh_degree=1)["degrees_to_use"] == 1
    assert step_scalars(5000, 5000, sh_interval=500)["degrees_to_use"] == 3


def test_regularizer_starts_at_step_500():
    assert step_scalars(499, 499)["op_reg"] == 0.0 and step_scalars(499, 499)["sc_reg"] == 0.0
    d = step_scalars(500, 500)
    assert d["op_reg"] == 0.01 and d["sc_reg"] == 0.01


def test_adam_bias_corrections():
    for t in (1, 2, 10, 3001):
        d = step_scalars(t, t)
        bc1 = np.float32(1.0 - float(np.float32(BETA1)) ** t)
        bc2 = np.float32(1.0 - float(np.float32(BETA2)) ** t)
        assert d["step_size"] == [float(np.float32(l) / bc1) for l in LR_INIT]
        assert d["bc2_sqrt"] == [float(np.sqrt(bc2))] * 6
    # at t = 1 the first moment's correction is 1 - 0.9f
    assert abs(step_scalars(1, 1)["step_size"][0] - LR_INIT[0] / 0.1) < 1e-9


def test_sgld_and_loss_constants():
    d = step_scalars(3001, 3001, width=1297, height=840)
    assert d["seed"] == 3001 and d["xyz_lr"] == LR_INIT[0]
    assert abs(d["max_disp"] - 3.0 * 0.0167) < 1e-12
    assert d["loss_inv_n"] == 1.0 / (1297 * 840 * 3)
    assert step_scalars(1, 1, cull_radius=0.0)["max_disp"] == 0.05
    assert "loss_inv_n" not in step_scalars(1, 1)
