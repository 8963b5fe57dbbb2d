"""Per-step scalars of the training step (learning rates, Adam bias
corrections, SH degree, regularizer gate, SGLD constants).

Pure Python: nothing here loads the engine library, so the CPU baseline and
the oracle's callers can use it on their own.
"""
from __future__ import annotations

import numpy as np

# Adam defaults (core/src/model.cpp:223, core/include/model.hpp:76-78)
LR_INIT = (0.00016, 0.005, 0.001, 0.0025, 0.000125, 0.05)
BETA1, BETA2, EPS = 0.9, 0.999, 1e-8
GROUPS = ("means", "scales", "quats", "features_dc", "features_rest", "opacities")


def step_scalars(step: int, adam_step: int, lr=LR_INIT, sh_degree=3, sh_interval=1000, op_reg=0.01, sc_reg=0.01,
                 width=None, height=None, noise_lr=5e5, cull_radius=3.0):
    """Per-step scalars of Model::fullIteration (core/src/model.cpp:901-975)."""
    # float betas raised to an int power in double, rounded once (model.cpp:915-916)
    bc1 = np.float32(1.0 - float(np.float32(BETA1)) ** adam_step)
    bc2 = np.float32(1.0 - float(np.float32(BETA2)) ** adam_step)
    d = dict(degrees_to_use=min(step // sh_interval, sh_degree),
             step_size=[float(np.float32(l) / bc1) for l in lr],
             bc2_sqrt=[float(np.sqrt(bc2))] * 6,
             beta1=BETA1, beta2=BETA2, eps=EPS,
             op_reg=op_reg if step >= 500 else 0.0, sc_reg=sc_reg if step >= 500 else 0.0, invis_scale=1.0,
             seed=step, noise_lr=noise_lr, xyz_lr=lr[0], max_disp=cull_radius * 0.0167 if cull_radius > 0 else 0.05)
    if width is not None:
        d["loss_inv_n"] = 1.0 / float(width * height * 3)
    return d
