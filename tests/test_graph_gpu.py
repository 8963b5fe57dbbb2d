"""CUDA graph mode of the training step: captured and replayed steps give
the same parameters as eager steps from the same state (GPU only)."""
import numpy as np
import pytest

from msplat_gb300 import engine as E
from msplat_gb300 import synthetic as S

from gpu_helpers import gt_image, rel_l2

pytestmark = pytest.mark.gpu


def _run(init, cams, gts, graphs, steps=6):
    import torch
    eng = E.Engine(0)
    eng.set_graphs(graphs)
    dg = E.DeviceGaussians(init)
    gt_d = [torch.from_numpy(g).cuda() for g in gts]
    for k in range(steps):
        cam = cams[k % len(cams)]
        st = E.step_scalars(600 + k, 600 + k, width=cam.width, height=cam.height)
        eng.train_step(dg, E.make_args(E.camera_dict(cam), st, do_sgld=True), gt_d[k % len(cams)].data_ptr())
    loss = eng.loss()
    launches = eng.stats().launches
    p, _ = dg.to_numpy()
    eng.close()
    return p, loss, launches


def test_graph_replay_matches_eager():
    sc = S.config_small(1)
    cams = sc.train_cams[:2]
    gts = [gt_image(sc.gt, c) for c in cams]
    init = S.init_from_gt(sc.gt, 1)
    pe, le, ne = _run(init, cams, gts, graphs=False)
    pg, lg, ng = _run(init, cams, gts, graphs=True)
    assert ne == ng                      # same kernels, replayed or not
    assert abs(le - lg) <= 1e-5 * abs(le)
    for k in E.GROUPS:
        d0 = pe[k] - getattr(init, k).reshape(pe[k].shape)
        d1 = pg[k] - getattr(init, k).reshape(pg[k].shape)
        assert rel_l2(d1, d0) <= 1e-4, k


def test_host_images_pipelined():
    """Steps that take their targets from page-locked host memory (uploaded
    on the copy stream into alternating buffers, overlapping the step
    before) give the steps from device targets; the loss sums read without
    waiting match the loss read with a wait."""
    import torch
    sc = S.config_small(5)
    cams = sc.train_cams[:3]
    gts = [gt_image(sc.gt, c) for c in cams]
    init = S.init_from_gt(sc.gt, 5)
    pd, ld, _ = _run(init, cams, gts, graphs=True, steps=7)
    eng = E.Engine(0)
    eng.set_graphs(True)
    dg = E.DeviceGaussians(init)
    host = [torch.from_numpy(g).pin_memory() for g in gts]
    sums = torch.zeros(7, dtype=torch.float32).pin_memory()
    for k in range(7):
        cam = cams[k % len(cams)]
        st = E.step_scalars(600 + k, 600 + k, width=cam.width, height=cam.height)
        eng.train_step_host(dg, E.make_args(E.camera_dict(cam), st, do_sgld=True), host[k % len(cams)].data_ptr())
        eng.loss_async(sums.data_ptr() + 4 * k)
    eng.synchronize()
    lh = eng.loss()
    cam = cams[6 % len(cams)]
    assert abs(float(sums[6]) / (cam.width * cam.height) - lh) <= 1e-6 * abs(lh)
    assert abs(lh - ld) <= 1e-5 * abs(ld)
    ph, _ = dg.to_numpy()
    eng.close()
    for k in E.GROUPS:
        base = getattr(init, k).reshape(pd[k].shape)
        assert rel_l2(ph[k] - base, pd[k] - base) <= 1e-4, k
