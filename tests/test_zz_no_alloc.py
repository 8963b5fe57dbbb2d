"""The allocation-free loss entry point (msplat_loss_ssim_l1_noalloc) against
the loss stage of the regular training step (GPU only).

The entry point serves callers that cannot call cudaMalloc (a host that owns
all device memory through its own allocator, or a loop that cannot take
cudaMalloc's implicit synchronisation): its only device state is the step
scalars, in the library's static device copy.  Two calls in a row must both
reproduce the training step's image gradient and loss, with the tolerance
the parity tests use for the image gradient (1e-5 relative L2), on a small
image with partial edge blocks and on one above 512 x 512 pixels.  This file
is collected last.
"""
import ctypes as C

import numpy as np
import pytest

from msplat_gb300 import _native as N
from msplat_gb300 import engine as E
from msplat_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _rel(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("size", [(203, 150, 130.0), (700, 413, 450.0)])
def test_noalloc_loss_matches_training_step(size):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    L = N.lib()
    L.msplat_loss_ssim_l1_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_float,
                                              C.c_float, C.c_void_p, C.c_void_p, C.c_void_p]
    L.msplat_loss_ssim_l1_noalloc.restype = C.c_int

    gt_scene = S.gaussians(3000, 11)
    cam = S.ring_cameras(4, size[0], size[1], size[2])[2]   # partial edge blocks
    cd = E.camera_dict(cam)
    W, H = cam.width, cam.height
    eng = E.Engine(0)
    ref = E.DeviceGaussians(gt_scene)
    eng.render(ref, E.make_args(cd, {"degrees_to_use": 3}))
    target = eng.read("out_img", np.float32, W * H * 3).reshape(H, W, 3)
    gt = (np.clip(target, 0, 1) * 255 + 0.5).astype(np.uint8)
    gt_d = torch.from_numpy(gt).cuda()
    mask = np.full((H, W), 255, np.uint8)
    mask[30:60, 40:90] = 0
    mask[H - 20:, W - 37:] = 0
    mask_d = torch.from_numpy(mask).cuda()

    dg = E.DeviceGaussians(S.init_from_gt(gt_scene, 11))
    step = E.step_scalars(10, 10, width=W, height=H)
    args = E.make_args(cd, step)
    eng.train_step(dg, args, gt_d.data_ptr(), mask_d.data_ptr())
    eng.synchronize()
    img = eng.read("out_img", np.float32, W * H * 3)
    v_ref = eng.read("v_img", np.float32, W * H * 3)
    loss_ref = eng.loss()
    eng.close()

    img_d = torch.from_numpy(img).cuda()
    torch.cuda.synchronize()
    for call in range(2):
        v_out = torch.full((W * H * 3,), float("nan"), dtype=torch.float32, device="cuda")
        loss_d = torch.full((1,), 123.0, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        rc = L.msplat_loss_ssim_l1_noalloc(img_d.data_ptr(), gt_d.data_ptr(), mask_d.data_ptr(), W, H,
                                           C.c_float(0.2), C.c_float(args.loss_inv_n), v_out.data_ptr(),
                                           loss_d.data_ptr(), None)
        assert rc == 0
        torch.cuda.synchronize()
        v = v_out.cpu().numpy()
        loss = float(loss_d.cpu().numpy()[0]) / (W * H)
        assert np.all(np.isfinite(v)), f"call {call}: non-finite gradient"
        assert _rel(v, v_ref) <= TOL, f"call {call}: gradient differs"
        assert abs(loss - loss_ref) <= TOL * max(1.0, abs(loss_ref)), f"call {call}: loss {loss} vs {loss_ref}"

    # a size beyond the kernel's grid is refused without touching the GPU
    rc = L.msplat_loss_ssim_l1_noalloc(img_d.data_ptr(), gt_d.data_ptr(), None, 16, 2100000, C.c_float(0.2),
                                       C.c_float(1.0), v_out.data_ptr(), loss_d.data_ptr(), None)
    assert rc == -3
