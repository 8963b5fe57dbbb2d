"""Tensor-core path of the learned relocation proposal (GPU only)."""
import ctypes as C

import numpy as np
import pytest

from msplat_gb300 import _native as N

pytestmark = pytest.mark.gpu


def _bf16_bits(x):
    """float32 values exactly representable in bfloat16 -> their 16-bit patterns."""
    b = np.ascontiguousarray(x, np.float32).view(np.uint32)
    assert np.all((b & 0xFFFF) == 0)
    return (b >> 16).astype(np.uint16)


@pytest.mark.parametrize("n,k", [(16, 16), (32, 32), (64, 64), (16, 64), (64, 16)])
def test_tc_gemm_probe(n, k):
    L = N.lib()
    L.msplat_tc_gemm_check.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int]
    rng = np.random.default_rng(n * 100 + k)
    A = rng.integers(-4, 5, (128, k)).astype(np.float32)
    B = rng.integers(-4, 5, (n, k)).astype(np.float32) * 0.5
    D = np.zeros((128, n), np.float32)
    a, b = _bf16_bits(A), _bf16_bits(B)
    rc = L.msplat_tc_gemm_check(a.ctypes.data, b.ctypes.data, D.ctypes.data, n, k)
    assert rc == 0
    np.testing.assert_array_equal(D, A @ B.T)      # small integers: exact in F32


def _mlp_lib():
    L = N.lib()
    vp = C.c_void_p
    L.msplat_mlp_pack.argtypes = [vp, vp, vp]
    L.msplat_mlp_forward.argtypes = [vp, C.c_int, vp, vp, vp, vp, vp]
    L.msplat_mlp_train_batch.argtypes = [vp, vp, C.c_int, vp, vp, vp, vp, vp, vp]
    L.msplat_mlp_adam.argtypes = [vp, vp, vp, vp, C.c_float, C.c_int, vp]
    return L


def _case(n, seed):
    from oracle import mlp_oracle as M
    rng = np.random.default_rng(seed)
    X = np.zeros((n, 32), np.float32)
    X[:, :M.N_IN] = M.bf16(rng.normal(0, 1, (n, M.N_IN)).astype(np.float32))
    T = rng.normal(0, 0.5, (n, 2)).astype(np.float32)
    P = M.init_params(seed)
    P[M.OFF["b1"][0]:M.OFF["b1"][0] + 64] = rng.normal(0, 0.1, 64)
    P[M.OFF["b3"][0]:M.OFF["b3"][0] + 2] = [0.3, -0.2]
    return X, T, P


def test_mlp_forward_and_gradients_match_oracle():
    torch = pytest.importorskip("torch")
    from oracle import mlp_oracle as M
    L = _mlp_lib()
    n = 300                                 # not a multiple of the 128-row tile
    X, T, P = _case(n, 2)
    dP = torch.from_numpy(P).cuda()
    img = torch.zeros(24576, dtype=torch.uint8, device="cuda")
    dX = torch.from_numpy(M.bf16_bits(X).view(np.int16)).cuda()
    dT = torch.from_numpy(T).cuda()
    out = torch.zeros((n, 2), dtype=torch.float32, device="cuda")
    G = torch.zeros_like(dP)
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert L.msplat_mlp_pack(dP.data_ptr(), img.data_ptr(), None) == 0
    assert L.msplat_mlp_forward(dX.data_ptr(), n, img.data_ptr(), dP.data_ptr(), out.data_ptr(), err.data_ptr(),
                                None) == 0
    assert L.msplat_mlp_train_batch(dX.data_ptr(), dT.data_ptr(), n, img.data_ptr(), dP.data_ptr(), G.data_ptr(),
                                    loss.data_ptr(), err.data_ptr(), None) == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    y_ref, _ = M.forward(X, P)
    y = out.cpu().numpy()
    assert np.abs(y - y_ref).max() <= 2e-3 * (1 + np.abs(y_ref).max()), np.abs(y - y_ref).max()
    l_ref, g_ref = M.loss_and_grad(X, T, P)
    assert abs(loss.item() - l_ref) <= 1e-3 * l_ref
    g = G.cpu().numpy()
    for k, (o, s) in M.OFF.items():
        sl = slice(o, o + int(np.prod(s)))
        a, b = g[sl], g_ref[sl]
        e = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
        print(k, e)
        assert e < 5e-3, (k, e)


def test_mlp_training_reduces_loss():
    torch = pytest.importorskip("torch")
    from oracle import mlp_oracle as M
    L = _mlp_lib()
    n = 4096
    rng = np.random.default_rng(9)
    X = np.zeros((n, 32), np.float32)
    X[:, :M.N_IN] = M.bf16(rng.normal(0, 1, (n, M.N_IN)).astype(np.float32))
    T = np.stack([np.tanh(X[:, 0] - 0.5 * X[:, 3]), 0.5 * X[:, 1] * X[:, 2]], 1).astype(np.float32)
    P = M.init_params(3)
    dP = torch.from_numpy(P).cuda()
    Mo, Vo, G = torch.zeros_like(dP), torch.zeros_like(dP), torch.zeros_like(dP)
    img = torch.zeros(24576, dtype=torch.uint8, device="cuda")
    dX = torch.from_numpy(M.bf16_bits(X).view(np.int16)).cuda()
    dT = torch.from_numpy(T).cuda()
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    losses = []
    for step in range(1, 301):
        L.msplat_mlp_pack(dP.data_ptr(), img.data_ptr(), None)
        loss.zero_()
        L.msplat_mlp_train_batch(dX.data_ptr(), dT.data_ptr(), n, img.data_ptr(), dP.data_ptr(), G.data_ptr(),
                                 loss.data_ptr(), err.data_ptr(), None)
        L.msplat_mlp_adam(dP.data_ptr(), G.data_ptr(), Mo.data_ptr(), Vo.data_ptr(), 3e-3, step, None)
        if step in (1, 300):
            torch.cuda.synchronize()
            losses.append(loss.item())
    assert int(err.item()) == 0
    print(losses)
    assert losses[1] < 0.2 * losses[0]


def test_learned_relocation_in_training():
    """A short MCMC run with the learned proposal: the MLP trains on the run's
    own pairs (snapshot at 500, labels and first training at 1000) and then
    weights the relocation draws; the run stays finite and learns."""
    pytest.importorskip("torch")
    from msplat_gb300 import api as A
    from msplat_gb300 import synthetic as S
    from gpu_helpers import gt_image
    gt = S.gaussians(3000, seed=31)
    cams = S.ring_cameras(6, 96, 64, 80.0)
    imgs = [gt_image(gt, c) for c in cams]
    rng = np.random.default_rng(2)
    xyz = (gt.means[:2000] + rng.normal(0, 0.03, (2000, 3))).astype(np.float32)
    rgb = rng.integers(0, 256, (2000, 3), dtype=np.uint8)
    ds = A.Dataset.from_arrays(cams, imgs, xyz, rgb, eval_mode=True, test_every=3)
    cfg = A.TrainingConfig(iterations=1500, cap_max=6000, bg_color=[0.0, 0.0, 0.0])
    t = A.GaussianTrainer(ds, cfg)
    t.set_learned_relocation(True)
    for _ in range(1200):
        t.step()
    st = t.learned_stats()
    assert st["enabled"] and st["rounds"] >= 1 and np.isfinite(st["last_loss"]), st
    assert t.splat_count > 2000                       # grew toward the cap
    m = t.evaluate()
    assert np.isfinite(m["psnr"]) and m["psnr"] > 15.0, m
