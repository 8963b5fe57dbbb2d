"""The C-ABI library loads and exports every function declared in include/*.h
(CPU only: nothing is called that needs a GPU)."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        src = re.sub(r"static\s+inline[^{]*\{.*?\n\}", "", src, flags=re.S)
        for m in re.finditer(r"\b(msplat_\w+)\s*\(", src):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from msplat_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_headers_declare_functions():
    assert len(declared_functions()) >= 10


@pytest.mark.parametrize("name", declared_functions())
def test_symbol_exported(lib, name):
    assert hasattr(lib, name), f"{name} declared in include/ but not exported"


def test_prepare_camera_matches_oracle():
    import numpy as np
    from msplat_gb300 import engine as E, synthetic as S
    from oracle import oracle as O
    for cam in S.config_small(0).train_cams[:4]:
        a = E.prepare_cam(cam.cam_to_world, cam.width, cam.height, cam.fx, cam.fy)
        b = O.prepare_cam(cam.cam_to_world, cam.width, cam.height, cam.fx, cam.fy)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


def test_null_handles_and_bad_arguments_rejected(lib):
    """Every entry point checks its handle and arguments before any CUDA
    call: a null engine or trainer, or an invalid argument, returns -1."""
    c = ctypes
    vp, fp = c.c_void_p, c.POINTER(c.c_float)
    lib.msplat_engine_set_tuning.argtypes = [vp, vp]
    lib.msplat_engine_get_tuning.argtypes = [vp, vp]
    lib.msplat_engine_set_graphs.argtypes = [vp, c.c_int]
    lib.msplat_engine_set_isect_budget.argtypes = [vp, c.c_longlong]
    lib.msplat_engine_synchronize.argtypes = [vp]
    lib.msplat_engine_read.argtypes = [vp, c.c_char_p, vp, c.c_longlong]
    lib.msplat_engine_last_error.argtypes = [vp]
    lib.msplat_engine_last_error.restype = c.c_char_p
    buf = (c.c_byte * 256)()
    assert lib.msplat_engine_set_tuning(None, buf) == -1
    assert lib.msplat_engine_get_tuning(None, buf) == -1
    assert lib.msplat_engine_set_graphs(None, 1) == -1
    assert lib.msplat_engine_set_isect_budget(None, 1 << 20) == -1
    assert lib.msplat_engine_synchronize(None) == -1
    assert lib.msplat_engine_read(None, b"out_img", buf, 4) == -1
    assert lib.msplat_engine_last_error(None) == b"null engine"

    lib.msplat_trainer_set_gaussians.argtypes = [vp, c.c_int, c.c_int, fp, fp, fp, fp, fp, fp]
    lib.msplat_trainer_set_learned_prune.argtypes = [vp, c.c_float]
    lib.msplat_trainer_set_batch_views.argtypes = [vp, c.c_int, c.c_float]
    lib.msplat_trainer_set_isect_budget.argtypes = [vp, c.c_float]
    lib.msplat_trainer_learned_eval.argtypes = [vp, fp]
    lib.msplat_trainer_splat_count.argtypes = [vp]
    mse = (c.c_float * 4)()
    assert lib.msplat_trainer_set_gaussians(None, 1, 15, None, None, None, None, None, None) == -1
    assert lib.msplat_trainer_set_learned_prune(None, 0.02) == -1
    assert lib.msplat_trainer_set_batch_views(None, 4, 0.0) == -1
    assert lib.msplat_trainer_set_isect_budget(None, 64.0) == -1
    assert lib.msplat_trainer_learned_eval(None, mse) == -1
    assert lib.msplat_trainer_splat_count(None) == 0


def test_dataset_from_memory_rejects_bad_arguments(lib):
    """msplat_dataset_create_from_memory returns NULL (no dataset, no CUDA
    call) for negative counts, missing arrays or empty image sizes."""
    c = ctypes
    vp = c.c_void_p
    f = lib.msplat_dataset_create_from_memory
    f.restype = vp
    f.argtypes = [c.c_int, vp, vp, vp, vp, vp, c.c_int, vp, vp, c.c_bool, c.c_int, c.c_bool]
    c2w = (c.c_float * 16)()
    intr = (c.c_float * 4)(100.0, 100.0, 32.0, 32.0)
    zero = (c.c_int * 2)(0, 64)
    assert f(-1, None, None, None, None, None, 0, None, None, False, 8, False) is None
    assert f(1, None, intr, zero, None, None, 0, None, None, False, 8, False) is None
    assert f(1, c2w, intr, zero, None, None, 0, None, None, False, 8, False) is None
    assert f(0, None, None, None, None, None, 5, None, None, False, 8, False) is None


def test_dataset_from_arrays_on_host():
    """Dataset.from_arrays builds the dataset on the host (no GPU): train/test
    split by test_every, an empty point cloud allowed, and an image size of
    zero refused with an error."""
    import numpy as np
    from msplat_gb300 import api as A, synthetic as S
    cams = S.config_small(0).train_cams[:3]
    imgs = [np.zeros((c.height, c.width, 3), np.uint8) for c in cams]
    xyz = np.zeros((10, 3), np.float32)
    rgb = np.full((10, 3), 128, np.uint8)
    ds = A.Dataset.from_arrays(cams, imgs, xyz, rgb, eval_mode=True, test_every=2)
    assert (ds.num_train, ds.num_test) == (1, 2)
    ds = A.Dataset.from_arrays(cams, imgs, np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint8))
    assert (ds.num_train, ds.num_test) == (3, 0)
    bad = S.config_small(0).train_cams[0]
    bad.width = 0
    with pytest.raises(RuntimeError):
        A.Dataset.from_arrays([bad], [np.zeros((1, 1, 3), np.uint8)], xyz, rgb)


def test_gaussian_files_round_trip(tmp_path):
    """msplat_write_ply / msplat_read_ply on the host: the finite rows come
    back bit for bit with the iteration, the dataset-frame mapping inverts to
    within float rounding, the .splat has 32 bytes per finite Gaussian, and
    bad arguments return -1."""
    import numpy as np
    from msplat_gb300 import api as A, synthetic as S
    g = S.gaussians(300, 2)
    arrs = [g.means, g.scales, g.quats, g.features_dc, g.features_rest, g.opacities[:, 0].copy()]
    arrs[0][4, 2] = np.nan
    A.write_ply(str(tmp_path / "a.ply"), arrs, step=1234)
    got, step = A.read_ply(str(tmp_path / "a.ply"))
    keep = np.ones(300, bool)
    keep[4] = False
    assert step == 1234 and got[0].shape[0] == 299
    for a, b in zip(got, arrs):
        assert np.array_equal(a, b[keep])
    crs = dict(keep_crs=True, scale=0.5, translation=(1.0, 2.0, 3.0))
    A.write_ply(str(tmp_path / "b.ply"), arrs, **crs)
    back, _ = A.read_ply(str(tmp_path / "b.ply"), **crs)
    np.testing.assert_allclose(back[0], arrs[0][keep], atol=1e-5)
    np.testing.assert_allclose(back[1], arrs[1][keep], atol=1e-5)
    A.write_splat(str(tmp_path / "c.splat"), arrs)
    assert (tmp_path / "c.splat").stat().st_size == 32 * 299
    L = A._lib()
    assert L.msplat_write_ply(None, 0, 15, None, None, None, None, None, None, 0, 0, 1.0, None) == -1
    assert L.msplat_ply_info(str(tmp_path / "missing.ply").encode(), None, None, None) == -2


def test_trainer_options_and_seed_gaussians():
    """The Python TrainerOptions defaults are msplat_default_trainer_options
    (the reference's: opacity 0.5, scale x0.1, decimation on, 30000-step LR
    decay, duty 1); msplat_seed_gaussians applies them on the host (opacity
    logits, decimation to half the cap above 75 %) and refuses options out
    of range."""
    import ctypes as C
    import numpy as np
    from msplat_gb300 import api as A
    d = A._TrainerOptions()
    A._lib().msplat_default_trainer_options(C.byref(d))
    o = A.TrainerOptions()
    assert (d.initOpacity, d.initScaleMult, d.seedDecimation, d.positionLrMaxSteps, d.regVisibilityDuty) == \
        (np.float32(o.init_opacity), np.float32(o.init_scale_mult), 1, o.position_lr_max_steps,
         np.float32(o.reg_visibility_duty))
    rng = np.random.default_rng(0)
    xyz = rng.normal(0, 1, (400, 3)).astype(np.float32)
    rgb = rng.integers(0, 256, (400, 3), dtype=np.uint8)
    g = A.seed_gaussians(xyz, rgb, cap_max=10_000)
    assert g[0].shape[0] == 400 and np.allclose(g[5], 0.0) and np.array_equal(g[0], xyz)
    g = A.seed_gaussians(xyz, rgb, cap_max=500, options=A.TrainerOptions(init_opacity=0.25))
    assert g[0].shape[0] == 250 and np.allclose(g[5], np.log(0.25 / 0.75))
    with pytest.raises(RuntimeError):
        A.seed_gaussians(xyz, rgb, options=A.TrainerOptions(init_opacity=1.5))
