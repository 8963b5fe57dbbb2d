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
