"""Checkpoint reader validation on the host (core/src/model.cpp:698-843 format).

msplat_checkpoint_info runs the same reader as msplat_trainer_load_checkpoint
without a trainer, so these run on the CPU: a well-formed file is accepted, and
a truncated file, a header N that disagrees with the tensors, a wrong row width,
a wrong byte count or an SH degree that disagrees with features_rest are all
rejected before anything is copied.
"""
import ctypes
import struct

import numpy as np
import pytest

GROUP_WIDTH = (3, 3, 4, 3, None, 1)


def write_ckpt(path, n=5, deg=1, step=7, override=None):
    """A checkpoint in the reference's layout; override(k, shape, nbytes, data)
    may change tensor k's record."""
    rest = (deg + 1) ** 2 - 1
    rng = np.random.default_rng(0)
    out = bytearray()
    out += struct.pack("<6I", 0x4C50534D, 1, step, n, deg, 3)
    out += np.arange(6, dtype=np.float32).tobytes() + struct.pack("<2f", 1.6e-4, 1.6e-6)
    for k in range(18):
        g = k % 6
        shape = [n, rest, 3] if g == 4 else ([n, 1] if g == 5 else [n, GROUP_WIDTH[g]])
        data = rng.normal(size=int(np.prod(shape))).astype(np.float32).tobytes()
        nbytes = len(data)
        if override is not None:
            shape, nbytes, data = override(k, shape, nbytes, data)
        out += struct.pack("<I", len(shape)) + struct.pack(f"<{len(shape)}q", *shape)
        out += struct.pack("<Q", nbytes) + data
    path.write_bytes(bytes(out))
    return path


@pytest.fixture(scope="module")
def lib():
    from msplat_gb300 import build
    L = ctypes.CDLL(build.build())
    L.msplat_checkpoint_info.argtypes = [ctypes.c_char_p] + [ctypes.POINTER(ctypes.c_int)] * 3
    L.msplat_checkpoint_info.restype = ctypes.c_int
    return L


def info(lib, path):
    n, d, it = ctypes.c_int(-1), ctypes.c_int(-1), ctypes.c_int(-1)
    rc = lib.msplat_checkpoint_info(str(path).encode(), ctypes.byref(n), ctypes.byref(d), ctypes.byref(it))
    return rc, n.value, d.value, it.value


@pytest.mark.parametrize("deg", [0, 1, 3])
def test_valid_checkpoint(lib, tmp_path, deg):
    p = write_ckpt(tmp_path / "ok.ckpt", n=9, deg=deg, step=123)
    assert info(lib, p) == (0, 9, deg, 123)


def test_truncated_checkpoint(lib, tmp_path):
    p = write_ckpt(tmp_path / "full.ckpt")
    raw = p.read_bytes()
    for cut in (10, 60, len(raw) // 2, len(raw) - 1):
        q = tmp_path / f"cut{cut}.ckpt"
        q.write_bytes(raw[:cut])
        assert info(lib, q)[0] == -1, cut


def test_wrong_n_in_header(lib, tmp_path):
    p = write_ckpt(tmp_path / "n.ckpt", n=5)
    raw = bytearray(p.read_bytes())
    raw[12:16] = struct.pack("<I", 6)          # header N = 6, tensors hold 5 rows
    p.write_bytes(bytes(raw))
    assert info(lib, p)[0] == -1
    raw[12:16] = struct.pack("<I", 4)          # fewer rows claimed than stored
    p.write_bytes(bytes(raw))
    assert info(lib, p)[0] == -1


def test_wrong_row_width(lib, tmp_path):
    def quats_wide(k, shape, nbytes, data):   # moment tensor of the quaternion group with 3 columns
        if k == 8:
            shape = [shape[0], 3]
            data = data[: shape[0] * 3 * 4]
            nbytes = len(data)
        return shape, nbytes, data
    assert info(lib, write_ckpt(tmp_path / "w.ckpt", override=quats_wide))[0] == -1


def test_byte_count_disagrees_with_shape(lib, tmp_path):
    def short_bytes(k, shape, nbytes, data):  # the stored byte count is below the shape's
        if k == 0:
            nbytes -= 4
            data = data[:nbytes]
        return shape, nbytes, data
    assert info(lib, write_ckpt(tmp_path / "b.ckpt", override=short_bytes))[0] == -1

    def long_bytes(k, shape, nbytes, data):   # above it (would over-read the host copy)
        if k == 13:
            data = data + b"\0" * 64
            nbytes = len(data)
        return shape, nbytes, data
    assert info(lib, write_ckpt(tmp_path / "c.ckpt", override=long_bytes))[0] == -1


def test_degree_disagrees_with_rest(lib, tmp_path):
    p = write_ckpt(tmp_path / "d.ckpt", deg=1)
    raw = bytearray(p.read_bytes())
    raw[16:20] = struct.pack("<I", 3)          # header degree 3, features_rest holds 3 bases
    p.write_bytes(bytes(raw))
    assert info(lib, p)[0] == -1
    raw[16:20] = struct.pack("<I", 9)          # no such degree
    p.write_bytes(bytes(raw))
    assert info(lib, p)[0] == -1


def test_missing_file(lib, tmp_path):
    assert info(lib, tmp_path / "missing.ckpt")[0] == -1
