"""Dataset ingestion on the host (no GPU): the PNG and JPEG decoders against
images encoded here from known pixels, and the COLMAP (binary and text),
Nerfstudio and Polycam layouts read through msplat_dataset_create
(core/src/input_data.cpp:244-261 and core/src/loaders/)."""
import ctypes as C
import json
import os
import struct
import zlib

import numpy as np
import pytest

from msplat_gb300 import _native as N
from msplat_gb300 import api as A


def _lib():
    L = N.lib()
    L.msplat_image_read.argtypes = [C.c_char_p, C.POINTER(C.c_float), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.msplat_dataset_camera.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_int),
                                        C.POINTER(C.c_float), C.POINTER(C.c_uint8)]
    L.msplat_dataset_points.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_uint8)]
    return L


def decode(path):
    L = _lib()
    w, h = C.c_int(), C.c_int()
    assert L.msplat_image_read(str(path).encode(), None, C.byref(w), C.byref(h)) == 0
    out = np.zeros((h.value, w.value, 3), np.float32)
    assert L.msplat_image_read(str(path).encode(), out.ctypes.data_as(C.POINTER(C.c_float)), None, None) == 0
    return out


# ---------------------------------------------------------------- PNG writer

def _png_chunk(t, d):
    return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)


def write_png(path, rows, color_type, depth, palette=None, level=6):
    """rows: list of raw (unfiltered) scanline bytes; each row gets filter y % 5."""
    h = len(rows)
    bits = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[color_type] * depth
    bpp = max(1, bits // 8)
    out = bytearray()
    prev = bytes(len(rows[0]))
    for y, row in enumerate(rows):
        ft = y % 5
        f = bytearray(len(row))
        for x in range(len(row)):
            a = row[x - bpp] if x >= bpp else 0
            b = prev[x]
            c = prev[x - bpp] if x >= bpp else 0
            pred = [0, a, b, (a + b) >> 1, _paeth(a, b, c)][ft]
            f[x] = (row[x] - pred) & 255
        out += bytes([ft]) + f
        prev = row
    w = (len(rows[0]) * 8) // bits
    ihdr = struct.pack(">IIBBBBB", w, h, depth, color_type, 0, 0, 0)
    data = b"\x89PNG\r\n\x1a\n" + _png_chunk(b"IHDR", ihdr)
    if palette is not None:
        data += _png_chunk(b"PLTE", bytes(palette))
    data += _png_chunk(b"IDAT", zlib.compress(bytes(out), level)) + _png_chunk(b"IEND", b"")
    open(path, "wb").write(data)


@pytest.mark.parametrize("level", [0, 1, 9])
def test_png_rgb8_all_filters(tmp_path, level):
    rng = np.random.default_rng(level)
    img = rng.integers(0, 256, (23, 37, 3), dtype=np.uint8)
    img[5:15, 10:30] = img[5, 10]          # runs for the LZ77 matches
    p = tmp_path / "a.png"
    write_png(p, [img[y].tobytes() for y in range(23)], 2, 8, level=level)
    np.testing.assert_array_equal(decode(p), img.astype(np.float32) / 255.0)


def test_png_other_types(tmp_path):
    rng = np.random.default_rng(7)
    g16 = rng.integers(0, 65536, (9, 11), dtype=np.uint16)
    write_png(tmp_path / "g16.png", [g16[y].astype(">u2").tobytes() for y in range(9)], 0, 16)
    d = decode(tmp_path / "g16.png")
    np.testing.assert_allclose(d[..., 0], g16 / 65535.0, atol=1e-6)
    assert np.array_equal(d[..., 0], d[..., 2])
    rgba = rng.integers(0, 256, (8, 6, 4), dtype=np.uint8)
    write_png(tmp_path / "rgba.png", [rgba[y].tobytes() for y in range(8)], 6, 8)
    np.testing.assert_array_equal(decode(tmp_path / "rgba.png"), rgba[..., :3] / np.float32(255.0))
    ga = rng.integers(0, 256, (5, 7, 2), dtype=np.uint8)
    write_png(tmp_path / "ga.png", [ga[y].tobytes() for y in range(5)], 4, 8)
    np.testing.assert_array_equal(decode(tmp_path / "ga.png")[..., 1], ga[..., 0] / np.float32(255.0))
    pal = rng.integers(0, 256, (16, 3), dtype=np.uint8)
    idx = rng.integers(0, 16, (6, 10), dtype=np.uint8)
    packed = [bytes((idx[y, x] << 4) | idx[y, x + 1] for x in range(0, 10, 2)) for y in range(6)]
    write_png(tmp_path / "p4.png", packed, 3, 4, palette=pal.ravel())
    np.testing.assert_array_equal(decode(tmp_path / "p4.png"), pal[idx] / np.float32(255.0))


# --------------------------------------------------------------- JPEG writer
# A baseline JPEG encoder written for the test from T.81: float DCT, one
# quantisation table per component class, Huffman tables of fixed code
# lengths (any canonical code is legal), optional restart intervals.

ZZ = np.array([0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13,
               6, 7, 14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51, 58, 59, 52, 45, 38,
               31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63])


def _dct_matrix():
    c = np.zeros((8, 8))
    for u in range(8):
        for x in range(8):
            c[u, x] = 0.5 * (np.sqrt(0.5) if u == 0 else 1.0) * np.cos((2 * x + 1) * u * np.pi / 16)
    return c


class _Bits:
    def __init__(self):
        self.out, self.acc, self.n = bytearray(), 0, 0

    def put(self, v, k):
        for i in range(k - 1, -1, -1):
            self.acc = (self.acc << 1) | ((v >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0)
                self.acc, self.n = 0, 0

    def flush(self):
        while self.n:
            self.put(1, 1)


def _table(symbols, length):
    codes = {s: (i, length) for i, s in enumerate(symbols)}
    counts = [0] * 16
    counts[length - 1] = len(symbols)
    return codes, bytes(counts) + bytes(symbols)


def write_jpeg(path, rgb, sub=1, q=1, restart=0):
    h, w, _ = rgb.shape
    x = rgb.astype(np.float64)
    Y = 0.299 * x[..., 0] + 0.587 * x[..., 1] + 0.114 * x[..., 2]
    Cb = -0.168736 * x[..., 0] - 0.331264 * x[..., 1] + 0.5 * x[..., 2] + 128
    Cr = 0.5 * x[..., 0] - 0.418688 * x[..., 1] - 0.081312 * x[..., 2] + 128
    mw, mh = 8 * sub, 8 * sub
    W2, H2 = -(-w // mw) * mw, -(-h // mh) * mh
    pad = lambda a: np.pad(a, ((0, H2 - h), (0, W2 - w)), mode="edge")
    Y, Cb, Cr = pad(Y), pad(Cb), pad(Cr)
    if sub == 2:
        Cb = Cb.reshape(H2 // 2, 2, W2 // 2, 2).mean(axis=(1, 3))
        Cr = Cr.reshape(H2 // 2, 2, W2 // 2, 2).mean(axis=(1, 3))
    D = _dct_matrix()
    dc_syms, ac_syms = list(range(12)), [0x00, 0xF0] + [(r << 4) | s for r in range(16) for s in range(1, 11)]
    dc_codes, dc_tab = _table(dc_syms, 4)
    ac_codes, ac_tab = _table(ac_syms, 8)
    bits = _Bits()
    pred = [0, 0, 0]

    def cat(v):
        return 0 if v == 0 else int(abs(v)).bit_length()

    def enc(v, s):
        return v if v >= 0 else v + (1 << s) - 1

    def block(plane, bx, by, ci):
        blk = plane[by * 8:by * 8 + 8, bx * 8:bx * 8 + 8] - 128.0
        F = D @ blk @ D.T
        qv = np.round(F.ravel()[ZZ] / q).astype(int)
        d = qv[0] - pred[ci]
        pred[ci] = qv[0]
        s = cat(d)
        bits.put(*dc_codes[s])
        bits.put(enc(d, s), s)
        run = 0
        for k in range(1, 64):
            if qv[k] == 0:
                run += 1
                continue
            while run > 15:
                bits.put(*ac_codes[0xF0])
                run -= 16
            s = cat(qv[k])
            bits.put(*ac_codes[(run << 4) | s])
            bits.put(enc(qv[k], s), s)
            run = 0
        if run:
            bits.put(*ac_codes[0x00])

    segs = bytearray(b"\xff\xd8")
    qt = bytes([q] * 64)
    segs += b"\xff\xdb" + struct.pack(">H", 67) + b"\x00" + qt
    segs += b"\xff\xc0" + struct.pack(">HBHHB", 17, 8, h, w, 3)
    segs += bytes([1, (sub << 4) | sub, 0, 2, 0x11, 0, 3, 0x11, 0])
    for tc, tab in ((0x00, dc_tab), (0x10, ac_tab)):
        segs += b"\xff\xc4" + struct.pack(">HB", 2 + 1 + len(tab), tc) + tab
    if restart:
        segs += b"\xff\xdd" + struct.pack(">HH", 4, restart)
    segs += b"\xff\xda" + struct.pack(">HB", 12, 3) + bytes([1, 0, 2, 0, 3, 0]) + bytes([0, 63, 0])
    n, rst = 0, 0
    for my in range(H2 // mh):
        for mx in range(W2 // mw):
            if restart and n and n % restart == 0:
                bits.flush()
                segs += bits.out
                bits.out = bytearray()
                segs += bytes([0xFF, 0xD0 + (rst & 7)])
                rst += 1
                pred[:] = [0, 0, 0]
            for vy in range(sub):
                for vx in range(sub):
                    block(Y, mx * sub + vx, my * sub + vy, 0)
            block(Cb, mx, my, 1)
            block(Cr, mx, my, 2)
            n += 1
    bits.flush()
    segs += bits.out + b"\xff\xd9"
    open(path, "wb").write(bytes(segs))


def _smooth(h, w):
    yy, xx = np.mgrid[0:h, 0:w]
    return np.stack([128 + 100 * np.sin(xx / 7.0), 128 + 90 * np.cos(yy / 5.0), (xx + yy) * 255.0 / (w + h)],
                    -1).clip(0, 255)


@pytest.mark.parametrize("sub,restart", [(1, 0), (2, 0), (1, 3), (2, 2)])
def test_jpeg_baseline(tmp_path, sub, restart):
    img = _smooth(37, 50)
    p = tmp_path / "a.jpg"
    write_jpeg(p, img, sub=sub, restart=restart)
    d = decode(p) * 255.0
    assert d.shape == img.shape
    err = np.abs(d - img)
    # q = 1: the error is the rounding of the coefficients and the colour
    # transform, plus chroma averaging when subsampled
    assert err.mean() < (1.5 if sub == 1 else 4.0), err.mean()
    assert err.max() < (6.0 if sub == 1 else 40.0), err.max()


def test_jpeg_real_files():
    sk = pytest.importorskip("sklearn")
    d = os.path.join(os.path.dirname(sk.__file__), "datasets", "images")
    for name in ("china.jpg", "flower.jpg"):
        p = os.path.join(d, name)
        if not os.path.exists(p):
            pytest.skip("sample images absent")
        img = decode(p)
        assert img.shape == (427, 640, 3)
        assert 0.2 < img.mean() < 0.8 and img.std() > 0.05


# -------------------------------------------------------------- layouts

def _pose(eye):
    eye = np.asarray(eye, np.float64)
    f = -eye / np.linalg.norm(eye)
    r = np.cross(f, [0, 0, 1.0])
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    c2w = np.eye(4)
    c2w[:3, 0], c2w[:3, 1], c2w[:3, 2], c2w[:3, 3] = r, u, -f, eye   # OpenGL axes
    return c2w


def _write_ply_points(path, xyz, rgb):
    head = ("ply\nformat binary_little_endian 1.0\nelement vertex %d\nproperty float x\nproperty float y\n"
            "property float z\nproperty uchar red\nproperty uchar green\nproperty uchar blue\nend_header\n" % len(xyz))
    rec = np.zeros(len(xyz), dtype=[("p", "<f4", 3), ("c", "u1", 3)])
    rec["p"], rec["c"] = xyz, rgb
    open(path, "wb").write(head.encode() + rec.tobytes())


def _scene(tmp_path):
    rng = np.random.default_rng(1)
    eyes = [(4 * np.cos(a), 4 * np.sin(a), 1.0 + 0.3 * k) for k, a in enumerate(np.linspace(0, 5, 5))]
    imgs = [rng.integers(0, 256, (24, 32, 3), dtype=np.uint8) for _ in eyes]
    xyz = rng.normal(0, 1, (50, 3)).astype(np.float32)
    rgb = rng.integers(0, 256, (50, 3), dtype=np.uint8)
    return eyes, imgs, xyz, rgb


def _check(ds, eyes, imgs, xyz, rgb, names_sorted, fx=30.0, eval_split=False):
    L = _lib()
    n = ds.num_train + ds.num_test
    assert n == len(eyes)
    # centre and scale as autoScaleAndCenter
    pos = np.array([_pose(e)[:3, 3] for e in eyes], np.float32)
    m = pos.mean(0)
    s = 1.0 / np.abs(pos - m).max()
    for i in range(ds.num_train):
        intr = np.zeros(4, np.float32)
        size = np.zeros(2, np.int32)
        c2w = np.zeros(16, np.float32)
        img = np.zeros((24, 32, 3), np.uint8)
        assert L.msplat_dataset_camera(ds.h, i, 0, intr.ctypes.data_as(C.POINTER(C.c_float)),
                                       size.ctypes.data_as(C.POINTER(C.c_int)),
                                       c2w.ctypes.data_as(C.POINTER(C.c_float)),
                                       img.ctypes.data_as(C.POINTER(C.c_uint8))) == 0
        k = names_sorted[i] if not eval_split else names_sorted[[j for j in range(n) if j % 2][i]]
        assert tuple(size) == (32, 24)
        np.testing.assert_allclose(intr, [fx, fx, 16.0, 12.0], rtol=1e-6)
        want = _pose(eyes[k]).astype(np.float32)
        np.testing.assert_allclose(c2w.reshape(4, 4)[:3, :3], want[:3, :3], atol=1e-5)
        np.testing.assert_allclose(c2w.reshape(4, 4)[:3, 3], (want[:3, 3] - m) * s, atol=1e-5)
        np.testing.assert_array_equal(img, imgs[k])
    pts = np.zeros((len(xyz), 3), np.float32)
    cols = np.zeros((len(xyz), 3), np.uint8)
    assert L.msplat_dataset_points(ds.h, pts.ctypes.data_as(C.POINTER(C.c_float)),
                                   cols.ctypes.data_as(C.POINTER(C.c_uint8))) == len(xyz)
    np.testing.assert_allclose(pts, (xyz - m) * s, atol=1e-5)
    np.testing.assert_array_equal(cols, rgb)


def test_nerfstudio_layout(tmp_path):
    eyes, imgs, xyz, rgb = _scene(tmp_path)
    os.makedirs(tmp_path / "images")
    frames = []
    order = [3, 0, 4, 1, 2]           # written unsorted; the loader sorts by file path
    for k in order:
        write_png(tmp_path / "images" / f"f{k}.png", [imgs[k][y].tobytes() for y in range(24)], 2, 8)
        frames.append({"file_path": f"images/f{k}", "transform_matrix": _pose(eyes[k]).tolist()})
    json.dump({"w": 32, "h": 24, "fl_x": 30.0, "fl_y": 30.0, "cx": 16.0, "cy": 12.0, "frames": frames,
               "ply_file_path": "points.ply"}, open(tmp_path / "transforms.json", "w"))
    _write_ply_points(tmp_path / "points.ply", xyz, rgb)
    ds = A.Dataset(str(tmp_path))
    _check(ds, eyes, imgs, xyz, rgb, list(range(5)))
    ds2 = A.Dataset(str(tmp_path), eval_mode=True, test_every=2)
    assert (ds2.num_train, ds2.num_test) == (2, 3)
    _check(ds2, eyes, imgs, xyz, rgb, list(range(5)), eval_split=True)


def _w2c(c2w_gl):
    c2w = c2w_gl.copy()
    c2w[:3, 1:3] *= -1                 # OpenGL -> OpenCV axes
    w2c = np.linalg.inv(c2w)
    R, t = w2c[:3, :3], w2c[:3, 3]
    # rotation matrix -> quaternion (w, x, y, z)
    w = np.sqrt(max(0.0, 1 + R[0, 0] + R[1, 1] + R[2, 2])) / 2
    x = np.copysign(np.sqrt(max(0.0, 1 + R[0, 0] - R[1, 1] - R[2, 2])) / 2, R[2, 1] - R[1, 2])
    y = np.copysign(np.sqrt(max(0.0, 1 - R[0, 0] + R[1, 1] - R[2, 2])) / 2, R[0, 2] - R[2, 0])
    z = np.copysign(np.sqrt(max(0.0, 1 - R[0, 0] - R[1, 1] + R[2, 2])) / 2, R[1, 0] - R[0, 1])
    return np.array([w, x, y, z]), t


@pytest.mark.parametrize("binary", [True, False])
def test_colmap_layout(tmp_path, binary):
    eyes, imgs, xyz, rgb = _scene(tmp_path)
    sp = tmp_path / "sparse" / "0"
    os.makedirs(sp)
    os.makedirs(tmp_path / "images")
    for k in range(5):
        write_png(tmp_path / "images" / f"im{k}.png", [imgs[k][y].tobytes() for y in range(24)], 2, 8)
    if binary:
        with open(sp / "cameras.bin", "wb") as f:
            f.write(struct.pack("<Q", 1) + struct.pack("<IiQQ", 1, 1, 32, 24) + struct.pack("<4d", 30, 30, 16, 12))
        with open(sp / "images.bin", "wb") as f:
            f.write(struct.pack("<Q", 5))
            for k in [2, 0, 4, 1, 3]:
                q, t = _w2c(_pose(eyes[k]))
                f.write(struct.pack("<I4d3dI", k + 1, *q, *t, 1) + f"im{k}.png".encode() + b"\0")
                f.write(struct.pack("<Q", 1) + struct.pack("<ddQ", 1.0, 2.0, 7))
        with open(sp / "points3D.bin", "wb") as f:
            f.write(struct.pack("<Q", len(xyz)))
            for i in range(len(xyz)):
                f.write(struct.pack("<Q3d3Bd", i, *xyz[i].astype(np.float64), *rgb[i], 0.5))
                f.write(struct.pack("<Q", 2) + struct.pack("<IIII", 1, 0, 2, 0))
    else:
        with open(sp / "cameras.txt", "w") as f:
            f.write("# comment\n1 PINHOLE 32 24 30 30 16 12\n")
        with open(sp / "images.txt", "w") as f:
            f.write("# images\n")
            for k in [2, 0, 4, 1, 3]:
                q, t = _w2c(_pose(eyes[k]))
                v = " ".join(repr(float(a)) for a in (*q, *t))
                f.write(f"{k + 1} {v} 1 im{k}.png\n")
                f.write("1.0 2.0 7\n")
        with open(sp / "points3D.txt", "w") as f:
            for i in range(len(xyz)):
                x, y, z = (float(v) for v in xyz[i])
                f.write(f"{i} {x!r} {y!r} {z!r} {rgb[i][0]} {rgb[i][1]} {rgb[i][2]} 0.5 1 0\n")
    ds = A.Dataset(str(tmp_path))
    _check(ds, eyes, imgs, xyz, rgb, list(range(5)))


def test_polycam_layout(tmp_path):
    eyes, imgs, xyz, rgb = _scene(tmp_path)
    kd = tmp_path / "keyframes" / "corrected_cameras"
    idir = tmp_path / "keyframes" / "corrected_images"
    os.makedirs(kd)
    os.makedirs(idir)
    for k in range(5):
        c2w = _pose(eyes[k])
        # the loader flips rows 1 and 2 of (R | t) into OpenGL axes
        R = c2w[:3, :3].copy()
        t = c2w[:3, 3].copy()
        R[1:] *= -1
        t[1:] *= -1
        d = {"width": 32, "height": 24, "fx": 30.0, "fy": 30.0, "cx": 16.0, "cy": 12.0,
             "t_20": t[0], "t_21": t[1], "t_22": t[2]}
        for a in range(3):
            for b in range(3):
                d[f"R_{a}{b}"] = R[a, b]
        json.dump(d, open(kd / f"{k:03d}.json", "w"))
        write_png(idir / f"{k:03d}.png", [imgs[k][y].tobytes() for y in range(24)], 2, 8)
    _write_ply_points(tmp_path / "keyframes" / "point_cloud.ply", xyz, rgb)
    ds = A.Dataset(str(tmp_path))
    _check(ds, eyes, imgs, xyz, rgb, list(range(5)))


def test_downscale_and_errors(tmp_path):
    eyes, imgs, xyz, rgb = _scene(tmp_path)
    os.makedirs(tmp_path / "images")
    frames = []
    for k in range(5):
        write_png(tmp_path / "images" / f"f{k}.png", [imgs[k][y].tobytes() for y in range(24)], 2, 8)
        frames.append({"file_path": f"images/f{k}.png", "transform_matrix": _pose(eyes[k]).tolist()})
    json.dump({"w": 32, "h": 24, "fl_x": 30.0, "fl_y": 30.0, "cx": 16.0, "cy": 12.0, "frames": frames},
              open(tmp_path / "transforms.json", "w"))
    _write_ply_points(tmp_path / "points3D.ply", xyz, rgb)
    ds = A.Dataset(str(tmp_path), downscale_factor=2.0)
    L = _lib()
    intr, size = np.zeros(4, np.float32), np.zeros(2, np.int32)
    img = np.zeros((12, 16, 3), np.uint8)
    L.msplat_dataset_camera(ds.h, 0, 0, intr.ctypes.data_as(C.POINTER(C.c_float)),
                            size.ctypes.data_as(C.POINTER(C.c_int)), None, img.ctypes.data_as(C.POINTER(C.c_uint8)))
    assert tuple(size) == (16, 12)
    np.testing.assert_allclose(intr, [15.0, 15.0, 8.0, 6.0])
    box = imgs[0].astype(np.float64).reshape(12, 2, 16, 2, 3).mean(axis=(1, 3))
    assert np.abs(img.astype(np.float64) - np.round(box)).max() <= 1
    with pytest.raises(RuntimeError):
        A.Dataset(str(tmp_path / "nothing_here"))
    os.remove(tmp_path / "images" / "f3.png")
    with pytest.raises(RuntimeError):
        A.Dataset(str(tmp_path))


def test_cli_arguments():
    from msplat_gb300 import cli
    a = cli.parse(["data", "-n", "7000", "-d", "0.5", "--eval", "--bg-color", "0", "0.5", "1", "--early-stop", "0.1"])
    assert (a.input, a.num_iters, a.downscale_factor, a.eval) == ("data", 7000, 1.0, True)
    assert a.bg_color == [0.0, 0.5, 1.0] and a.early_stop == 0.1 and a.cap_max == 1_000_000
    # the reference CLI's model options (cli/msplat.mm:90-131)
    a = cli.parse(["data", "--init-opacity", "0.2", "--init-scale", "0.5", "--no-seed-decimation",
                   "--position-lr-max-steps", "7000", "--reg-visibility-duty", "0.25"])
    assert (a.init_opacity, a.init_scale, a.no_seed_decimation, a.position_lr_max_steps,
            a.reg_visibility_duty) == (0.2, 0.5, True, 7000, 0.25)
    d = cli.parse(["data"])
    assert (d.init_opacity, d.init_scale, d.no_seed_decimation, d.position_lr_max_steps,
            d.reg_visibility_duty) == (0.5, 0.1, False, 30000, 1.0)


def test_colmap_mask_dir(tmp_path):
    """--mask-dir (Camera::loadMask): "<dir>/<name>.png" or the name with its
    extension swapped; resized to the image by area averaging; a pixel
    trains where the mask's first channel is above 0.5; an all-white mask or
    a missing one leaves the camera unmasked."""
    eyes, imgs, xyz, rgb = _scene(tmp_path)
    sp = tmp_path / "sparse" / "0"
    os.makedirs(sp)
    os.makedirs(tmp_path / "images")
    md = tmp_path / "masks"
    os.makedirs(md)
    for k in range(5):
        write_png(tmp_path / "images" / f"im{k}.png", [imgs[k][y].tobytes() for y in range(24)], 2, 8)
    with open(sp / "cameras.bin", "wb") as f:
        f.write(struct.pack("<Q", 1) + struct.pack("<IiQQ", 1, 1, 32, 24) + struct.pack("<4d", 30, 30, 16, 12))
    with open(sp / "images.bin", "wb") as f:
        f.write(struct.pack("<Q", 5))
        for k in range(5):
            q, t = _w2c(_pose(eyes[k]))
            f.write(struct.pack("<I4d3dI", k + 1, *q, *t, 1) + f"im{k}.png".encode() + b"\0")
            f.write(struct.pack("<Q", 0))
    with open(sp / "points3D.bin", "wb") as f:
        f.write(struct.pack("<Q", len(xyz)))
        for i in range(len(xyz)):
            f.write(struct.pack("<Q3d3Bd", i, *xyz[i].astype(np.float64), *rgb[i], 0.5) + struct.pack("<Q", 0))
    m0 = np.full((24, 32), 255, np.uint8)
    m0[4:10, 6:20] = 0
    write_png(md / "im0.png.png", [m0[y].tobytes() for y in range(24)], 0, 8)          # appended name, grey PNG
    m1 = np.full((12, 16), 255, np.uint8)
    m1[:6] = 0
    write_png(md / "im1.png", [m1[y].tobytes() for y in range(12)], 0, 8)              # swapped name, half size
    write_png(md / "im2.png.png", [bytes([255] * 32)] * 24, 0, 8)                     # all white: unmasked
    ds = A.Dataset(str(tmp_path), mask_dir=str(md))
    assert np.array_equal(ds.mask(0), np.where(m0 > 127, 255, 0).astype(np.uint8))
    want1 = np.full((24, 32), 255, np.uint8)
    want1[:12] = 0
    assert np.array_equal(ds.mask(1), want1)
    assert ds.mask(2) is None and ds.mask(3) is None and ds.mask(4) is None
    assert A.Dataset(str(tmp_path)).mask(0) is None


def test_validation_hold_out(tmp_path):
    """--val / --val-image (InputData::getCameras): one training camera
    becomes the only test camera — "random" picks std::mt19937(42)'s first
    draw (1608637542) modulo the count, a name picks the first camera whose
    path contains it; eval-mode datasets refuse."""
    eyes, imgs, xyz, rgb = _scene(tmp_path)
    os.makedirs(tmp_path / "images")
    frames = []
    for k in range(5):
        write_png(tmp_path / "images" / f"f{k}.png", [imgs[k][y].tobytes() for y in range(24)], 2, 8)
        frames.append({"file_path": f"images/f{k}.png", "transform_matrix": _pose(eyes[k]).tolist()})
    json.dump({"w": 32, "h": 24, "fl_x": 30.0, "fl_y": 30.0, "cx": 16.0, "cy": 12.0, "frames": frames,
               "ply_file_path": "points.ply"}, open(tmp_path / "transforms.json", "w"))
    _write_ply_points(tmp_path / "points.ply", xyz, rgb)
    ds = A.Dataset(str(tmp_path))
    before = [ds.camera(i)["image"] for i in range(5)]
    assert ds.hold_out("random") == 1608637542 % 5
    assert (ds.num_train, ds.num_test) == (4, 1)
    assert np.array_equal(ds.camera(0, use_test=True)["image"], before[1608637542 % 5])
    ds = A.Dataset(str(tmp_path))
    assert ds.hold_out("f3") == 3 and np.array_equal(ds.camera(0, use_test=True)["image"], before[3])
    ds = A.Dataset(str(tmp_path), eval_mode=True, test_every=2)
    with pytest.raises(RuntimeError):
        ds.hold_out()
    from msplat_gb300 import cli
    a = cli.parse(["data", "--val-render", "out", "--val-image", "f3"])
    assert (a.val, a.val_render, a.val_image) == (False, "out", "f3")


def test_cli_cameras_json(tmp_path):
    """The CLI's cameras.json (InputData::saveCameras): every camera in the
    loader's order (the eval split and a --val camera put back in place),
    file names, sizes, intrinsics, the rotation with the pose's columns 1 and
    2 negated (OpenCV axes) and the position, in the dataset's own frame
    with keep_crs; keys in std::map order as nlohmann writes them."""
    from msplat_gb300 import cli
    eyes, imgs, xyz, rgb = _scene(tmp_path)
    os.makedirs(tmp_path / "images")
    frames = []
    for k in range(5):
        write_png(tmp_path / "images" / f"f{k}.png", [imgs[k][y].tobytes() for y in range(24)], 2, 8)
        frames.append({"file_path": f"images/f{k}.png", "transform_matrix": _pose(eyes[k]).tolist()})
    json.dump({"w": 32, "h": 24, "fl_x": 30.0, "fl_y": 30.0, "cx": 16.0, "cy": 12.0, "frames": frames,
               "ply_file_path": "points.ply"}, open(tmp_path / "transforms.json", "w"))
    _write_ply_points(tmp_path / "points.ply", xyz, rgb)
    full = A.Dataset(str(tmp_path))
    pos = np.array([_pose(e)[:3, 3] for e in eyes], np.float32)
    for kind in ("plain", "eval", "val"):
        if kind == "eval":
            ds, held, every = A.Dataset(str(tmp_path), eval_mode=True, test_every=2), -1, 2
        else:
            ds, every = A.Dataset(str(tmp_path)), 0
            held = ds.hold_out("f3") if kind == "val" else -1
        for keep in (False, True):
            path = tmp_path / f"cams_{kind}_{int(keep)}.json"
            cli.save_cameras(str(path), ds, keep, every, held)
            cams = json.load(open(path))
            assert [c["file_path"] for c in cams] == [f"f{k}.png" for k in range(5)]
            assert list(cams[0].keys()) == sorted(cams[0].keys())
            for k, c in enumerate(cams):
                m = full.camera(k)["cam_to_world"]
                assert (c["width"], c["height"], c["fx"], c["cx"]) == (32, 24, 30.0, 16.0)
                R = np.array(c["rotation"], np.float32)
                assert np.array_equal(R[:, 0], m[:3, 0]) and np.array_equal(R[:, 1:], -m[:3, 1:3])
                want = pos[k] if keep else m[:3, 3]
                np.testing.assert_allclose(c["translation"], want, atol=2e-6 if keep else 0)
