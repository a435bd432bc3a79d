"""Input formats of the reference's command line (host only, no GPU):
Wavefront OBJ into the loadOBJ3 layout (main.h:620-679), the ACCV binary
depth of loadDepth (main.cu:35-64) and greyscale PNG depth / label images
(README.md: "640x480 png images"), and the command-line drop-in's argument
and input errors."""
import os
import struct
import subprocess
import zlib

import numpy as np
import pytest

import qpso
import scene

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "q-pso_gb300", "_build", "qpso_main")


# ---- writers used by the tests (and by the GPU test of the command line) ----
def write_obj(path, soa, F, quads=False):
    """Every face corner as its own vertex, printed with 9 significant
    digits (exact float32 round trip)."""
    lines = ["# test mesh", "o mesh"]
    for f in range(F):
        for j in range(3):
            x, y, z = soa[f + j * F], soa[3 * F + f + j * F], soa[6 * F + f + j * F]
            lines.append("v %.9g %.9g %.9g" % (x, y, z))
    for f in range(F):
        a = 3 * f + 1
        lines.append("f %d/%d/%d %d//%d %d" % (a, a, a, a + 1, a + 1, a + 2))
    with open(path, "w") as fp:
        fp.write("\n".join(lines) + "\n")


def write_accv(path, img):
    img = np.ascontiguousarray(img, np.uint16)
    with open(path, "wb") as fp:
        fp.write(struct.pack("<ii", img.shape[0], img.shape[1]))
        fp.write(img.tobytes())


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)


def write_png_gray(path, img, bits=16, level=6, filters=(0,), corrupt_crc=False, interlace=0):
    """Greyscale PNG with the given row filters (cycled) and zlib level."""
    img = np.asarray(img)
    h, w = img.shape
    bpp = bits // 8
    raw = bytearray()
    prev = bytes(w * bpp)
    for y in range(h):
        row = img[y].astype(">u2").tobytes() if bits == 16 else img[y].astype(np.uint8).tobytes()
        ft = filters[y % len(filters)]
        out = bytearray()
        for i in range(len(row)):
            a = row[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            pred = [0, a, b, (a + b) >> 1, _paeth(a, b, c)][ft]
            out.append((row[i] - pred) & 0xFF)
        raw += bytes([ft]) + out
        prev = row

    def chunk(t, d):
        crc = zlib.crc32(t + d) & 0xFFFFFFFF
        if corrupt_crc and t == b"IDAT":
            crc ^= 1
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", crc)

    ihdr = struct.pack(">IIBBBBB", w, h, bits, 0, 0, 0, interlace)
    comp = zlib.compress(bytes(raw), level)
    half = len(comp) // 2  # two IDAT chunks
    data = (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", ihdr) + chunk(b"tEXt", b"k\x00v") +
            chunk(b"IDAT", comp[:half]) + chunk(b"IDAT", comp[half:]) + chunk(b"IEND", b""))
    with open(path, "wb") as fp:
        fp.write(data)
    return comp


def write_png_color(path, img, filters=(0, 1, 2, 3, 4), level=6, bits=8):
    """RGB (h, w, 3), RGBA (h, w, 4) or grey + alpha (h, w, 2) PNG."""
    img = np.asarray(img)
    h, w, ch = img.shape
    ctype = {2: 4, 3: 2, 4: 6}[ch]
    bpp = ch * bits // 8
    raw = bytearray()
    prev = bytes(w * bpp)
    for y in range(h):
        row = img[y].astype(">u2").tobytes() if bits == 16 else img[y].astype(np.uint8).tobytes()
        ft = filters[y % len(filters)]
        out = bytearray()
        for i in range(len(row)):
            a = row[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            pred = [0, a, b, (a + b) >> 1, _paeth(a, b, c)][ft]
            out.append((row[i] - pred) & 0xFF)
        raw += bytes([ft]) + out
        prev = row

    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF)

    ihdr = struct.pack(">IIBBBBB", w, h, bits, ctype, 0, 0, 0)
    data = (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", ihdr) + chunk(b"IDAT", zlib.compress(bytes(raw), level)) +
            chunk(b"IEND", b""))
    with open(path, "wb") as fp:
        fp.write(data)


def write_ppm(path, rgb, comment=True):
    h, w, _ = rgb.shape
    head = b"P6\n" + (b"# made by the tests\n" if comment else b"") + b"%d %d\n255\n" % (w, h)
    with open(path, "wb") as fp:
        fp.write(head + np.ascontiguousarray(rgb, np.uint8).tobytes())


def _block_types(comp):
    """BTYPE of the first deflate block of a zlib stream."""
    return (comp[2] >> 1) & 3


# ---- OBJ ----
def test_obj_round_trip_is_exact(tmp_path):
    soa, F = scene.make_mesh("ellipsoid", 300, 80.0, seed=2)
    p = str(tmp_path / "m.obj")
    write_obj(p, soa, F)
    got, n = qpso.obj_load(p)
    assert n == F
    np.testing.assert_array_equal(got, np.asarray(soa, np.float32))


def test_obj_polygons_negative_indices_and_junk(tmp_path):
    p = tmp_path / "q.obj"
    p.write_text("""# quad and pentagon
mtllib x.mtl
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
vn 0 0 1
vt 0 0
g side
usemtl red
f 1/1/1 2/1/1 3/1/1 4/1/1
v 2 0 1
v 3 0 1
v 3 1 1
v 2.5 2 1
v 2 1 1
f -5 -4 -3 -2 -1
l 1 2
s off
""")
    soa, F = qpso.obj_load(str(p))
    assert F == 2 + 3  # quad -> 2 fan triangles, pentagon -> 3
    V = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [2, 0, 1], [3, 0, 1], [3, 1, 1],
                  [2.5, 2, 1], [2, 1, 1]], np.float32)
    tris = [(0, 1, 2), (0, 2, 3), (4, 5, 6), (4, 6, 7), (4, 7, 8)]
    for f, t in enumerate(tris):
        for j in range(3):
            for c in range(3):
                assert soa[f + j * F + c * 3 * F] == V[t[j], c]


@pytest.mark.parametrize("text", ["v 0 0 0\nv 1 0 0\nf 1 2 3\n",   # index out of range
                                  "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2\n",  # two corners
                                  "v 0 0 nan\nv 1 0 0\nv 0 1 0\nf 1 2 3\n",
                                  "v 0 0 0\n"])  # no face
def test_obj_malformed(tmp_path, text):
    p = tmp_path / "bad.obj"
    p.write_text(text)
    with pytest.raises(qpso.QpsoError) as e:
        qpso.obj_load(str(p))
    assert e.value.status == qpso.ERR_ARG


def test_missing_files(tmp_path):
    with pytest.raises(qpso.QpsoError) as e:
        qpso.obj_load(str(tmp_path / "none.obj"))
    assert e.value.status == qpso.ERR_NOT_FOUND
    with pytest.raises(qpso.QpsoError) as e:
        qpso.image_u16_load(str(tmp_path / "none.png"))
    assert e.value.status == qpso.ERR_NOT_FOUND


# ---- depth images ----
def _depth(seed=0, h=48, w=64):
    rng = np.random.default_rng(seed)
    d = rng.integers(0, 65536, (h, w)).astype(np.uint16)
    d[10:20, 5:30] = 1234  # runs that compress to back-references
    d[30:] = 0
    return d


def test_accv_round_trip_and_size_check(tmp_path):
    d = _depth(1, 480, 640)
    p = str(tmp_path / "d.bin")
    write_accv(p, d)
    np.testing.assert_array_equal(qpso.image_u16_load(p), d)
    with open(p, "ab") as fp:
        fp.write(b"\0")  # one byte too many
    with pytest.raises(qpso.QpsoError):
        qpso.image_u16_load(p)


@pytest.mark.parametrize("level", [0, 1, 9])
@pytest.mark.parametrize("filters", [(0,), (1,), (2,), (3,), (4,), (0, 1, 2, 3, 4)])
def test_png16_all_filters_and_block_types(tmp_path, level, filters):
    """Level 0 gives stored blocks, level 1 fixed-Huffman ones on small
    inputs, level 9 dynamic ones; every row filter type."""
    d = _depth(2)
    p = str(tmp_path / "d.png")
    comp = write_png_gray(p, d, 16, level, filters)
    assert _block_types(comp) == (0 if level == 0 else 2)
    np.testing.assert_array_equal(qpso.image_u16_load(p), d)


def test_png_fixed_huffman_block(tmp_path):
    d = np.full((3, 5), 300, np.uint16)
    p = str(tmp_path / "tiny.png")
    assert _block_types(write_png_gray(p, d, 16, 1)) == 1
    np.testing.assert_array_equal(qpso.image_u16_load(p), d)


def test_png8_labels(tmp_path):
    lab = np.zeros((40, 50), np.uint8)
    lab[5:15, 5:20] = 1
    lab[20:35, 30:45] = 7
    p = str(tmp_path / "l.png")
    write_png_gray(p, lab, 8, 9, (0, 1, 2, 3, 4))
    np.testing.assert_array_equal(qpso.image_u16_load(p), lab.astype(np.uint16))


def test_png_rejects_bad_crc_and_interlace(tmp_path):
    d = _depth(3, 8, 8)
    p = str(tmp_path / "c.png")
    write_png_gray(p, d, 16, 6, corrupt_crc=True)
    with pytest.raises(qpso.QpsoError) as e:
        qpso.image_u16_load(p)
    assert e.value.status == qpso.ERR_ARG
    write_png_gray(p, d, 16, 6, interlace=1)
    with pytest.raises(qpso.QpsoError):
        qpso.image_u16_load(p)
    with open(p, "wb") as fp:  # truncated
        fp.write(b"\x89PNG\r\n\x1a\n\0\0")
    with pytest.raises(qpso.QpsoError):
        qpso.image_u16_load(p)


# ---- command line (argument and input errors need no GPU) ----
def test_cli_usage_and_input_errors(tmp_path):
    r = subprocess.run([CLI], capture_output=True, text=True)
    assert r.returncode == 0 and "Usage:" in r.stdout
    r = subprocess.run([CLI, str(tmp_path / "none.obj"), "rgb.png", "d.png", "0"], capture_output=True,
                       text=True)
    assert r.returncode == 1 and "none.obj" in r.stderr
    soa, F = scene.make_mesh("box", 12, 50.0, seed=0)
    obj = str(tmp_path / "m.obj")
    write_obj(obj, soa, F)
    dep = str(tmp_path / "d.bin")
    write_accv(dep, _depth(4))
    # no label map: the frame is segmented from the colour image, which must exist
    r = subprocess.run([CLI, obj, str(tmp_path / "rgb.png"), dep, "0"], capture_output=True, text=True)
    assert r.returncode == 1 and "rgb.png" in r.stderr and "not found" in r.stderr
    rgb = str(tmp_path / "small.ppm")
    write_ppm(rgb, np.zeros((10, 12, 3), np.uint8))
    r = subprocess.run([CLI, obj, rgb, dep, "0"], capture_output=True, text=True)
    assert r.returncode == 1 and "size differs" in r.stderr
    r = subprocess.run([CLI, obj, "rgb.png", dep, "x"], capture_output=True, text=True)
    assert r.returncode == 1 and "cluster_idx" in r.stderr
    r = subprocess.run([CLI, obj, "rgb.png", dep, "0", "--particles"], capture_output=True, text=True)
    assert r.returncode == 1 and "missing value" in r.stderr


# ---- colour images ----
def test_colour_png_and_ppm_to_bgr(tmp_path):
    rng = np.random.default_rng(4)
    rgb = rng.integers(0, 256, (23, 31, 3)).astype(np.uint8)
    bgr = rgb[..., ::-1]
    p = str(tmp_path / "c.png")
    write_png_color(p, rgb)
    np.testing.assert_array_equal(qpso.image_bgr8_load(p), bgr)
    alpha = rng.integers(0, 256, (23, 31, 1)).astype(np.uint8)
    write_png_color(p, np.concatenate([rgb, alpha], 2), filters=(4, 3))
    np.testing.assert_array_equal(qpso.image_bgr8_load(p), bgr)
    write_png_color(p, rgb.astype(np.uint16) * 256 + 3, bits=16)
    np.testing.assert_array_equal(qpso.image_bgr8_load(p), bgr)
    grey = rgb[..., 0]
    write_png_color(p, np.stack([grey, alpha[..., 0]], 2))
    np.testing.assert_array_equal(qpso.image_bgr8_load(p), np.repeat(grey[..., None], 3, 2))
    write_png_gray(p, grey, bits=8)
    np.testing.assert_array_equal(qpso.image_bgr8_load(p), np.repeat(grey[..., None], 3, 2))
    q = str(tmp_path / "c.ppm")
    write_ppm(q, rgb)
    np.testing.assert_array_equal(qpso.image_bgr8_load(q), bgr)
    write_ppm(q, rgb, comment=False)
    np.testing.assert_array_equal(qpso.image_bgr8_load(q), bgr)


@pytest.mark.parametrize("data", [b"P6\n4 4\n65535\n" + bytes(96), b"P6\n4 4\n255\n" + bytes(10), b"P5\n1 1\n255\n\x00",
                                  b"P6\n-1 4\n255\n"])
def test_bad_colour_images_are_refused(tmp_path, data):
    p = str(tmp_path / "bad.ppm")
    with open(p, "wb") as fp:
        fp.write(data)
    with pytest.raises(qpso.QpsoError) as e:
        qpso.image_bgr8_load(p)
    assert e.value.status == qpso.ERR_ARG
