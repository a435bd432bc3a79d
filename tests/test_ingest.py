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


# ---- the JPEG writer (cluster images of the command line) -------------------

_JPEG_ZIG = np.array([0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48, 41, 34, 27, 20,
                      13, 6, 7, 14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51, 58, 59,
                      52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63])


def _jpeg_decode(data: bytes):
    """A baseline sequential JPEG decoder (ITU-T T.81, Annex F), enough for
    the writer's files (4:4:4, one scan, no restart intervals): returns
    (height, width, 3) B G R and the parsed tables."""
    i, q, huff, comps, scan = 2, {}, {}, [], None
    assert data[:2] == b"\xff\xd8"
    while scan is None:
        assert data[i] == 0xFF
        marker, n = data[i + 1], int.from_bytes(data[i + 2:i + 4], "big")
        seg = data[i + 4:i + 2 + n]
        if marker == 0xDB:
            q[seg[0] & 15] = np.frombuffer(seg[1:65], np.uint8).astype(np.int32)
        elif marker == 0xC0:
            h, w = int.from_bytes(seg[1:3], "big"), int.from_bytes(seg[3:5], "big")
            comps = [(seg[6 + 3 * k], seg[7 + 3 * k], seg[8 + 3 * k]) for k in range(seg[5])]
        elif marker == 0xC4:
            j = 0
            while j < len(seg):
                tc_th, bits = seg[j], seg[j + 1:j + 17]
                vals = seg[j + 17:j + 17 + sum(bits)]
                codes, code, k = {}, 0, 0
                for length in range(1, 17):
                    for _ in range(bits[length - 1]):
                        codes[(length, code)] = vals[k]
                        k += 1
                        code += 1
                    code <<= 1
                huff[tc_th] = (codes, bytes(vals))
                j += 17 + sum(bits)
        elif marker == 0xDA:
            scan = {seg[1 + 2 * k]: seg[2 + 2 * k] for k in range(seg[0])}
        i += 2 + n
    # entropy-coded data up to EOI, stuffed zero bytes removed
    end = data.index(b"\xff\xd9", i)
    raw = data[i:end].replace(b"\xff\x00", b"\xff")
    bits = np.unpackbits(np.frombuffer(raw, np.uint8))
    pos = 0

    def read(nb):
        nonlocal pos
        v = 0
        for _ in range(nb):
            v = (v << 1) | int(bits[pos])
            pos += 1
        return v

    def symbol(codes):
        code = 0
        for length in range(1, 17):
            code = (code << 1) | read(1)
            if (length, code) in codes:
                return codes[(length, code)]
        raise AssertionError("no Huffman code matches")

    def extend(v, s):
        return v if s == 0 or v >= (1 << (s - 1)) else v - (1 << s) + 1

    c8 = np.array([[(np.sqrt(0.125) if u == 0 else 0.5) * np.cos((2 * x + 1) * u * np.pi / 16) for x in range(8)]
                   for u in range(8)])
    planes = [np.zeros(((h + 7) // 8 * 8, (w + 7) // 8 * 8)) for _ in comps]
    pred = [0] * len(comps)
    for by in range(0, h, 8):
        for bx in range(0, w, 8):
            for ci, (cid, _hv, tq) in enumerate(comps):
                td, ta = scan[cid] >> 4, scan[cid] & 15
                zz = np.zeros(64)
                s = symbol(huff[td][0])
                pred[ci] += extend(read(s), s)
                zz[0] = pred[ci]
                k = 1
                while k < 64:
                    rs = symbol(huff[0x10 | ta][0])
                    r, s = rs >> 4, rs & 15
                    if s == 0:
                        if r != 15:
                            break
                        k += 16
                        continue
                    k += r
                    zz[k] = extend(read(s), s)
                    k += 1
                coef = np.zeros(64)
                coef[_JPEG_ZIG] = zz * q[tq]
                planes[ci][by:by + 8, bx:bx + 8] = c8.T @ coef.reshape(8, 8) @ c8 + 128.0
    Y, Cb, Cr = (p[:h, :w] for p in planes)
    R = Y + 1.402 * (Cr - 128)
    G = Y - 0.344136 * (Cb - 128) - 0.714136 * (Cr - 128)
    B = Y + 1.772 * (Cb - 128)
    img = np.clip(np.rint(np.stack([B, G, R], -1)), 0, 255).astype(np.uint8)
    return img, {"huff": huff, "q": q, "comps": comps, "size": (h, w)}


def test_jpeg_writer_round_trip(tmp_path):
    import qpso

    H, W = 37, 53  # not multiples of 8: padded blocks
    yy, xx = np.mgrid[0:H, 0:W]
    bgr = np.stack([(xx * 4) % 256, (yy * 6) % 256, 128 + 60 * np.sin(xx / 5.0) * np.cos(yy / 7.0)], -1)
    bgr = bgr.astype(np.uint8)
    bgr[10:20, 20:30] = 0  # a black cut-out, as in a cluster image
    p = str(tmp_path / "c.jpg")
    qpso.image_jpeg_write(p, bgr, 95)
    data = open(p, "rb").read()
    assert data[:2] == b"\xff\xd8" and data[-2:] == b"\xff\xd9"
    img, info = _jpeg_decode(data)
    assert info["size"] == (H, W) and [c[1] for c in info["comps"]] == [0x11] * 3
    # the Annex K tables: each AC table codes exactly EOB, ZRL and every
    # (run, size) with size 1..10
    want = {0x00, 0xF0} | {(r << 4) | s for r in range(16) for s in range(1, 11)}
    for tc_th in (0x10, 0x11):
        assert set(info["huff"][tc_th][1]) == want and len(info["huff"][tc_th][1]) == 162
    err = img.astype(np.float64) - bgr
    psnr = 10 * np.log10(255.0 ** 2 / np.mean(err ** 2))
    assert psnr > 34.0, psnr


def test_jpeg_writer_quality_and_arguments(tmp_path):
    import qpso

    rng = np.random.default_rng(2)
    bgr = rng.integers(0, 256, (16, 24, 3), dtype=np.uint8)
    sizes = []
    for qual in (10, 50, 95, 100):
        p = str(tmp_path / ("q%d.jpg" % qual))
        qpso.image_jpeg_write(p, bgr, qual)
        data = open(p, "rb").read()
        img, _ = _jpeg_decode(data)
        assert img.shape == bgr.shape
        sizes.append(len(data))
    assert sizes == sorted(sizes)  # higher quality, larger file
    with pytest.raises(qpso.QpsoError):
        qpso.image_jpeg_write(str(tmp_path / "x.jpg"), bgr, 0)
    with pytest.raises(qpso.QpsoError):
        qpso.image_jpeg_write(str(tmp_path / "no_such_dir" / "x.jpg"), bgr, 90)


@pytest.mark.parametrize("shape", [(1, 1), (8, 8), (9, 1), (480, 640)], ids=["1x1", "8x8", "9x1", "640x480"])
def test_jpeg_writer_small_and_black_frames(tmp_path, shape):
    """A single pixel, one exact block, a one-pixel column, and a full
    black frame with one coloured patch (what a cluster image mostly is:
    blocks that code as DC 0 and end-of-block)."""
    import qpso

    H, W = shape
    bgr = np.zeros((H, W, 3), np.uint8)
    bgr[: max(1, H // 8), : max(1, W // 8)] = (40, 200, 90)
    p = str(tmp_path / "s.jpg")
    qpso.image_jpeg_write(p, bgr, 95)
    img, info = _jpeg_decode(open(p, "rb").read())
    assert info["size"] == (H, W)
    assert np.abs(img.astype(np.int32) - bgr).max() <= 24
    # 8x8 blocks that hold no patch pixel are black in, and exactly black
    # out: their level-shifted DC, -1024, is a multiple of quality 95's
    # DC step (2), and every AC coefficient is 0
    ph, pw = max(1, H // 8), max(1, W // 8)
    by0, bx0 = (ph + 7) // 8 * 8, (pw + 7) // 8 * 8
    assert not img[by0:].any() and not img[:, bx0:].any()
