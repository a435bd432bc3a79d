"""The oracle's restatement of the segmentation stages around the graph
stage (oracle/qpso_seg_front.c) against independent numpy restatements of
the same published definitions, and against the properties the algorithms
guarantee.  CPU only.

The reference computes these stages with OpenCV 2.4, which is not
available here, so their parity with the reference is unpinned; these
tests pin the oracle to its own stated definitions, and the GPU tests pin
the kernels to the oracle bit for bit.
"""
import math
from fractions import Fraction

import numpy as np
import pytest

import scene
from oracle import pyoracle as po


def test_hsv_and_gray_follow_the_published_formulas():
    rng = np.random.default_rng(3)
    bgr = rng.integers(0, 256, (64, 80, 3)).astype(np.uint8)
    bgr[0, :6] = [[0, 0, 0], [255, 255, 255], [10, 10, 10], [0, 0, 255], [0, 255, 0], [255, 0, 0]]
    h, s, v, g = po.bgr_to_hsv_gray(bgr)
    for (y, x) in [(0, i) for i in range(6)] + [tuple(p) for p in rng.integers(0, [64, 80], (400, 2))]:
        b, gg, r = (int(c) for c in bgr[y, x])
        mx, mn = max(r, gg, b), min(r, gg, b)
        d = mx - mn
        assert v[y, x] == mx
        want_s = 0 if mx == 0 else math.floor(Fraction(255 * d, mx) + Fraction(1, 2))
        assert s[y, x] == want_s
        if d == 0:
            want_h = 0
        else:
            if mx == r:
                hh = Fraction(60 * (gg - b), d)
            elif mx == gg:
                hh = 120 + Fraction(60 * (b - r), d)
            else:
                hh = 240 + Fraction(60 * (r - gg), d)
            if hh < 0:
                hh += 360
            want_h = math.floor(hh / 2 + Fraction(1, 2))
        assert h[y, x] == want_h
        assert abs(int(g[y, x]) - (0.299 * r + 0.587 * gg + 0.114 * b)) <= 0.5 + 1e-9


def test_gauss_taps():
    t5, t7 = po.gauss_taps(5), po.gauss_taps(7)
    assert t5.sum() == 256 and t7.sum() == 256
    assert list(t5) == list(t5[::-1]) and list(t7) == list(t7[::-1])
    for taps, k in ((t5, 5), (t7, 7)):
        sigma = 0.3 * ((k - 1) * 0.5 - 1) + 0.8
        g = np.exp(-((np.arange(k) - k // 2) ** 2) / (2 * sigma * sigma))
        assert np.abs(taps - g / g.sum() * 256).max() <= 1.0


def _blur_np(src, k):
    taps = po.gauss_taps(k).astype(np.int64)
    c = k // 2
    p = np.pad(src.astype(np.int64), c, mode="reflect")  # numpy "reflect" is reflect-101
    rows = sum(taps[i] * p[c:-c, i:i + src.shape[1]] for i in range(k))
    rp = np.pad(rows, ((c, c), (0, 0)), mode="reflect")
    cols = sum(taps[i] * rp[i:i + src.shape[0], :] for i in range(k))
    return ((cols + 32768) >> 16).astype(np.uint8)


@pytest.mark.parametrize("k", [5, 7])
def test_blur_is_the_integer_separable_filter(k):
    rng = np.random.default_rng(k)
    img = rng.integers(0, 256, (37, 53)).astype(np.uint8)
    np.testing.assert_array_equal(po.blur_u8(img, k), _blur_np(img, k))


def test_orientation_bins_match_atan2_away_from_the_edges():
    rng = np.random.default_rng(5)
    for x, y in rng.integers(-4080, 4081, (3000, 2)):
        deg = math.degrees(math.atan2(-y, -x)) + 180.0
        edges = [22.5, 67.5, 112.5, 157.5, 202.5, 247.5, 292.5, 337.5]
        if min(abs(deg - e) for e in edges) < 1e-3 or (x == 0 and y == 0):
            continue
        if deg < 22.5 or 157.5 <= deg < 202.5 or deg >= 337.5:
            want = 0
        elif deg < 67.5 or 202.5 <= deg < 247.5:
            want = 45
        elif deg < 112.5 or 247.5 <= deg < 292.5:
            want = 90
        else:
            want = 135
        assert po.orient_bin(int(x), int(y)) == want, (x, y, deg)
    assert po.orient_bin(0, 0) == 0


def _smooth_np(d, beta, gamma):
    """numpy restatement of the depth smoothing with the same float order."""
    H, W = d.shape
    alfa = np.float32(np.float32(0.0028) / np.float32(1e6))
    fdc = (d.astype(np.int64) ** 2).astype(np.float32) * alfa
    tdc = np.float32(gamma) * fdc
    C = np.zeros((H, W), bool)
    di = d.astype(np.int64)
    for r in range(1, H - 1):
        for c in range(1, W - 1):
            if np.float32(abs(di[r, c + 1] - di[r, c])) >= tdc[r, c]:
                C[r, c] = C[r, c + 1] = C[r, c - 1] = True
            if np.float32(abs(di[r + 1, c] - di[r, c])) >= tdc[r, c]:
                C[r, c] = C[r + 1, c] = C[r - 1, c] = True
    mod = np.where(C, 0, d).astype(np.uint16)
    ys, xs = np.nonzero(C)
    if len(ys):
        yy, xx = np.mgrid[0:H, 0:W]
        d2 = np.full((H, W), np.iinfo(np.int64).max, np.int64)
        for y0, x0 in zip(ys, xs):
            d2 = np.minimum(d2, (yy - y0) ** 2 + (xx - x0) ** 2)
        T = np.sqrt(d2.astype(np.float32)).astype(np.float32) * np.float32(0.70710677)
    else:
        T = np.full((H, W), np.inf, np.float32)
    B = np.float32(beta) * fdc
    R = np.where(B < T, B, T).astype(np.float32)
    rows = np.cumsum(mod.astype(np.float32), axis=1, dtype=np.float32)
    I = np.zeros((H + 1, W + 1), np.float32)
    I[1:, 1:] = np.cumsum(rows, axis=0, dtype=np.float32)
    Z = np.zeros((H + 1, W + 1), np.int64)
    Z[1:, 1:] = np.cumsum(np.cumsum(mod == 0, axis=1), axis=0)
    out = np.zeros((H, W), np.uint16)
    for r in range(15, H - 15):
        for c in range(15, W - 15):
            radi = int(np.float32(R[r, c] + np.float32(0.5)))
            if radi == 0:
                out[r, c] = d[r, c]
                continue
            x0, x1 = max(c - radi, 0), min(c + radi + 1, W)
            y0, y1 = max(r - radi, 0), min(r + radi + 1, H)
            den = (x1 - x0) * (y1 - y0)
            nz = Z[y1, x1] + Z[y0, x0] - Z[y1, x0] - Z[y0, x1]
            if den == nz:
                out[r, c] = d[r, c]
                continue
            s = np.float32(np.float32(np.float32(I[y1, x1] + I[y0, x0]) - I[y1, x0]) - I[y0, x1])
            v = np.float32(np.float32(np.float32(1.0) / np.float32(den - nz)) * s) + np.float32(0.5)
            out[r, c] = 0 if v <= 0 else 65535 if v >= 65535 else int(v)
    return out, C, R


def test_depth_smoothing_matches_a_numpy_restatement():
    depth, _, _ = scene.segmentation_frame_c5()
    d = depth[100:160, 200:275].copy()
    d[5:9, 10:14] = 0
    got, C, R = po.depth_smooth(d, with_maps=True)
    want, Cw, Rw = _smooth_np(d, 2000.0, 18000.0)
    np.testing.assert_array_equal(C.astype(bool), Cw)
    np.testing.assert_array_equal(R, Rw)
    np.testing.assert_array_equal(got, want)


def test_depth_smoothing_averages_a_flat_patch_and_keeps_the_border_zero():
    d = np.full((60, 70), 1000, np.uint16)
    d[30, 35] = 0  # a dropout pixel: its neighbours are marked, it keeps its depth
    out = po.depth_smooth(d)
    assert (out[:15] == 0).all() and (out[-15:] == 0).all() and (out[:, :15] == 0).all()
    inner = out[15:-15, 15:-15]
    assert inner[30 - 15, 35 - 15] == 0
    assert (np.delete(inner.ravel(), (30 - 15) * inner.shape[1] + 35 - 15) == 1000).all()


def test_telea_fills_only_the_mask_and_keeps_constants():
    img = np.full((24, 30), 77, np.uint8)
    mask = np.zeros_like(img)
    mask[5:12, 8:20] = 1
    out = po.telea(np.where(mask, 0, img), mask, radius=5)
    np.testing.assert_array_equal(out, img)
    # no mask: unchanged
    rng = np.random.default_rng(1)
    a = rng.integers(1, 255, (20, 20)).astype(np.uint8)
    np.testing.assert_array_equal(po.telea(a, np.zeros_like(a), 6), a)


def test_telea_continues_a_ramp():
    yy, xx = np.mgrid[0:40, 0:50]
    ramp = (40 + 3 * xx).astype(np.uint8)
    mask = np.zeros(ramp.shape, np.uint8)
    mask[12:28, 18:30] = 1
    out = po.telea(np.where(mask, 0, ramp), mask, radius=8)
    assert (out[mask == 0] == ramp[mask == 0]).all()
    assert np.abs(out[mask == 1].astype(int) - ramp[mask == 1].astype(int)).max() <= 3


def test_eikonal_update_and_arrival_times():
    import ctypes as C

    f = po.lib().qo_eikonal2
    f.restype = C.c_float
    f.argtypes = [C.c_float, C.c_float]
    assert f(0.0, 0.0) == np.float32((0.0 + 0.0 + math.sqrt(2.0)) / 2)
    assert f(0.0, 1.5) == 1.0
    assert f(2.0, float("inf")) == 3.0
    assert f(float("inf"), float("inf")) == float("inf")
    # a masked 5 x 5 square in a known frame: times grow inwards, symmetric
    mask = np.zeros((9, 9), np.uint8)
    mask[2:7, 2:7] = 1
    T = np.zeros(mask.shape, np.float32)
    g = po.lib().qo_telea_times
    g.restype = C.c_int32
    it = g(mask.ctypes.data_as(C.c_void_p), 9, 9, T.ctypes.data_as(C.c_void_p))
    assert it > 0
    assert (T[mask == 0] == 0).all()
    np.testing.assert_array_equal(T, T.T)
    np.testing.assert_array_equal(T, T[::-1, ::-1])
    # the corner from two known neighbours; the edge from the known pixel
    # and the edge pixels beside it (as the march computes them); growing inwards
    assert T[2, 2] == np.float32(math.sqrt(2.0) / 2)
    assert abs(T[2, 4] - 1.0) < 1e-3 and 1.9 < T[3, 4] < 2.0
    assert T[2, 4] < T[3, 4] < T[4, 4]


def _resize_np(src, dw, dh):
    sh, sw = src.shape

    def coef(n_d, n_s):
        out = []
        for dx in range(n_d):
            f = np.float32((dx + 0.5) * (n_s / n_d) - 0.5)
            s = int(np.floor(f))
            f = np.float32(f - np.float32(s))
            if s < 0:
                f, s = np.float32(0), 0
            if s >= n_s - 1:
                f, s = np.float32(0), n_s - 1
            a0 = int(np.rint(np.float32(np.float32(1.0) - f) * np.float32(2048.0)))
            out.append((s, min(s + 1, n_s - 1), a0))
        return out

    cx, cy = coef(dw, sw), coef(dh, sh)
    out = np.empty((dh, dw), np.uint8)
    s64 = src.astype(np.int64)
    for y, (y0, y1, b0) in enumerate(cy):
        for x, (x0, x1, a0) in enumerate(cx):
            r0 = a0 * s64[y0, x0] + (2048 - a0) * s64[y0, x1]
            r1 = a0 * s64[y1, x0] + (2048 - a0) * s64[y1, x1]
            out[y, x] = (b0 * r0 + (2048 - b0) * r1 + (1 << 21)) >> 22
    return out


def test_bilinear_resize():
    rng = np.random.default_rng(8)
    src = rng.integers(0, 256, (12, 16)).astype(np.uint8)
    np.testing.assert_array_equal(po.resize_bilinear_u8(src, 80, 60), _resize_np(src, 80, 60))
    np.testing.assert_array_equal(po.resize_bilinear_u8(src, 7, 5), _resize_np(src, 7, 5))


def test_inpainting_fills_every_hole_of_a_frame():
    depth, _, _ = scene.segmentation_frame_c5()
    sm = po.depth_smooth(depth)
    out, small = po.inpaint_depth(sm, with_small=True)
    assert small.shape == (96, 128)
    assert (small > 0).all()
    assert (out > 0).all()
    keep = sm != 0
    np.testing.assert_array_equal(out[keep], sm[keep])
    # filled values stay inside the frame's depth range
    assert out.max() <= sm.max() and out.min() >= 1


def test_cluster_records_from_exact_moments():
    depth, gt, bgr = scene.segmentation_frame_c5()
    h, s, v, _ = po.bgr_to_hsv_gray(bgr)
    labels = gt + 1  # plane is set 0, objects 1..15
    n_sets = int(labels.max()) + 1
    recs = po.seg_clusters(labels, n_sets, depth, v, keep_all=True)
    fp = po.seg_front_params()
    assert [r.label for r in recs] == list(range(n_sets))
    for r in recs:
        ys, xs = np.nonzero(labels == r.label)
        assert r.pixels == len(xs) and r.num_points == len(xs) + 1
        assert (r.min_x, r.max_x, r.min_y, r.max_y) == (xs.min(), xs.max() + 1, ys.min(), ys.max() + 1)
        z = depth[ys, xs].astype(np.float64)
        ok = z > 0
        cen = [((xs[ok] - fp.cx) * z[ok] / fp.fx).mean(), ((ys[ok] - fp.cy) * z[ok] / fp.fy).mean(), z[ok].mean()]
        np.testing.assert_allclose(list(r.centroid_mm), cen, rtol=1e-5, atol=1e-3)
        ev = np.sort(np.linalg.eigvalsh(np.cov(np.stack([xs, ys]).astype(np.float64), bias=True)))[::-1]
        np.testing.assert_allclose(list(r.eig), ev, rtol=1e-9, atol=1e-9)
        assert r.nan_ratio == np.float32(np.float32((~ok).sum()) / np.float32(len(xs) + 1))
    # the plane spans the frame: too eccentric or too spread for an object
    assert not recs[0].kept


def test_end_to_end_oracle_segments_the_objects():
    """From the colour image and depth alone, the kept clusters of the C5
    segmentation frame cover most of the large objects."""
    depth, gt, bgr = scene.segmentation_frame_c5()
    r = po.segment_rgbd(bgr, depth)
    assert (r["inpainted"] > 0).all()
    assert 0.0 <= r["saliency"].min() and r["saliency"].max() <= 1.0
    found = 0
    for k in range(int(gt.max()) + 1):
        m = gt == k
        if m.sum() < 900:
            continue
        best = 0.0
        for c in r["clusters"]:
            lab = r["labels"] == c.label
            best = max(best, (lab & m).sum() / (lab | m).sum())
        found += best > 0.5
    assert found >= 6
