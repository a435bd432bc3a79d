"""The pixel graph that feeds the segmentation (no GPU): the oracle's
restatement of the reference's Gaussian smoothing (GraphCannySeg.h:423-489),
depth normalisation (GraphCannySeg.cpp:1105-1127) and edge weight (the HSV
+ depth + saliency branch of diff, GraphCannySeg.h:2051-2288, over the edge
loop GraphCannySeg.cpp:1174-1210), bit for bit against the reference's own
code compiled for the host (oracle/build.py build_seg_pin) and against
fixtures frozen from it (tests/golden/ref_seg_graph.npz).

Equal weights are common (integer depth makes many neighbours' depth
differences zero), and their order after the reference's std::sort belongs
to the C++ library.  Given the order the reference's sort produced, the
oracle's cluster lists equal the reference's; with its own order (ties by
edge index) the oracle is deterministic everywhere."""
import os

import numpy as np
import pytest

from oracle import pyoracle as po

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "ref_seg_graph.npz")


def scene_planes(H, W, seed, n_rect=5, dropout=0.03):
    """A synthetic HSV + depth + saliency frame: a tilted background plane
    with rectangles of other colours and depths, 0-2 mm depth noise,
    dropped depth pixels, and a forward-difference saliency of V."""
    rng = np.random.default_rng(seed)
    h8 = np.full((H, W), 20, np.uint8)
    s8 = np.full((H, W), 60, np.uint8)
    v8 = np.full((H, W), 120, np.uint8)
    d = (900 + np.arange(H)[:, None] * 2 + np.arange(W)[None, :]).astype(np.int32)
    for _ in range(n_rect):
        y0, x0 = rng.integers(0, max(1, H - 4)), rng.integers(0, max(1, W - 4))
        y1, x1 = y0 + rng.integers(2, max(3, H // 2)), x0 + rng.integers(2, max(3, W // 2))
        h8[y0:y1, x0:x1] = rng.integers(0, 181)
        s8[y0:y1, x0:x1] = rng.integers(0, 256)
        v8[y0:y1, x0:x1] = rng.integers(0, 256)
        d[y0:y1, x0:x1] = rng.integers(500, 880)
    d = d + rng.integers(0, 3, (H, W))
    d[rng.random((H, W)) < dropout] = 0
    vf = v8.astype(np.float32)
    gx, gy = np.zeros_like(vf), np.zeros_like(vf)
    gx[:, :-1] = np.abs(np.diff(vf, axis=1))
    gy[:-1, :] = np.abs(np.diff(vf, axis=0))
    sal = ((gx + gy) / 510.0).astype(np.float32)
    return h8, s8, v8, d.astype(np.uint16), sal


def random_planes(H, W, seed):
    rng = np.random.default_rng(seed)
    h8 = rng.integers(0, 181, (H, W)).astype(np.uint8)
    s8 = rng.integers(0, 256, (H, W)).astype(np.uint8)
    v8 = rng.integers(0, 256, (H, W)).astype(np.uint8)
    d = rng.integers(300, 2000, (H, W)).astype(np.uint16)
    d[rng.random((H, W)) < 0.1] = 0
    sal = rng.random((H, W)).astype(np.float32)
    return h8, s8, v8, d, sal


FRAMES = [("scene", 24, 32, 1), ("scene", 48, 64, 2), ("random", 24, 32, 3), ("random", 7, 5, 4),
          ("scene", 1, 30, 5), ("scene", 30, 1, 6), ("random", 2, 2, 7)]


def frame(kind, H, W, seed):
    return (scene_planes if kind == "scene" else random_planes)(H, W, seed)


def _reference_or_skip(*args):
    ref = po.graph_reference(*args)
    if ref is None:
        pytest.skip("reference sources absent (the golden test covers the oracle)")
    return ref


@pytest.mark.parametrize("sigma", [0.8, 0.3, 2.0, 0.001])
@pytest.mark.parametrize("shape", [(24, 32), (1, 17), (17, 1), (5, 3)])
def test_smooth_equals_reference(sigma, shape):
    rng = np.random.default_rng(int(sigma * 1000) + shape[0])
    plane = rng.integers(0, 256, shape).astype(np.float32)
    want = po.smooth_reference(plane, sigma)
    if want is None:
        pytest.skip("reference sources absent")
    got = po.smooth(plane, sigma)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("fr", FRAMES)
def test_graph_equals_reference(fr):
    """Smoothed planes, normalised depth and every edge (ends, order and
    weight bits) equal the reference's."""
    h8, s8, v8, d, sal = frame(*fr)
    sp = po.seg_params()
    e_ref, sm_ref, dn_ref = _reference_or_skip(h8, s8, v8, d, sal, sp)
    for i, pl in enumerate((h8, s8, v8)):
        assert np.array_equal(po.smooth(pl.astype(np.float32), sp.sigma).view(np.uint32), sm_ref[i].view(np.uint32))
    dn = po.depth_norm(d)
    assert np.array_equal(dn.view(np.uint32), dn_ref.view(np.uint32))
    e = po.graph_edges(sm_ref[0], sm_ref[1], sm_ref[2], dn_ref, sal, sp)
    assert len(e) == len(e_ref)
    assert np.array_equal(e["a"], e_ref["a"]) and np.array_equal(e["b"], e_ref["b"])
    assert np.array_equal(e["w"].view(np.uint32), e_ref["w"].view(np.uint32))


def test_weight_branches_are_exercised():
    """The weight's branches: a zero depth next to a valid one and equal
    depths (the saliency term alone) occur in the frames above; a dark
    neighbour (v < 0.03) pins the HSV distance, so hue and saturation no
    longer matter; hue differences of 180 degrees or more wrap around."""
    sp = po.seg_params()
    f32 = np.float32
    h8, s8, v8, d, sal = random_planes(24, 32, 3)
    sm = [po.smooth(p.astype(f32), sp.sigma) for p in (h8, s8, v8)]
    e = po.graph_edges(sm[0], sm[1], sm[2], po.depth_norm(d), sal, sp)
    a, b = e["a"], e["b"]
    dz = d.ravel()
    assert ((dz[a] == 0) != (dz[b] == 0)).any()

    h8s, s8s, v8s, ds, sals = scene_planes(48, 64, 2)
    sms = [po.smooth(p.astype(f32), sp.sigma) for p in (h8s, s8s, v8s)]
    dns = po.depth_norm(ds).ravel()
    es = po.graph_edges(sms[0], sms[1], sms[2], dns.reshape(ds.shape), sals, sp)
    same = dns[es["a"]] == dns[es["b"]]
    want = (f32(sp.ks) * sals.ravel()[es["a"][same]]) / (f32(sp.kx) + f32(sp.ks))
    assert same.sum() > 100 and np.array_equal(es["w"][same], want.astype(f32))

    # 1 x 2 frame, pivot then a dark neighbour (V = 2 < 0.03 * 255)
    dnorm = np.array([[0.25, 0.75]], f32)
    zero = np.zeros((1, 2), f32)
    w = []
    for hue_, sat in [(0, 0), (170, 250), (90, 30)]:
        hp = np.array([[hue_, 0]], f32)
        spl = np.array([[sat, 255]], f32)
        vp = np.array([[200, 2]], f32)
        w.append(po.graph_edges(hp, spl, vp, dnorm, zero, sp)["w"][0])
    assert w[0] == w[1] == w[2] and w[0] > 0

    # hue wrap-around: 350 and 10 degrees are as far apart as 10 and 30
    spl = np.array([[200, 120]], f32)
    vp = np.array([[200, 180]], f32)
    wrap = po.graph_edges(np.array([[175, 5]], f32), spl, vp, dnorm, zero, sp)["w"][0]
    plain = po.graph_edges(np.array([[5, 15]], f32), spl, vp, dnorm, zero, sp)["w"][0]
    other = po.graph_edges(np.array([[5, 45]], f32), spl, vp, dnorm, zero, sp)["w"][0]
    assert wrap == plain and plain != other


def test_depth_norm_leaves_out_the_last_pixel():
    """The reference's min/max ranges end at the last pixel's address, so
    a last pixel above every other maps above 1 (and one below, below 0)."""
    d = np.array([[500, 700], [900, 4000]], np.uint16)
    dn = po.depth_norm(d)
    assert dn[0, 0] == 0.0 and dn[1, 0] == 1.0 and dn[1, 1] > 1.0
    want = po.graph_reference(*(np.zeros((2, 2), np.uint8),) * 3, d, np.zeros((2, 2), np.float32), po.seg_params())
    if want is not None:
        assert np.array_equal(dn.view(np.uint32), want[2].view(np.uint32))


@pytest.mark.parametrize("fr", [f for f in FRAMES if f[1] * f[2] >= 100])
def test_segmentation_in_the_references_edge_order_equals_reference(fr):
    """From the reference's pixel graph in the order its std::sort left it,
    the oracle's forest, merge and listing equal the reference's."""
    h8, s8, v8, d, sal = frame(*fr)
    sp = po.seg_params(min_size=20.0)
    H, W = h8.shape
    e_ref, _, _ = _reference_or_skip(h8, s8, v8, d, sal, sp)
    lists_ref, ns_ref, sorted_ref = po.segment_graph_reference(H, W, e_ref, sp.k, sp.min_size, True)
    lists, ns, _ = po.segment_graph(H * W, sorted_ref, sp.k, sp.min_size, True, presorted=True)
    assert ns == ns_ref and len(lists) == len(lists_ref)
    assert all(np.array_equal(x, y) for x, y in zip(lists, lists_ref))


@pytest.mark.parametrize("fr", FRAMES)
def test_end_to_end_is_the_composition(fr):
    """qo_segment_planes is smoothing, normalisation, graph and
    segment_graph (own tie order) composed."""
    h8, s8, v8, d, sal = frame(*fr)
    sp = po.seg_params(min_size=20.0)
    H, W = h8.shape
    lists, ns = po.segment_planes(h8, s8, v8, d, sal, sp)
    sm = [po.smooth(p.astype(np.float32), sp.sigma) for p in (h8, s8, v8)]
    e = po.graph_edges(sm[0], sm[1], sm[2], po.depth_norm(d), sal, sp)
    want, ns2, _ = po.segment_graph(H * W, e, sp.k, sp.min_size, True)
    assert ns == ns2 and all(np.array_equal(x, y) for x, y in zip(lists, want))


def test_oracle_equals_golden_graph():
    """The oracle's graph against the reference's, frozen by
    tests/golden/make_golden.py (runs where the reference is absent)."""
    g = np.load(GOLDEN)
    sp = po.seg_params()
    for c in range(len(g["hw"])):
        H, W = (int(x) for x in g["hw"][c])
        p0, p1 = g["pix_off"][c], g["pix_off"][c + 1]
        h8, s8, v8 = (g[k][p0:p1].reshape(H, W) for k in ("h8", "s8", "v8"))
        d, sal = g["depth"][p0:p1].reshape(H, W), g["sal"][p0:p1].reshape(H, W)
        sm = [po.smooth(p.astype(np.float32), sp.sigma) for p in (h8, s8, v8)]
        e = po.graph_edges(sm[0], sm[1], sm[2], po.depth_norm(d), sal, sp)
        e0, e1 = g["edge_off"][c], g["edge_off"][c + 1]
        assert len(e) == e1 - e0, c
        assert np.array_equal(e["a"], g["edge_a"][e0:e1]) and np.array_equal(e["b"], g["edge_b"][e0:e1]), c
        assert np.array_equal(e["w"].view(np.uint32), g["edge_w"][e0:e1].view(np.uint32)), c


def test_bad_arguments_are_refused():
    with pytest.raises(ValueError):
        po.smooth(np.zeros((0, 4), np.float32), 0.8)
    # all pixels but the last equal: 0/0 weights, refused rather than sorted
    flat = np.full((4, 4), 800, np.uint16)
    z = np.zeros((4, 4), np.uint8)
    with pytest.raises(ValueError):
        po.segment_planes(z, z, z, flat, np.zeros((4, 4), np.float32), po.seg_params())
