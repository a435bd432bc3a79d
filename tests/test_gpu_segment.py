"""The segmentation graph stage on the GPU (qpso_segment_planes) against the
oracle, which is pinned against the reference's own code
(test_segmentation_core.py, test_segmentation_graph.py).

The GPU smooths, normalises, weighs every edge and radix-sorts; the host
runs the merge passes.  Checked here:
  * the edge weights against the oracle's: bit-equal where no
    transcendental enters (equal depths: the saliency term alone), within
    a few ulps elsewhere (CUDA's cos and log2f where the reference calls the
    C library's);
  * the labels: exactly the oracle's segmentation of the GPU's own weights,
    which needs the GPU's sort to be the stable order (ties by edge index);
  * a NaN weight (flat depth) refused with QPSO_ERR_ARG, the context still
    usable after it."""
import numpy as np
import pytest

import qpso
from oracle import pyoracle as po
from tests.test_segmentation_graph import FRAMES, frame

pytestmark = pytest.mark.gpu

GPU_FRAMES = FRAMES + [("scene", 480, 640, 11), ("random", 96, 128, 12)]


def _labels_from_lists(lists, n):
    lab = np.full(n, -1, np.int32)
    for i, L in enumerate(lists):
        lab[L] = i
    return lab


@pytest.mark.parametrize("fr", GPU_FRAMES)
def test_segment_planes_against_oracle(gpu_ctx, fr):
    h8, s8, v8, d, sal = frame(*fr)
    H, W = h8.shape
    labels, n, w = gpu_ctx.segment_planes(h8, s8, v8, d, sal, qpso.seg_params(min_size=20.0), weights=True)
    sp = po.seg_params(min_size=20.0)
    sm = [po.smooth(p.astype(np.float32), sp.sigma) for p in (h8, s8, v8)]
    dn = po.depth_norm(d)
    e = po.graph_edges(sm[0], sm[1], sm[2], dn, sal, sp)
    assert len(w) == len(e) == qpso.segment_num_edges(W, H)
    if len(e):
        wo = e["w"]
        assert (w >= 0).all() and (wo >= 0).all()
        ulps = np.abs(w.view(np.int32).astype(np.int64) - wo.view(np.int32).astype(np.int64))
        assert ulps.max() <= 4, (int(ulps.max()), int((ulps > 0).sum()))
        flat = dn.ravel()[e["a"]] == dn.ravel()[e["b"]]
        assert np.array_equal(w[flat].view(np.uint32), wo[flat].view(np.uint32))
    lists, ns, _ = po.segment_graph(H * W, po.edges_array(e["a"], e["b"], w), sp.k, sp.min_size, True)
    assert n == ns
    assert np.array_equal(labels.ravel(), _labels_from_lists(lists, H * W))


def test_segment_planes_defaults_and_one_pixel(gpu_ctx):
    """The reference main's constants (min_size 500) on a full frame, and a
    1 x 1 frame (no edges: one cluster)."""
    h8, s8, v8, d, sal = frame("scene", 480, 640, 13)
    labels, n = gpu_ctx.segment_planes(h8, s8, v8, d, sal)
    sizes = np.bincount(labels.ravel())
    assert n == len(sizes) and (sizes >= 500).all()
    one = np.zeros((1, 1), np.uint8)
    labels, n = gpu_ctx.segment_planes(one, one, one, np.full((1, 1), 700, np.uint16),
                                       np.zeros((1, 1), np.float32))
    assert n == 1 and labels.tolist() == [[0]]


def test_segment_planes_refuses_nan_weights(gpu_ctx):
    """Every pixel but the last at one depth: the reference's normalisation
    divides by zero and its sort would see NaNs; refused here, and the
    context keeps working."""
    z = np.zeros((6, 8), np.uint8)
    flat = np.full((6, 8), 800, np.uint16)
    with pytest.raises(qpso.QpsoError) as ei:
        gpu_ctx.segment_planes(z, z, z, flat, np.zeros((6, 8), np.float32))
    assert ei.value.status == qpso.ERR_ARG
    h8, s8, v8, d, sal = frame("scene", 24, 32, 1)
    labels, n = gpu_ctx.segment_planes(h8, s8, v8, d, sal, qpso.seg_params(min_size=20.0))
    assert n >= 1 and labels.min() == 0 and labels.max() == n - 1


def _streamed_vs_oracle(ctx, h8, s8, v8, d, sal, prm):
    """Labels of the streamed merge (the GPU joins the weight-0 edges, the
    host the rest) against the oracle's merge of the GPU's own weights."""
    H, W = h8.shape
    _, _, w = ctx.segment_planes(h8, s8, v8, d, sal, prm, weights=True)
    labels, n = ctx.segment_planes(h8, s8, v8, d, sal, prm)
    a, b = qpso.segment_edge_ends(W, H)
    lists, ns, _ = po.segment_graph(H * W, po.edges_array(a, b, w), prm.k, prm.min_size, True)
    assert n == ns
    assert np.array_equal(labels.ravel(), _labels_from_lists(lists, H * W))
    return w


@pytest.mark.parametrize("k", [-0.001, 0.0, 0.005, 0.05])
def test_streamed_merge_against_oracle(gpu_ctx, k):
    """k < 0: no set admits weight 0 beyond its own, the GPU leaves
    singletons and the host runs every edge; k >= 0: the weight-0 edges are
    joined on the GPU first."""
    h8, s8, v8, d, sal = frame("scene", 480, 640, 11)
    w = _streamed_vs_oracle(gpu_ctx, h8, s8, v8, d, sal, qpso.seg_params(k=k, min_size=50.0))
    assert (w == 0).mean() > 0.05  # the frame has a weight-0 run to join


def test_streamed_merge_mostly_zero_weights(gpu_ctx):
    """A frame of one colour with one brighter, raised block: nearly every
    weight is 0, so the host is left a couple of hundred edges."""
    H, W = 96, 128
    h8 = np.full((H, W), 40, np.uint8)
    s8 = np.full((H, W), 90, np.uint8)
    v8 = np.full((H, W), 150, np.uint8)
    v8[40:52, 60:80] = 210
    d = np.full((H, W), 1000, np.uint16)
    d[40:52, 60:80] = 1300
    sal = np.zeros((H, W), np.float32)
    w = _streamed_vs_oracle(gpu_ctx, h8, s8, v8, d, sal, qpso.seg_params(min_size=20.0))
    assert 0 < (w > 0).sum() < 0.05 * len(w)
