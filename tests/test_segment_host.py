"""Host side of the library's segmentation graph stage (no GPU): the edge
enumeration the GPU kernel indexes by (the same function, compiled for the
host), the smoothing mask and the merge passes, against the oracle, which
is pinned against the reference's own code (test_segmentation_core.py,
test_segmentation_graph.py)."""
import ctypes as C

import numpy as np
import pytest

import qpso
from oracle import pyoracle as po
from tests.test_segmentation_graph import FRAMES, frame


@pytest.mark.parametrize("shape", [(1, 1), (1, 9), (9, 1), (2, 2), (23, 37), (480, 640)])
def test_edge_order_is_the_references(shape):
    """The closed-form edge index (seg_edge_base) enumerates the reference's
    edge loop: same ends in the same order, (W-1)(4H-3) + H-1 edges."""
    H, W = shape
    a, b = qpso.segment_edge_ends(W, H)
    want = po.grid_edges(H, W, lambda x, y: np.zeros(len(x), np.float32))
    assert qpso.segment_num_edges(W, H) == len(want) == (W - 1) * (4 * H - 3) + H - 1
    assert np.array_equal(a, want["a"]) and np.array_equal(b, want["b"])


def test_num_edges_limits():
    assert qpso.segment_num_edges(0, 5) == 0 and qpso.segment_num_edges(5, 0) == 0
    assert qpso.segment_num_edges(1 << 13, 1 << 13) == (8191) * (4 * 8192 - 3) + 8191  # 2^26 pixels
    assert qpso.segment_num_edges((1 << 13) + 1, 1 << 13) == 0  # above 2^26 pixels


@pytest.mark.parametrize("sigma", [0.8, 0.3, 2.0, 0.001, 7.75, 1e-9])
def test_gauss_mask_equals_oracle(sigma):
    got = qpso.segment_gauss_mask(sigma)
    want = np.empty(64, np.float32)
    n = po.lib().qo_gauss_mask(C.c_float(sigma), want.ctypes.data_as(C.c_void_p), 64)
    assert len(got) == n and np.array_equal(got.view(np.uint32), want[:n].view(np.uint32))
    if sigma == 0.8:
        assert len(got) == 5 and abs(float(got[0]) + 2 * float(got[1:].sum()) - 1.0) < 1e-6


def _labels_from_lists(lists, n):
    lab = np.full(n, -1, np.int32)
    for i, L in enumerate(lists):
        lab[L] = i
    return lab


@pytest.mark.parametrize("fr", FRAMES)
@pytest.mark.parametrize("min_size", [0.0, 20.0, 500.0])
def test_merge_passes_equal_oracle(fr, min_size):
    """qpso_segment_edges over the oracle's weights: the same sets, numbered
    the same way, as the oracle's segment_graph with its tie order."""
    h8, s8, v8, d, sal = frame(*fr)
    H, W = h8.shape
    sp = po.seg_params(min_size=min_size)
    sm = [po.smooth(p.astype(np.float32), sp.sigma) for p in (h8, s8, v8)]
    e = po.graph_edges(sm[0], sm[1], sm[2], po.depth_norm(d), sal, sp)
    lists, ns, _ = po.segment_graph(H * W, e, sp.k, sp.min_size, True)
    labels, n = qpso.segment_edges(W, H, e["w"], qpso.seg_params(min_size=min_size))
    assert n == ns
    assert np.array_equal(labels.ravel(), _labels_from_lists(lists, H * W))


def test_merge_passes_with_many_ties():
    """Quantised weights (most edges tied): ties by edge index on both sides."""
    H, W = 30, 40
    rng = np.random.default_rng(5)
    w = (rng.integers(0, 4, qpso.segment_num_edges(W, H)) / 8.0).astype(np.float32)
    prm = qpso.seg_params(k=0.3, min_size=15.0)
    a, b = qpso.segment_edge_ends(W, H)
    lists, ns, _ = po.segment_graph(H * W, po.edges_array(a, b, w), prm.k, prm.min_size, True)
    labels, n = qpso.segment_edges(W, H, w, prm)
    assert n == ns > 1 and np.array_equal(labels.ravel(), _labels_from_lists(lists, H * W))


def test_merge_passes_refuse_nan_and_bad_sizes():
    w = np.zeros(qpso.segment_num_edges(4, 3), np.float32)
    w[5] = np.nan
    with pytest.raises(qpso.QpsoError):
        qpso.segment_edges(4, 3, w)
    with pytest.raises(qpso.QpsoError):
        qpso.segment_edges(4, 3, np.zeros(len(w), np.float32), qpso.seg_params(sigma=8.0))
    labels, n = qpso.segment_edges(1, 1, np.zeros(0, np.float32))
    assert n == 1 and labels.tolist() == [[0]]


def test_default_constants_equal_oracle():
    """qpso_seg_params_init and the oracle's defaults: the reference main's
    constants (main.h:58-65, main.cu:1214-1217), field for field."""
    a, b = qpso.seg_params(), po.seg_params()
    for f, _ in qpso.SegParams._fields_:
        assert np.float32(getattr(a, f)) == np.float32(getattr(b, f)), f
    assert np.float32(a.k) == np.float32(50) / np.float32(10000) and a.min_size == 500.0


def test_empty_images_are_refused():
    for w, h in [(0, 3), (3, 0), (0, 0)]:
        with pytest.raises(qpso.QpsoError):
            qpso.segment_edges(w, h, np.zeros(0, np.float32))
        with pytest.raises(qpso.QpsoError):
            qpso.segment_edge_ends(w, h)
