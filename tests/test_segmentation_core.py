"""The segmentation core that numbers the clusters (no GPU): the oracle's
restatement of the reference's disjoint-set forest, segment_graph, the
small-component merge and collectSets (GraphCannySeg.cpp:231-352,
1243-1248, 1301-1373) against the reference's own code compiled for the
host (oracle/build.py build_seg_pin), and against fixtures frozen from it
(tests/golden/ref_seg.npz) where the reference sources are absent.

It also pins a property of the reference's cluster records that the command
line relies on: every collectSets list repeats one pixel (the first pixel's
parent), so a cluster of n pixels reaches the fitness as
num_point_SegmentedCluster = n + 1 (main.cu:1322, GraphCannySeg.h:1831)."""
import os

import numpy as np
import pytest

from oracle import pyoracle as po

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "ref_seg.npz")
REF_K = float(np.float32(50) / np.float32(10000))  # kfloat = k / 10000, k = 50 (main.h:58, main.cu:1214)


def region_weights(H, W, n_rect, rng, tie_levels=0):
    """Piecewise-constant regions (random rectangles painted over each
    other): small weights inside a region, large across a boundary.  With
    tie_levels > 0 every weight is rounded to one of that many levels."""
    lab = np.zeros((H, W), np.int32)
    for r in range(1, n_rect + 1):
        y0, x0 = rng.integers(0, max(1, H - 2)), rng.integers(0, max(1, W - 2))
        y1, x1 = rng.integers(y0 + 1, H + 1), rng.integers(x0 + 1, W + 1)
        lab[y0:y1, x0:x1] = r
    flat = lab.ravel()
    inside = rng.uniform(0.0, 0.004, size=4 * H * W)
    across = rng.uniform(0.05, 1.0, size=4 * H * W)
    state = {"i": 0}

    def weight(a, b):
        n = len(a)
        i = state["i"]
        state["i"] += n
        w = np.where(flat[a] == flat[b], inside[i:i + n], across[i:i + n])
        if tie_levels:
            w = np.round(w * tie_levels / 1.0) / tie_levels
        return w.astype(np.float32)

    return po.grid_edges(H, W, weight)


CASES = [  # (H, W, rectangles, k, min_size, merge, seed)
    (12, 16, 3, REF_K, 0.0, False, 1),
    (12, 16, 3, REF_K, 10.0, True, 2),
    (24, 32, 6, REF_K, 20.0, True, 3),
    (24, 32, 6, 0.05, 20.0, True, 4),
    (24, 32, 0, 0.5, 0.0, False, 5),
    (30, 40, 8, 0.01, 500.0, True, 6),
    (48, 64, 10, REF_K, 50.0, True, 7),
    (1, 40, 2, 0.02, 3.0, True, 8),
    (40, 1, 2, 0.02, 3.0, True, 9),
]


def _case_edges(case):
    H, W, n_rect, k, min_size, merge, seed = case
    rng = np.random.default_rng(seed)
    if n_rect == 0:
        return po.grid_edges(H, W, lambda a, b: rng.uniform(0, 1, len(a)).astype(np.float32))
    return region_weights(H, W, n_rect, rng)


def _same_lists(a, b):
    return len(a) == len(b) and all(np.array_equal(x, y) for x, y in zip(a, b))


def _check_structure(lists, num_sets, n_vertices):
    """collectSets' listing: one list per set in the order of its smallest
    pixel, that pixel first, a repeated entry, every pixel of the image in
    exactly one set."""
    assert len(lists) == num_sets
    seen = np.zeros(n_vertices, np.int32)
    firsts = []
    for L in lists:
        members = np.unique(L)
        assert len(L) == len(members) + 1
        assert L[0] == members.min() and L[1] in members
        seen[members] += 1
        firsts.append(L[0])
    assert (seen == 1).all()
    assert firsts == sorted(firsts)


@pytest.mark.parametrize("case", CASES)
def test_oracle_equals_reference_code(case):
    H, W, _, k, min_size, merge, _ = case
    edges = _case_edges(case)
    want = po.segment_graph_reference(H, W, edges, k, min_size, merge)
    if want is None:
        pytest.skip("reference sources absent (the golden test covers the oracle)")
    got = po.segment_graph(H * W, edges, k, min_size, merge)
    assert got[1] == want[1]
    assert np.array_equal(got[2]["w"], want[2]["w"])
    assert _same_lists(got[0], want[0])
    _check_structure(got[0], got[1], H * W)


def test_ties_follow_the_given_order():
    """Equal weights: the reference's std::sort decides their order.  Given
    the order it produced, the oracle's forest and listing equal the
    reference's; the oracle's own sort keeps ties in input order."""
    H, W = 24, 32
    edges = region_weights(H, W, 6, np.random.default_rng(11), tie_levels=16)
    assert len(np.unique(edges["w"])) < len(edges) // 10
    want = po.segment_graph_reference(H, W, edges, 0.05, 20.0, True)
    if want is None:
        pytest.skip("reference sources absent")
    got = po.segment_graph(H * W, want[2], 0.05, 20.0, True, presorted=True)
    assert got[1] == want[1] and _same_lists(got[0], want[0])
    own = po.segment_graph(H * W, edges, 0.05, 20.0, True)
    assert np.array_equal(own[2]["w"], want[2]["w"])
    order = np.lexsort((np.arange(len(edges)), edges["w"]))
    assert np.array_equal(own[2]["a"], edges["a"][order]) and np.array_equal(own[2]["b"], edges["b"][order])
    _check_structure(own[0], own[1], H * W)


def test_reference_cluster_size_is_pixels_plus_one():
    """SegResults.num_points is the length of the set's collectSets list
    (GraphCannySeg.h:1831, SegResults ctor GraphCannySeg.cpp:361-372), one
    more than the cluster's pixels; a label map of the same sets counts the
    pixels.  The command line adds the one back when it fills the solve."""
    H, W = 30, 40
    edges = region_weights(H, W, 8, np.random.default_rng(21))
    res = po.segment_graph_reference(H, W, edges, REF_K, 30.0, True)
    if res is None:
        res = po.segment_graph(H * W, edges, REF_K, 30.0, True)
    lists = res[0]
    labels = np.full(H * W, -1, np.int32)
    for i, L in enumerate(lists):
        labels[L] = i
    counts = np.bincount(labels, minlength=len(lists))
    assert (labels >= 0).all()
    assert [len(L) for L in lists] == list(counts + 1)


def test_oracle_equals_golden():
    """The oracle against outputs of the reference's own code frozen by
    tests/golden/make_golden.py (runs where the reference is absent)."""
    g = np.load(GOLDEN)
    for c in range(len(g["case_hw"])):
        H, W = (int(x) for x in g["case_hw"][c])
        k, min_size = (float(x) for x in g["case_k_min"][c])
        merge = bool(g["case_merge"][c])
        e0, e1 = g["edge_off"][c], g["edge_off"][c + 1]
        edges = po.edges_array(g["edge_a"][e0:e1], g["edge_b"][e0:e1], g["edge_w"][e0:e1])
        got_lists, ns, _ = po.segment_graph(H * W, edges, k, min_size, merge, presorted=bool(g["presorted"][c]))
        l0, l1 = g["list_off"][c], g["list_off"][c + 1]
        offs = g["list_bounds"][l0:l1]
        pts = g["points"]
        want = [pts[offs[i]:offs[i + 1]] for i in range(len(offs) - 1)]
        assert ns == int(g["num_sets"][c]), c
        assert _same_lists(got_lists, want), c


def test_bad_arguments_are_refused():
    e = po.edges_array([0], [5], [0.1])
    with pytest.raises(ValueError):
        po.segment_graph(4, e, 0.1, 0.0)
    e = po.edges_array([0], [1], [float("nan")])
    with pytest.raises(ValueError):
        po.segment_graph(4, e, 0.1, 0.0)
    lists, ns, _ = po.segment_graph(3, po.edges_array([], [], []), 0.1, 0.0)
    assert ns == 3 and [list(L) for L in lists] == [[0, 0], [1, 1], [2, 2]]
