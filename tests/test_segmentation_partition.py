"""Partition agreement with the reference's own segment_graph on full-size
frames.

The reference sorts the edges with std::sort (GraphCannySeg.cpp:1303), which
is unstable, so the order of equal weights is the C++ library's.  This
library (and the oracle) order equal weights by edge index.  The test runs,
on the same edge weights (the oracle's, which equal the reference's own
graph code bit for bit: test_segmentation_graph.py):

  * the reference's segment_graph + small-component merge, compiled from its
    sources (oracle/ref_pin, needs them: skipped elsewhere);
  * the oracle's, with ties by edge index (what the GPU path computes);

on the production-size C2 frame and the stress configuration's 15-object
frame (640x480, from the colour image and depth through the oracle's front
stages), and measures how many pixels land in the same set after canonical
relabelling (sets numbered by their smallest pixel on both sides).  The
measured agreement is recorded in the design notes; the test holds it to a
bound.  CPU only.
"""
import numpy as np
import pytest

import scene
from oracle import pyoracle as po


def _frame_edges(bgr, depth):
    sp = po.seg_params()
    fp = po.seg_front_params()
    h8, s8, v8, gray = po.bgr_to_hsv_gray(bgr)
    inp = po.inpaint_depth(po.depth_smooth(depth, fp), fp)
    sal = po.canny_saliency(gray, inp, fp)
    sm = [po.smooth(p.astype(np.float32), sp.sigma) for p in (h8, s8, v8)]
    return po.graph_edges(sm[0], sm[1], sm[2], po.depth_norm(inp), sal, sp), sp


def _frames():
    w2 = scene.workload_c2()
    d2, _, rgb2 = w2["frames"][0]
    d5, _, rgb5 = scene.segmentation_frame_c5()
    return {"c2": (rgb2, d2), "c5": (rgb5, d5)}


@pytest.mark.parametrize("name", ["c2", "c5"])
def test_partition_agreement_with_the_reference_sort(name):
    if po.segpin() is None:
        pytest.skip("the reference's segmentation code is not built here")
    bgr, depth = _frames()[name]
    H, W = depth.shape
    edges, sp = _frame_edges(bgr, depth)
    ref = po.segment_graph_reference(H, W, edges, sp.k, sp.min_size, True)
    ours = po.segment_graph(H * W, edges, sp.k, sp.min_size, True)
    lab_r = po.labels_from_lists(ref[0], H, W)
    lab_o = po.labels_from_lists(ours[0], H, W)
    agree = float((lab_r == lab_o).mean())
    sizes_r = sorted(len(x) for x in ref[0])
    sizes_o = sorted(len(x) for x in ours[0])
    print("%s: sets %d (reference) %d (index ties), pixel agreement %.6f, differing pixels %d"
          % (name, len(ref[0]), len(ours[0]), agree, int((lab_r != lab_o).sum())))
    # measured: C2 0 differing pixels of 307,200 (17 sets each), C5 1 (31 sets
    # each); held to at most 0.01% of the pixels and the same set count
    assert len(ref[0]) == len(ours[0])
    assert agree >= 0.9999
    assert np.abs(np.array(sizes_r) - np.array(sizes_o)).sum() <= 2e-4 * H * W
