"""The segmentation from a colour image and raw depth on the GPU
(qpso_segment_rgbd) against the oracle, stage by stage, bit for bit:

  * the HSV planes and grey image (cvtColor BGR2HSV / BGR2GRAY);
  * the smoothed depth (dynamicDepthSmoothing: exact distance transform,
    float summed-area tables in the stated order);
  * the inpainted depth (inpaintDepth: Telea's fast marching on the
    shrunk map, bilinear growth);
  * the Canny edge map after the depth test, and the saliency map;
  * the labels: exactly the oracle's merge over the GPU's own edge weights
    of those planes (the weights themselves are checked in
    test_gpu_segment.py);
  * the cluster records of PostSegmFilter (exact moments, same filter).

Frames: the production-size C2 frame (8 objects), the 15-object frame of
the stress configuration, a small crop whose shrunk map is not a multiple
of the sampling grid, and the 15-object frame at twice the size (1280x960):
its 256x192 shrunk map is too large for shared memory, so both inpainting
kernels run from global memory; and the 15-object frame's depth times 40
(up to 65535 mm), whose row sums pass 2^24, where float rounding enters the
summed-area tables."""
import numpy as np
import pytest

import qpso
import scene
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def _frames():
    w2 = scene.workload_c2()
    d2, _, rgb2 = w2["frames"][0]
    d5, _, rgb5 = scene.segmentation_frame_c5()
    big = (np.ascontiguousarray(np.repeat(np.repeat(rgb5, 2, axis=0), 2, axis=1)),
           np.ascontiguousarray(np.repeat(np.repeat(d5, 2, axis=0), 2, axis=1)))
    return {"c2": (rgb2, d2), "c5": (rgb5, d5),
            "crop": (np.ascontiguousarray(rgb5[60:223, 90:338]), np.ascontiguousarray(d5[60:223, 90:338])),
            "big": big,
            "far": (rgb5, np.ascontiguousarray(np.minimum(d5.astype(np.int64) * 40, 65535).astype(np.uint16)))}


FRAMES = _frames()


def _rec(c):
    return (c.label, c.num_points, c.pixels, c.min_x, c.max_x, c.min_y, c.max_y, tuple(c.centroid_mm),
            c.nan_ratio, c.dark_ratio, tuple(c.eig), c.eccentricity, c.far, c.kept)


@pytest.mark.parametrize("name", ["crop", "c2", "c5", "big", "far"])
def test_front_stages_equal_the_oracle(gpu_ctx, name):
    bgr, depth = FRAMES[name]
    out = gpu_ctx.segment_rgbd(bgr, depth, planes=True)
    h, s, v, gray = po.bgr_to_hsv_gray(bgr)
    for k, want in (("h", h), ("s", s), ("v", v), ("gray", gray)):
        np.testing.assert_array_equal(out[k], want, err_msg=k)
    sm = po.depth_smooth(depth)
    np.testing.assert_array_equal(out["smoothed"], sm)
    inp = po.inpaint_depth(sm)
    np.testing.assert_array_equal(out["inpainted"], inp)
    sal, edges = po.canny_saliency(gray, inp, with_edges=True)
    np.testing.assert_array_equal(out["edges"], edges)
    np.testing.assert_array_equal(out["saliency"].view(np.uint32), sal.view(np.uint32))


@pytest.mark.parametrize("name", ["crop", "c2", "c5"])
def test_labels_and_clusters_equal_the_oracle(gpu_ctx, name):
    bgr, depth = FRAMES[name]
    out = gpu_ctx.segment_rgbd(bgr, depth, planes=True)
    H, W = depth.shape
    sp = po.seg_params()
    # the GPU graph stage's weights of the same planes, merged by the oracle
    lab2, n2, w = gpu_ctx.segment_planes(out["h"], out["s"], out["v"], out["inpainted"], out["saliency"],
                                         weights=True)
    a, b = qpso.segment_edge_ends(W, H)
    lists, ns, _ = po.segment_graph(H * W, po.edges_array(a, b, w), sp.k, sp.min_size, True)
    want = po.labels_from_lists(lists, H, W)
    np.testing.assert_array_equal(out["labels"], want)
    np.testing.assert_array_equal(lab2, want)
    assert out["n_sets"] == n2 == len(lists)
    # the cluster filter: the oracle's records of the same label map
    recs = po.seg_clusters(out["labels"], out["n_sets"], out["inpainted"], out["v"])
    assert [_rec(c) for c in out["clusters"]] == [_rec(c) for c in recs]
    every = gpu_ctx.segment_clusters(out["labels"], out["n_sets"], out["inpainted"], out["v"], keep_all=True)
    every_o = po.seg_clusters(out["labels"], out["n_sets"], out["inpainted"], out["v"], keep_all=True)
    assert [_rec(c) for c in every] == [_rec(c) for c in every_o]
    assert len(every) == out["n_sets"]


def test_end_to_end_partition_matches_the_oracle_pipeline(gpu_ctx):
    """Against the oracle's own end-to-end run (its weights call the C
    library's cos and log2f, the GPU's CUDA's): the same partition, or
    pixel-level agreement above 99.9%."""
    bgr, depth = FRAMES["c5"]
    out = gpu_ctx.segment_rgbd(bgr, depth)
    ref = po.segment_rgbd(bgr, depth)
    a, b = out["labels"].ravel(), ref["labels"].ravel()
    # canonical relabelling: both number sets by their smallest pixel
    agree = (a == b).mean()
    assert agree > 0.999, agree


def test_segment_rgbd_rejects_bad_arguments(gpu_ctx):
    bgr, depth = FRAMES["crop"]
    with pytest.raises(qpso.QpsoError) as e:
        gpu_ctx.segment_rgbd(bgr[:2, :2], depth[:2, :2])
    assert e.value.status == qpso.ERR_ARG
    with pytest.raises(qpso.QpsoError) as e:
        gpu_ctx.segment_rgbd(bgr, depth, front=qpso.seg_front_params(inpaint_radius=0))
    assert e.value.status == qpso.ERR_ARG
    # still usable
    out = gpu_ctx.segment_rgbd(bgr, depth)
    assert out["n_sets"] >= 1
