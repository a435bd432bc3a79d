/*
 * seg_api.h -- the C entry points of libqpso_segpin.so: the reference's own
 * graph segmentation code run on given inputs: its Gaussian smoothing, its
 * pixel graph with the edge weights of the HSV + depth + saliency branch of
 * diff(), and its segmentation of an edge list with the disjoint sets
 * listed as its collectSets lists them (GraphCannySeg.cpp:305-352).
 *
 * TEST INFRASTRUCTURE ONLY (see seg_prelude.h).
 */
#pragma once

extern "C" {

/* Runs segment_graph(num_vertices, num_edges, edges) with k, then (when
 * merge != 0) the merge of components smaller than min_size over the same
 * sorted edges, then collectSets(H, W) with H * W == num_vertices.
 *
 * In:  ea, eb, ew   -- the edges (a, b, w), num_edges of them.
 * Out: sa, sb, sw   -- the edges in the order the reference's std::sort
 *                      left them (num_edges each);
 *      offsets      -- num_lists + 1 offsets into points;
 *      points       -- pixel indices of every list, in list order
 *                      (capacity num_vertices + num_vertices);
 *      num_lists    -- number of lists collectSets produced;
 *      num_sets     -- universe::num_sets() after the segmentation.
 * Returns 0, or -1 on bad sizes. */
int sp_segment(int num_vertices, int num_edges, const int *ea, const int *eb, const float *ew, float k,
               float min_size, int merge, int H, int W, int *sa, int *sb, float *sw, int *offsets,
               int *points, int *num_lists, int *num_sets)
{
    if (num_vertices <= 0 || num_edges < 0 || H * W != num_vertices) return -1;
    std::vector<GraphCanny::edge> edges(num_edges > 0 ? num_edges : 1);
    for (int i = 0; i < num_edges; ++i) edges[i] = GraphCanny::edge(ea[i], eb[i], ew[i]);
    GraphCanny::GraphCannySeg<int> seg(k, min_size);
    GraphCanny::universe *u = seg.segment_graph(num_vertices, num_edges, edges.data());
    if (merge) seg.merge_small(u, edges.data(), num_edges);
    for (int i = 0; i < num_edges; ++i) {
        sa[i] = edges[i].a;
        sb[i] = edges[i].b;
        sw[i] = edges[i].w;
    }
    *num_sets = u->num_sets();
    std::vector<std::vector<cv::Point3i> > xyi;
    u->collectSets(xyi, H, W);
    int n = 0;
    offsets[0] = 0;
    for (size_t s = 0; s < xyi.size(); ++s) {
        for (size_t j = 0; j < xyi[s].size(); ++j) points[n++] = xyi[s][j].z;
        offsets[s + 1] = n;
    }
    *num_lists = (int)xyi.size();
    delete u;
    return 0;
}

/* smooth(src, sigma) (GraphCannySeg.h:478-489) of a W x H float plane. */
int sp_smooth(int W, int H, const float *src, float sigma, float *dst)
{
    if (W <= 0 || H <= 0) return -1;
    GraphCanny::image<float> in(W, H, false);
    std::memcpy(in.data, src, sizeof(float) * (size_t)W * H);
    GraphCanny::image<float> *out = GraphCanny::smooth(&in, sigma);
    std::memcpy(dst, out->data, sizeof(float) * (size_t)W * H);
    delete out;
    return 0;
}

/* segment_image's pixel graph (GraphCannySeg.cpp:1053-1210) for an HSV
 * image (8-bit planes, H in 0..180), the inpainted depth (mm) and the
 * saliency: the planes as floats, each smoothed with sigma, the depth
 * normalised to [0, 1] by the reference's fragment, then the reference's
 * edge loop with GraphCannySeg<hsv>::diff.  Writes the edges (a, b, w) in
 * the reference's order (capacity 4 W H) and, when not NULL, the three
 * smoothed planes (3 W H) and the normalised depth (W H).  Returns the
 * number of edges, or -1 on bad sizes. */
int sp_graph(int W, int H, const uint8_t *h8, const uint8_t *s8, const uint8_t *v8, const uint16_t *depth,
             const float *saliency, float sigma, float kdv, float kdc, float kx, float ky, float ks, int *ea,
             int *eb, float *ew, float *smooth_out, float *norm_out)
{
    if (W <= 0 || H <= 0) return -1;
    using GraphCanny::image;
    const size_t n = (size_t)W * H;
    GraphCanny::GraphCannySeg<GraphCanny::hsv> seg(0.f, 0.f);
    seg.mWidth = (uint)W;
    seg.mHeight = (uint)H;
    seg.mKdv = kdv;
    seg.mKdc = kdc;
    seg.mKx = kx;
    seg.mKy = ky;
    seg.mKs = ks;
    image<uint16_t> dimg(W, H, false);
    std::memcpy(dimg.data, depth, sizeof(uint16_t) * n);
    seg.mInpaintedDepth = &dimg;
    std::vector<float> sal(saliency, saliency + n);
    seg.mSaliencyMyCannyPtr = sal.data();
    image<float> hp(W, H, false), sp(W, H, false), vp(W, H, false);
    for (size_t i = 0; i < n; ++i) {
        hp.data[i] = static_cast<float>(h8[i]);
        sp.data[i] = static_cast<float>(s8[i]);
        vp.data[i] = static_cast<float>(v8[i]);
    }
    image<float> *sh = GraphCanny::smooth(&hp, sigma);
    image<float> *ss = GraphCanny::smooth(&sp, sigma);
    image<float> *sv = GraphCanny::smooth(&vp, sigma);
    image<float> *dn = seg.depth_norm();
    std::vector<GraphCanny::edge> edges(4 * n);
    const int m = seg.build_edges(sh, ss, sv, dn, edges.data());
    for (int i = 0; i < m; ++i) {
        ea[i] = edges[i].a;
        eb[i] = edges[i].b;
        ew[i] = edges[i].w;
    }
    if (smooth_out) {
        std::memcpy(smooth_out, sh->data, sizeof(float) * n);
        std::memcpy(smooth_out + n, ss->data, sizeof(float) * n);
        std::memcpy(smooth_out + 2 * n, sv->data, sizeof(float) * n);
    }
    if (norm_out) std::memcpy(norm_out, dn->data, sizeof(float) * n);
    delete sh;
    delete ss;
    delete sv;
    delete dn;
    return m;
}

}  // extern "C"
