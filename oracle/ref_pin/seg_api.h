/*
 * seg_api.h -- the C entry points of libqpso_segpin.so: the reference's own
 * segmentation core run on one edge list, with its disjoint sets listed as
 * its collectSets lists them (GraphCannySeg.cpp:305-352).
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

}  // extern "C"
