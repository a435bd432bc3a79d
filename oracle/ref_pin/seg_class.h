/*
 * seg_class.h -- a stand-in for the GraphCannySeg<T> class template with
 * just the members that segment_graph (GraphCannySeg.cpp:1301-1373) and the
 * small-component merge (GraphCannySeg.cpp:1243-1248) read: mK (the
 * threshold constant k) and mMin_size, both float as in the reference
 * (GraphCannySeg.cpp:384-386).
 *
 * TEST INFRASTRUCTURE ONLY (see seg_prelude.h).
 */
#pragma once

namespace GraphCanny {
template <class T>
class GraphCannySeg {
public:
    GraphCannySeg(float k, float min_size) : mK(k), mMin_size(min_size) {}
    universe *segment_graph(int num_vertices, int num_edges, edge *edges);
    void merge_small(universe *u, edge *edges, int num);
    float mK;
    float mMin_size;
};
}  // namespace GraphCanny
