/*
 * seg_class.h -- the body of a stand-in for the GraphCannySeg<T> class
 * template: the members that the reference's edge weight diff()
 * (GraphCannySeg.h:1876-2397), segment_graph (GraphCannySeg.cpp:1301-1373)
 * and the segment_image fragments (GraphCannySeg.cpp:1105-1127 depth
 * normalisation, 1174-1210 pixel graph, 1243-1248 small-component merge)
 * read, with the reference's types (GraphCannySeg.h:623-663).  The
 * generated unit includes this file inside the class body, before diff().
 *
 * TEST INFRASTRUCTURE ONLY (see seg_prelude.h).
 */
    GraphCannySeg(float k, float min_size) : mK(k), mMin_size(min_size) {}
    universe *segment_graph(int num_vertices, int num_edges, edge *edges);
    void merge_small(universe *u, edge *edges, int num);
    image<float> *depth_norm();
    int build_edges(image<float> *smooth_h, image<float> *smooth_s, image<float> *smooth_v,
                    image<float> *depth_mm_norm, edge *edges);

    float mK;
    float mMin_size;
    float mKx = 0.f, mKy = 0.f, mKs = 0.f;
    float mKdv = 0.f, mKdc = 0.f;
    uint mWidth = 0, mHeight = 0;
    const float c_mapVeS = 1.f / 255.f;
    float *mSaliencyMyCannyPtr = nullptr;
    image<uint16_t> *mInpaintedDepth = nullptr;
    std::vector<float> DrgbV, DdepthV;
