/*
 * seg_prelude.h -- stand-ins for the names the reference's graph
 * segmentation (its Gaussian smoothing, edge weight, disjoint-set forest,
 * segment_graph and set listing in GraphCannySeg.h/.cpp) takes from OpenCV,
 * so that those pieces compile on the host without it.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/build.py (build_seg_pin) writes a
 * translation unit that includes this file, then the reference's pieces
 * read from its sources where they lie (with seg_class.h inside the
 * stand-in class), then seg_api.h; the unit exists only while g++ runs.
 */
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <math.h>
#include <sys/types.h>
#include <typeinfo>
#include <vector>

typedef unsigned char uchar;

namespace cv {
/* cv::Mat: named only in signatures of image<T> members never called */
struct Mat {};
/* cv::Point3i: three ints with a (x, y, z) constructor (collectSets) */
struct Point3i {
    int x, y, z;
    Point3i() : x(0), y(0), z(0) {}
    Point3i(int x_, int y_, int z_) : x(x_), y(y_), z(z_) {}
};
/* cv::Mat_<uchar>: only ptr<uchar>(0) is named (printSet, never called) */
template <class T>
struct Mat_ {
    T *data = nullptr;
    template <class U>
    U *ptr(int) { return reinterpret_cast<U *>(data); }
};
}  // namespace cv
