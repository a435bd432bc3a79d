// qpso_checks.h -- argument checks shared by the entry points of the C ABI.
//
// The allocating entry points (qpso_api.cu) and the one that allocates
// nothing (qpso_noalloc.cu) validate cameras and cluster fields with these
// functions, so that they accept and refuse the same inputs.  Each returns
// nullptr when the argument is valid, else the message the caller reports
// with QPSO_ERR_ARG.  Host only.
#pragma once

#include <cmath>
#include <cstdint>

#include "qpso.h"
#include "qpso_device.cuh"

namespace qpso {

// A frame's camera: size in [1, 8192] per side, finite intrinsics, a known
// projection.
inline const char* camera_error(const qpso_camera& c) {
  if (c.width <= 0 || c.height <= 0 || c.width > 8192 || c.height > 8192)
    return "frame size must be in [1, 8192]";
  if (!(std::isfinite(c.fx) && std::isfinite(c.fy) && std::isfinite(c.cx) && std::isfinite(c.cy)))
    return "non-finite intrinsics";
  if (c.projection != QPSO_PROJ_FP32 && c.projection != QPSO_PROJ_REF_ACCV) return "unknown projection";
  return nullptr;
}

// The fields of a solve descriptor that describe the cluster and how it is
// rendered, against a frame of width x height: the pixel count
// (num_point_SegmentedCluster, main.cu:1322), a non-empty AABB inside the
// raster domain (the image grown by kGuard per side), the label selector
// and the raster mode.
inline const char* cluster_error(const qpso_solve_desc& d, int32_t width, int32_t height) {
  if (d.num_points == 0) return "num_points must be > 0";
  if (!(d.cl_min_x < d.cl_max_x && d.cl_min_y < d.cl_max_y))
    return "cluster AABB must be non-empty (min < max)";
  if (d.cl_min_x < -kGuard || d.cl_max_x > width + kGuard || d.cl_min_y < -kGuard ||
      d.cl_max_y > height + kGuard)
    return "cluster AABB outside the raster domain";
  if (d.cluster_label < 0 && d.cluster_label != -1) return "cluster_label must be >= 0 or -1";
  if (d.raster_mode != QPSO_RASTER_REF && d.raster_mode != QPSO_RASTER_EDGE)
    return "raster_mode must be QPSO_RASTER_REF or QPSO_RASTER_EDGE";
  return nullptr;
}

}  // namespace qpso
