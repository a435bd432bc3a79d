// scene.cpp -- host-side synthetic RGB-D scene rendering for the benchmark
// and test workloads (not part of the solve path).
//
// Draws a mesh (loadOBJ3 SoA layout, metres) at a pose into a float depth
// buffer in mm with correct pinhole coverage: pixel centres inside the
// triangle (edge functions, either winding), perspective-correct depth by
// interpolating 1/z, nearest surface wins and writes its label.
#include <algorithm>
#include <cmath>
#include <cstdint>

extern "C" {

void qs_render_depth(const float* soa, uint32_t F, const float* pose, const float* K, int32_t w,
                     int32_t h, float* zbuf, int32_t* label, int32_t label_value) {
  const double tx = pose[0], ty = pose[1], tz = pose[2];
  const double q0 = pose[3], q1 = pose[4], q2 = pose[5], q3 = pose[6];
  // rotation matrix of the unit quaternion (q0 scalar)
  const double R[9] = {1 - 2 * (q2 * q2 + q3 * q3), 2 * (q1 * q2 - q0 * q3), 2 * (q1 * q3 + q0 * q2),
                       2 * (q1 * q2 + q0 * q3), 1 - 2 * (q1 * q1 + q3 * q3), 2 * (q2 * q3 - q0 * q1),
                       2 * (q1 * q3 - q0 * q2), 2 * (q2 * q3 + q0 * q1), 1 - 2 * (q1 * q1 + q2 * q2)};
  const double fx = K[0], fy = K[1], cx = K[2], cy = K[3];
  for (uint32_t f = 0; f < F; ++f) {
    double u[3], v[3], iz[3];
    bool ok = true;
    for (int j = 0; j < 3; ++j) {
      const double x = soa[f + (size_t)j * F], y = soa[f + (size_t)(3 + j) * F],
                   z = soa[f + (size_t)(6 + j) * F];
      const double X = R[0] * x + R[1] * y + R[2] * z + tx;
      const double Y = R[3] * x + R[4] * y + R[5] * z + ty;
      const double Z = R[6] * x + R[7] * y + R[8] * z + tz;
      if (Z <= 1e-4) ok = false;
      u[j] = cx + fx * X / Z;
      v[j] = cy + fy * Y / Z;
      iz[j] = 1.0 / (Z * 1000.0);
    }
    if (!ok) continue;
    const double area = (u[1] - u[0]) * (v[2] - v[0]) - (u[2] - u[0]) * (v[1] - v[0]);
    if (std::fabs(area) < 1e-12) continue;
    const int x0 = std::max(0, (int)std::floor(std::min({u[0], u[1], u[2]})));
    const int x1 = std::min(w - 1, (int)std::ceil(std::max({u[0], u[1], u[2]})));
    const int y0 = std::max(0, (int)std::floor(std::min({v[0], v[1], v[2]})));
    const int y1 = std::min(h - 1, (int)std::ceil(std::max({v[0], v[1], v[2]})));
    for (int y = y0; y <= y1; ++y) {
      const double py = y;
      for (int x = x0; x <= x1; ++x) {
        const double px = x;
        double b0 = (u[1] - px) * (v[2] - py) - (u[2] - px) * (v[1] - py);
        double b1 = (u[2] - px) * (v[0] - py) - (u[0] - px) * (v[2] - py);
        double b2 = (u[0] - px) * (v[1] - py) - (u[1] - px) * (v[0] - py);
        b0 /= area;
        b1 /= area;
        b2 /= area;
        if (b0 < 0 || b1 < 0 || b2 < 0) continue;
        const double zi = b0 * iz[0] + b1 * iz[1] + b2 * iz[2];
        const float z = (float)(1.0 / zi);
        float* zp = zbuf + (size_t)y * w + x;
        if (z < *zp) {
          *zp = z;
          if (label) label[(size_t)y * w + x] = label_value;
        }
      }
    }
  }
}

}  // extern "C"
