// qpso_seg_front.cu -- the stages of the reference's segmentation around its
// graph stage (GraphCannySeg<hsv>::run, GraphCannySeg.cpp:1438-1459) on the
// GPU: the colour conversions, the depth smoothing, the depth inpainting and
// the Canny saliency before segment_image, and the per-set moments that
// PostSegmFilter (GraphCannySeg.h:1639-1873) tests after it.
//
// Every stage is defined exactly (integers where the data are integers, a
// fixed order of float operations elsewhere) so that the kernels equal the
// oracle's restatement bit for bit; the definitions, and where they depart
// from OpenCV's own rounding, are stated beside each kernel.  The reference
// runs these stages with OpenCV 2.4 on the CPU.
//
// Data layout: one frame of W x H pixels, planes row-major.  All stages run
// on one stream with no host round trip; their outputs land in the graph
// stage's input slots (HSV planes, inpainted depth, saliency), so a frame
// goes from the colour image and raw depth to the label map with two copies
// in and one label map out.
//
// This unit is compiled with -ffp-contract=off for its host code too.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "qpso.h"
#include "qpso_internal.cuh"

namespace qpso {

namespace {

constexpr int kTaps = 16;

struct FrontConst {
  int32_t W, H;
  float alfa, beta, gamma;
  int32_t blur5[kTaps], blur7[kTaps];
  float canny_low, canny_high;
  int32_t dth, plus_d, point_3d;
  float g_angle, l_angle;
  float kinv[4];  // 1/fx, -cx/fx, 1/fy, -cy/fy
};

__device__ __forceinline__ int32_t refl101(int32_t i, int32_t n) {
  if (n == 1) return 0;
  while (i < 0 || i >= n) {
    if (i < 0) i = -i;
    if (i >= n) i = 2 * (n - 1) - i;
  }
  return i;
}

#define GRID_STRIDE(t, n) \
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (n); t += (size_t)gridDim.x * blockDim.x)

// ---- colour conversions ----------------------------------------------------
// cvtColor BGR2HSV (convertMat2Image, GraphCannySeg.h:708-721) and BGR2GRAY
// (constructor, GraphCannySeg.cpp:404): V = max, S = 255 (V - min) / V,
// H = the hue in degrees / 2, each the exact rational rounded half up; grey
// with the 14-bit weights of 0.299 / 0.587 / 0.114.
__global__ void front_colour_kernel(const uint8_t* __restrict__ bgr, size_t n, uint8_t* __restrict__ hsv,
                                    uint8_t* __restrict__ gray) {
  GRID_STRIDE(i, n) {
    const int b = bgr[3 * i], g = bgr[3 * i + 1], r = bgr[3 * i + 2];
    const int mx = max(r, max(g, b)), mn = min(r, min(g, b)), d = mx - mn;
    int h = 0;
    if (d != 0) {
      int num, off;
      if (mx == r) {
        num = g - b;
        off = 0;
      } else if (mx == g) {
        num = b - r;
        off = 60;
      } else {
        num = r - g;
        off = 120;
      }
      int hd = 30 * num + off * d;
      if (hd < 0) hd += 180 * d;
      h = (2 * hd + d) / (2 * d);
    }
    hsv[i] = (uint8_t)h;
    hsv[n + i] = mx == 0 ? 0 : (uint8_t)((510 * d + mx) / (2 * mx));
    hsv[2 * n + i] = (uint8_t)mx;
    gray[i] = (uint8_t)((4899 * r + 9617 * g + 1868 * b + 8192) >> 14);
  }
}

// ---- dynamicDepthSmoothing (GraphCannySeg.cpp:426-634) ----------------------
// Depth-change map as a gather: pixel p is marked when it, or its left or
// right neighbour, is an interior pivot whose |z(x+1) - z(x)| reaches
// gamma Fdc(pivot), or when it, or the pixel above or below, is one whose
// |z(y+1) - z(y)| does.  misc[0] |= 1 when any pixel is marked.
__device__ __forceinline__ float fdc_of(uint16_t z, float alfa) { return (float)((int64_t)z * z) * alfa; }

__device__ __forceinline__ bool cond_x(const uint16_t* d, int32_t x, int32_t y, const FrontConst& c) {
  if (x < 1 || x >= c.W - 1 || y < 1 || y >= c.H - 1) return false;
  const size_t p = (size_t)y * c.W + x;
  const float tdc = c.gamma * fdc_of(d[p], c.alfa);
  return (float)abs((int)d[p + 1] - (int)d[p]) >= tdc;
}

__device__ __forceinline__ bool cond_y(const uint16_t* d, int32_t x, int32_t y, const FrontConst& c) {
  if (x < 1 || x >= c.W - 1 || y < 1 || y >= c.H - 1) return false;
  const size_t p = (size_t)y * c.W + x;
  const float tdc = c.gamma * fdc_of(d[p], c.alfa);
  return (float)abs((int)d[p + c.W] - (int)d[p]) >= tdc;
}

__global__ void smooth_cmap_kernel(const uint16_t* __restrict__ d, uint8_t* __restrict__ cm, uint32_t* misc,
                                   FrontConst c) {
  const size_t n = (size_t)c.W * c.H;
  bool any = false;
  GRID_STRIDE(p, n) {
    const int32_t y = (int32_t)(p / c.W), x = (int32_t)(p - (size_t)y * c.W);
    const bool m = cond_x(d, x, y, c) || cond_x(d, x - 1, y, c) || cond_x(d, x + 1, y, c) ||
                   cond_y(d, x, y, c) || cond_y(d, x, y - 1, c) || cond_y(d, x, y + 1, c);
    cm[p] = m;
    any |= m;
  }
  if (__any_sync(0xffffffffu, any) && (threadIdx.x & 31) == 0) atomicOr(misc, 1u);
}

// Horizontal distance to the nearest marked pixel of the row (kInf: none):
// min(x - L, R - x) with L the last marked pixel at or before x and R the
// first at or after it.  One warp per row, 32 pixels at a time: L is a
// running maximum (left to right), R a running minimum (right to left),
// each a warp scan plus the carry from the previous 32.
constexpr int32_t kInf = 0x3fffffff;

__global__ void edt_rows_kernel(const uint8_t* __restrict__ cm, int32_t* __restrict__ g, FrontConst c) {
  const int32_t r = (int32_t)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= c.H) return;  // whole warps
  const uint8_t* row = cm + (size_t)r * c.W;
  int32_t* gr = g + (size_t)r * c.W;
  int32_t carry = -kInf;
  for (int32_t x0 = 0; x0 < c.W; x0 += 32) {
    const int32_t x = x0 + lane;
    int32_t L = (x < c.W && row[x]) ? x : -kInf;
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t y = __shfl_up_sync(0xffffffffu, L, o);
      if (lane >= o) L = max(L, y);
    }
    L = max(L, carry);
    carry = __shfl_sync(0xffffffffu, L, 31);
    if (x < c.W) gr[x] = L == -kInf ? kInf : x - L;
  }
  carry = kInf;
  const int32_t last0 = ((c.W - 1) / 32) * 32;
  for (int32_t x0 = last0; x0 >= 0; x0 -= 32) {
    const int32_t x = x0 + lane;
    int32_t R = (x < c.W && row[x]) ? x : kInf;
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t y = __shfl_down_sync(0xffffffffu, R, o);
      if (lane + o < 32) R = min(R, y);
    }
    R = min(R, carry);
    carry = __shfl_sync(0xffffffffu, R, 0);
    if (x < c.W && R != kInf && R - x < gr[x]) gr[x] = R - x;
  }
}

// R = min(B, T): T the exact Euclidean distance (outward search over rows
// while dy^2 < the best squared distance), times sqrt(1/2) in float.
__global__ void smooth_radius_kernel(const uint16_t* __restrict__ d, const int32_t* __restrict__ g,
                                     const uint32_t* misc, float* __restrict__ R, FrontConst c) {
  const size_t n = (size_t)c.W * c.H;
  const bool any = misc[0] & 1u;
  GRID_STRIDE(p, n) {
    const int32_t r = (int32_t)(p / c.W), x = (int32_t)(p - (size_t)r * c.W);
    float T;
    if (!any) {
      T = __int_as_float(0x7f800000);
    } else {
      int64_t best = g[p] == kInf ? INT64_MAX : (int64_t)g[p] * g[p];
      for (int32_t dy = 1; (int64_t)dy * dy < best; ++dy) {
        if (r - dy < 0 && r + dy >= c.H) break;
        if (r - dy >= 0) {
          const int32_t gg = g[(size_t)(r - dy) * c.W + x];
          if (gg != kInf) {
            const int64_t d2 = (int64_t)dy * dy + (int64_t)gg * gg;
            if (d2 < best) best = d2;
          }
        }
        if (r + dy < c.H) {
          const int32_t gg = g[(size_t)(r + dy) * c.W + x];
          if (gg != kInf) {
            const int64_t d2 = (int64_t)dy * dy + (int64_t)gg * gg;
            if (d2 < best) best = d2;
          }
        }
      }
      T = __fmul_rn(__fsqrt_rn((float)best), 0.70710677f);
    }
    const float B = __fmul_rn(c.beta, fdc_of(d[p], c.alfa));
    R[p] = B < T ? B : T;
  }
}

// Summed-area tables of ModDepth (float, the running row sum added to the
// entry above, in that order) and of its zeros (int).  Rows: one thread per
// row, sequential in x; columns: one thread per column, sequential in y.
// Row prefix sums of the unmarked depths (float, in order) and of the zero
// pixels.  One warp per row, 32 pixels at a time with an integer warp scan:
// while the row's total stays at or below 2^24 every partial sum is an
// integer that float holds exactly, so each in-order float addition is
// exact and the integer prefix is the same value.  A row whose total
// exceeds 2^24 is summed again in order by one lane.
__global__ void integral_rows_kernel(const uint16_t* __restrict__ d, const uint8_t* __restrict__ cm,
                                     float* __restrict__ rs, int32_t* __restrict__ rz, FrontConst c) {
  const int32_t y = (int32_t)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (y >= c.H) return;  // whole warps
  const size_t row = (size_t)y * c.W;
  unsigned long long cs = 0;  // carries: depth sum (checked against 2^24 below), zero count
  int32_t cz = 0;
  for (int32_t x0 = 0; x0 < c.W; x0 += 32) {
    const int32_t x = x0 + lane;
    unsigned long long v = 0;
    int32_t z = 0;
    if (x < c.W) {
      v = cm[row + x] ? 0u : d[row + x];
      z = v == 0u;
    }
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long sv = __shfl_up_sync(0xffffffffu, v, o);
      const int32_t sz = __shfl_up_sync(0xffffffffu, z, o);
      if (lane >= o) {
        v += sv;
        z += sz;
      }
    }
    v += cs;
    z += cz;
    if (x < c.W) {
      rs[row + x] = (float)v;
      rz[row + x] = z;
    }
    cs = __shfl_sync(0xffffffffu, v, 31);
    cz = __shfl_sync(0xffffffffu, z, 31);
  }
  __syncwarp();  // the lanes' stores before lane 0 rewrites the row
  if (cs > (1ull << 24) && lane == 0) {  // rounding enters: the reference's order
    float s = 0.0f;
    for (int32_t x = 0; x < c.W; ++x) {
      const uint16_t v = cm[row + x] ? 0 : d[row + x];
      s = __fadd_rn(s, (float)v);
      rs[row + x] = s;
    }
  }
}

// Column prefix sums of the row sums, in order (float: here rounding
// enters), one thread per column; the loads run eight rows ahead of the
// additions.
__global__ void integral_cols_kernel(const float* __restrict__ rs, const int32_t* __restrict__ rz,
                                     float* __restrict__ I, int32_t* __restrict__ N, FrontConst c) {
  const int32_t x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x > c.W) return;
  const size_t s1 = (size_t)c.W + 1;
  float acc = 0.0f;
  int32_t za = 0;
  I[x] = 0.0f;
  N[x] = 0;
  for (int32_t y0 = 0; y0 < c.H; y0 += 8) {
    float fv[8];
    int32_t zv[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int32_t y = y0 + j;
      fv[j] = 0.0f;
      zv[j] = 0;
      if (x > 0 && y < c.H) {
        fv[j] = rs[(size_t)y * c.W + x - 1];
        zv[j] = rz[(size_t)y * c.W + x - 1];
      }
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int32_t y = y0 + j;
      if (y < c.H) {
        if (x > 0) {
          acc = __fadd_rn(acc, fv[j]);
          za += zv[j];
        }
        I[(size_t)(y + 1) * s1 + x] = acc;
        N[(size_t)(y + 1) * s1 + x] = za;
      }
    }
  }
}

__global__ void smooth_out_kernel(const uint16_t* __restrict__ d, const float* __restrict__ R,
                                  const float* __restrict__ I, const int32_t* __restrict__ N,
                                  uint16_t* __restrict__ out, FrontConst c) {
  const size_t n = (size_t)c.W * c.H;
  const size_t s1 = (size_t)c.W + 1;
  GRID_STRIDE(p, n) {
    const int32_t r = (int32_t)(p / c.W), x = (int32_t)(p - (size_t)r * c.W);
    uint16_t o = 0;
    if (r >= 15 && r < c.H - 15 && x >= 15 && x < c.W - 15) {
      const int radi = (int)__fadd_rn(R[p], 0.5f);
      if (radi == 0) {
        o = d[p];
      } else {
        const int32_t x0 = max(x - radi, 0), x1 = min(x + radi + 1, c.W);
        const int32_t y0 = max(r - radi, 0), y1 = min(r + radi + 1, c.H);
        const int32_t den = (x1 - x0) * (y1 - y0);
        const int32_t nz = N[y1 * s1 + x1] + N[y0 * s1 + x0] - N[y1 * s1 + x0] - N[y0 * s1 + x1];
        if (den == nz) {
          o = d[p];
        } else {
          const float sum = __fsub_rn(__fsub_rn(__fadd_rn(I[y1 * s1 + x1], I[y0 * s1 + x0]), I[y1 * s1 + x0]),
                                      I[y0 * s1 + x1]);
          const float v = __fadd_rn(__fmul_rn(__frcp_rn((float)(den - nz)), sum), 0.5f);
          o = v <= 0.0f ? 0 : v >= 65535.0f ? 65535 : (uint16_t)v;
        }
      }
    }
    out[p] = o;
  }
}

// ---- inpaintDepth (GraphCannySeg.h:1164-1230) ------------------------------

// misc[2] = min, misc[3] = max of the smoothed depth (initialised 0xFFFF / 0)
__global__ void minmax_u16_kernel(const uint16_t* __restrict__ d, size_t n, uint32_t* misc) {
  uint32_t lo = 0xFFFFu, hi = 0u;
  GRID_STRIDE(t, n) {
    const uint32_t v = d[t];
    lo = v < lo ? v : lo;
    hi = v > hi ? v : hi;
  }
  lo = __reduce_min_sync(0xffffffffu, lo);
  hi = __reduce_max_sync(0xffffffffu, hi);
  if ((threadIdx.x & 31) == 0) {
    atomicMin(misc + 2, lo);
    atomicMax(misc + 3, hi);
  }
}

struct InpaintDims {
  int32_t sw, sh;  // the shrunk map
};

__device__ __forceinline__ uint8_t to_gray8(uint16_t z, uint32_t mn, uint32_t mx) {
  const double alpha = 255.0 / (double)(mx - mn);
  const double beta = -(double)mn * 255.0 / (double)(mx - mn);
  const float f = __fadd_rn(__fmul_rn((float)z, (float)alpha), (float)beta);
  const float q = rintf(f);
  return (uint8_t)(q < 0.0f ? 0.0f : q > 255.0f ? 255.0f : q);
}

// the shrunk 8-bit map: samples at (5x + 2, 5y + 2), and its zero mask
__global__ void inpaint_shrink_kernel(const uint16_t* __restrict__ sm, const uint32_t* misc,
                                      uint8_t* __restrict__ small, FrontConst c, InpaintDims s) {
  const uint32_t mn = misc[2], mx = misc[3];
  if (mx == mn) return;
  GRID_STRIDE(t, (size_t)s.sw * s.sh) {
    const int32_t y = (int32_t)(t / s.sw), x = (int32_t)(t - (size_t)y * s.sw);
    const int32_t sy = min(5 * y + 2, c.H - 1), sx = min(5 * x + 2, c.W - 1);
    small[t] = to_gray8(sm[(size_t)sy * c.W + sx], mn, mx);
  }
}

// Telea's inpainting of the shrunk map's zero pixels, by arrival time.  The
// times T are the fixed point of the upwind eikonal update (Jacobi
// iterations), and the masked pixels are filled in increasing T, each from
// the pixels of smaller T only, so every pixel of one time (a level) is
// independent of the others.  Two kernels:
//   telea_levels_kernel (one CTA): T, then the masked pixels grouped by
//     level in increasing T: order[lvl[l] .. lvl[l + 1]) holds level l,
//     ctrl[0] the number of levels;
//   telea_fill_kernel (cooperative, one CTA per SM): the levels in turn,
//     their pixels spread over the CTAs (a CTA per pixel, or a warp per
//     pixel when a level has more pixels than CTAs), a grid barrier between
//     levels.  A pixel's sums over the disc of `radius` are in 32.32 fixed
//     point, so they do not depend on the order of terms.
// State lives in shared memory when it fits, else in global memory.

__device__ __forceinline__ float eikonal2(float a, float b) {
  const float inf = __int_as_float(0x7f800000);
  if (a == inf && b == inf) return inf;
  const float d = __fsub_rn(a, b);
  if (fabsf(d) >= 1.0f) return __fadd_rn(a < b ? a : b, 1.0f);
  return __fmul_rn(__fadd_rn(__fadd_rn(a, b), __fsqrt_rn(__fsub_rn(2.0f, __fmul_rn(d, d)))), 0.5f);
}

__device__ __forceinline__ float grad1(bool km, float am, bool kp, float ap, float a0) {
  if (km && kp) return __fmul_rn(__fsub_rn(ap, am), 0.5f);
  if (kp) return __fsub_rn(ap, a0);
  if (km) return __fsub_rn(a0, am);
  return 0.0f;
}

__host__ __device__ __forceinline__ size_t a16(size_t b) { return (b + 15) & ~(size_t)15; }

// ctrl words: [0] levels, [1] barrier arrivals, [2] barrier generation
__global__ void __launch_bounds__(1024) telea_levels_kernel(const uint8_t* __restrict__ img_io, const uint32_t* misc,
                                                             int32_t w, int32_t h, float* __restrict__ T_out,
                                                             int32_t* __restrict__ order, int32_t* __restrict__ lvl,
                                                             uint32_t* ctrl, unsigned char* __restrict__ gmem,
                                                             int use_smem) {
  extern __shared__ __align__(16) unsigned char tsm[];
  __shared__ uint32_t s_min[32];
  __shared__ uint32_t s_L, s_cnt;
  if (threadIdx.x == 0) {
    ctrl[0] = 0u;
    ctrl[1] = 0u;
    ctrl[2] = 0u;
  }
  if (misc[3] == misc[2]) return;  // flat depth: nothing is filled
  const size_t n = (size_t)w * h;
  unsigned char* base = use_smem ? tsm : gmem;
  float* T = reinterpret_cast<float*>(base);
  float* U = reinterpret_cast<float*>(base + a16(n * 4));
  uint8_t* img = base + 2 * a16(n * 4);
  const float inf = __int_as_float(0x7f800000);
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, wid = tid >> 5, nw = nt >> 5;
  for (size_t i = tid; i < n; i += nt) {
    const uint8_t v = img_io[i];
    img[i] = v;
    T[i] = v == 0 ? inf : 0.0f;
  }
  __syncthreads();
  // arrival times: Jacobi iterations of the upwind update to the fixed point
  const int cap = 4 * (w + h) + 8;
  bool converged = false;
  for (int it = 0; it <= cap; ++it) {
    int changed = 0;
    for (size_t p = tid; p < n; p += nt) {
      float v = 0.0f;
      if (img[p] == 0) {
        const int32_t y = (int32_t)(p / w), x = (int32_t)(p - (size_t)y * w);
        const float l = x > 0 ? T[p - 1] : inf, r = x + 1 < w ? T[p + 1] : inf;
        const float u = y > 0 ? T[p - w] : inf, d = y + 1 < h ? T[p + w] : inf;
        v = eikonal2(l < r ? l : r, u < d ? u : d);
        changed |= v != T[p];
      }
      U[p] = v;
    }
    changed = __syncthreads_or(changed);
    float* t = T;
    T = U;
    U = t;
    if (!changed) {
      converged = true;
      break;
    }
  }
  if (!converged) return;  // cannot happen: the iterates only fall (as the oracle, nothing is filled)
  for (size_t i = tid; i < n; i += nt) T_out[i] = T[i];
  // the levels: masked pixels (T > 0) grouped by T in increasing order
  float last = 0.0f;
  uint32_t total = 0, nlev = 0;
  for (;;) {
    uint32_t lo = 0x7f800000u;  // the next time (non-negative floats order as their bits)
    for (size_t p = tid; p < n; p += nt) {
      const float t = T[p];
      if (t > last) lo = min(lo, __float_as_uint(t));
    }
    lo = __reduce_min_sync(0xffffffffu, lo);
    if (lane == 0) s_min[wid] = lo;
    if (tid == 0) s_cnt = 0;
    __syncthreads();
    if (wid == 0) {
      uint32_t v = lane < nw ? s_min[lane] : 0x7f800000u;
      v = __reduce_min_sync(0xffffffffu, v);
      if (lane == 0) s_L = v;
    }
    __syncthreads();
    const float L = __uint_as_float(s_L);
    if (L == inf) break;
    for (size_t p0 = (size_t)(tid & ~31); p0 < n; p0 += nt) {  // whole warps
      const size_t p = p0 + lane;
      const bool on = p < n && T[p] == L;
      const unsigned bal = __ballot_sync(0xffffffffu, on);
      uint32_t at = 0;
      if (lane == 0 && bal) at = atomicAdd(&s_cnt, (uint32_t)__popc(bal));
      at = __shfl_sync(0xffffffffu, at, 0);
      if (on) order[total + at + __popc(bal & ((1u << lane) - 1u))] = (int32_t)p;
    }
    __syncthreads();
    if (tid == 0) lvl[nlev] = (int32_t)total;
    total += s_cnt;
    ++nlev;
    last = L;
    __syncthreads();  // s_cnt is read before the next level resets it
  }
  if (tid == 0) {
    lvl[nlev] = (int32_t)total;
    __threadfence();
    ctrl[0] = nlev;
  }
}

// Grid barrier of the cooperative fill kernel, with a limit: a wait longer
// than one second sets misc[7] and returns false (every CTA then leaves).
__device__ bool fill_barrier(uint32_t* ctrl, uint32_t* misc) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile uint32_t* gen = ctrl + 2;
    const uint32_t g = *gen;
    __threadfence();
    const uint32_t arrived = atomicAdd(ctrl + 1, 1u) + 1u;
    int ok = 1;
    if (arrived == gridDim.x) {
      ctrl[1] = 0u;
      __threadfence();
      atomicExch(ctrl + 2, g + 1u);
    } else {
      unsigned long long t0;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
      while (*gen == g) {
        if (*(volatile uint32_t*)(misc + 7) != 0u) {
          ok = 0;
          break;
        }
        unsigned long long now;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
        if (now - t0 > 1000000000ull) {
          atomicOr(misc + 7, 1u);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// A lane's (or thread's) share of pixel q's sums: offsets o = first, first +
// step, ... of the disc, those whose pixel has T < L.  The map is read from
// shared memory (kSmem) or from L2 (other CTAs write it).
template <bool kSmem>
__device__ __forceinline__ void telea_terms(const float* __restrict__ T, const uint8_t* img, const short2* off,
                                            const float* olen, const float* odst, int32_t w, int32_t h, int32_t x,
                                            int32_t y, float L, float gtx, float gty, int n_off, int first, int step,
                                            bool unit_dir, long long& num, long long& den) {
  for (int o = first; o < n_off; o += step) {
    const int32_t dx = off[o].x, dy = off[o].y;
    const int32_t kx = x + dx, ky = y + dy;
    if (kx < 0 || kx >= w || ky < 0 || ky >= h) continue;
    const size_t k = (size_t)ky * w + kx;
    const float tk = T[k];
    if (!(tk < L)) continue;
    const int32_t rx = -dx, ry = -dy;
    const float dir = unit_dir ? 1.0f
                               : __fdiv_rn(fabsf(__fadd_rn(__fmul_rn((float)rx, gtx), __fmul_rn((float)ry, gty))),
                                           olen[o]);
    const float lev = __fdiv_rn(1.0f, __fadd_rn(1.0f, fabsf(__fsub_rn(tk, L))));
    const float wt = __fmul_rn(__fmul_rn(dir, odst[o]), lev);
    const bool ixm = kx > 0 && T[k - 1] < L, ixp = kx + 1 < w && T[k + 1] < L;
    const bool iym = ky > 0 && T[k - w] < L, iyp = ky + 1 < h && T[k + w] < L;
    auto at = [&](size_t i) { return kSmem ? (float)img[i] : (float)__ldcg(img + i); };
    const float a0 = at(k);
    const float gix = grad1(ixm, ixm ? at(k - 1) : 0.0f, ixp, ixp ? at(k + 1) : 0.0f, a0);
    const float giy = grad1(iym, iym ? at(k - w) : 0.0f, iyp, iyp ? at(k + w) : 0.0f, a0);
    const float val = __fadd_rn(a0, __fadd_rn(__fmul_rn(gix, (float)rx), __fmul_rn(giy, (float)ry)));
    // x * 2^32 is exact in float as in double, so these equal
    // llrint((double)x * 2^32) without the (slow) double pipe
    den += __float2ll_rn(__fmul_rn(wt, 4294967296.0f));
    num += __float2ll_rn(__fmul_rn(__fmul_rn(wt, val), 4294967296.0f));
  }
}

// T's gradient at pixel q (finite neighbours)
__device__ __forceinline__ void telea_tgrad(const float* __restrict__ T, int32_t w, int32_t h, int32_t qx, int32_t qy,
                                            float L, float& gtx, float& gty) {
  const float inf = __int_as_float(0x7f800000);
  const size_t q = (size_t)qy * w + qx;
  const bool fxm = qx > 0 && T[q - 1] != inf, fxp = qx + 1 < w && T[q + 1] != inf;
  const bool fym = qy > 0 && T[q - w] != inf, fyp = qy + 1 < h && T[q + w] != inf;
  gtx = grad1(fxm, fxm ? T[q - 1] : 0.0f, fxp, fxp ? T[q + 1] : 0.0f, L);
  gty = grad1(fym, fym ? T[q - w] : 0.0f, fyp, fyp ? T[q + w] : 0.0f, L);
}

__device__ __forceinline__ uint8_t telea_round(long long num, long long den) {
  const double v = rint((double)num / (double)den);
  return (uint8_t)(v < 0.0 ? 0.0 : v > 255.0 ? 255.0 : v);
}

template <bool kSmem>
__global__ void __launch_bounds__(256) telea_fill_kernel(uint8_t* img_io, const float* __restrict__ Tg,
                                                         const int32_t* __restrict__ order,
                                                         const int32_t* __restrict__ lvl, uint32_t* ctrl,
                                                         uint32_t* misc, int32_t w, int32_t h, int32_t radius,
                                                         int n_off) {
  extern __shared__ __align__(16) unsigned char fsm[];
  __shared__ long long s_red[8][2];
  __shared__ long long s_sum[2];
  const uint32_t nlev = ctrl[0];
  if (nlev == 0u) return;  // CTA-uniform
  const size_t n = (size_t)w * h;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, wid = tid >> 5, nw = nt >> 5;
  // layout: offsets | lengths | 1 / lengths^2 [| T | map]
  const size_t ob = a16((size_t)n_off * 4);
  short2* off = reinterpret_cast<short2*>(fsm);
  float* olen = reinterpret_cast<float*>(fsm + ob);
  float* odst = reinterpret_cast<float*>(fsm + 2 * ob);
  const float* T = Tg;
  uint8_t* img = img_io;
  if (kSmem) {
    float* Ts = reinterpret_cast<float*>(fsm + 3 * ob);
    uint8_t* ims = fsm + 3 * ob + a16(n * 4);
    for (size_t i = tid; i < n; i += nt) {
      Ts[i] = Tg[i];
      ims[i] = __ldcg(img_io + i);
    }
    T = Ts;
    img = ims;
  }
  if (tid == 0) {  // disc offsets in raster order
    int k = 0;
    for (int32_t dy = -radius; dy <= radius; ++dy)
      for (int32_t dx = -radius; dx <= radius; ++dx)
        if ((dx || dy) && dx * dx + dy * dy <= radius * radius) off[k++] = make_short2((short)dx, (short)dy);
  }
  __syncthreads();
  for (int k = tid; k < n_off; k += nt) {
    const float len2 = (float)(off[k].x * off[k].x + off[k].y * off[k].y);
    olen[k] = __fsqrt_rn(len2);
    odst[k] = __fdiv_rn(1.0f, len2);
  }
  __syncthreads();
  const int G = (int)gridDim.x;
  for (uint32_t l = 0; l < nlev; ++l) {
    const int32_t s = lvl[l], e = lvl[l + 1];
    const float L = Tg[order[s]];
    if (e - s <= G) {  // a CTA per pixel
      for (int32_t i = s + (int32_t)blockIdx.x; i < e; i += G) {
        const int32_t q = order[i];
        const int32_t qx = q % w, qy = q / w;
        float gtx, gty;
        telea_tgrad(T, w, h, qx, qy, L, gtx, gty);
        uint8_t val = 0;
        for (int pass = 0; pass < 2; ++pass) {
          long long num = 0, den = 0;
          telea_terms<kSmem>(T, img, off, olen, odst, w, h, qx, qy, L, gtx, gty, n_off, tid, nt, pass == 1, num,
                             den);
          for (int sft = 16; sft > 0; sft >>= 1) {
            num += __shfl_down_sync(0xffffffffu, num, sft);
            den += __shfl_down_sync(0xffffffffu, den, sft);
          }
          if (lane == 0) {
            s_red[wid][0] = num;
            s_red[wid][1] = den;
          }
          __syncthreads();
          if (tid == 0) {
            long long tn = 0, td = 0;
            for (int k = 0; k < nw; ++k) {
              tn += s_red[k][0];
              td += s_red[k][1];
            }
            s_sum[0] = tn;
            s_sum[1] = td;
          }
          __syncthreads();
          const long long tn = s_sum[0], td = s_sum[1];
          __syncthreads();  // s_sum is rewritten by the next pass or pixel
          if (td > 0) {
            val = telea_round(tn, td);
            break;
          }
        }
        // the level's own pixels are not read while it is filled (T < L only)
        if (tid == 0) {
          img_io[q] = val;
          if (kSmem) img[q] = val;
        }
      }
    } else {  // a warp per pixel
      for (int32_t i = s + (int32_t)blockIdx.x * nw + wid; i < e; i += G * nw) {
        const int32_t q = order[i];
        const int32_t qx = q % w, qy = q / w;
        float gtx, gty;
        telea_tgrad(T, w, h, qx, qy, L, gtx, gty);
        uint8_t val = 0;
        for (int pass = 0; pass < 2; ++pass) {
          long long num = 0, den = 0;
          telea_terms<kSmem>(T, img, off, olen, odst, w, h, qx, qy, L, gtx, gty, n_off, lane, 32, pass == 1, num,
                             den);
          for (int sft = 16; sft > 0; sft >>= 1) {
            num += __shfl_down_sync(0xffffffffu, num, sft);
            den += __shfl_down_sync(0xffffffffu, den, sft);
          }
          den = __shfl_sync(0xffffffffu, den, 0);
          num = __shfl_sync(0xffffffffu, num, 0);
          if (den > 0) {
            val = telea_round(num, den);
            break;
          }
        }
        if (lane == 0) {
          img_io[q] = val;
          if (kSmem) img[q] = val;
        }
      }
    }
    if (l + 1 == nlev) break;
    if (!fill_barrier(ctrl, misc)) return;
    if (kSmem)  // the level's values from the other CTAs (L2: not this SM's L1)
      for (int32_t i = s + tid; i < e; i += nt) {
        const int32_t q = order[i];
        img[q] = __ldcg(img_io + q);
      }
    __syncthreads();
  }
}

// Grow the inpainted map back to full size where it is needed and fill the
// depth: bilinear with half-pixel centres and 11-bit weights, then
// gray * (uint16)((max - min) / 255) + min at pixels without depth.
struct LinCoef {
  int32_t s0, s1, a0;
};

__device__ __forceinline__ LinCoef lin_coef(int32_t dx, int32_t sw, int32_t dw) {
  float f = (float)__dsub_rn(__dmul_rn((double)dx + 0.5, __ddiv_rn((double)sw, (double)dw)), 0.5);
  int32_t s = (int32_t)floorf(f);
  f = __fsub_rn(f, (float)s);
  if (s < 0) {
    f = 0.0f;
    s = 0;
  }
  if (s >= sw - 1) {
    f = 0.0f;
    s = sw - 1;
  }
  LinCoef c;
  c.s0 = s;
  c.s1 = s + 1 < sw ? s + 1 : sw - 1;
  c.a0 = (int32_t)rintf(__fmul_rn(__fsub_rn(1.0f, f), 2048.0f));
  return c;
}

__global__ void inpaint_fill_kernel(const uint16_t* __restrict__ sm, const uint32_t* misc,
                                    const uint8_t* __restrict__ small, uint16_t* __restrict__ out, FrontConst c,
                                    InpaintDims s) {
  const size_t n = (size_t)c.W * c.H;
  const uint32_t mn = misc[2], mx = misc[3];
  const uint16_t dgs = mx == mn ? 0 : (uint16_t)((double)(mx - mn) / 255.0);
  GRID_STRIDE(p, n) {
    const uint16_t z = sm[p];
    if (z != 0 || mx == mn || s.sw < 1 || s.sh < 1) {
      out[p] = z;
      continue;
    }
    int gv = to_gray8(z, mn, mx);
    if (gv == 0) {
      const int32_t y = (int32_t)(p / c.W), x = (int32_t)(p - (size_t)y * c.W);
      const LinCoef cx = lin_coef(x, s.sw, c.W), cy = lin_coef(y, s.sh, c.H);
      const int64_t r0 = (int64_t)cx.a0 * small[(size_t)cy.s0 * s.sw + cx.s0] +
                         (int64_t)(2048 - cx.a0) * small[(size_t)cy.s0 * s.sw + cx.s1];
      const int64_t r1 = (int64_t)cx.a0 * small[(size_t)cy.s1 * s.sw + cx.s0] +
                         (int64_t)(2048 - cx.a0) * small[(size_t)cy.s1 * s.sw + cx.s1];
      const int64_t v = ((int64_t)cy.a0 * r0 + (int64_t)(2048 - cy.a0) * r1 + (1 << 21)) >> 22;
      gv = (int)(v < 0 ? 0 : v > 255 ? 255 : v);
    }
    out[p] = (uint16_t)(gv * dgs + mn);
  }
}

// ---- myCannyWithOri2 (GraphCannySeg.cpp:638-1050) ---------------------------

// integer separable Gaussian (taps summing to 256), border reflect-101
__global__ void blur_rows_kernel(const uint8_t* __restrict__ src, int32_t* __restrict__ tmp, FrontConst c,
                                 int k7) {
  const size_t n = (size_t)c.W * c.H;
  const int32_t* taps = k7 ? c.blur7 : c.blur5;
  const int ks = k7 ? 7 : 5, hc = ks / 2;
  GRID_STRIDE(p, n) {
    const int32_t y = (int32_t)(p / c.W), x = (int32_t)(p - (size_t)y * c.W);
    const uint8_t* row = src + (size_t)y * c.W;
    int32_t s = 0;
    for (int i = 0; i < ks; ++i) s += taps[i] * row[refl101(x + i - hc, c.W)];
    tmp[p] = s;
  }
}

__global__ void blur_cols_kernel(const int32_t* __restrict__ tmp, uint8_t* __restrict__ dst, FrontConst c,
                                 int k7) {
  const size_t n = (size_t)c.W * c.H;
  const int32_t* taps = k7 ? c.blur7 : c.blur5;
  const int ks = k7 ? 7 : 5, hc = ks / 2;
  GRID_STRIDE(p, n) {
    const int32_t y = (int32_t)(p / c.W), x = (int32_t)(p - (size_t)y * c.W);
    int64_t s = 0;
    for (int i = 0; i < ks; ++i) s += (int64_t)taps[i] * tmp[(size_t)refl101(y + i - hc, c.H) * c.W + x];
    dst[p] = (uint8_t)((s + 32768) >> 16);
  }
}

__device__ __forceinline__ int orient_bin(int32_t x, int32_t y) {
  if (y < 0 || (y == 0 && x < 0)) {
    x = -x;
    y = -y;
  }
  if (x == 0 && y == 0) return 0;
  const int64_t a = x < 0 ? -(int64_t)x : x, b = y;
  if ((a + b) * (a + b) < 2 * a * a) return 0;
  if (b > a && (b - a) * (b - a) > 2 * a * a) return 90;
  return x >= 0 ? 45 : 135;
}

// Scharr dx and -dy (reflect-101), magnitude and orientation bin
__global__ void scharr_kernel(const uint8_t* __restrict__ bl, float* __restrict__ G, uint8_t* __restrict__ bin,
                              FrontConst c) {
  const size_t n = (size_t)c.W * c.H;
  GRID_STRIDE(p, n) {
    const int32_t y = (int32_t)(p / c.W), x = (int32_t)(p - (size_t)y * c.W);
    const int32_t xm = refl101(x - 1, c.W), xp = refl101(x + 1, c.W);
    const int32_t ym = refl101(y - 1, c.H), yp = refl101(y + 1, c.H);
#define B_(yy, xx) ((int32_t)bl[(size_t)(yy) * c.W + (xx)])
    const int32_t dx = 3 * (B_(ym, xp) - B_(ym, xm)) + 10 * (B_(y, xp) - B_(y, xm)) + 3 * (B_(yp, xp) - B_(yp, xm));
    const int32_t dy = 3 * (B_(yp, xm) - B_(ym, xm)) + 10 * (B_(yp, x) - B_(ym, x)) + 3 * (B_(yp, xp) - B_(ym, xp));
#undef B_
    G[p] = __fsqrt_rn(__fadd_rn((float)(dx * dx), (float)(dy * dy)));
    bin[p] = (uint8_t)orient_bin(dx, -dy);
  }
}

// non-maximum suppression over the interior; misc[4] = max (float bits)
__global__ void nms_kernel(const float* __restrict__ G, const uint8_t* __restrict__ bin, float* __restrict__ BW,
                           uint32_t* misc, FrontConst c) {
  const size_t n = (size_t)c.W * c.H;
  float mx = 0.0f;
  GRID_STRIDE(p, n) {
    const int32_t i = (int32_t)(p / c.W), j = (int32_t)(p - (size_t)i * c.W);
    float v = 0.0f;
    if (i >= 1 && i < c.H - 1 && j >= 1 && j < c.W - 1) {
      float a, b;
      switch (bin[p]) {
        case 0: a = G[p + 1]; b = G[p - 1]; break;
        case 45: a = G[p + c.W - 1]; b = G[p - c.W + 1]; break;
        case 90: a = G[p + c.W]; b = G[p - c.W]; break;
        default: a = G[p + c.W + 1]; b = G[p - c.W - 1]; break;
      }
      const float g = G[p];
      const float m3 = g >= a ? (g >= b ? g : b) : (a >= b ? a : b);
      if (g == m3) v = g;
    }
    BW[p] = v;
    mx = v > mx ? v : mx;
  }
  const uint32_t bits = __reduce_max_sync(0xffffffffu, __float_as_uint(mx));  // non-negative floats
  if ((threadIdx.x & 31) == 0) atomicMax(misc + 4, bits);
}

__device__ __forceinline__ void back_project(const float* kinv, int32_t u, int32_t v, uint16_t z, float* o) {
  const float p0 = (float)(u * (int32_t)z), p1 = (float)(v * (int32_t)z), p2 = (float)z;
  o[0] = (float)__dadd_rn(__dmul_rn((double)kinv[0], (double)p0), __dmul_rn((double)kinv[1], (double)p2));
  o[1] = (float)__dadd_rn(__dmul_rn((double)kinv[2], (double)p1), __dmul_rn((double)kinv[3], (double)p2));
  o[2] = p2;
}

__device__ float angle3(const float* p1, const float* p0, const float* p2) {
  float a[3], b[3], cr[3];
  for (int k = 0; k < 3; ++k) {
    a[k] = __fsub_rn(p1[k], p0[k]);
    b[k] = __fsub_rn(p2[k], p0[k]);
  }
  const float la = (float)__dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn((double)a[0], a[0]), __dmul_rn((double)a[1], a[1])),
                                               __dmul_rn((double)a[2], a[2])));
  const float lb = (float)__dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn((double)b[0], b[0]), __dmul_rn((double)b[1], b[1])),
                                               __dmul_rn((double)b[2], b[2])));
  const float dot = (float)__dadd_rn(__dadd_rn(__dmul_rn((double)a[0], b[0]), __dmul_rn((double)a[1], b[1])),
                                     __dmul_rn((double)a[2], b[2]));
  const float cs = __fdiv_rn(dot, __fmul_rn(la, lb));
  cr[0] = __fsub_rn(__fmul_rn(a[1], b[2]), __fmul_rn(a[2], b[1]));
  cr[1] = __fsub_rn(__fmul_rn(a[2], b[0]), __fmul_rn(a[0], b[2]));
  cr[2] = __fsub_rn(__fmul_rn(a[0], b[1]), __fmul_rn(a[1], b[0]));
  const float lc = (float)__dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn((double)cr[0], cr[0]), __dmul_rn((double)cr[1], cr[1])),
                                               __dmul_rn((double)cr[2], cr[2])));
  const float sn = __fdiv_rn(lc, __fmul_rn(la, lb));
  float th = (float)atan2((double)sn, (double)cs);
  if (cr[0] < 0.0f) th = -th;
  return th;
}

// one hysteresis pass (8 neighbours, outside the image = 0), the border
// of max(plusD, point3D) + 1 pixels zeroed, and the depth test
__global__ void hyst_depth_kernel(const float* __restrict__ BW, const uint8_t* __restrict__ bin,
                                  const uint16_t* __restrict__ inp, const uint32_t* misc, uint8_t* __restrict__ mag,
                                  FrontConst c) {
  const size_t n = (size_t)c.W * c.H;
  const float mx = __uint_as_float(misc[4]);
  const float tl = (float)__dmul_rn((double)c.canny_low, (double)mx);
  const float th = (float)__dmul_rn((double)c.canny_high, (double)mx);
  const int32_t pd = c.plus_d, p3 = c.point_3d;
  const int32_t sp = (pd > p3 ? pd : p3) + 1;
  GRID_STRIDE(p, n) {
    const int32_t i = (int32_t)(p / c.W), j = (int32_t)(p - (size_t)i * c.W);
    uint8_t m = 0;
    const float v = BW[p];
    if (!(v < tl)) {
      if (v > th) {
        m = 255;
      } else {
        for (int dy = -1; dy <= 1 && !m; ++dy)
          for (int dx = -1; dx <= 1; ++dx) {
            if (!dx && !dy) continue;
            const int32_t y = i + dy, x = j + dx;
            if (y < 0 || y >= c.H || x < 0 || x >= c.W) continue;
            if (BW[(size_t)y * c.W + x] > th) {
              m = 255;
              break;
            }
          }
      }
    }
    if (i < sp || i > c.H - sp || j < sp || j > c.W - sp) m = 0;
    if (m) {
      int32_t ex, ey;
      switch (bin[p]) {
        case 0: ex = 1; ey = 0; break;
        case 45: ex = 1; ey = -1; break;
        case 90: ex = 0; ey = -1; break;
        default: ex = -1; ey = -1; break;
      }
#define Z_(xx, yy) inp[(size_t)(yy) * c.W + (xx)]
      const int z0 = Z_(j, i);
      const uint16_t dp2 = (uint16_t)abs(z0 - (int)Z_(j + ex * pd, i + ey * pd));
      const uint16_t dm2 = (uint16_t)abs(z0 - (int)Z_(j - ex * pd, i - ey * pd));
      if (dp2 < c.dth && dm2 < c.dth) {
        float q0[3], q1[3], q2[3];
        back_project(c.kinv, j, i, Z_(j, i), q0);
        back_project(c.kinv, j + ex * p3, i + ey * p3, Z_(j + ex * p3, i + ey * p3), q1);
        back_project(c.kinv, j - ex * p3, i - ey * p3, Z_(j - ex * p3, i - ey * p3), q2);
        const float theta = angle3(q1, q0, q2);
        if (theta > c.g_angle || theta < c.l_angle) m = 0;
      }
#undef Z_
    }
    mag[p] = m;
  }
}

// misc[5] = min, misc[6] = max of an 8-bit map (initialised 255 / 0)
__global__ void minmax_u8_kernel(const uint8_t* __restrict__ a, size_t n, uint32_t* misc) {
  uint32_t lo = 255u, hi = 0u;
  GRID_STRIDE(t, n) {
    const uint32_t v = a[t];
    lo = v < lo ? v : lo;
    hi = v > hi ? v : hi;
  }
  lo = __reduce_min_sync(0xffffffffu, lo);
  hi = __reduce_max_sync(0xffffffffu, hi);
  if ((threadIdx.x & 31) == 0) {
    atomicMin(misc + 5, lo);
    atomicMax(misc + 6, hi);
  }
}

__global__ void saliency_kernel(const uint8_t* __restrict__ mb, const uint32_t* misc, float* __restrict__ sal,
                                size_t n) {
  const uint32_t mn = misc[5], mx = misc[6];
  const float a = mx == mn ? 0.0f : (float)__ddiv_rn(1.0, (double)(mx - mn));
  const float b = mx == mn ? 0.0f : (float)__ddiv_rn(-(double)mn * 1.0, (double)(mx - mn));
  GRID_STRIDE(t, n) sal[t] = mx == mn ? 0.0f : __fadd_rn(__fmul_rn((float)mb[t], a), b);
}

__global__ void front_misc_init_kernel(uint32_t* misc) {
  misc[0] = 0;        // any marked pixel
  misc[1] = 0;
  misc[2] = 0xFFFFu;  // smoothed depth min
  misc[3] = 0;        // and max
  misc[4] = 0;        // max of the suppressed gradient (float bits)
  misc[5] = 255u;     // blurred edge map min
  misc[6] = 0;        // and max
  misc[7] = 0;
}

int grid_of(size_t work, int threads, int sms) {
  const size_t blocks = (work + threads - 1) / threads;
  const size_t cap = (size_t)sms * 8;
  return (int)(blocks < 1 ? 1 : blocks < cap ? blocks : cap);
}

size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

int disc_count(int32_t radius) {
  int k = 0;
  for (int32_t dy = -radius; dy <= radius; ++dy)
    for (int32_t dx = -radius; dx <= radius; ++dx)
      if ((dx || dy) && dx * dx + dy * dy <= radius * radius) ++k;
  return k;
}

// telea_levels_kernel's state (times, their next iterate, the map)
size_t telea_levels_bytes(size_t n) { return 2 * a16(n * 4) + a16(n); }
// telea_fill_kernel's shared memory: the disc, and with kSmem the times and map
size_t telea_fill_bytes(size_t n, int n_off, bool smem) {
  return 3 * a16((size_t)n_off * 4) + (smem ? a16(n * 4) + a16(n) : 0);
}
// global buffers: times, level order, level offsets, control words, and the
// levels kernel's state when it does not fit in shared memory
size_t telea_ws_bytes(size_t n) {
  return al256(4 * n) + al256(4 * n) + al256(4 * (n + 1)) + al256(16) + al256(telea_levels_bytes(n));
}

}  // namespace

// ---- host side ---------------------------------------------------------------

int seg_gauss_taps(int ksize, int32_t* taps) {
  if (ksize < 1 || (ksize & 1) == 0 || ksize > 31) return -1;
  const double sigma = 0.3 * ((ksize - 1) * 0.5 - 1.0) + 0.8;
  const int c = ksize / 2;
  double g[31], sum = 0.0;
  for (int i = 0; i < ksize; ++i) {
    const double x = (double)(i - c);
    g[i] = std::exp(-(x * x) / (2.0 * sigma * sigma));
    sum += g[i];
  }
  int32_t tot = 0;
  for (int i = 0; i < ksize; ++i) {
    taps[i] = (int32_t)std::floor(g[i] / sum * 256.0 + 0.5);
    tot += taps[i];
  }
  taps[c] += 256 - tot;
  return ksize;
}

size_t seg_front_workspace_bytes(int32_t W, int32_t H, int32_t radius) {
  (void)radius;  // the inpainting disc lives in shared memory
  const size_t n = (size_t)W * H, n1 = (size_t)(W + 1) * (H + 1);
  const int32_t sw = (int32_t)std::rint(W * 0.2), sh = (int32_t)std::rint(H * 0.2);
  return al256(3 * n) + al256(n) + al256(2 * n) + al256(n) + al256(4 * n) + al256(4 * n) + 2 * al256(4 * n) +
         2 * al256(4 * n1) + al256(2 * n) + al256((size_t)(sw > 0 ? sw : 1) * (sh > 0 ? sh : 1)) +
         al256(4 * n) + al256(4 * n) + al256(n) + al256(4 * n) + al256(n) + al256(n) + al256(64) +
         al256(telea_ws_bytes((size_t)(sw > 0 ? sw : 1) * (sh > 0 ? sh : 1)));
}

cudaError_t seg_front_run(const SegFrontArgs& a, void* ws, int sms, size_t smem_optin, cudaStream_t st) {
  const int32_t W = a.W, H = a.H;
  const size_t n = (size_t)W * H, n1 = (size_t)(W + 1) * (H + 1);
  char* p = static_cast<char*>(ws);
  auto take = [&](size_t b) {
    char* q = p;
    p += al256(b);
    return q;
  };
  uint8_t* d_bgr = (uint8_t*)take(3 * n);
  uint8_t* d_gray = (uint8_t*)take(n);
  uint16_t* d_raw = (uint16_t*)take(2 * n);
  uint8_t* d_cm = (uint8_t*)take(n);
  int32_t* d_g = (int32_t*)take(4 * n);
  float* d_R = (float*)take(4 * n);
  float* d_rs = (float*)take(4 * n);
  int32_t* d_rz = (int32_t*)take(4 * n);
  float* d_I = (float*)take(4 * n1);
  int32_t* d_N = (int32_t*)take(4 * n1);
  uint16_t* d_sm = (uint16_t*)take(2 * n);
  const int32_t sw = (int32_t)std::rint(W * 0.2), sh = (int32_t)std::rint(H * 0.2);
  uint8_t* d_small = (uint8_t*)take((size_t)(sw > 0 ? sw : 1) * (sh > 0 ? sh : 1));
  int32_t* d_tmp = (int32_t*)take(4 * n);
  float* d_G = (float*)take(4 * n);
  uint8_t* d_bin = (uint8_t*)take(n);
  float* d_BW = (float*)take(4 * n);
  uint8_t* d_mag = (uint8_t*)take(n);
  uint8_t* d_mb = (uint8_t*)take(n);
  uint32_t* d_misc = (uint32_t*)take(64);
  const int n_off = disc_count(a.radius);
  const size_t ns = (size_t)(sw > 0 ? sw : 1) * (sh > 0 ? sh : 1);
  unsigned char* d_telea = (unsigned char*)take(telea_ws_bytes(ns));
  float* d_T = reinterpret_cast<float*>(d_telea);
  int32_t* d_order = reinterpret_cast<int32_t*>(d_telea + al256(4 * ns));
  int32_t* d_lvl = reinterpret_cast<int32_t*>(d_telea + 2 * al256(4 * ns));
  uint32_t* d_ctrl = reinterpret_cast<uint32_t*>(d_telea + 2 * al256(4 * ns) + al256(4 * (ns + 1)));
  unsigned char* d_lstate = d_telea + 2 * al256(4 * ns) + al256(4 * (ns + 1)) + al256(16);

  FrontConst c{};
  c.W = W;
  c.H = H;
  c.alfa = 0.0028f / 1e6f;
  c.beta = a.beta;
  c.gamma = a.gamma;
  seg_gauss_taps(5, c.blur5);
  seg_gauss_taps(7, c.blur7);
  c.canny_low = a.canny_low;
  c.canny_high = a.canny_high;
  c.dth = a.dth;
  c.plus_d = a.plus_d;
  c.point_3d = a.point_3d;
  c.g_angle = a.g_angle;
  c.l_angle = a.l_angle;
  c.kinv[0] = 1.0f / a.fx;
  c.kinv[1] = -a.cx / a.fx;
  c.kinv[2] = 1.0f / a.fy;
  c.kinv[3] = -a.cy / a.fy;

  cudaError_t e;
  if ((e = cudaMemcpyAsync(d_bgr, a.bgr_host, 3 * n, cudaMemcpyHostToDevice, st)) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(d_raw, a.depth_host, 2 * n, cudaMemcpyHostToDevice, st)) != cudaSuccess) return e;
  const int T = 256;
  front_misc_init_kernel<<<1, 1, 0, st>>>(d_misc);
  front_colour_kernel<<<grid_of(n, T, sms), T, 0, st>>>(d_bgr, n, a.hsv_out, d_gray);
  // depth smoothing
  smooth_cmap_kernel<<<grid_of(n, T, sms), T, 0, st>>>(d_raw, d_cm, d_misc, c);
  edt_rows_kernel<<<(H + 7) / 8, 256, 0, st>>>(d_cm, d_g, c);  // a warp per row
  smooth_radius_kernel<<<grid_of(n, T, sms), T, 0, st>>>(d_raw, d_g, d_misc, d_R, c);
  integral_rows_kernel<<<(H + 7) / 8, 256, 0, st>>>(d_raw, d_cm, d_rs, d_rz, c);  // a warp per row
  integral_cols_kernel<<<(W + 1 + 127) / 128, 128, 0, st>>>(d_rs, d_rz, d_I, d_N, c);
  smooth_out_kernel<<<grid_of(n, T, sms), T, 0, st>>>(d_raw, d_R, d_I, d_N, d_sm, c);
  // inpainting
  minmax_u16_kernel<<<grid_of(n, T, sms), T, 0, st>>>(d_sm, n, d_misc);
  InpaintDims dims{sw, sh};
  if (sw >= 1 && sh >= 1) {
    inpaint_shrink_kernel<<<grid_of((size_t)sw * sh, T, sms), T, 0, st>>>(d_sm, d_misc, d_small, c, dims);
    // the levels (one CTA; its static shared memory must fit beside the state)
    const size_t lb = telea_levels_bytes(ns);
    const int lsm = lb + 1024 <= smem_optin ? 1 : 0;
    if (lsm && lb > 48 * 1024 &&
        (e = cudaFuncSetAttribute(telea_levels_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lb)) !=
            cudaSuccess)
      return e;
    telea_levels_kernel<<<1, 1024, lsm ? lb : 0, st>>>(d_small, d_misc, sw, sh, d_T, d_order, d_lvl, d_ctrl,
                                                       d_lstate, lsm);
    // the fill: one CTA per SM, all resident (cooperative launch)
    const size_t fbs = telea_fill_bytes(ns, n_off, true);
    const bool fsm = fbs + 2048 <= smem_optin;
    void (*kf)(uint8_t*, const float*, const int32_t*, const int32_t*, uint32_t*, uint32_t*, int32_t, int32_t,
               int32_t, int) = fsm ? telea_fill_kernel<true> : telea_fill_kernel<false>;
    const size_t fdyn = fsm ? fbs : telea_fill_bytes(ns, n_off, false);
    if (fdyn > 48 * 1024 &&
        (e = cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fdyn)) != cudaSuccess)
      return e;
    int per_sm = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kf, 256, fdyn)) != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned)sms);
    lc.blockDim = dim3(256);
    lc.dynamicSmemBytes = fdyn;
    lc.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    lc.attrs = attr;
    lc.numAttrs = 1;
    if ((e = cudaLaunchKernelEx(&lc, kf, d_small, (const float*)d_T, (const int32_t*)d_order, (const int32_t*)d_lvl,
                                d_ctrl, d_misc, sw, sh, a.radius, n_off)) != cudaSuccess)
      return e;
  }
  inpaint_fill_kernel<<<grid_of(n, T, sms), T, 0, st>>>(d_sm, d_misc, d_small, a.inpainted_out, c, dims);
  // Canny saliency
  blur_rows_kernel<<<grid_of(n, T, sms), T, 0, st>>>(d_gray, d_tmp, c, 0);
  blur_cols_kernel<<<grid_of(n, T, sms), T, 0, st>>>(d_tmp, d_mb, c, 0);
  scharr_kernel<<<grid_of(n, T, sms), T, 0, st>>>(d_mb, d_G, d_bin, c);
  nms_kernel<<<grid_of(n, T, sms), T, 0, st>>>(d_G, d_bin, d_BW, d_misc, c);
  hyst_depth_kernel<<<grid_of(n, T, sms), T, 0, st>>>(d_BW, d_bin, a.inpainted_out, d_misc, d_mag, c);
  blur_rows_kernel<<<grid_of(n, T, sms), T, 0, st>>>(d_mag, d_tmp, c, 1);
  blur_cols_kernel<<<grid_of(n, T, sms), T, 0, st>>>(d_tmp, d_mb, c, 1);
  minmax_u8_kernel<<<grid_of(n, T, sms), T, 0, st>>>(d_mb, n, d_misc);
  saliency_kernel<<<grid_of(n, T, sms), T, 0, st>>>(d_mb, d_misc, a.saliency_out, n);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  // optional copies of the intermediate planes
  if (a.gray_host && (e = cudaMemcpyAsync(a.gray_host, d_gray, n, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return e;
  if (a.smoothed_host &&
      (e = cudaMemcpyAsync(a.smoothed_host, d_sm, 2 * n, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return e;
  if (a.edges_host && (e = cudaMemcpyAsync(a.edges_host, d_mag, n, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return e;
  // misc[7]: the inpainting fill's grid barrier expired
  if (a.err_pinned && (e = cudaMemcpyAsync(a.err_pinned, d_misc + 7, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return e;
  return cudaSuccess;
}

// ---- per-set moments for the cluster filter ----------------------------------

// One warp takes 32 consecutive pixels.  When they all belong to one set
// (the common case inside a segment), the warp reduces its sums with
// shuffles and one lane adds them; otherwise every lane adds its own.
__device__ __forceinline__ unsigned long long warp_sum64(unsigned long long v) {
  for (int s = 16; s > 0; s >>= 1) v += __shfl_down_sync(0xffffffffu, v, s);
  return v;
}

__global__ void set_moments_kernel(const int32_t* __restrict__ labels, const uint16_t* __restrict__ inp,
                                   const uint8_t* __restrict__ v8, int32_t W, int32_t H, int32_t n_sets,
                                   SetMoments* __restrict__ acc) {
  const size_t n = (size_t)W * H;
  const int lane = threadIdx.x & 31;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t base = blockIdx.x * (size_t)blockDim.x + (threadIdx.x & ~31u); base < n; base += stride) {
    const size_t p = base + lane;
    const int32_t k = p < n ? labels[p] : -1;
    const bool valid = k >= 0 && k < n_sets;
    const int32_t y = valid ? (int32_t)(p / W) : 0, x = valid ? (int32_t)(p - (size_t)y * W) : 0;
    const uint64_t z = valid ? inp[p] : 0;
    const uint8_t v = valid ? v8[p] : 255;
    unsigned long long f[15];
    f[0] = valid;
    f[1] = (unsigned long long)x;
    f[2] = (unsigned long long)y;
    f[3] = (unsigned long long)((int64_t)x * x);
    f[4] = (unsigned long long)((int64_t)y * y);
    f[5] = (unsigned long long)((int64_t)x * y);
    f[6] = valid && z;
    f[7] = z;
    f[8] = (unsigned long long)x * z;
    f[9] = (unsigned long long)y * z;
    f[10] = valid && !z;
    f[11] = v < 8;
    f[12] = v >= 8 && v < 16;
    f[13] = v >= 16 && v < 24;
    const int32_t k0 = __shfl_sync(0xffffffffu, k, 0);
    const bool uniform = __all_sync(0xffffffffu, valid && k == k0);
    if (uniform) {
      for (int i = 0; i < 14; ++i) f[i] = warp_sum64(f[i]);
      const int32_t mnx = __reduce_min_sync(0xffffffffu, x), mxx = __reduce_max_sync(0xffffffffu, x);
      const int32_t mny = __reduce_min_sync(0xffffffffu, y), mxy = __reduce_max_sync(0xffffffffu, y);
      if (lane == 0) {
        SetMoments* a = acc + k0;
        unsigned long long* dst[14] = {&a->n,  &a->sx, &a->sy,  &a->sxx,   &a->syy,   &a->sxy,   &a->nz,
                                       &a->sz, &a->suz, &a->svz, &a->nzero, &a->vb[0], &a->vb[1], &a->vb[2]};
        for (int i = 0; i < 14; ++i)
          if (f[i]) atomicAdd(dst[i], f[i]);
        atomicMin(&a->minx, mnx);
        atomicMax(&a->maxx, mxx);
        atomicMin(&a->miny, mny);
        atomicMax(&a->maxy, mxy);
      }
    } else if (valid) {
      SetMoments* a = acc + k;
      unsigned long long* dst[14] = {&a->n,  &a->sx, &a->sy,  &a->sxx,   &a->syy,   &a->sxy,   &a->nz,
                                     &a->sz, &a->suz, &a->svz, &a->nzero, &a->vb[0], &a->vb[1], &a->vb[2]};
      for (int i = 0; i < 14; ++i)
        if (f[i]) atomicAdd(dst[i], f[i]);
      atomicMin(&a->minx, x);
      atomicMax(&a->maxx, x);
      atomicMin(&a->miny, y);
      atomicMax(&a->maxy, y);
    }
  }
}

// The same sums for frames with few sets: each block accumulates into a
// shared-memory copy of the table (warp sums first, then shared atomics)
// and adds its non-empty records to the global table once.
__global__ void set_moments_smem_kernel(const int32_t* __restrict__ labels, const uint16_t* __restrict__ inp,
                                        const uint8_t* __restrict__ v8, int32_t W, int32_t H, int32_t n_sets,
                                        SetMoments* __restrict__ acc) {
  extern __shared__ __align__(16) unsigned char msm[];
  SetMoments* sm = reinterpret_cast<SetMoments*>(msm);
  for (int32_t k = threadIdx.x; k < n_sets; k += blockDim.x) {
    SetMoments z{};
    z.minx = z.miny = 0x7fffffff;
    z.maxx = z.maxy = -1;
    sm[k] = z;
  }
  __syncthreads();
  const size_t n = (size_t)W * H;
  const int lane = threadIdx.x & 31;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t base = blockIdx.x * (size_t)blockDim.x + (threadIdx.x & ~31u); base < n; base += stride) {
    const size_t p = base + lane;
    const int32_t k = p < n ? labels[p] : -1;
    const bool valid = k >= 0 && k < n_sets;
    const int32_t y = valid ? (int32_t)(p / W) : 0, x = valid ? (int32_t)(p - (size_t)y * W) : 0;
    const uint64_t z = valid ? inp[p] : 0;
    const uint8_t v = valid ? v8[p] : 255;
    unsigned long long f[14];
    f[0] = valid;
    f[1] = (unsigned long long)x;
    f[2] = (unsigned long long)y;
    f[3] = (unsigned long long)((int64_t)x * x);
    f[4] = (unsigned long long)((int64_t)y * y);
    f[5] = (unsigned long long)((int64_t)x * y);
    f[6] = valid && z;
    f[7] = z;
    f[8] = (unsigned long long)x * z;
    f[9] = (unsigned long long)y * z;
    f[10] = valid && !z;
    f[11] = v < 8;
    f[12] = v >= 8 && v < 16;
    f[13] = v >= 16 && v < 24;
    const int32_t k0 = __shfl_sync(0xffffffffu, k, 0);
    const bool uniform = __all_sync(0xffffffffu, valid && k == k0);
    int32_t mnx = x, mxx = x, mny = y, mxy = y;
    int32_t kk = k;
    bool act = valid;
    if (uniform) {
      for (int i = 0; i < 14; ++i) f[i] = warp_sum64(f[i]);
      mnx = __reduce_min_sync(0xffffffffu, x);
      mxx = __reduce_max_sync(0xffffffffu, x);
      mny = __reduce_min_sync(0xffffffffu, y);
      mxy = __reduce_max_sync(0xffffffffu, y);
      kk = k0;
      act = lane == 0;
    }
    if (act) {
      SetMoments* a = sm + kk;
      unsigned long long* dst[14] = {&a->n,  &a->sx, &a->sy,  &a->sxx,   &a->syy,   &a->sxy,   &a->nz,
                                     &a->sz, &a->suz, &a->svz, &a->nzero, &a->vb[0], &a->vb[1], &a->vb[2]};
      for (int i = 0; i < 14; ++i)
        if (f[i]) atomicAdd(dst[i], f[i]);
      atomicMin(&a->minx, mnx);
      atomicMax(&a->maxx, mxx);
      atomicMin(&a->miny, mny);
      atomicMax(&a->maxy, mxy);
    }
  }
  __syncthreads();
  for (int32_t k = threadIdx.x; k < n_sets; k += blockDim.x) {
    const SetMoments& m = sm[k];
    if (m.n == 0) continue;
    SetMoments* a = acc + k;
    const unsigned long long src[14] = {m.n,  m.sx, m.sy,  m.sxx,   m.syy,   m.sxy,   m.nz,
                                        m.sz, m.suz, m.svz, m.nzero, m.vb[0], m.vb[1], m.vb[2]};
    unsigned long long* dst[14] = {&a->n,  &a->sx, &a->sy,  &a->sxx,   &a->syy,   &a->sxy,   &a->nz,
                                   &a->sz, &a->suz, &a->svz, &a->nzero, &a->vb[0], &a->vb[1], &a->vb[2]};
    for (int i = 0; i < 14; ++i)
      if (src[i]) atomicAdd(dst[i], src[i]);
    atomicMin(&a->minx, m.minx);
    atomicMax(&a->maxx, m.maxx);
    atomicMin(&a->miny, m.miny);
    atomicMax(&a->maxy, m.maxy);
  }
}

__global__ void set_moments_init_kernel(SetMoments* acc, int32_t n_sets) {
  for (int32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n_sets; k += gridDim.x * blockDim.x) {
    SetMoments m{};
    m.minx = m.miny = 0x7fffffff;
    m.maxx = m.maxy = -1;
    acc[k] = m;
  }
}

cudaError_t launch_set_moments(const int32_t* labels, const uint16_t* inp, const uint8_t* v8, int32_t W, int32_t H,
                               int32_t n_sets, SetMoments* acc, int sms, cudaStream_t st) {
  if (n_sets <= 0) return cudaSuccess;
  set_moments_init_kernel<<<(n_sets + 255) / 256, 256, 0, st>>>(acc, n_sets);
  if (n_sets <= 256) {
    const int grid = std::min(grid_of((size_t)W * H, 256, sms), 2 * sms);
    set_moments_smem_kernel<<<grid, 256, n_sets * sizeof(SetMoments), st>>>(labels, inp, v8, W, H, n_sets, acc);
  } else {
    set_moments_kernel<<<grid_of((size_t)W * H, 256, sms), 256, 0, st>>>(labels, inp, v8, W, H, n_sets, acc);
  }
  return cudaGetLastError();
}

// The record of one set from its exact moments, with PostSegmFilter's
// tests (GraphCannySeg.h:1700-1765): centroid norm > far_obj_z; PCA
// eccentricity > max_ecc or eigenvalues above max_l1 / max_l2
// (computePCA, GraphCannySeg.cpp:1376-1435: eigenvalues of the covariance
// normalised by the point count); a share of pixels without depth >= 0.3;
// a share in the three darkest of 32 value bins >= 0.3.  The shares divide
// by the reference's list length n + 1.  Host code of this unit is built
// without floating-point contraction, like the oracle's restatement.
void seg_cluster_record(const SetMoments& m, int32_t label, const qpso_seg_front_params& fp, qpso_seg_cluster* r) {
  std::memset(r, 0, sizeof(*r));
  const int64_t n = (int64_t)m.n;
  r->label = label;
  r->num_points = (uint32_t)(n + 1);
  r->pixels = (uint32_t)n;
  r->min_x = m.minx;
  r->max_x = m.maxx + 1;
  r->min_y = m.miny;
  r->max_y = m.maxy + 1;
  const double cx = fp.cx, cy = fp.cy, fx = fp.fx, fy = fp.fy;
  if (m.nz > 0) {
    r->centroid_mm[0] = (float)(((double)m.suz - cx * (double)m.sz) / (fx * (double)m.nz));
    r->centroid_mm[1] = (float)(((double)m.svz - cy * (double)m.sz) / (fy * (double)m.nz));
    r->centroid_mm[2] = (float)((double)m.sz / (double)m.nz);
  }
  const float cxm = r->centroid_mm[0], cym = r->centroid_mm[1], czm = r->centroid_mm[2];
  const float l2c = std::sqrt(czm * czm + cym * cym + cxm * cxm);
  const double dn = (double)n;
  const double mx = (double)m.sx / dn, my = (double)m.sy / dn;
  const double vxx = ((double)m.sxx - (double)m.sx * mx) / dn;
  const double vyy = ((double)m.syy - (double)m.sy * my) / dn;
  const double vxy = ((double)m.sxy - (double)m.sx * my) / dn;
  const double hm = 0.5 * (vxx + vyy);
  const double hd = 0.5 * (vxx - vyy);
  const double rt = std::sqrt(hd * hd + vxy * vxy);
  r->eig[0] = hm + rt;
  r->eig[1] = hm - rt;
  r->eccentricity = r->eig[0] > 0.0 ? std::sqrt(1.0 - r->eig[1] / r->eig[0]) : 0.0;
  const float area = (float)(n + 1);
  r->nan_ratio = (float)m.nzero / area;
  r->dark_ratio = ((float)m.vb[0] / area + (float)m.vb[1] / area) + (float)m.vb[2] / area;
  r->far = l2c > fp.far_obj_z;
  r->kept = !r->far && !(r->eccentricity > fp.max_ecc || r->eig[0] > fp.max_l1 || r->eig[1] > fp.max_l2) &&
            !(r->nan_ratio >= 0.3f) && !(r->dark_ratio >= 0.3f);
}

}  // namespace qpso
