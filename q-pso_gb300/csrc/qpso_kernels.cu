// qpso_kernels.cu -- the fused Q-PSO iteration on sm_103a.
//
// One work item = one chunk of `ppb` particles of one solve instance, run by
// one CTA.  Per item: the PSO step (InitQPSO main.cu:72-198 on the first
// iteration, UpdateParticlesEquationKernel main.cu:858-1060 afterwards),
// then per particle the transform + fixed-point raster into an int32 depth
// tile in shared memory (RenderFixedPointKernelAABB main.cu:305-419,
// renderFixedPointAABB main.h:1306-1491, smem atomicMin instead of global
// atomics into a 1.2 MB-per-particle buffer), the render AABB
// (ComputeAABBFinalReductionKernel main.cu:423-546, here a warp-shuffle
// reduction), the fitness (ComputeFitnessKernel main.cu:550-764) and the
// personal best.  The CTA that finishes an instance's last chunk of an
// iteration does the argmin and the global best (thrust::min_element +
// UpdatePersonalAndGlobalBest, main.cu:1691-1704, 768-855).
//
// Fitness counting.  The reference walks every pixel of the window
// (render AABB union cluster AABB) and counts, per pixel, rendered /
// observed combinations.  Pixels outside the render AABB are never
// rendered, so their only contribution is "observed but not rendered".
// Here the number of observed pixels in the window comes from a
// summed-area table of (obs != 0) in O(1), and only the tile pixels (a
// conservative superset of the rendered ones) are scanned:
//   n_seg_not_rendered = observed(window) - observed_and_rendered.
// Every count is an exact integer, so the result equals the direct walk.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <vector>

#include "qpso_internal.cuh"

namespace qpso {

constexpr int kMaxPpb = 16;
constexpr int kMaxThreads = 1024;

// Bring a global line into L1 ahead of its use (no register is written).
__device__ __forceinline__ void prefetch_l1(const void* p) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void add128(uint64_t& lo, uint64_t& hi, uint64_t v) {
  lo += v;
  hi += (lo < v) ? 1ull : 0ull;
}

struct Partial {
  uint32_t nR, nNo, nSegR;
  uint64_t lo, hi;
  int32_t rminx, rmaxx, rminy, rmaxy;
  unsigned long long writes;
};

__device__ __forceinline__ void warp_reduce(Partial& a) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a.nR += __shfl_xor_sync(0xffffffffu, a.nR, o);
    a.nNo += __shfl_xor_sync(0xffffffffu, a.nNo, o);
    a.nSegR += __shfl_xor_sync(0xffffffffu, a.nSegR, o);
    const uint64_t lo = __shfl_xor_sync(0xffffffffu, a.lo, o);
    const uint64_t hi = __shfl_xor_sync(0xffffffffu, a.hi, o);
    a.hi += hi;
    add128(a.lo, a.hi, lo);
    a.rminx = min(a.rminx, __shfl_xor_sync(0xffffffffu, a.rminx, o));
    a.rmaxx = max(a.rmaxx, __shfl_xor_sync(0xffffffffu, a.rmaxx, o));
    a.rminy = min(a.rminy, __shfl_xor_sync(0xffffffffu, a.rminy, o));
    a.rmaxy = max(a.rmaxy, __shfl_xor_sync(0xffffffffu, a.rmaxy, o));
    a.writes += __shfl_xor_sync(0xffffffffu, a.writes, o);
  }
}

// Observed pixels (obs != 0) in [x0,x1) x [y0,y1), clipped to the image.
__device__ __forceinline__ uint32_t sat_count(const int32_t* sat, int32_t w, int32_t h, int64_t x0,
                                              int64_t x1, int64_t y0, int64_t y1) {
  x0 = x0 < 0 ? 0 : (x0 > w ? w : x0);
  x1 = x1 < 0 ? 0 : (x1 > w ? w : x1);
  y0 = y0 < 0 ? 0 : (y0 > h ? h : y0);
  y1 = y1 < 0 ? 0 : (y1 > h ? h : y1);
  if (x0 >= x1 || y0 >= y1) return 0;
  const int64_t W1 = (int64_t)w + 1;
  const int32_t a = __ldg(sat + y1 * W1 + x1), b = __ldg(sat + y0 * W1 + x1);
  const int32_t c = __ldg(sat + y1 * W1 + x0), d = __ldg(sat + y0 * W1 + x0);
  return (uint32_t)(a - b - c + d);
}

// The summed-area table's words that sat_count reads, brought into L1.
__device__ __forceinline__ void sat_prefetch(const int32_t* sat, int32_t w, int32_t h, int64_t x0, int64_t x1,
                                             int64_t y0, int64_t y1) {
  x0 = x0 < 0 ? 0 : (x0 > w ? w : x0);
  x1 = x1 < 0 ? 0 : (x1 > w ? w : x1);
  y0 = y0 < 0 ? 0 : (y0 > h ? h : y0);
  y1 = y1 < 0 ? 0 : (y1 > h ? h : y1);
  if (x0 >= x1 || y0 >= y1) return;
  const int64_t W1 = (int64_t)w + 1;
  prefetch_l1(sat + y1 * W1 + x1);
  prefetch_l1(sat + y0 * W1 + x1);
  prefetch_l1(sat + y1 * W1 + x0);
  prefetch_l1(sat + y0 * W1 + x0);
}

// Per-particle bookkeeping of the meshlet path.
struct PartCtl {
  int32_t bound[4];                 // conservative pixel bound (domain-clipped)
  int32_t tx0, tw, cw, th, ncol, nrow, npass;
  int32_t x0, y0, cwp, thp;         // current band
  int32_t box[4];                   // render AABB (shared-memory atomics)
  uint32_t nR, nNo, nSegR;
  uint64_t lo, hi;
};

constexpr int kCullCap = 512;  // meshlets whose per-particle rectangles are kept
constexpr int kLaneRasterMax = 64;  // larger face rectangles are rasterised by the whole warp

// Dynamic shared memory of the fused kernels.
struct FusedSmem {
  int4* vcache;          // [warps][vcap] snapped X, Y and depth bits, per warp
  int vcap;              // vertex cache slots per warp: the launch's largest meshlet
  int4* mbox;            // [ppb][kCullCap] meshlet rectangles (minx, maxx, miny, maxy)
  uint32_t* live;        // [ppb * kCullCap] listed items of a culled pass (particle << 28 | meshlet)
  int32_t* tiles;        // [ppb][tile_px] depth tiles
};

struct SmemCtl {
  float pose[kMaxPpb][8];  // d 0..6: the particle's pose; 7: its personal-best fitness
  int32_t bound[4];
  uint32_t claim;
  uint32_t n_live;     // listed items of the current pass and meshlet chunk
  uint8_t grp_live[kMaxPpb][kCullCap / kMletGroup];  // groups of a chunk that meet the band
  uint32_t next_item;  // items claimed so far beyond each warp's first
  int last;
  int maxpass;
  Partial warp[kMaxThreads / 32];
  float argv[kMaxThreads / 32];
  uint32_t argi[kMaxThreads / 32];
  PartCtl part[kMaxPpb];
};

// Conservative pixel bound of every face's raster rectangle at pose s: the
// mesh AABB's eight corners, projected (all at least 5 cm in front of the
// camera, so float error stays far below the 1 px margin), bound every
// projected vertex because x/z is linear-fractional.  Falls back to the
// whole raster domain.
__device__ void pose_bound(const Instance& I, const float* s, int32_t b[4]) {
  const int32_t dx0 = -kGuard, dx1 = I.cam.width + kGuard;
  const int32_t dy0 = -kGuard, dy1 = I.cam.height + kGuard;
  float ulo = 3.0e38f, uhi = -3.0e38f, vlo = 3.0e38f, vhi = -3.0e38f;
  bool ok = true;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const float x = (c & 1) ? I.mesh_hi[0] : I.mesh_lo[0];
    const float y = (c & 2) ? I.mesh_hi[1] : I.mesh_lo[1];
    const float z = (c & 4) ? I.mesh_hi[2] : I.mesh_lo[2];
    float u, v, zz;
    project(s, x, y, z, I.cam, u, v, zz);
    ok = ok && (zz >= 50.0f);  // 50 mm
    ulo = fminf(ulo, u);
    uhi = fmaxf(uhi, u);
    vlo = fminf(vlo, v);
    vhi = fmaxf(vhi, v);
  }
  if (!ok || !(ulo == ulo) || !(vlo == vlo) || !(uhi == uhi) || !(vhi == vhi)) {
    b[0] = dx0; b[1] = dx1; b[2] = dy0; b[3] = dy1;
    return;
  }
  const float fx0 = fmaxf(floorf(ulo) - 1.0f, (float)dx0), fx1 = fminf(floorf(uhi) + 2.0f, (float)dx1);
  const float fy0 = fmaxf(floorf(vlo) - 1.0f, (float)dy0), fy1 = fminf(floorf(vhi) + 2.0f, (float)dy1);
  b[0] = (int32_t)fx0;
  b[1] = (int32_t)fx1;
  b[2] = (int32_t)fy0;
  b[3] = (int32_t)fy1;
  if (b[1] < b[0]) b[1] = b[0];
  if (b[3] < b[2]) b[3] = b[2];
}

// Render + score one particle whose pose sits in shared memory.  All
// threads of the CTA call this.  Returns the fitness on thread 0.
__device__ float render_score(const Instance& I, const float* s, int32_t* tile, int tile_px,
                              SmemCtl& ctl) {
  const int tid = threadIdx.x, T = blockDim.x;
  const int32_t W = I.cam.width, H = I.cam.height;
  const int32_t dx0 = -kGuard, dx1 = W + kGuard, dy0 = -kGuard, dy1 = H + kGuard;
  const bool edge = I.prm.raster_mode == kRasterEdge;
  if (tid == 0) pose_bound(I, s, ctl.bound);
  __syncthreads();
  const int32_t bx0 = ctl.bound[0], bx1 = ctl.bound[1], by0 = ctl.bound[2], by1 = ctl.bound[3];

  // tiling of the bound: columns in chunks of cw (multiple of 8), rows in
  // bands of th so that cw * th <= tile_px
  const int32_t tx0 = bx0 & ~7;  // floor to a multiple of 8 (two's complement)
  const int32_t tw = ((bx1 - tx0) + 7) & ~7;
  const int32_t bh = by1 - by0;
  int32_t cw = tw < tile_px ? tw : (tile_px & ~7);
  if (cw < 8) cw = 8;
  const int32_t th = tile_px / cw;
  const int32_t ncol = tw > 0 ? (tw + cw - 1) / cw : 0;
  const int32_t nrow = (bh > 0 && th > 0) ? (bh + th - 1) / th : 0;
  const int32_t npass = (ncol * nrow) > 0 ? ncol * nrow : 1;  // >= 1 pass for the AABB

  Partial acc;
  acc.nR = acc.nNo = acc.nSegR = 0;
  acc.lo = acc.hi = 0;
  acc.rminx = kAabbInitMin;
  acc.rmaxx = kAabbInitMax;
  acc.rminy = kAabbInitMin;
  acc.rmaxy = kAabbInitMax;
  acc.writes = 0;
  bool bound_violation = false;

  const uint32_t F = I.F;
  const float* __restrict__ mesh = I.mesh;
  const uint16_t* __restrict__ obs = I.obs;
  const bool vec_obs = (W & 3) == 0;

  for (int32_t pass = 0; pass < npass; ++pass) {
    int32_t x0 = 0, y0 = 0, cwp = 0, thp = 0;
    if (ncol * nrow > 0) {
      const int32_t pr = pass / ncol, pc = pass - pr * ncol;
      x0 = tx0 + pc * cw;
      y0 = by0 + pr * th;
      cwp = min(cw, tx0 + tw - x0);
      thp = min(th, by1 - y0);
    }
    const int32_t npx = cwp * thp;
    // fill with the background depth, 16 bytes per store
    {
      int4* t4 = reinterpret_cast<int4*>(tile);
      const int4 bg = make_int4(kDepthBg, kDepthBg, kDepthBg, kDepthBg);
      for (int i = tid; i < (npx >> 2); i += T) t4[i] = bg;
    }
    __syncthreads();
    for (uint32_t f = tid; f < F; f += T) {
      float u[3], v[3], z[3];
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const float mx = __ldg(mesh + f + (size_t)j * F);
        const float my = __ldg(mesh + f + (size_t)(3 + j) * F);
        const float mz = __ldg(mesh + f + (size_t)(6 + j) * F);
        project(s, mx, my, mz, I.cam, u[j], v[j], z[j]);
      }
      FaceSetup fs;
      setup_face(u[0], v[0], z[0], u[1], v[1], z[1], u[2], v[2], z[2], fs, edge);
      if (pass == 0) {
        acc.rminx = min(acc.rminx, fs.minx);
        acc.rmaxx = max(acc.rmaxx, fs.maxx);
        acc.rminy = min(acc.rminy, fs.miny);
        acc.rmaxy = max(acc.rmaxy, fs.maxy);
      }
      if (!fs.live) continue;
      if (pass == 0) {
        // the rectangle inside the domain must lie inside the bound
        const int32_t ca = max(fs.minx, dx0), cb = min(fs.maxx, dx1);
        const int32_t ra = max(fs.miny, dy0), rb = min(fs.maxy, dy1);
        if (ca < cb && ra < rb && (ca < bx0 || cb > bx1 || ra < by0 || rb > by1))
          bound_violation = true;
      }
      const int32_t xa = max(fs.minx, x0), xb = min(fs.maxx, x0 + cwp);
      const int32_t ya = max(fs.miny, y0), yb = min(fs.maxy, y0 + thp);
      if (xa >= xb || ya >= yb) continue;
      if (!edge) acc.writes += (unsigned long long)(xb - xa) * (unsigned long long)(yb - ya);
      for (int32_t y = ya; y < yb; ++y) {
        int32_t CX2 = wsub(wadd(fs.c2, wmul(y, fs.fdx23)), wmul(xa, fs.fdy23));
        int32_t CX3 = wsub(wadd(fs.c3, wmul(y, fs.fdx31)), wmul(xa, fs.fdy31));
        int32_t CX1 = edge ? wsub(wadd(fs.c1, wmul(y, fs.fdx12)), wmul(xa, fs.fdy12)) : 1;
        int32_t* row = tile + (y - y0) * cwp - x0;
        for (int32_t x = xa; x < xb; ++x) {
          if (!edge || (CX1 > 0 && CX2 > 0 && CX3 > 0)) {
            const int32_t cx2 = wadd(CX2, 0xF) >> 8;
            const int32_t cx3 = wadd(CX3, 0xF) >> 8;
            float depth = fs.z1;
            depth = depth + (float)cx2 * fs.z2;
            depth = depth + (float)cx3 * fs.z3;
            const int32_t d = __float2int_rn(depth);
            atomicMin(row + x, d);  // a depth at or above the background leaves the tile as it is
            if (edge) acc.writes += 1ull;
          }
          CX2 = wsub(CX2, fs.fdy23);
          CX3 = wsub(CX3, fs.fdy31);
          if (edge) CX1 = wsub(CX1, fs.fdy12);
        }
      }
    }
    __syncthreads();
    // scan the tile: rendered pixels only, 4 pixels per step
    if (npx > 0) {
      const int32_t gpr = cwp >> 2;
      const int32_t ng = gpr * thp;
      for (int32_t g = tid; g < ng; g += T) {
        const int32_t r = g / gpr;
        const int32_t c = (g - r * gpr) << 2;
        const int4 zz = *reinterpret_cast<const int4*>(tile + r * cwp + c);
        if (zz.x >= kDepthBg && zz.y >= kDepthBg && zz.z >= kDepthBg && zz.w >= kDepthBg) continue;
        const int32_t y = y0 + r, x = x0 + c;
        uint32_t k[4] = {0u, 0u, 0u, 0u};
        if (y >= 0 && y < H) {
          const uint16_t* orow = obs + (size_t)y * (size_t)W;
          if (vec_obs && x >= 0 && x + 3 < W) {
            const uint2 q = __ldg(reinterpret_cast<const uint2*>(orow + x));
            k[0] = q.x & 0xffffu;
            k[1] = q.x >> 16;
            k[2] = q.y & 0xffffu;
            k[3] = q.y >> 16;
          } else {
#pragma unroll
            for (int e = 0; e < 4; ++e)
              if (x + e >= 0 && x + e < W) k[e] = __ldg(orow + x + e);
          }
        }
        const int32_t zr[4] = {zz.x, zz.y, zz.z, zz.w};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          if (zr[e] < kDepthBg) {
            acc.nR += 1;
            if (k[e] == 0u) {
              acc.nNo += 1;
            } else {
              const int32_t dd = wsub(zr[e], (int32_t)k[e]);
              const int64_t d64 = dd;
              add128(acc.lo, acc.hi, (uint64_t)(d64 * d64));
              acc.nSegR += 1;
            }
          }
        }
      }
    }
    __syncthreads();
  }
  if (bound_violation) atomicOr(I.err, kErrBound);

  // block reduction
  warp_reduce(acc);
  const int wid = tid >> 5, lane = tid & 31, nw = T >> 5;
  if (lane == 0) ctl.warp[wid] = acc;
  __syncthreads();
  float fitv = 0.f;
  if (tid == 0) {
    Partial t = ctl.warp[0];
    for (int i = 1; i < nw; ++i) {
      const Partial& o = ctl.warp[i];
      t.nR += o.nR;
      t.nNo += o.nNo;
      t.nSegR += o.nSegR;
      t.hi += o.hi;
      add128(t.lo, t.hi, o.lo);
      t.rminx = min(t.rminx, o.rminx);
      t.rmaxx = max(t.rmaxx, o.rmaxx);
      t.rminy = min(t.rminy, o.rminy);
      t.rmaxy = max(t.rmaxy, o.rmaxy);
      t.writes += o.writes;
    }
    const SolveParams& prm = I.prm;
    const int32_t minX = min(t.rminx, prm.cl_min_x), maxX = max(t.rmaxx, prm.cl_max_x);
    const int32_t minY = min(t.rminy, prm.cl_min_y), maxY = max(t.rmaxy, prm.cl_max_y);
    const int64_t Ww = (int64_t)maxX - minX, Hh = (int64_t)maxY - minY;
    uint32_t observed = 0;
    if (Ww > 0 && Hh > 0) {
      const int64_t area = Ww * Hh;
      const int64_t pad = (1024 - area % 1024) % 1024;
      const int64_t L = pad < Ww ? pad : Ww;
      observed = sat_count(I.sat, W, H, minX, maxX, minY, maxY) +
                 sat_count(I.sat, W, H, minX, (int64_t)minX + L, maxY, (int64_t)maxY + 1);
    }
    const uint32_t nSNR = observed - t.nSegR;
    fitv = fitness_from_counts(nSNR, t.nR, t.nNo, t.lo, t.hi, prm.num_points);
    atomicAdd(I.stats, t.writes);
    atomicAdd(I.stats + 1, (unsigned long long)npass);
  }
  return fitv;
}

// ------------------------------------------------------------------------
// Meshlet path: the fused kernels' render + score of up to kMaxPpb
// particles at once.  Warps work independently on (particle, meshlet)
// items: every unique vertex of the meshlet is transformed once into the
// warp's vertex cache (28.4 snapped X, Y and depth z), the faces are set up
// from the cache and rasterised into the particle's int32 tile in shared
// memory; the CTA synchronises only between passes.  The tile is scanned
// over the exact render AABB only.

// Exact i / d for i < 2^16 and 1 <= d <= 2^10 through a float reciprocal:
// (i + 0.5) / d is at least 1/(2d) away from the next integer.
__device__ __forceinline__ int32_t small_div(int32_t i, float rd) {
  return __float2int_rz(((float)i + 0.5f) * rd);
}

struct BlockSums {
  uint32_t nR, nNo, nSegR;
  uint64_t lo, hi;
};

// Per-particle tiling of its conservative bound (same rule as render_score).
__device__ __forceinline__ void plan_tiles(PartCtl& pc, int tile_px) {
  const int32_t bx0 = pc.bound[0], bx1 = pc.bound[1], by0 = pc.bound[2], by1 = pc.bound[3];
  pc.tx0 = bx0 & ~7;
  pc.tw = ((bx1 - pc.tx0) + 7) & ~7;
  const int32_t bh = by1 - by0;
  int32_t cw = pc.tw < tile_px ? pc.tw : (tile_px & ~7);
  if (cw < 8) cw = 8;
  pc.cw = cw;
  pc.th = tile_px / cw;
  pc.ncol = pc.tw > 0 ? (pc.tw + cw - 1) / cw : 0;
  pc.nrow = (bh > 0 && pc.th > 0) ? (bh + pc.th - 1) / pc.th : 0;
  pc.npass = (pc.ncol * pc.nrow) > 0 ? pc.ncol * pc.nrow : 1;
}

__device__ __forceinline__ FusedSmem carve_smem(unsigned char* dyn, int ppb, int vcap) {
  FusedSmem sm;
  size_t o = 0;
  sm.vcache = reinterpret_cast<int4*>(dyn + o);
  sm.vcap = vcap;
  o += (size_t)(blockDim.x >> 5) * vcap * 16;
  sm.mbox = reinterpret_cast<int4*>(dyn + o);
  o += (size_t)ppb * kCullCap * 16;
  sm.live = reinterpret_cast<uint32_t*>(dyn + o);
  o += (size_t)ppb * kCullCap * 4;
  sm.tiles = reinterpret_cast<int32_t*>(dyn + o);
  return sm;
}

// Half-open rectangle overlap test (face rectangles are [min, max)).
__device__ __forceinline__ bool rect_overlaps(const int4& b, const PartCtl& pc) {
  return pc.cwp > 0 && pc.thp > 0 && b.x < pc.x0 + pc.cwp && b.y > pc.x0 && b.z < pc.y0 + pc.thp &&
         b.w > pc.y0;
}

__device__ __forceinline__ int32_t clamp_px(float f, int32_t lo, int32_t hi) {
  return (int32_t)fminf(fmaxf(f, (float)lo), (float)hi);
}

// Conservative pixel rectangle (minx, maxx, miny, maxy; half-open) of an
// object-space box under `pose`: its 8 corners projected, widened by the
// particle bound's margin, clipped to the raster domain.  Every vertex
// inside the box projects inside the corners' hull when all corners lie in
// front of the 50 mm plane (depth is affine in the object coordinates);
// false when one does not, or a corner does not project to a number.
template <bool kRefProj>
__device__ __forceinline__ bool box_rect(const float* pose, const Camera& cam, float4 lo, float4 hi,
                                         int32_t dx0, int32_t dx1, int32_t dy0, int32_t dy1, int4& r) {
  float ulo = 3.0e38f, uhi = -3.0e38f, vlo = 3.0e38f, vhi = -3.0e38f;
  bool ok = true;
#pragma unroll 1
  for (int c = 0; c < 8; ++c) {
    float u, v, zz;
    project_t<kRefProj>(pose, (c & 1) ? hi.x : lo.x, (c & 2) ? hi.y : lo.y, (c & 4) ? hi.z : lo.z, cam, u, v, zz);
    ok = ok && zz >= 50.0f && u == u && v == v;
    ulo = fminf(ulo, u);
    uhi = fmaxf(uhi, u);
    vlo = fminf(vlo, v);
    vhi = fmaxf(vhi, v);
  }
  r = make_int4(clamp_px(floorf(ulo) - 1.0f, dx0, dx1), clamp_px(floorf(uhi) + 2.0f, dx0, dx1),
                clamp_px(floorf(vlo) - 1.0f, dy0, dy1), clamp_px(floorf(vhi) + 2.0f, dy0, dy1));
  return ok;
}

// Render + score particles 0..np-1 whose poses are in ctl.pose.  All
// threads call this; fitness k is returned in fit_out[k] (shared memory).
// When a particle's conservative bound needs several tile passes, later
// passes load and transform only the meshlets that overlap a live band:
// pass 0 records every meshlet's screen rectangle per particle when the
// mesh has at most kCullCap meshlets; larger meshes project each meshlet's
// object-space box instead (checked in pass 0 against the real rectangle).
template <bool kEdge, bool kRefProj, bool kFacePipe>
__device__ void render_score_mlets_mode(const Instance& I, int np, const FusedSmem& sm, int tile_px,
                                        SmemCtl& ctl, float* fit_out) {
  const int tid = threadIdx.x, T = blockDim.x;
  const int lane = tid & 31, wid = tid >> 5, nw = T >> 5;
  const int32_t W = I.cam.width, H = I.cam.height;
  const int32_t dx0 = -kGuard, dx1 = W + kGuard, dy0 = -kGuard, dy1 = H + kGuard;
  const uint32_t nm = I.n_mlets;
  const bool cull_ok = nm <= (uint32_t)kCullCap;
  int32_t* tiles = sm.tiles;
  int4* vcache = sm.vcache;
  int4* mbox = sm.mbox;

  // 1. conservative bound of every particle: the union of its meshlets'
  //    projected object-space boxes (box_rect; a box with a corner closer
  //    than 50 mm bounds nothing and stands for the whole domain), far
  //    tighter than the projected box of the whole mesh.  Four lanes
  //    project one box's corners, two each; one shared atomic per warp and
  //    side.
  if (tid < np) {
    PartCtl& pc = ctl.part[tid];
    pc.bound[0] = dx1;
    pc.bound[1] = dx0;
    pc.bound[2] = dy1;
    pc.bound[3] = dy0;
  }
  if (tid == 0) ctl.maxpass = 1;
  if (cull_ok)
    for (int i = tid; i < np * (int)nm; i += T)
      mbox[(i / nm) * kCullCap + (i % nm)] = make_int4(kAabbInitMin, kAabbInitMax, kAabbInitMin, kAabbInitMax);
  __syncthreads();
  // (group boxes would be cheaper for large meshes, but their looser
  // bound costs more tile passes than the projections save)
  const float4* grp_box = I.mlet_box + 2 * nm;
  const uint32_t nbox = nm;
  const float4* boxes = I.mlet_box;
  for (int k = 0; k < np; ++k) {
    PartCtl& pc = ctl.part[k];
    const uint32_t n4 = nbox * 4u;
    for (uint32_t b = (uint32_t)(tid & ~31); b < n4; b += (uint32_t)T) {  // whole warps
      // lanes 4j..4j+3 project the corners of one box: corner c (z low)
      // and corner c + 4 (z high)
      const uint32_t i = b + (uint32_t)lane, m = i >> 2, c = i & 3u;
      float ulo = 0.f, uhi = 0.f, vlo = 0.f, vhi = 0.f;
      bool ok = true;
      if (m < nbox) {
        const float4 blo = __ldg(boxes + 2 * m), bhi = __ldg(boxes + 2 * m + 1);
        const float x = (c & 1u) ? bhi.x : blo.x, y = (c & 2u) ? bhi.y : blo.y;
        float u0, v0, z0, u1, v1, z1;
        project_t<kRefProj>(ctl.pose[k], x, y, blo.z, I.cam, u0, v0, z0);
        project_t<kRefProj>(ctl.pose[k], x, y, bhi.z, I.cam, u1, v1, z1);
        ok = z0 >= 50.0f && u0 == u0 && v0 == v0 && z1 >= 50.0f && u1 == u1 && v1 == v1;
        ulo = fminf(u0, u1);
        uhi = fmaxf(u0, u1);
        vlo = fminf(v0, v1);
        vhi = fmaxf(v0, v1);
      }
#pragma unroll
      for (int o = 1; o < 4; o <<= 1) {
        ulo = fminf(ulo, __shfl_xor_sync(0xffffffffu, ulo, o));
        uhi = fmaxf(uhi, __shfl_xor_sync(0xffffffffu, uhi, o));
        vlo = fminf(vlo, __shfl_xor_sync(0xffffffffu, vlo, o));
        vhi = fmaxf(vhi, __shfl_xor_sync(0xffffffffu, vhi, o));
      }
      ok = ((__ballot_sync(0xffffffffu, !ok) >> (lane & ~3)) & 0xfu) == 0u;
      int32_t rx0 = INT32_MAX, rx1 = INT32_MIN, ry0 = INT32_MAX, ry1 = INT32_MIN;
      if (m < nbox) {
        // the rectangle of box_rect(); a box that bounds nothing stands for
        // the whole domain
        const int4 r = ok ? make_int4(clamp_px(floorf(ulo) - 1.0f, dx0, dx1), clamp_px(floorf(uhi) + 2.0f, dx0, dx1),
                                      clamp_px(floorf(vlo) - 1.0f, dy0, dy1), clamp_px(floorf(vhi) + 2.0f, dy0, dy1))
                          : make_int4(dx0, dx1, dy0, dy1);
        if (r.x < r.y && r.z < r.w) {
          rx0 = r.x;
          rx1 = r.y;
          ry0 = r.z;
          ry1 = r.w;
        }
      }
      rx0 = __reduce_min_sync(0xffffffffu, rx0);
      rx1 = __reduce_max_sync(0xffffffffu, rx1);
      ry0 = __reduce_min_sync(0xffffffffu, ry0);
      ry1 = __reduce_max_sync(0xffffffffu, ry1);
      if (lane == 0 && rx0 < rx1) {
        atomicMin(&pc.bound[0], rx0);
        atomicMax(&pc.bound[1], rx1);
        atomicMin(&pc.bound[2], ry0);
        atomicMax(&pc.bound[3], ry1);
      }
    }
  }
  __syncthreads();
  if (tid < np) {
    PartCtl& pc = ctl.part[tid];
    if (pc.bound[1] <= pc.bound[0] || pc.bound[3] <= pc.bound[2]) {  // nothing inside the domain
      pc.bound[0] = pc.bound[1] = dx1;
      pc.bound[2] = pc.bound[3] = dy1;
    }
    plan_tiles(pc, tile_px);
    pc.box[0] = kAabbInitMin;
    pc.box[1] = kAabbInitMax;
    pc.box[2] = kAabbInitMin;
    pc.box[3] = kAabbInitMax;
    pc.nR = pc.nNo = pc.nSegR = 0;
    pc.lo = pc.hi = 0;
    atomicMax(&ctl.maxpass, pc.npass);
  }
  __syncthreads();
  const int maxpass = ctl.maxpass;
  unsigned long long writes = 0;
  bool violation = false;

  for (int pass = 0; pass < maxpass; ++pass) {
    // 2a. band of every particle still active in this pass
    if (tid == 0) ctl.next_item = (uint32_t)nw;
    if (tid < np) {
      PartCtl& pc = ctl.part[tid];
      pc.x0 = pc.y0 = pc.cwp = pc.thp = 0;
      if (pass < pc.npass && pc.ncol * pc.nrow > 0) {
        const int32_t pr = pass / pc.ncol, pcol = pass - pr * pc.ncol;
        pc.x0 = pc.tx0 + pcol * pc.cw;
        pc.y0 = pc.bound[2] + pr * pc.th;
        pc.cwp = min(pc.cw, pc.tx0 + pc.tw - pc.x0);
        pc.thp = min(pc.th, pc.bound[3] - pc.y0);
      }
    }
    __syncthreads();
    // 2b. clear the tiles of the active particles
    for (int k = 0; k < np; ++k) {
      const PartCtl& pc = ctl.part[k];
      int4* t4 = reinterpret_cast<int4*>(tiles + (size_t)k * tile_px);
      const int4 bg = make_int4(kDepthBg, kDepthBg, kDepthBg, kDepthBg);
      const int n4 = (pc.cwp * pc.thp) >> 2;
      for (int i = tid; i < n4; i += T) t4[i] = bg;
    }
    __syncthreads();
    // 2c. every warp takes (particle, meshlet) items on its own: vertices
    //     into its private cache, then the faces into the particle's tile.
    //     Pass 0 takes every item.  A later pass first lists, with one
    //     thread per item, the meshlets that overlap the particle's band
    //     (their pass-0 rectangle, or for meshes above kCullCap meshlets the
    //     projection of their object-space box, kCullCap meshlets at a
    //     time), then the warps share out the listed items.
    const bool cull = pass > 0;
    const bool check_boxes = !cull_ok && maxpass > 1;
    int4* vc = vcache + wid * sm.vcap;
    for (uint32_t mc = 0; mc < (cull ? nm : 1u); mc += (uint32_t)kCullCap) {
      uint32_t n_items = (uint32_t)np * nm;
      if (cull) {
        const uint32_t nmc = min((uint32_t)kCullCap, nm - mc);
        if (!cull_ok) {
          // meshes above kCullCap meshlets: first the groups of this chunk
          // (kCullCap / kMletGroup per particle) that meet the band, so that
          // only their meshlets' boxes are projected
          const uint32_t g0 = mc / kMletGroup, gn = (nmc + kMletGroup - 1) / kMletGroup;
          for (uint32_t i = (uint32_t)tid; i < (uint32_t)np * gn; i += (uint32_t)T) {
            const uint32_t k = i / gn, g = g0 + (i - k * gn);
            const PartCtl& pc = ctl.part[k];
            bool ov = false;
            if (pass < pc.npass) {
              int4 r;
              ov = !box_rect<kRefProj>(ctl.pose[k], I.cam, __ldg(grp_box + 2 * g), __ldg(grp_box + 2 * g + 1), dx0, dx1,
                             dy0, dy1, r) ||
                   rect_overlaps(r, pc);
            }
            ctl.grp_live[k][i - k * gn] = ov ? 1 : 0;
          }
        }
        const uint32_t nt = (uint32_t)np * nmc;
        if (tid == 0) {
          ctl.n_live = 0;
          ctl.next_item = (uint32_t)nw;
        }
        __syncthreads();
        for (uint32_t b = (uint32_t)(tid & ~31); b < nt; b += (uint32_t)T) {  // whole warps
          const uint32_t i = b + (uint32_t)lane;
          bool ov = false;
          uint32_t k = 0, m = 0;
          if (i < nt) {
            k = i / nmc;
            m = mc + (i - k * nmc);
            const PartCtl& pc = ctl.part[k];
            if (pass < pc.npass) {
              if (cull_ok) {
                ov = rect_overlaps(mbox[k * kCullCap + m], pc);
              } else if (ctl.grp_live[k][(m - mc) / kMletGroup]) {
                int4 r;
                ov = !box_rect<kRefProj>(ctl.pose[k], I.cam, __ldg(I.mlet_box + 2 * m), __ldg(I.mlet_box + 2 * m + 1),
                               dx0, dx1, dy0, dy1, r) ||
                     rect_overlaps(r, pc);
              }
            }
          }
          const unsigned bal = __ballot_sync(0xffffffffu, ov);
          uint32_t at = 0;
          if (lane == 0 && bal) at = atomicAdd(&ctl.n_live, (uint32_t)__popc(bal));
          at = __shfl_sync(0xffffffffu, at, 0);
          if (ov) sm.live[at + (uint32_t)__popc(bal & ((1u << lane) - 1u))] = (k << 28) | m;
        }
        __syncthreads();
        n_items = ctl.n_live;
      }
      // a warp's first item is its index, later ones come from a shared
      // counter: items differ in cost (back-facing meshlets raster nothing)
      // and the barrier after the items waits for the slowest warp
      for (uint32_t item = wid; item < n_items;
           item = __shfl_sync(0xffffffffu, lane == 0 ? atomicAdd(&ctl.next_item, 1u) : 0u, 0)) {
        int k;
        uint32_t m;
        if (cull) {
          const uint32_t e = sm.live[item];
          k = (int)(e >> 28);
          m = e & 0x0fffffffu;
        } else if (np == 1) {  // one particle per CTA: no division
          k = 0;
          m = item;
        } else {
          k = (int)(item / nm);
          m = item - (uint32_t)k * nm;
        }
        PartCtl& pc = ctl.part[k];
        const uint2 hw = __ldg(reinterpret_cast<const uint2*>(I.mlets + m));
        MeshletHdr h;
        h.off = hw.x;
        h.nv = (uint16_t)(hw.y & 0xffffu);
        h.nf = (uint16_t)(hw.y >> 16);
        const int nv = h.nv, nf = h.nf;
        const float4* gv = reinterpret_cast<const float4*>(I.mlet_blob + h.off);
        const uint32_t* gf = reinterpret_cast<const uint32_t*>(I.mlet_blob + h.off + nv * 16);
        const float* pose = ctl.pose[k];
        // kFacePipe: the lane's face words are loaded a round ahead, the
        // first before the transform, so that their latency hides behind
        // it (it costs the plain step kernel's default variant spills)
        uint32_t fi_next = 0u;
        if (kFacePipe) fi_next = lane < nf ? __ldg(gf + lane) : 0u;
        for (int v = lane; v < nv; v += 32) {
          const float4 qv = __ldg(gv + v);
          float u, vv, z;
          project_t<kRefProj>(pose, qv.x, qv.y, qv.z, I.cam, u, vv, z);
          vc[v] = make_int4(__float2int_rn(16.0f * u), __float2int_rn(16.0f * vv), __float_as_int(z), 0);
        }
        __syncwarp();
        // the meshlet's own rectangle starts empty; the render AABB it is
        // merged into starts from the reference's 50000 / -1
        int32_t bminx = INT32_MAX, bmaxx = INT32_MIN, bminy = INT32_MAX, bmaxy = INT32_MIN;
        int32_t* tile = tiles + (size_t)k * tile_px;
        const int32_t x0 = pc.x0, y0 = pc.y0, cwp = pc.cwp, thp = pc.thp;
        // faces: a lane rasterises its own face when the clipped rectangle has
        // at most kLaneRasterMax pixels; larger rectangles are rasterised by the
        // whole warp (set-up broadcast by shuffles, pixels strided over lanes)
        for (int base = 0; base < nf; base += 32) {
          const int f = base + lane;
          uint32_t fi = 0u;
          if (kFacePipe) {
            fi = fi_next;
            if (f + 32 < nf) fi_next = __ldg(gf + f + 32);
          }
          FaceSetup fs;
          int32_t xa = 0, xb = 0, ya = 0, yb = 0;
          bool big = false;
          if (f < nf) {
            if (!kFacePipe) fi = __ldg(gf + f);
            const int4 a = vc[fi & 1023u], bb = vc[(fi >> 10) & 1023u], c = vc[(fi >> 20) & 1023u];
            setup_face_fixed(a.x, a.y, __int_as_float(a.z), bb.x, bb.y, __int_as_float(bb.z), c.x, c.y,
                             __int_as_float(c.z), fs, kEdge);
            bminx = min(bminx, fs.minx);
            bmaxx = max(bmaxx, fs.maxx);
            bminy = min(bminy, fs.miny);
            bmaxy = max(bmaxy, fs.maxy);
            if (fs.live) {
              xa = max(fs.minx, x0);
              xb = min(fs.maxx, x0 + cwp);
              ya = max(fs.miny, y0);
              yb = min(fs.maxy, y0 + thp);
              if (xa < xb && ya < yb) {
                const int32_t n = (xb - xa) * (yb - ya);
                if (!kEdge) writes += (unsigned long long)n;
                if (n > kLaneRasterMax) {
                  big = true;
                } else {
                  // edge values at the row's first pixel, one step per row;
                  // REF mode folds the rounding bias 0xF of the depth
                  // weights into them (exact: 32-bit wrapping sums), EDGE
                  // mode tests their signs and adds it per pixel
                  const int32_t bias = kEdge ? 0 : 0xF;
                  int32_t R2 = wadd(wsub(wadd(fs.c2, wmul(ya, fs.fdx23)), wmul(xa, fs.fdy23)), bias);
                  int32_t R3 = wadd(wsub(wadd(fs.c3, wmul(ya, fs.fdx31)), wmul(xa, fs.fdy31)), bias);
                  int32_t R1 = kEdge ? wsub(wadd(fs.c1, wmul(ya, fs.fdx12)), wmul(xa, fs.fdy12)) : 1;
                  int32_t* row = tile + (ya - y0) * cwp - x0;
                  for (int32_t y = ya; y < yb; ++y) {
                    int32_t CX2 = R2, CX3 = R3, CX1 = R1;
                    // each pixel is one dependent chain (shift, convert,
                    // depth, convert, atomic) linked to the next only by the
                    // edge steps: eight in flight per lane in REF mode (EDGE
                    // mode's inside tests would spill in the variants that
                    // carry both modes)
#pragma unroll (kEdge ? 1 : 8)
                    for (int32_t x = xa; x < xb; ++x) {
                      if (!kEdge || (CX1 > 0 && CX2 > 0 && CX3 > 0)) {
                        const int32_t cx2 = (kEdge ? wadd(CX2, 0xF) : CX2) >> 8;
                        const int32_t cx3 = (kEdge ? wadd(CX3, 0xF) : CX3) >> 8;
                        float depth = fs.z1;
                        depth = depth + (float)cx2 * fs.z2;
                        depth = depth + (float)cx3 * fs.z3;
                        const int32_t d = __float2int_rn(depth);
                        atomicMin(row + x, d);  // a depth at or above the background leaves the tile as it is
                        if (kEdge) writes += 1ull;
                      }
                      CX2 = wsub(CX2, fs.fdy23);
                      CX3 = wsub(CX3, fs.fdy31);
                      if (kEdge) CX1 = wsub(CX1, fs.fdy12);
                    }
                    R2 = wadd(R2, fs.fdx23);
                    R3 = wadd(R3, fs.fdx31);
                    if (kEdge) R1 = wadd(R1, fs.fdx12);
                    row += cwp;
                  }
                }
              }
            }
          }
          unsigned bigmask = __ballot_sync(0xffffffffu, big);
          while (bigmask) {
            const int src = __ffs(bigmask) - 1;
            bigmask &= bigmask - 1;
            // REF mode: the rounding bias folded in, as in the lane path
            const int32_t c2 = wadd(__shfl_sync(0xffffffffu, fs.c2, src), kEdge ? 0 : 0xF);
            const int32_t c3 = wadd(__shfl_sync(0xffffffffu, fs.c3, src), kEdge ? 0 : 0xF);
            const int32_t fdx23 = __shfl_sync(0xffffffffu, fs.fdx23, src);
            const int32_t fdx31 = __shfl_sync(0xffffffffu, fs.fdx31, src);
            const int32_t fdy23 = __shfl_sync(0xffffffffu, fs.fdy23, src);
            const int32_t fdy31 = __shfl_sync(0xffffffffu, fs.fdy31, src);
            const float z1 = __shfl_sync(0xffffffffu, fs.z1, src);
            const float z2 = __shfl_sync(0xffffffffu, fs.z2, src);
            const float z3 = __shfl_sync(0xffffffffu, fs.z3, src);
            const int32_t bxa = __shfl_sync(0xffffffffu, xa, src);
            const int32_t bxb = __shfl_sync(0xffffffffu, xb, src);
            const int32_t bya = __shfl_sync(0xffffffffu, ya, src);
            const int32_t byb = __shfl_sync(0xffffffffu, yb, src);
            int32_t c1 = 0, fdx12 = 0, fdy12 = 0;
            if (kEdge) {
              c1 = __shfl_sync(0xffffffffu, fs.c1, src);
              fdx12 = __shfl_sync(0xffffffffu, fs.fdx12, src);
              fdy12 = __shfl_sync(0xffffffffu, fs.fdy12, src);
            }
            const int32_t w = bxb - bxa;
            const int32_t n = w * (byb - bya);
            const float rw = 1.0f / (float)w;
            for (int32_t pix = lane; pix < n; pix += 32) {
              const int32_t r = small_div(pix, rw);
              const int32_t x = bxa + (pix - r * w), y = bya + r;
              const int32_t CX2 = wsub(wadd(c2, wmul(y, fdx23)), wmul(x, fdy23));
              const int32_t CX3 = wsub(wadd(c3, wmul(y, fdx31)), wmul(x, fdy31));
              if (kEdge) {
                const int32_t CX1 = wsub(wadd(c1, wmul(y, fdx12)), wmul(x, fdy12));
                if (!(CX1 > 0 && CX2 > 0 && CX3 > 0)) continue;
                writes += 1ull;
              }
              const int32_t cx2 = (kEdge ? wadd(CX2, 0xF) : CX2) >> 8;
              const int32_t cx3 = (kEdge ? wadd(CX3, 0xF) : CX3) >> 8;
              float depth = z1;
              depth = depth + (float)cx2 * z2;
              depth = depth + (float)cx3 * z3;
              const int32_t d = __float2int_rn(depth);
              atomicMin(tile + (y - y0) * cwp + (x - x0), d);
            }
          }
        }
        if (pass == 0) {
          bminx = __reduce_min_sync(0xffffffffu, bminx);
          bmaxx = __reduce_max_sync(0xffffffffu, bmaxx);
          bminy = __reduce_min_sync(0xffffffffu, bminy);
          bmaxy = __reduce_max_sync(0xffffffffu, bmaxy);
          // the bound must hold every live face's rectangle (clipped to the
          // domain), or the band passes could miss pixels: the meshlet's
          // union of rectangles, live faces or not, inside the bound
          // settles it for all of them; otherwise (not met in practice: the
          // bound holds the meshlet's projected box) face by face
          {
            const int32_t ux0 = max(bminx, dx0), ux1 = min(bmaxx, dx1);
            const int32_t uy0 = max(bminy, dy0), uy1 = min(bmaxy, dy1);
            if (ux0 < ux1 && uy0 < uy1 &&
                (ux0 < pc.bound[0] || ux1 > pc.bound[1] || uy0 < pc.bound[2] || uy1 > pc.bound[3])) {
              for (int f = lane; f < nf; f += 32) {
                const uint32_t fi = __ldg(gf + f);
                const int4 a = vc[fi & 1023u], bb = vc[(fi >> 10) & 1023u], c = vc[(fi >> 20) & 1023u];
                FaceSetup fs;
                setup_face_fixed(a.x, a.y, __int_as_float(a.z), bb.x, bb.y, __int_as_float(bb.z), c.x, c.y,
                                 __int_as_float(c.z), fs, kEdge);
                if (fs.live) {
                  const int32_t ca = max(fs.minx, dx0), cb = min(fs.maxx, dx1);
                  const int32_t ra = max(fs.miny, dy0), rb = min(fs.maxy, dy1);
                  if (ca < cb && ra < rb &&
                      (ca < pc.bound[0] || cb > pc.bound[1] || ra < pc.bound[2] || rb > pc.bound[3]))
                    violation = true;
                }
              }
            }
          }
          if (lane == 0) {
            atomicMin(&pc.box[0], bminx);
            atomicMax(&pc.box[1], bmaxx);
            atomicMin(&pc.box[2], bminy);
            atomicMax(&pc.box[3], bmaxy);
            if (cull_ok) {
              int4* mb = mbox + k * kCullCap + m;
              mb->x = max(bminx, dx0);
              mb->y = min(bmaxx, dx1);
              mb->z = max(bminy, dy0);
              mb->w = min(bmaxy, dy1);
            }
          }
          if (check_boxes) {
            // the projected box must contain the meshlet's rectangle, or the
            // later passes could skip pixels it writes
            int32_t cx0 = INT32_MAX, cx1 = INT32_MIN, cy0 = INT32_MAX, cy1 = INT32_MIN;
            bool ok = true;
            if (lane < 8) {
              const float4 blo = __ldg(I.mlet_box + 2 * m), bhi = __ldg(I.mlet_box + 2 * m + 1);
              const float x = (lane & 1) ? bhi.x : blo.x;
              const float y = (lane & 2) ? bhi.y : blo.y;
              const float z = (lane & 4) ? bhi.z : blo.z;
              float u, v, zz;
              project_t<kRefProj>(pose, x, y, z, I.cam, u, v, zz);
              ok = zz >= 50.0f && u == u && v == v;
              cx0 = clamp_px(floorf(u) - 1.0f, dx0, dx1);
              cx1 = clamp_px(floorf(u) + 2.0f, dx0, dx1);
              cy0 = clamp_px(floorf(v) - 1.0f, dy0, dy1);
              cy1 = clamp_px(floorf(v) + 2.0f, dy0, dy1);
            }
            ok = __all_sync(0xffffffffu, ok);
            cx0 = __reduce_min_sync(0xffffffffu, cx0);
            cx1 = __reduce_max_sync(0xffffffffu, cx1);
            cy0 = __reduce_min_sync(0xffffffffu, cy0);
            cy1 = __reduce_max_sync(0xffffffffu, cy1);
            const int32_t ax0 = max(bminx, dx0), ax1 = min(bmaxx, dx1);
            const int32_t ay0 = max(bminy, dy0), ay1 = min(bmaxy, dy1);
            if (ok && ax0 < ax1 && ay0 < ay1 && (ax0 < cx0 || ax1 > cx1 || ay0 < cy0 || ay1 > cy1))
              violation = true;
          }
        }
        __syncwarp();
      }
      if (cull) __syncthreads();  // the list is rebuilt for the next chunk
    }
    __syncthreads();
    // the render AABB is final after pass 0's items: one thread per particle
    // (from the last warp) brings the fitness's summed-area words into L1
    if (pass == 0 && tid >= T - np) {
      const PartCtl& pc = ctl.part[T - 1 - tid];
      const SolveParams& prm = I.prm;
      const int32_t minX = min(pc.box[0], prm.cl_min_x), maxX = max(pc.box[1], prm.cl_max_x);
      const int32_t minY = min(pc.box[2], prm.cl_min_y), maxY = max(pc.box[3], prm.cl_max_y);
      const int64_t Ww = (int64_t)maxX - minX, Hh = (int64_t)maxY - minY;
      if (Ww > 0 && Hh > 0) {
        const int64_t pad = (1024 - (Ww * Hh) % 1024) % 1024;
        const int64_t L = pad < Ww ? pad : Ww;
        sat_prefetch(I.sat, W, H, minX, maxX, minY, maxY);
        sat_prefetch(I.sat, W, H, minX, (int64_t)minX + L, maxY, (int64_t)maxY + 1);
      }
    }
    // 2e. scan every active particle's tile over its render AABB
    for (int k = 0; k < np; ++k) {
      PartCtl& pc = ctl.part[k];
      if (pass >= pc.npass) continue;  // CTA-uniform
      const int32_t x0 = pc.x0, y0 = pc.y0, cwp = pc.cwp;
      const int32_t sx0 = max(pc.box[0], x0), sx1 = min(pc.box[1], x0 + cwp);
      const int32_t sy0 = max(pc.box[2], y0), sy1 = min(pc.box[3], y0 + pc.thp);
      BlockSums acc = {0u, 0u, 0u, 0, 0};
      if (sx0 < sx1 && sy0 < sy1) {
        const int32_t gx0 = x0 + ((sx0 - x0) & ~3);
        const int32_t gpr = (sx1 - gx0 + 3) >> 2;
        const int32_t ng = gpr * (sy1 - sy0);
        const float rg = 1.0f / (float)gpr;
        const int32_t* tile = tiles + (size_t)k * tile_px;
        const uint16_t* __restrict__ obs = I.obs;
        const bool vec_obs = (W & 3) == 0;
        // two groups of four pixels per iteration: both groups' loads are in
        // flight before either is counted
        for (int32_t g0 = tid; g0 < ng; g0 += 2 * T) {
          int4 zz[2];
          uint32_t kk[2][4];
#pragma unroll
          for (int j = 0; j < 2; ++j) {
            const int32_t gi = g0 + j * T;
            zz[j] = make_int4(kDepthBg, kDepthBg, kDepthBg, kDepthBg);
            kk[j][0] = kk[j][1] = kk[j][2] = kk[j][3] = 0u;
            if (gi < ng) {
              const int32_t r = small_div(gi, rg);
              const int32_t x = gx0 + ((gi - r * gpr) << 2);
              const int32_t y = sy0 + r;
              zz[j] = *reinterpret_cast<const int4*>(tile + (y - y0) * cwp + (x - x0));
              const bool any = zz[j].x < kDepthBg || zz[j].y < kDepthBg || zz[j].z < kDepthBg || zz[j].w < kDepthBg;
              if (any && y >= 0 && y < H) {
                const uint16_t* orow = obs + (size_t)y * (size_t)W;
                if (vec_obs && x >= 0 && x + 3 < W) {
                  const uint2 qo = __ldg(reinterpret_cast<const uint2*>(orow + x));
                  kk[j][0] = qo.x & 0xffffu;
                  kk[j][1] = qo.x >> 16;
                  kk[j][2] = qo.y & 0xffffu;
                  kk[j][3] = qo.y >> 16;
                } else {
#pragma unroll
                  for (int e = 0; e < 4; ++e)
                    if (x + e >= 0 && x + e < W) kk[j][e] = __ldg(orow + x + e);
                }
              }
            }
          }
#pragma unroll
          for (int j = 0; j < 2; ++j) {
            const int32_t zr[4] = {zz[j].x, zz[j].y, zz[j].z, zz[j].w};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              if (zr[e] < kDepthBg) {
                acc.nR += 1;
                if (kk[j][e] == 0u) {
                  acc.nNo += 1;
                } else {
                  // the wrapped 32-bit difference squared: its magnitude
                  // times itself, one 32 x 32 -> 64-bit product
                  const int32_t d = wsub(zr[e], (int32_t)kk[j][e]);
                  const uint32_t ad = d < 0 ? 0u - (uint32_t)d : (uint32_t)d;
                  add128(acc.lo, acc.hi, (uint64_t)ad * ad);
                }
              }
            }
          }
        }
      }
      acc.nSegR = acc.nR - acc.nNo;  // rendered pixels with an observation
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        acc.nR += __shfl_xor_sync(0xffffffffu, acc.nR, o);
        acc.nNo += __shfl_xor_sync(0xffffffffu, acc.nNo, o);
        acc.nSegR += __shfl_xor_sync(0xffffffffu, acc.nSegR, o);
        const uint64_t lo = __shfl_xor_sync(0xffffffffu, acc.lo, o);
        const uint64_t hi = __shfl_xor_sync(0xffffffffu, acc.hi, o);
        acc.hi += hi;
        add128(acc.lo, acc.hi, lo);
      }
      if (lane == 0) {
        ctl.warp[wid].nR = acc.nR;
        ctl.warp[wid].nNo = acc.nNo;
        ctl.warp[wid].nSegR = acc.nSegR;
        ctl.warp[wid].lo = acc.lo;
        ctl.warp[wid].hi = acc.hi;
      }
      __syncthreads();
      if (wid == 0) {  // the warps' partial sums, reduced by warp 0
        BlockSums t = {0u, 0u, 0u, 0, 0};
        if (lane < nw) {
          t.nR = ctl.warp[lane].nR;
          t.nNo = ctl.warp[lane].nNo;
          t.nSegR = ctl.warp[lane].nSegR;
          t.lo = ctl.warp[lane].lo;
          t.hi = ctl.warp[lane].hi;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          t.nR += __shfl_xor_sync(0xffffffffu, t.nR, o);
          t.nNo += __shfl_xor_sync(0xffffffffu, t.nNo, o);
          t.nSegR += __shfl_xor_sync(0xffffffffu, t.nSegR, o);
          const uint64_t lo = __shfl_xor_sync(0xffffffffu, t.lo, o);
          const uint64_t hi = __shfl_xor_sync(0xffffffffu, t.hi, o);
          t.hi += hi;
          add128(t.lo, t.hi, lo);
        }
        if (lane == 0) {
          pc.nR += t.nR;
          pc.nNo += t.nNo;
          pc.nSegR += t.nSegR;
          pc.hi += t.hi;
          add128(pc.lo, pc.hi, t.lo);
        }
      }
      __syncthreads();
    }
  }
  if (violation) atomicOr(I.err, kErrBound);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) writes += __shfl_xor_sync(0xffffffffu, writes, o);
  if (lane == 0 && writes) atomicAdd(I.stats, writes);
  // 3. window, observed count from the summed-area table, fitness
  if (tid < np) {
    const PartCtl& pc = ctl.part[tid];
    const SolveParams& prm = I.prm;
    const int32_t minX = min(pc.box[0], prm.cl_min_x), maxX = max(pc.box[1], prm.cl_max_x);
    const int32_t minY = min(pc.box[2], prm.cl_min_y), maxY = max(pc.box[3], prm.cl_max_y);
    const int64_t Ww = (int64_t)maxX - minX, Hh = (int64_t)maxY - minY;
    uint32_t observed = 0;
    if (Ww > 0 && Hh > 0) {
      const int64_t area = Ww * Hh;
      const int64_t pad = (1024 - area % 1024) % 1024;
      const int64_t L = pad < Ww ? pad : Ww;
      observed = sat_count(I.sat, W, H, minX, maxX, minY, maxY) +
                 sat_count(I.sat, W, H, minX, (int64_t)minX + L, maxY, (int64_t)maxY + 1);
    }
    fit_out[tid] = fitness_from_counts(observed - pc.nSegR, pc.nR, pc.nNo, pc.lo, pc.hi, prm.num_points);
    atomicAdd(I.stats + 1, (unsigned long long)pc.npass);
  }
  __syncthreads();
}

// Render + score in the instance's raster mode and camera projection
// (uniform per instance).  The fused kernels are compiled in three
// variants, so that the default path's code and registers carry neither
// the EDGE raster nor the reference projection:
//   kVar 0: REF raster, fp32 projection (the default);
//   kVar 1: REF or EDGE raster, fp32 projection;
//   kVar 2: either raster, either projection.
template <int kVar, bool kFacePipe = true>
__device__ __forceinline__ void render_score_mlets(const Instance& I, int np, const FusedSmem& sm, int tile_px,
                                                   SmemCtl& ctl, float* fit_out) {
  const bool edge = kVar >= 1 && I.prm.raster_mode == kRasterEdge;
  const bool ref = kVar == 2 && I.cam.proj == kProjRefAccv;
  if (kVar == 2 && edge && ref)
    render_score_mlets_mode<true, true, kFacePipe>(I, np, sm, tile_px, ctl, fit_out);
  else if (kVar == 2 && ref)
    render_score_mlets_mode<false, true, kFacePipe>(I, np, sm, tile_px, ctl, fit_out);
  else if (kVar >= 1 && edge)
    render_score_mlets_mode<true, false, kFacePipe>(I, np, sm, tile_px, ctl, fit_out);
  else
    render_score_mlets_mode<false, false, kFacePipe>(I, np, sm, tile_px, ctl, fit_out);
}

// PSO step + render + score + personal best for one work item.
// dep_wait: the plain kernel is launched as a programmatic dependent of
// the previous iteration's launch, so its CTAs may start while that launch
// still runs; they wait (griddepcontrol.wait) before the first read of what
// it writes: the swarm state, the global best and the counters.  The mesh
// and the instance record are written before the first launch.
template <int kVar, bool kFacePipe = true>
__device__ void process_item(const Instance& I, uint32_t chunk, uint32_t iter, unsigned char* dyn,
                             int tile_px, int vcap, SmemCtl& ctl, bool dep_wait) {
  const int tid = threadIdx.x;
  const uint32_t P = I.prm.num_particles;
  const uint32_t p0 = chunk * I.ppb;
  const uint32_t np = min(I.ppb, P - p0);
  // while the PSO update runs, the other warps bring the meshlet boxes and
  // headers that the bound and the first items read into L1
  // (meshes of up to kCullCap meshlets; every line lies inside the arrays)
  if (tid >= 32 && I.n_mlets <= (uint32_t)kCullCap) {
    const uint32_t nm = I.n_mlets;
    const uint32_t box_lines = (nm + 3u) / 4u;   // 4 boxes (2 float4 each) per 128-byte line
    const uint32_t hdr_lines = (nm + 15u) / 16u;  // 16 headers (8 bytes each) per line
    for (uint32_t i = (uint32_t)tid - 32u; i < box_lines + hdr_lines; i += blockDim.x - 32u) {
      if (i < box_lines)
        prefetch_l1(reinterpret_cast<const char*>(I.mlet_box) + (size_t)i * 128u);
      else
        prefetch_l1(reinterpret_cast<const char*>(I.mlets) + (size_t)(i - box_lines) * 128u);
    }
  }
  // the iteration's uniforms depend on nothing the previous launch writes:
  // drawn while it finishes (the empty asm keeps them before the wait)
  float u[12];
  if (dep_wait && tid < (int)np && iter > 0) {
    draw_group(I.prm.seed, I.prm.stream, p0 + tid, iter, u);
    asm volatile("" ::"f"(u[0]), "f"(u[1]), "f"(u[2]), "f"(u[3]), "f"(u[4]), "f"(u[5]), "f"(u[6]), "f"(u[7]),
                 "f"(u[8]), "f"(u[9]), "f"(u[10]), "f"(u[11]));
  }
  if (dep_wait) asm volatile("griddepcontrol.wait;" ::: "memory");
  if (tid < (int)np) {
    const uint32_t p = p0 + tid;
    float s[7], v[7];
    if (iter == 0) {
      init_particle(I.prm, p, s, v);
#pragma unroll
      for (int d = 0; d < 7; ++d) I.pbest[p + (size_t)d * P] = s[d];
      I.pbest_fit[p] = kBestInit;
      ctl.pose[tid][7] = kBestInit;
    } else {
      float b[7], g[7];
      // the personal-best fitness is read here, with the state, rather than
      // after the render: one L2 round trip fewer at the end of the item
      ctl.pose[tid][7] = __ldcg(I.pbest_fit + p);
#pragma unroll
      for (int d = 0; d < 7; ++d) {
        s[d] = __ldcg(I.pos + p + (size_t)d * P);
        v[d] = __ldcg(I.vel + p + (size_t)d * P);
        b[d] = __ldcg(I.pbest + p + (size_t)d * P);
        g[d] = __ldcg(I.gbest + 1 + d);
      }
      if (!dep_wait) draw_group(I.prm.seed, I.prm.stream, p, iter, u);
      update_particle_drawn(I.prm, s, v, b, g, u);
    }
#pragma unroll
    for (int d = 0; d < 7; ++d) {
      I.pos[p + (size_t)d * P] = s[d];
      I.vel[p + (size_t)d * P] = v[d];
      ctl.pose[tid][d] = s[d];
    }
  }
  __syncthreads();
  render_score_mlets<kVar, kFacePipe>(I, (int)np, carve_smem(dyn, (int)I.ppb, vcap), tile_px, ctl, ctl.argv);
  if (tid < (int)np) {
    const uint32_t p = p0 + tid;
    const float fv = ctl.argv[tid];
    I.fit[p] = fv;
    if (fv < ctl.pose[tid][7]) {
      I.pbest_fit[p] = fv;
#pragma unroll
      for (int d = 0; d < 7; ++d) I.pbest[p + (size_t)d * P] = ctl.pose[tid][d];
    }
  }
  __syncthreads();
}

// Shared memory of the fused kernels: one vertex cache per warp, ppb
// meshlet-rectangle tables, ppb depth tiles.
size_t fused_smem_bytes(int threads, int ppb, int tile_px, int vcap) {
  return (size_t)(threads / 32) * vcap * 16 + (size_t)ppb * kCullCap * 20 +
         (size_t)ppb * tile_px * 4;
}

// After a work item: every CTA folds its particles' (fitness, index) into
// the instance's key with one 64-bit atomicMin, and the CTA that completes
// the instance's last chunk of the iteration reads (and resets) the key and
// updates the global best (main.cu:1691-1704 and 826-852).  The fitness is
// never NaN and never -0 (a sum of non-negative terms, +inf for an empty
// render), so its bits order as the values do, and the smallest key is the
// first minimum that thrust::min_element returns.
__device__ __forceinline__ unsigned long long fit_key(float f, uint32_t p) {
  return ((unsigned long long)__float_as_uint(f) << 32) | p;
}

__device__ void instance_epilogue(const Instance& I, uint32_t chunk, uint32_t iter, SmemCtl& ctl) {
  const int tid = threadIdx.x;
  if (tid < 32) {
    const uint32_t P = I.prm.num_particles;
    const uint32_t p0 = chunk * I.ppb;
    const uint32_t np = min(I.ppb, P - p0);
    unsigned long long k = ~0ull;
    if ((uint32_t)tid < np) k = fit_key(ctl.argv[tid], p0 + (uint32_t)tid);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long ok = __shfl_xor_sync(0xffffffffu, k, o);
      k = ok < k ? ok : k;
    }
    if (tid == 0) {
      atomicMin(I.argkey, k);
      __threadfence();
      const uint32_t t = atomicAdd(I.done, 1u);
      ctl.last = (t == I.chunks - 1) ? 1 : 0;
    }
  }
  __syncthreads();
  if (!ctl.last) return;
  if (tid == 0) {
    __threadfence();
    const uint32_t P = I.prm.num_particles;
    const unsigned long long key = atomicExch(I.argkey, ~0ull);  // read, and reset for the next iteration
    float g[8];
#pragma unroll
    for (int d = 0; d < 8; ++d) g[d] = __ldcg(I.gbest + d);
    const uint32_t bi = (uint32_t)(key & 0xffffffffull);
    const float bv = __uint_as_float((uint32_t)(key >> 32));
    if (key != ~0ull && bv < g[0]) {
      g[0] = bv;
#pragma unroll
      for (int d = 0; d < 7; ++d) g[1 + d] = __ldcg(I.pos + bi + (size_t)d * P);
#pragma unroll
      for (int d = 0; d < 8; ++d) I.gbest[d] = g[d];
    }
    if (I.trace) {
      float* tr = I.trace + (size_t)iter * 8;
#pragma unroll
      for (int d = 0; d < 8; ++d) tr[d] = g[d];
    }
    *I.done = 0u;
    __threadfence();
  }
  __syncthreads();
}

// Plain form: one launch per iteration of one instance, one CTA per chunk.
template <int kVar>
__global__ void __launch_bounds__(kMaxThreads) qpso_step_kernel(const Instance* __restrict__ inst,
                                                                uint32_t iter, int tile_px, int vcap) {
  extern __shared__ int4 dyn_smem[];
  __shared__ SmemCtl ctl;
  const Instance& I = *inst;
  // the next iteration's launch may place its CTAs now; they wait for this
  // grid to complete before reading anything it writes
  asm volatile("griddepcontrol.launch_dependents;");
  process_item<kVar, kVar != 0>(I, blockIdx.x, iter, reinterpret_cast<unsigned char*>(dyn_smem), tile_px, vcap, ctl,
                                true);
  instance_epilogue(I, blockIdx.x, iter, ctl);
}

// Batched form: every iteration of every instance in one cooperative
// launch, scheduled as a dataflow queue with no grid-wide barrier.  The
// queue starts with iteration 0 of every instance (most expensive first);
// CTAs claim the chunks of the entry at its head, and the CTA that completes
// an instance's iteration updates its global best and appends the
// instance's next iteration.  Instances are independent, so an instance
// waits only for its own previous iteration, and the items of other
// instances fill the gap.

// One attempt to claim a chunk: 0 = chunk `chunk` of iteration `iter` of
// instance `inst`; 1 = every entry has been claimed; 3 = nothing ready now
// (the head entry's iteration is not appended yet).
__device__ int try_claim_queue_item(const BatchArgs& A, uint32_t& inst, uint32_t& iter, uint32_t& chunk) {
  volatile uint32_t* vhead = &A.qctl->head;
  const uint32_t total = A.qctl->total;
  while (true) {
    const uint32_t h = *vhead;
    if (h >= total) return 1;
    QEntry* e = A.queue + h;
    if (!*(volatile uint32_t*)&e->ready) return 3;
    __threadfence();
    const uint32_t in = *(volatile uint32_t*)&e->inst, it = *(volatile uint32_t*)&e->iter;
    const uint32_t c = atomicAdd(&e->next, 1u);
    if (c < A.inst[in].chunks) {
      __threadfence();
      inst = in;
      iter = it;
      chunk = c;
      return 0;
    }
    atomicCAS(&A.qctl->head, h, h + 1u);  // every chunk of the head entry is claimed
  }
}

// Claim with a bounded wait: 0 = claimed, 1 = every entry claimed, 2 =
// error or wait limit.  A wait (every open iteration is in progress) ends
// when another CTA appends or after timeout_ns, and it always ends: the
// iterations in progress run in resident CTAs and append on completion.
__device__ int claim_queue_item(const BatchArgs& A, uint32_t& inst, uint32_t& iter, uint32_t& chunk) {
  unsigned long long t0 = 0ull;
  while (true) {
    const int r = try_claim_queue_item(A, inst, iter, chunk);
    if (r != 3) return r;
    if (*(volatile uint32_t*)A.err != 0u) return 2;
    const unsigned long long now = global_ns();
    if (t0 == 0ull) {
      t0 = now;
    } else if (now - t0 > A.timeout_ns) {
      atomicOr(A.err, kErrTimeout);
      return 2;
    }
    __nanosleep(256);
  }
}

// Append iteration `iter` of instance `inst` (thread 0 of the CTA that
// completed the instance's previous iteration).
__device__ void append_queue_item(const BatchArgs& A, uint32_t inst, uint32_t iter) {
  const uint32_t slot = atomicAdd(&A.qctl->tail, 1u);
  if (slot >= A.qctl->total) {  // cannot happen: one entry per (instance, iteration)
    atomicOr(A.err, kErrTimeout);
    return;
  }
  QEntry* e = A.queue + slot;
  e->inst = inst;
  e->iter = iter;
  __threadfence();
  atomicExch(&e->ready, 1u);
}

template <int kVar>
__global__ void __launch_bounds__(kMaxThreads) qpso_batch_kernel(BatchArgs A, int tile_px, int vcap) {
  extern __shared__ int4 dyn_smem[];
  __shared__ SmemCtl ctl;
  __shared__ uint32_t q[4];  // claim result, instance, iteration, chunk
  while (true) {
    if (threadIdx.x == 0) q[0] = (uint32_t)claim_queue_item(A, q[1], q[2], q[3]);
    __syncthreads();
    const uint32_t state = q[0], in = q[1], it = q[2], chunk = q[3];
    __syncthreads();
    if (state != 0u) return;
    const Instance& I = A.inst[in];
    process_item<kVar>(I, chunk, it, reinterpret_cast<unsigned char*>(dyn_smem), tile_px, vcap, ctl, false);
    instance_epilogue(I, chunk, it, ctl);
    if (ctl.last && threadIdx.x == 0 && it + 1 < I.prm.iterations) append_queue_item(A, in, it + 1);
  }
}

// Serving form: one cooperative launch per scheduling epoch runs the same
// dataflow queue over the active requests (continuous batching: the set of
// requests changes between epochs).  Request `in` runs its iterations
// cur_iter .. end_iter[in] - 1: the queue starts with every request's
// current iteration, and the CTA that completes one advances the request's
// counter and appends its next iteration while it is below end_iter.
template <int kVar>
__global__ void __launch_bounds__(kMaxThreads) qpso_epoch_kernel(BatchArgs A, const uint32_t* __restrict__ end_iter,
                                                                 int tile_px, int vcap) {
  extern __shared__ int4 dyn_smem[];
  __shared__ SmemCtl ctl;
  __shared__ uint32_t q[4];  // claim result, instance, iteration, chunk
  while (true) {
    if (threadIdx.x == 0) q[0] = (uint32_t)claim_queue_item(A, q[1], q[2], q[3]);
    __syncthreads();
    const uint32_t state = q[0], in = q[1], it = q[2], chunk = q[3];
    __syncthreads();
    if (state != 0u) return;
    Instance& I = A.inst[in];
    process_item<kVar>(I, chunk, it, reinterpret_cast<unsigned char*>(dyn_smem), tile_px, vcap, ctl, false);
    instance_epilogue(I, chunk, it, ctl);
    if (ctl.last && threadIdx.x == 0) {
      I.cur_iter = it + 1;
      if (it + 1 < end_iter[in]) append_queue_item(A, in, it + 1);
    }
  }
}

// Wait-expiry check for the batched kernel's bounded wait for work: the
// queue's only entry is never appended, so every CTA's claim waits out
// timeout_ns and returns with kErrTimeout set; nothing else is touched.
__global__ void qpso_queue_probe_kernel(QCtl* qctl, QEntry* queue, uint32_t* err,
                                        unsigned long long timeout_ns) {
  if (threadIdx.x != 0) return;
  BatchArgs A;
  A.inst = nullptr;  // read only for a ready entry
  A.queue = queue;
  A.qctl = qctl;
  A.err = err;
  A.timeout_ns = timeout_ns;
  uint32_t inst, iter, chunk;
  claim_queue_item(A, inst, iter, chunk);
}

// ------------------------------------------------------------------------
// Per-solve preparation.

// Cluster-masked observed depth (main.cu:1548-1557 builds it from
// GraphCannySeg's clusterDepth): depth where label == cluster, else 0.
// blockIdx.y selects the preparation job.
// The cluster-masked depth obs (depth where the label matches, else 0) and
// the summed-area table of (obs != 0): sat[y][x] = #{(i,j): i<y, j<x,
// obs!=0}.  Pass 1: one warp per row writes the row's obs and the inclusive
// scan of its mask into sat[y+1][1..w].
__global__ void sat_rows_kernel(const PrepDesc* __restrict__ jobs) {
  const PrepDesc J = jobs[blockIdx.y];
  const int32_t w = J.width, h = J.height;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t W1 = (int64_t)w + 1;
  if (warp == 0)
    for (int32_t x = lane; x <= w; x += 32) J.sat[x] = 0;
  for (int32_t y = warp; y < h; y += (gridDim.x * blockDim.x) >> 5) {
    int32_t carry = 0;
    int32_t* out = J.sat + (int64_t)(y + 1) * W1;
    if (lane == 0) out[0] = 0;
    for (int32_t x0 = 0; x0 < w; x0 += 32) {
      const int32_t x = x0 + lane;
      int32_t v = 0;
      if (x < w) {
        const int64_t i = (int64_t)y * w + x;
        const uint16_t d = J.depth[i];
        const uint16_t o = (J.labels == nullptr || J.labels[i] == J.label) ? d : (uint16_t)0;
        J.obs[i] = o;
        v = o != 0 ? 1 : 0;
      }
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
      }
      if (x < w) out[x + 1] = carry + v;
      carry += __shfl_sync(0xffffffffu, v, 31);
    }
  }
}

// Pass 2: running sums down the columns.  A CTA takes 32 columns; its 8
// warps split the rows into 8 segments: each thread sums its segment, the
// segments' offsets come from shared memory, and each thread writes its
// segment's running sums.  Integer sums, so the split changes nothing.
constexpr int kSatSegs = 8;

__global__ void __launch_bounds__(32 * kSatSegs) sat_cols_kernel(const PrepDesc* __restrict__ jobs) {
  __shared__ int32_t seg_sum[kSatSegs][32];
  const PrepDesc J = jobs[blockIdx.y];
  const int32_t w = J.width, h = J.height;
  const int64_t W1 = (int64_t)w + 1;
  const int lane = threadIdx.x & 31, seg = threadIdx.x >> 5;
  const int32_t x = blockIdx.x * 32 + lane;
  const int32_t rows = (h + kSatSegs - 1) / kSatSegs;
  const int32_t y0 = 1 + seg * rows, y1 = min(h, y0 + rows - 1);  // rows y0 .. y1 of sat
  int32_t* col = J.sat + x;
  int32_t s = 0;
  if (x <= w)
    for (int32_t y = y0; y <= y1; ++y) s += col[(int64_t)y * W1];
  seg_sum[seg][lane] = s;
  __syncthreads();
  if (x > w) return;
  int32_t run = 0;
  for (int k = 0; k < seg; ++k) run += seg_sum[k][lane];
  for (int32_t y = y0; y <= y1; ++y) {
    run += col[(int64_t)y * W1];
    col[(int64_t)y * W1] = run;
  }
}

// Mesh AABB over all 3F vertices (min/max of each coordinate).
__global__ void mesh_aabb_kernel(const float* __restrict__ mesh, uint32_t F, float* __restrict__ out) {
  __shared__ float red[6][32];
  float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
  const size_t n = 3 * (size_t)F;
  for (size_t i = threadIdx.x; i < n; i += blockDim.x) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float v = mesh[i + c * n];
      lo[c] = fminf(lo[c], v);
      hi[c] = fmaxf(hi[c], v);
    }
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo[c] = fminf(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], o));
      hi[c] = fmaxf(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], o));
    }
  }
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0)
    for (int c = 0; c < 3; ++c) {
      red[c][wid] = lo[c];
      red[3 + c][wid] = hi[c];
    }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = blockDim.x >> 5;
    for (int c = 0; c < 3; ++c) {
      float a = red[c][0], b = red[3 + c][0];
      for (int i = 1; i < nw; ++i) {
        a = fminf(a, red[c][i]);
        b = fmaxf(b, red[3 + c][i]);
      }
      out[c] = a;
      out[3 + c] = b;
    }
  }
}

// Render one pose into a caller window of the raster domain (for parity
// tests and the best-pose render-out): window [x0, x0+ww) x [y0, y0+wh),
// ww*wh <= tile_px, int32 depth with the background value where nothing
// was written.  box receives the render AABB.  One CTA.
__global__ void render_window_kernel(const Instance* __restrict__ inst, const float* __restrict__ pose,
                                     int32_t x0, int32_t y0, int32_t ww, int32_t wh,
                                     int32_t* __restrict__ out, int32_t* __restrict__ box) {
  extern __shared__ int4 dyn_smem[];
  int32_t* tile = reinterpret_cast<int32_t*>(dyn_smem);
  __shared__ float s[8];
  __shared__ int32_t red[4][32];
  const Instance& I = *inst;
  const int tid = threadIdx.x, T = blockDim.x;
  if (tid < 7) s[tid] = pose[tid];
  const int32_t n = ww * wh;
  for (int i = tid; i < n; i += T) tile[i] = kDepthBg;
  __syncthreads();
  const int32_t dx0 = -kGuard, dx1 = I.cam.width + kGuard, dy0 = -kGuard, dy1 = I.cam.height + kGuard;
  int32_t b0 = kAabbInitMin, b1 = kAabbInitMax, b2 = kAabbInitMin, b3 = kAabbInitMax;
  for (uint32_t f = tid; f < I.F; f += T) {
    float u[3], v[3], z[3];
    for (int j = 0; j < 3; ++j)
      project(s, I.mesh[f + (size_t)j * I.F], I.mesh[f + (size_t)(3 + j) * I.F],
              I.mesh[f + (size_t)(6 + j) * I.F], I.cam, u[j], v[j], z[j]);
    FaceSetup fs;
    setup_face(u[0], v[0], z[0], u[1], v[1], z[1], u[2], v[2], z[2], fs);
    b0 = min(b0, fs.minx);
    b1 = max(b1, fs.maxx);
    b2 = min(b2, fs.miny);
    b3 = max(b3, fs.maxy);
    if (!fs.live) continue;
    const int32_t xa = max(max(fs.minx, x0), dx0), xb = min(min(fs.maxx, x0 + ww), dx1);
    const int32_t ya = max(max(fs.miny, y0), dy0), yb = min(min(fs.maxy, y0 + wh), dy1);
    for (int32_t y = ya; y < yb; ++y) {
      int32_t CX2 = wsub(wadd(fs.c2, wmul(y, fs.fdx23)), wmul(xa, fs.fdy23));
      int32_t CX3 = wsub(wadd(fs.c3, wmul(y, fs.fdx31)), wmul(xa, fs.fdy31));
      for (int32_t x = xa; x < xb; ++x) {
        const int32_t cx2 = wadd(CX2, 0xF) >> 8;
        const int32_t cx3 = wadd(CX3, 0xF) >> 8;
        float depth = fs.z1;
        depth = depth + (float)cx2 * fs.z2;
        depth = depth + (float)cx3 * fs.z3;
        atomicMin(tile + (y - y0) * ww + (x - x0), __float2int_rn(depth));
        CX2 = wsub(CX2, fs.fdy23);
        CX3 = wsub(CX3, fs.fdy31);
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    b0 = min(b0, __shfl_xor_sync(0xffffffffu, b0, o));
    b1 = max(b1, __shfl_xor_sync(0xffffffffu, b1, o));
    b2 = min(b2, __shfl_xor_sync(0xffffffffu, b2, o));
    b3 = max(b3, __shfl_xor_sync(0xffffffffu, b3, o));
  }
  const int wid = tid >> 5, lane = tid & 31;
  if (lane == 0) {
    red[0][wid] = b0;
    red[1][wid] = b1;
    red[2][wid] = b2;
    red[3][wid] = b3;
  }
  __syncthreads();
  for (int i = tid; i < n; i += T) out[i] = tile[i];
  if (tid == 0) {
    for (int i = 1; i < (T >> 5); ++i) {
      b0 = min(b0, red[0][i]);
      b1 = max(b1, red[1][i]);
      b2 = min(b2, red[2][i]);
      b3 = max(b3, red[3][i]);
    }
    b0 = min(b0, red[0][0]);
    b1 = max(b1, red[1][0]);
    b2 = min(b2, red[2][0]);
    b3 = max(b3, red[3][0]);
    box[0] = b0;
    box[1] = b1;
    box[2] = b2;
    box[3] = b3;
  }
}

// Score explicit poses of one instance (no PSO state change): pose k goes
// to fit_out[k] and its integer counts to counts_out[k*8 ..].
__global__ void __launch_bounds__(kMaxThreads) score_poses_kernel(const Instance* __restrict__ inst,
                                                                  const float* __restrict__ poses,
                                                                  uint32_t n, int tile_px,
                                                                  float* __restrict__ fit_out) {
  extern __shared__ int4 dyn_smem[];
  __shared__ SmemCtl ctl;
  int32_t* tile = reinterpret_cast<int32_t*>(dyn_smem);
  for (uint32_t k = blockIdx.x; k < n; k += gridDim.x) {
    if (threadIdx.x < 7) ctl.pose[0][threadIdx.x] = poses[(size_t)k * 7 + threadIdx.x];
    __syncthreads();
    const float fv = render_score(*inst, ctl.pose[0], tile, tile_px, ctl);
    if (threadIdx.x == 0) fit_out[k] = fv;
    __syncthreads();
  }
}

// Score explicit poses with the meshlet path, ppb poses per CTA pass.
template <int kVar>
__global__ void __launch_bounds__(kMaxThreads) score_poses_mlet_kernel(const Instance* __restrict__ inst,
                                                                       const float* __restrict__ poses,
                                                                       uint32_t n, int tile_px,
                                                                       float* __restrict__ fit_out, int vcap) {
  extern __shared__ int4 dyn_smem[];
  __shared__ SmemCtl ctl;
  const Instance& I = *inst;
  unsigned char* dyn = reinterpret_cast<unsigned char*>(dyn_smem);
  const FusedSmem sm = carve_smem(dyn, (int)I.ppb, vcap);
  const uint32_t groups = (n + I.ppb - 1) / I.ppb;
  for (uint32_t gi = blockIdx.x; gi < groups; gi += gridDim.x) {
    const uint32_t k0 = gi * I.ppb;
    const int np = (int)min(I.ppb, n - k0);
    if ((int)threadIdx.x < np * 7) ctl.pose[threadIdx.x / 7][threadIdx.x % 7] = poses[(size_t)k0 * 7 + threadIdx.x];
    __syncthreads();
    render_score_mlets<kVar>(I, np, sm, tile_px, ctl, ctl.argv);
    if ((int)threadIdx.x < np) fit_out[k0 + threadIdx.x] = ctl.argv[threadIdx.x];
    __syncthreads();
  }
}

// Writes the instance and preparation records of a scoring call into
// caller-independent scratch and clears its header words (error bits,
// counters), so nothing is copied from the host.
__global__ void noalloc_init_kernel(Instance I, PrepDesc J, Instance* di, PrepDesc* dj) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  *di = I;
  *dj = J;
  for (int d = 0; d < 8; ++d) I.gbest[d] = 0.f;
  *I.done = 0u;
  *I.err = 0u;
  I.stats[0] = 0ull;
  I.stats[1] = 0ull;
}

__global__ void copy_flags_kernel(const uint32_t* src, uint32_t* dst) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *dst = *src;
}

// ------------------------------------------------------------------------
// Host launch wrappers.

size_t smem_ctl_bytes() { return sizeof(SmemCtl); }

// Opt in to more than 48 KB of dynamic shared memory.  The attribute is
// set once per kernel, device and size: calling cudaFuncSetAttribute on
// every launch costs host time that starves back-to-back iteration launches.
template <typename K>
static cudaError_t ensure_smem(K kernel, size_t bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  struct Entry {
    const void* fn;
    int dev;
    size_t bytes;
  };
  static std::mutex mu;
  static std::vector<Entry> done;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> g(mu);
  for (const Entry& x : done)
    if (x.fn == (const void*)kernel && x.dev == dev && x.bytes >= bytes) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) {
    for (Entry& x : done)
      if (x.fn == (const void*)kernel && x.dev == dev) {
        x.bytes = bytes;
        return e;
      }
    done.push_back(Entry{(const void*)kernel, dev, bytes});
  }
  return e;
}

cudaError_t launch_prep(const PrepDesc* jobs, int n, int max_w, int max_h, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  dim3 g2((max_h * 32 + 255) / 256, n);
  sat_rows_kernel<<<g2, 256, 0, st>>>(jobs);
  dim3 g3((max_w + 1 + 31) / 32, n);
  sat_cols_kernel<<<g3, 32 * kSatSegs, 0, st>>>(jobs);
  return cudaGetLastError();
}

cudaError_t launch_mesh_aabb(const float* mesh, uint32_t F, float* out, cudaStream_t st) {
  mesh_aabb_kernel<<<1, 1024, 0, st>>>(mesh, F, out);
  return cudaGetLastError();
}

cudaError_t launch_step(const Instance* inst, uint32_t iter, uint32_t chunks, const TileConfig& cfg,
                        cudaStream_t st, int var, int vcap) {
  const size_t smem = fused_smem_bytes(cfg.threads, cfg.ppb, cfg.tile_px, vcap);
  auto* k = var == 2 ? qpso_step_kernel<2> : var == 1 ? qpso_step_kernel<1> : qpso_step_kernel<0>;
  cudaError_t e = ensure_smem(k, smem);
  if (e != cudaSuccess) return e;
  // a programmatic dependent of the previous launch in the stream (the
  // kernel waits for it before touching its outputs)
  cudaLaunchConfig_t lc = {};
  lc.gridDim = dim3(chunks);
  lc.blockDim = dim3(cfg.threads);
  lc.dynamicSmemBytes = smem;
  lc.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  lc.attrs = attr;
  lc.numAttrs = 1;
  return cudaLaunchKernelEx(&lc, k, inst, iter, cfg.tile_px, vcap);
}

// The largest tile (a multiple of 8 pixels) with which `per_sm` CTAs of the
// fused kernel (plain or batched form) are resident on one SM, or 0: the
// shared memory left per CTA, then checked with the occupancy calculator
// (allocation granularity), stepping down 256 pixels at a time.  The
// kernel's dynamic shared memory limit is only ever raised (ensure_smem).
template <typename K>
static int tile_for_occupancy_k(K kernel, int threads, int ppb, int vcap, int per_sm) {
  int dev = 0, smem_sm = 0, reserved = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess)
    return 0;
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess) return 0;
  const long per_cta = (long)smem_sm / per_sm - reserved - (long)fa.sharedSizeBytes;
  const long rest = (long)fused_smem_bytes(threads, ppb, 0, vcap);
  long tile = ((per_cta - rest) / (4L * ppb)) & ~7L;
  for (int step = 0; step < 16 && tile >= 64; ++step, tile -= 256) {
    const size_t dyn = fused_smem_bytes(threads, ppb, (int)tile, vcap);
    if (ensure_smem(kernel, dyn) != cudaSuccess) continue;
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kernel, threads, dyn) != cudaSuccess) return 0;
    if (blocks >= per_sm) return (int)tile;
  }
  return 0;
}

int tile_for_occupancy(int threads, int ppb, int vcap, int per_sm, bool batched, int var) {
  if (batched)
    return var == 2   ? tile_for_occupancy_k(qpso_batch_kernel<2>, threads, ppb, vcap, per_sm)
           : var == 1 ? tile_for_occupancy_k(qpso_batch_kernel<1>, threads, ppb, vcap, per_sm)
                      : tile_for_occupancy_k(qpso_batch_kernel<0>, threads, ppb, vcap, per_sm);
  return var == 2   ? tile_for_occupancy_k(qpso_step_kernel<2>, threads, ppb, vcap, per_sm)
         : var == 1 ? tile_for_occupancy_k(qpso_step_kernel<1>, threads, ppb, vcap, per_sm)
                    : tile_for_occupancy_k(qpso_step_kernel<0>, threads, ppb, vcap, per_sm);
}

cudaError_t batch_max_grid(const TileConfig& cfg, int var, int vcap, int* blocks_per_sm) {
  const size_t smem = fused_smem_bytes(cfg.threads, cfg.ppb, cfg.tile_px, vcap);
  auto* k = var == 2 ? qpso_batch_kernel<2> : var == 1 ? qpso_batch_kernel<1> : qpso_batch_kernel<0>;
  cudaError_t e = ensure_smem(k, smem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k, cfg.threads, smem);
}

cudaError_t launch_batch(const BatchArgs& args, int grid, const TileConfig& cfg, cudaStream_t st, int var,
                         int vcap) {
  const size_t smem = fused_smem_bytes(cfg.threads, cfg.ppb, cfg.tile_px, vcap);
  auto* k = var == 2 ? qpso_batch_kernel<2> : var == 1 ? qpso_batch_kernel<1> : qpso_batch_kernel<0>;
  cudaError_t e = ensure_smem(k, smem);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t lc = {};
  lc.gridDim = dim3(grid);
  lc.blockDim = dim3(cfg.threads);
  lc.dynamicSmemBytes = smem;
  lc.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  lc.attrs = attr;
  lc.numAttrs = 1;
  return cudaLaunchKernelEx(&lc, k, args, cfg.tile_px, vcap);
}

cudaError_t launch_score(const Instance* inst, const float* poses, uint32_t n, float* fit_out,
                         const TileConfig& cfg, int grid, cudaStream_t st) {
  const size_t smem = (size_t)cfg.tile_px * sizeof(int32_t);
  cudaError_t e = ensure_smem(score_poses_kernel, smem);
  if (e != cudaSuccess) return e;
  score_poses_kernel<<<grid, cfg.threads, smem, st>>>(inst, poses, n, cfg.tile_px, fit_out);
  return cudaGetLastError();
}

// ------------------------------------------------------------------------
// The reference's host render of one pose (RenderCPU, main.h:2012-2043), the
// depth image of results/<rgb>-<N>-best.csv, on the GPU: the kernels'
// projection, then CPUfixedPointRender (main.h:1857-1991), which snaps with
// iround(v) = (int)(v + 0.5f) and keeps depth as a float in a float buffer
// (background 60000) written where `depth < previous`.  The minimum over
// faces is order-free, so the buffer holds order-preserving integer keys of
// the floats and takes atomicMin; -0 is stored as +0 and NaN is never
// written (`NaN < x` is false).  Writes are clipped to the image.

struct Pose8 {
  float s[8];
};

__device__ __forceinline__ uint32_t depth_key(float d) {
  const uint32_t b = __float_as_uint(d == 0.0f ? 0.0f : d);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

__device__ __forceinline__ float depth_from_key(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

__device__ __forceinline__ int32_t iround_ref(float v) { return __float2int_rz(v + 0.5f); }

__global__ void host_render_fill_kernel(uint32_t* keys, uint32_t n) {
  const uint32_t bg = depth_key((float)kDepthBg);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) keys[i] = bg;
}

// one warp per face: every lane sets the face up, the lanes stride over its
// clipped rectangle
__global__ void __launch_bounds__(256) host_render_kernel(const float* __restrict__ mesh, uint32_t F,
                                                          Pose8 pose, Camera cam, uint32_t* keys) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t f = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (f >= F) return;  // warp-uniform
  int32_t X[3], Y[3];
  float Z[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    float u, v;
    project(pose.s, __ldg(mesh + f + (size_t)j * F), __ldg(mesh + f + (size_t)(3 + j) * F),
            __ldg(mesh + f + (size_t)(6 + j) * F), cam, u, v, Z[j]);
    X[j] = iround_ref(16.0f * u);
    Y[j] = iround_ref(16.0f * v);
  }
  FaceSetup fs;
  setup_face_fixed(X[0], Y[0], Z[0], X[1], Y[1], Z[1], X[2], Y[2], Z[2], fs);
  if (!fs.live) return;
  // rectangle [minx, maxx) x [miny, maxy) (extents below 2^31: the wrapped
  // differences are positive) clipped to the image
  const int64_t xa = max((int64_t)fs.minx, (int64_t)0);
  const int64_t xb = min((int64_t)fs.minx + (int64_t)(uint32_t)wsub(fs.maxx, fs.minx), (int64_t)cam.width);
  const int64_t ya = max((int64_t)fs.miny, (int64_t)0);
  const int64_t yb = min((int64_t)fs.miny + (int64_t)(uint32_t)wsub(fs.maxy, fs.miny), (int64_t)cam.height);
  if (xa >= xb || ya >= yb) return;
  const int32_t w = (int32_t)(xb - xa);
  const int32_t n = w * (int32_t)(yb - ya);
  for (int32_t pix = (int32_t)lane; pix < n; pix += 32) {
    const int32_t r = pix / w;
    const int32_t x = (int32_t)xa + (pix - r * w), y = (int32_t)ya + r;
    const int32_t CX2 = wsub(wadd(fs.c2, wmul(y, fs.fdx23)), wmul(x, fs.fdy23));
    const int32_t CX3 = wsub(wadd(fs.c3, wmul(y, fs.fdx31)), wmul(x, fs.fdy31));
    const int32_t cx2 = wadd(CX2, 0xF) >> 8;
    const int32_t cx3 = wadd(CX3, 0xF) >> 8;
    float d = fs.z1;
    d = d + (float)cx2 * fs.z2;
    d = d + (float)cx3 * fs.z3;
    if (d == d) atomicMin(keys + (size_t)y * (size_t)cam.width + (size_t)x, depth_key(d));
  }
}

__global__ void host_render_decode_kernel(uint32_t* keys, uint32_t n) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    keys[i] = __float_as_uint(depth_from_key(keys[i]));
}

cudaError_t launch_host_render(const float* mesh, uint32_t F, const float pose[7], const Camera& cam,
                               float* out, cudaStream_t st) {
  Pose8 p;
  for (int k = 0; k < 7; ++k) p.s[k] = pose[k];
  p.s[7] = 0.f;
  const uint32_t n = (uint32_t)cam.width * (uint32_t)cam.height;
  uint32_t* keys = reinterpret_cast<uint32_t*>(out);
  host_render_fill_kernel<<<(n + 255) / 256, 256, 0, st>>>(keys, n);
  host_render_kernel<<<(unsigned)(((uint64_t)F * 32 + 255) / 256), 256, 0, st>>>(mesh, F, p, cam, keys);
  host_render_decode_kernel<<<(n + 255) / 256, 256, 0, st>>>(keys, n);
  return cudaGetLastError();
}

// ------------------------------------------------------------------------
// Cluster records of a label map (the fields of the segmentation's
// SegResults that the solve reads): per label the pixel count, bounding
// rectangle and exact integer sums for the centroid of the pixels with
// depth.  One thread per pixel, global atomics (once per frame).

__global__ void label_max_kernel(const int32_t* __restrict__ labels, uint32_t n, int32_t* out) {
  int32_t m = -1;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    m = max(m, __ldg(labels + i));
  m = __reduce_max_sync(0xffffffffu, m);
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

__global__ void cluster_init_kernel(ClusterAcc* acc, int32_t nlab) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nlab) return;
  ClusterAcc a;
  a.sum_z = a.sum_xz = a.sum_yz = 0ull;
  a.n = a.nz = 0u;
  a.minx = a.miny = INT32_MAX;
  a.maxx = a.maxy = INT32_MIN;
  acc[i] = a;
}

__global__ void cluster_stats_kernel(const uint16_t* __restrict__ depth, const int32_t* __restrict__ labels,
                                     int32_t W, int32_t H, ClusterAcc* acc, int32_t nlab) {
  const uint32_t n = (uint32_t)W * (uint32_t)H;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int32_t l = __ldg(labels + i);
    if (l < 0 || l >= nlab) continue;
    const int32_t x = (int32_t)(i % (uint32_t)W), y = (int32_t)(i / (uint32_t)W);
    ClusterAcc& a = acc[l];
    atomicAdd(&a.n, 1u);
    atomicMin(&a.minx, x);
    atomicMax(&a.maxx, x + 1);
    atomicMin(&a.miny, y);
    atomicMax(&a.maxy, y + 1);
    const uint32_t z = __ldg(depth + i);
    if (z) {
      atomicAdd(&a.nz, 1u);
      atomicAdd(&a.sum_z, (unsigned long long)z);
      atomicAdd(&a.sum_xz, (unsigned long long)z * (unsigned long long)x);
      atomicAdd(&a.sum_yz, (unsigned long long)z * (unsigned long long)y);
    }
  }
}

cudaError_t launch_label_max(const int32_t* labels, uint32_t n, int32_t* out, cudaStream_t st) {
  const int32_t init = -1;
  cudaError_t e = cudaMemcpyAsync(out, &init, 4, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  label_max_kernel<<<304, 256, 0, st>>>(labels, n, out);
  return cudaGetLastError();
}

cudaError_t launch_cluster_stats(const uint16_t* depth, const int32_t* labels, int32_t W, int32_t H,
                                 ClusterAcc* acc, int32_t nlab, cudaStream_t st) {
  cluster_init_kernel<<<(nlab + 255) / 256, 256, 0, st>>>(acc, nlab);
  cluster_stats_kernel<<<608, 256, 0, st>>>(depth, labels, W, H, acc, nlab);
  return cudaGetLastError();
}

cudaError_t launch_score_mlets(const Instance* inst, const float* poses, uint32_t n, float* fit_out,
                               const TileConfig& cfg, int grid, cudaStream_t st, int var, int vcap) {
  const size_t smem = fused_smem_bytes(cfg.threads, cfg.ppb, cfg.tile_px, vcap);
  auto* k = var == 2 ? score_poses_mlet_kernel<2> : var == 1 ? score_poses_mlet_kernel<1> : score_poses_mlet_kernel<0>;
  cudaError_t e = ensure_smem(k, smem);
  if (e != cudaSuccess) return e;
  k<<<grid, cfg.threads, smem, st>>>(inst, poses, n, cfg.tile_px, fit_out, vcap);
  return cudaGetLastError();
}

// qpso_refine on the device: one thread per candidate of the round
__global__ void refine_gen_kernel(const RefineState* __restrict__ st, float* __restrict__ cand, uint32_t K) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K) return;
  float pose[7];
  for (int k = 0; k < 7; ++k) pose[k] = st->pose[k];
  // the stream's draws in the host order: 6 per random candidate, rounds
  // one after another
  const uint64_t draw0 = ((uint64_t)st->round * (K - 12u) + (i >= 12u ? i - 12u : 0u)) * 6u;
  float c[7];
  refine_candidate(pose, i, st->step_t, st->step_r, st->rng_seed, draw0, c);
  for (int k = 0; k < 7; ++k) cand[(size_t)i * 7 + k] = c[k];
}

// The round's first smallest fitness (the fitness is never NaN and never
// -0, so its bits order as its values do), then the state's update.
__global__ void __launch_bounds__(1024) refine_pick_kernel(RefineState* __restrict__ st,
                                                           const float* __restrict__ cand,
                                                           const float* __restrict__ fits, uint32_t K) {
  __shared__ unsigned long long best[32];
  unsigned long long key = ~0ull;
  for (uint32_t i = threadIdx.x; i < K; i += blockDim.x)
    key = min(key, ((unsigned long long)__float_as_uint(fits[i]) << 32) | i);
  for (int o = 16; o > 0; o >>= 1) key = min(key, __shfl_xor_sync(0xffffffffu, key, o));
  if ((threadIdx.x & 31) == 0) best[threadIdx.x >> 5] = key;
  __syncthreads();
  if (threadIdx.x < 32) {
    key = threadIdx.x < (blockDim.x >> 5) ? best[threadIdx.x] : ~0ull;
    for (int o = 16; o > 0; o >>= 1) key = min(key, __shfl_xor_sync(0xffffffffu, key, o));
    if (threadIdx.x == 0) {
      const uint32_t j = (uint32_t)(key & 0xffffffffu);
      const float fj = fits[j];
      if (fj < st->fit) {
        st->fit = fj;
        for (int k = 0; k < 7; ++k) st->pose[k] = cand[(size_t)j * 7 + k];
      } else {
        st->step_t = st->step_t * 0.5f;
        st->step_r = st->step_r * 0.5f;
      }
      st->round += 1;
    }
  }
}

cudaError_t launch_refine_gen(const RefineState* st, float* cand, uint32_t K, cudaStream_t s) {
  refine_gen_kernel<<<(K + 127) / 128, 128, 0, s>>>(st, cand, K);
  return cudaGetLastError();
}

cudaError_t launch_refine_pick(RefineState* st, const float* cand, const float* fits, uint32_t K, cudaStream_t s) {
  refine_pick_kernel<<<1, 1024, 0, s>>>(st, cand, fits, K);
  return cudaGetLastError();
}

cudaError_t launch_render_window(const Instance* inst, const float* pose, int32_t x0, int32_t y0,
                                 int32_t w, int32_t h, int32_t* out, int32_t* box, int threads,
                                 cudaStream_t st) {
  const size_t smem = (size_t)w * (size_t)h * sizeof(int32_t);
  cudaError_t e = ensure_smem(render_window_kernel, smem < 16 ? 16 : smem);
  if (e != cudaSuccess) return e;
  render_window_kernel<<<1, threads, smem < 16 ? 16 : smem, st>>>(inst, pose, x0, y0, w, h, out, box);
  return cudaGetLastError();
}

cudaError_t epoch_max_grid(const TileConfig& cfg, int var, int vcap, int* blocks_per_sm) {
  const size_t smem = fused_smem_bytes(cfg.threads, cfg.ppb, cfg.tile_px, vcap);
  auto* k = var == 2 ? qpso_epoch_kernel<2> : var == 1 ? qpso_epoch_kernel<1> : qpso_epoch_kernel<0>;
  cudaError_t e = ensure_smem(k, smem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k, cfg.threads, smem);
}

cudaError_t launch_epoch(const BatchArgs& args, const uint32_t* end_iter, int grid, const TileConfig& cfg,
                         cudaStream_t st, int var, int vcap) {
  const size_t smem = fused_smem_bytes(cfg.threads, cfg.ppb, cfg.tile_px, vcap);
  auto* k = var == 2 ? qpso_epoch_kernel<2> : var == 1 ? qpso_epoch_kernel<1> : qpso_epoch_kernel<0>;
  cudaError_t e = ensure_smem(k, smem);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t lc = {};
  lc.gridDim = dim3(grid);
  lc.blockDim = dim3(cfg.threads);
  lc.dynamicSmemBytes = smem;
  lc.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  lc.attrs = attr;
  lc.numAttrs = 1;
  return cudaLaunchKernelEx(&lc, k, args, end_iter, cfg.tile_px, vcap);
}

cudaError_t launch_noalloc_init(const Instance& I, const PrepDesc& J, Instance* di, PrepDesc* dj,
                                cudaStream_t st) {
  noalloc_init_kernel<<<1, 32, 0, st>>>(I, J, di, dj);
  return cudaGetLastError();
}

cudaError_t launch_copy_flags(const uint32_t* src, uint32_t* dst, cudaStream_t st) {
  copy_flags_kernel<<<1, 32, 0, st>>>(src, dst);
  return cudaGetLastError();
}

cudaError_t launch_queue_probe(QCtl* qctl, QEntry* queue, uint32_t* err, uint32_t grid,
                               unsigned long long timeout_ns, cudaStream_t st) {
  qpso_queue_probe_kernel<<<grid, 32, 0, st>>>(qctl, queue, err, timeout_ns);
  return cudaGetLastError();
}

}  // namespace qpso
