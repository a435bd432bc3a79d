// qpso_segment.cu -- the graph stage of the reference's segmentation
// (segment_image, GraphCannySeg.cpp:1053-1250) on the GPU, and its
// sequential merge pass on the host.
//
// GPU, one stream, no waits between kernels:
//   1. the three 8-bit HSV planes smoothed with the reference's Gaussian
//      (smooth, GraphCannySeg.h:423-489): a pass along the rows, then one
//      along the columns, edges clamped, the mask's taps added in order and
//      every product rounded on its own (no contraction);
//   2. the depth range over every pixel but the last (the reference's
//      min/max ranges end at the last pixel's address,
//      GraphCannySeg.cpp:1105-1115);
//   3. every edge of the pixel graph, written at its index in the
//      reference's edge order (GraphCannySeg.cpp:1174-1210) with the
//      HSV + depth + saliency weight of diff (GraphCannySeg.h:2051-2288),
//      as a 64-bit key: the weight's order bits above the edge index;
//   4. a least-significant-digit radix sort of the keys.  It is stable and
//      the keys are distinct, so equal weights end in edge-index order.
// segment_graph's merge pass (GraphCannySeg.cpp:1301-1373) is a sequential
// union-find over about 4 edges per pixel.  The GPU joins the weight-0
// edges, which come first and whose result does not depend on their order
// (connected components); the host runs the pass over the rest, streamed
// as the copies land.  For the small-component merge
// (GraphCannySeg.cpp:1243-1248) the GPU lists the edges that can still
// join two sets and the host runs the merge over that list.  The GPU then
// numbers the sets in the order of their smallest pixel (collectSets,
// GraphCannySeg.cpp:305-352).
//
// This unit is compiled with -ffp-contract=off for its host code too: the
// mask and the thresholds are float expressions that must round like the
// reference's.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "qpso_internal.cuh"

namespace qpso {

// Edges before pixel (x, y) in the reference's order.  A pixel with
// x < W-1 has 1 + 2 [y < H-1] + [y > 0] edges (right, down, down-right,
// up-right); the last pixel of a row has [y < H-1] (down).  Summing rows:
// start(y) = (W-1) (y + 2 min(y, H-1) + max(y-1, 0)) + min(y, H-1).
__host__ __device__ inline uint64_t seg_edge_base(int32_t x, int32_t y, int32_t W, int32_t H) {
  const uint64_t ym = (uint64_t)(y < H - 1 ? y : H - 1);
  const uint64_t start = (uint64_t)(W - 1) * ((uint64_t)y + 2 * ym + (uint64_t)(y > 0 ? y - 1 : 0)) + ym;
  const uint64_t per = 1u + 2u * (y < H - 1) + (y > 0);
  return start + (uint64_t)x * per;
}

uint64_t seg_num_edges(int32_t W, int32_t H) {
  return W <= 0 || H <= 0 ? 0 : seg_edge_base(0, H, W, H);
}

namespace {

constexpr int kMaskCap = 32;
constexpr int kRsThreads = 256;  // one thread per digit value
constexpr int kRsItems = 16;
constexpr int kRsTile = kRsThreads * kRsItems;  // keys per radix-sort block

struct SegConst {
  float mask[kMaskCap];
  int32_t len;
  int32_t W, H;
  float kdv, kdc, kx, ks;
};

// ---- 1. smoothing ------------------------------------------------------

__global__ void seg_rows_kernel(const uint8_t* __restrict__ in, float* __restrict__ out, SegConst c) {
  const size_t n = (size_t)c.W * c.H;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < 3 * n; t += (size_t)gridDim.x * blockDim.x) {
    const size_t plane = t / n, p = t - plane * n;
    const int32_t y = (int32_t)(p / (size_t)c.W), x = (int32_t)(p - (size_t)y * c.W);
    const uint8_t* row = in + plane * n + (size_t)y * c.W;
    float sum = c.mask[0] * (float)row[x];
    for (int i = 1; i < c.len; ++i) {
      const int32_t xl = x - i > 0 ? x - i : 0;
      const int32_t xr = x + i < c.W - 1 ? x + i : c.W - 1;
      sum = sum + c.mask[i] * ((float)row[xl] + (float)row[xr]);
    }
    out[t] = sum;
  }
}

__global__ void seg_cols_kernel(const float* __restrict__ in, float* __restrict__ out, SegConst c) {
  const size_t n = (size_t)c.W * c.H;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < 3 * n; t += (size_t)gridDim.x * blockDim.x) {
    const size_t plane = t / n, p = t - plane * n;
    const int32_t y = (int32_t)(p / (size_t)c.W), x = (int32_t)(p - (size_t)y * c.W);
    const float* col = in + plane * n + x;
    float sum = c.mask[0] * col[(size_t)y * c.W];
    for (int i = 1; i < c.len; ++i) {
      const int32_t yu = y - i > 0 ? y - i : 0;
      const int32_t yd = y + i < c.H - 1 ? y + i : c.H - 1;
      sum = sum + c.mask[i] * (col[(size_t)yu * c.W] + col[(size_t)yd * c.W]);
    }
    out[t] = sum;
  }
}

// ---- 2. depth range ----------------------------------------------------

// mm[0] / mm[1] hold the first pixel's depth on entry
__global__ void seg_range_kernel(const uint16_t* __restrict__ d, size_t m, uint32_t* mm) {
  uint32_t lo = 0xFFFFu, hi = 0u;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < m; t += (size_t)gridDim.x * blockDim.x) {
    const uint32_t v = d[t];
    lo = v < lo ? v : lo;
    hi = v > hi ? v : hi;
  }
  lo = __reduce_min_sync(0xffffffffu, lo);
  hi = __reduce_max_sync(0xffffffffu, hi);
  if ((threadIdx.x & 31) == 0) {
    atomicMin(mm, lo);
    atomicMax(mm + 1, hi);
  }
}

// ---- 3. edges ------------------------------------------------------------

// mapminmax(d, min, max, 0, 1) = (1 - 0) (d - min) / (max - min) + 0
__device__ __forceinline__ float seg_norm_depth(uint16_t d, float mn, float mx) {
  return (1.0f - 0.0f) * ((float)d - mn) / (mx - mn) + 0.0f;
}

// The HSV + depth + saliency branch of diff.  The reference's deg2rad is
// M_PI / 180.0f without parentheses, so the angle and everything the cosine
// touches are double; the chroma term rounds to float once.  cos and log2f
// are CUDA's here and the C library's in the reference: the weights agree
// to an ulp or so.
__device__ float seg_weight(const float* __restrict__ sh, const float* __restrict__ ss,
                            const float* __restrict__ sv, size_t p, size_t q, float z_pivot, float z_current,
                            float sal_p, const SegConst& c) {
  const float c_map = 1.f / 255.f;
  const float h1 = sh[q] * 2.0f, s1 = ss[q] * c_map, v1 = sv[q] * c_map;
  const float h2 = sh[p] * 2.0f, s2 = ss[p] * c_map, v2 = sv[p] * c_map;
  const float delta_v = c.kdv * fabsf(v1 - v2);
  const float delta_h = fabsf(h1 - h2);
  const float theta = delta_h < 180.0f ? delta_h : 360.0f - delta_h;
  const double ang = (double)theta * 3.14159265358979323846 / 180.0;
  const double chord = (double)(s1 * s1 + s2 * s2) - (double)(2.0f * s1 * s2) * cos(ang);
  const float delta_c = (float)((double)c.kdc * sqrt(chord));
  float dist = sqrtf(delta_v * delta_v + delta_c * delta_c);
  if (isnan(dist) || isinf(dist)) dist = 0.0f;
  if (v1 < 0.03f) dist = 0.01f;
  dist = dist / sqrtf(c.kdv * c.kdv + c.kdc * c.kdc);
  const float dd = fabsf(z_pivot - z_current);
  return (c.kx * dd * log2f(1.0f + dist) + c.ks * sal_p) / (c.kx + c.ks);
}

// order bits of a float (ascending as unsigned); -0 is taken as +0, which
// the reference's operator< does not tell apart either
__device__ __forceinline__ uint32_t seg_order_bits(float w) {
  const uint32_t u = __float_as_uint(w == 0.0f ? 0.0f : w);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__global__ void seg_edges_kernel(const float* __restrict__ sm, const uint16_t* __restrict__ depth,
                                 const float* __restrict__ sal, const uint32_t* __restrict__ mm, SegConst c,
                                 uint64_t n_edges, uint64_t* __restrict__ keys, float* __restrict__ wout,
                                 int32_t* __restrict__ ea, int32_t* __restrict__ eb, uint32_t* err) {
  const size_t n = (size_t)c.W * c.H;
  const float* sh = sm;
  const float* ss = sm + n;
  const float* sv = sm + 2 * n;
  const float mn = (float)mm[0], mx = (float)mm[1];
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const int32_t y = (int32_t)(t / (size_t)c.W), x = (int32_t)(t - (size_t)y * c.W);
    uint64_t e = seg_edge_base(x, y, c.W, c.H);
    const float zp = seg_norm_depth(depth[t], mn, mx);
    const float sp = sal[t];
    const int32_t nx[4] = {x + 1, x, x + 1, x + 1};
    const int32_t ny[4] = {y, y + 1, y + 1, y - 1};
    const bool has[4] = {x < c.W - 1, y < c.H - 1, x < c.W - 1 && y < c.H - 1, x < c.W - 1 && y > 0};
    for (int k = 0; k < 4; ++k) {
      if (!has[k]) continue;
      const size_t q = (size_t)ny[k] * c.W + nx[k];
      const float w = seg_weight(sh, ss, sv, t, q, zp, seg_norm_depth(depth[q], mn, mx), sp, c);
      if (e >= n_edges) {
        atomicOr(err, 1u);
        break;
      }
      if (isnan(w)) atomicOr(err, 2u);
      keys[e] = ((uint64_t)seg_order_bits(w) << 32) | e;
      wout[e] = w;
      ea[e] = (int32_t)t;
      eb[e] = (int32_t)q;
      ++e;
    }
  }
}

// ---- 4. radix sort -------------------------------------------------------

__global__ void rs_hist_kernel(const uint64_t* __restrict__ keys, uint32_t n, int shift, uint32_t* hist,
                               uint32_t nblk) {
  __shared__ uint32_t h[kRsThreads];
  h[threadIdx.x] = 0;
  __syncthreads();
  const size_t base = (size_t)blockIdx.x * kRsTile;
  for (int i = 0; i < kRsItems; ++i) {
    const size_t j = base + (size_t)i * kRsThreads + threadIdx.x;
    if (j < n) atomicAdd(&h[(uint32_t)(keys[j] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[(size_t)threadIdx.x * nblk + blockIdx.x] = h[threadIdx.x];
}

// Exclusive prefix sums of the histogram's digit rows (digit-major: row d
// holds the counts of digit d in tiles 0 .. nblk - 1), one CTA of
// kRsThreads per row, in place; row totals into tot[d].
__global__ void rs_rowscan_kernel(uint32_t* hist, uint32_t nblk, uint32_t* tot) {
  __shared__ uint32_t wsum[kRsThreads / 32];
  uint32_t* row = hist + (size_t)blockIdx.x * nblk;
  const uint32_t per = (nblk + kRsThreads - 1) / kRsThreads;
  const uint32_t lo = threadIdx.x * per, hi = min(lo + per, nblk);
  uint32_t s = 0;
  for (uint32_t i = lo; i < hi; ++i) s += row[i];
  // exclusive scan of the threads' sums
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = s;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[warp] = x;
  __syncthreads();
  uint32_t before = 0;
  for (int w = 0; w < warp; ++w) before += wsum[w];
  uint32_t run = before + x - s;
  for (uint32_t i = lo; i < hi; ++i) {
    const uint32_t v = row[i];
    row[i] = run;
    run += v;
  }
  if (threadIdx.x == kRsThreads - 1) tot[blockIdx.x] = before + x;
}

// Stable scatter of one block's tile: keys go out in tile order within each
// digit.  Each round takes 256 consecutive keys; a key's place is the
// digit's running position + the same digit's count in earlier warps of the
// round + its rank among equal digits of its own warp.
__global__ void rs_scatter_kernel(const uint64_t* __restrict__ in, uint64_t* __restrict__ out, uint32_t n,
                                  int shift, const uint32_t* __restrict__ offs, const uint32_t* __restrict__ tot,
                                  uint32_t nblk, uint32_t* err) {
  __shared__ uint32_t base[kRsThreads];
  __shared__ uint32_t wcnt[kRsThreads / 32][kRsThreads];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  {
    // digit d's first position: the keys of smaller digits (exclusive scan
    // of the row totals), then this tile's place in row d
    const uint32_t t = tot[threadIdx.x];
    uint32_t x = t;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wcnt[0][warp] = x;
    __syncthreads();
    uint32_t before = 0;
    for (int w = 0; w < warp; ++w) before += wcnt[0][w];
    base[threadIdx.x] = before + x - t + offs[(size_t)threadIdx.x * nblk + blockIdx.x];
    __syncthreads();  // wcnt is cleared below
  }
  const size_t tile = (size_t)blockIdx.x * kRsTile;
  for (int r = 0; r < kRsItems; ++r) {
    for (int w = 0; w < kRsThreads / 32; ++w) wcnt[w][threadIdx.x] = 0u;
    __syncthreads();
    const size_t j = tile + (size_t)r * kRsThreads + threadIdx.x;
    const bool valid = j < n;
    const uint64_t key = valid ? in[j] : 0ull;
    const uint32_t d = valid ? (uint32_t)(key >> shift) & 255u : 256u;
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
    if (valid && rank == 0) wcnt[warp][d] = __popc(peers);
    __syncthreads();
    uint32_t total = 0;
    for (int w = 0; w < kRsThreads / 32; ++w) {
      const uint32_t cnt = wcnt[w][threadIdx.x];
      wcnt[w][threadIdx.x] = total;
      total += cnt;
    }
    __syncthreads();
    if (valid) {
      const uint32_t pos = base[d] + wcnt[warp][d] + rank;
      if (pos < n)
        out[pos] = key;
      else
        atomicOr(err, 4u);
    }
    __syncthreads();
    base[threadIdx.x] += total;
    __syncthreads();
  }
}

__global__ void seg_misc_init_kernel(const uint16_t* __restrict__ d, uint32_t* misc) {
  misc[0] = d[0];
  misc[1] = d[0];
  misc[2] = 0;
  misc[3] = 0;
}

int grid_for(size_t work, int threads, int sms) {
  const size_t blocks = (work + threads - 1) / threads;
  const size_t cap = (size_t)sms * 8;
  return (int)(blocks < 1 ? 1 : blocks < cap ? blocks : cap);
}

int bit_length(uint64_t v) {
  int b = 0;
  while (v) {
    ++b;
    v >>= 1;
  }
  return b;
}

}  // namespace

// ---- host: mask, edge list, merge pass -----------------------------------

int seg_gauss_mask(float sigma, float* mask, int capacity) {
  if (!(sigma >= 0.01f)) sigma = 0.01f;  // std::max(sigma, 0.01F); NaN is refused by the caller
  const int len = (int)std::ceil((double)sigma * 4.0) + 1;
  if (len > capacity) return -1;
  for (int i = 0; i < len; ++i) {
    const float q = (float)i / sigma;
    const float q2 = q * q;
    mask[i] = (float)std::exp(-0.5 * (double)q2);
  }
  float sum = 0.0f;
  for (int i = 1; i < len; ++i) sum += std::fabs(mask[i]);
  sum = 2.0f * sum + std::fabs(mask[0]);
  for (int i = 0; i < len; ++i) mask[i] /= sum;
  return len;
}

void seg_edge_ends(int32_t W, int32_t H, int32_t* a, int32_t* b) {
  for (int32_t y = 0; y < H; ++y)
    for (int32_t x = 0; x < W; ++x) {
      uint64_t e = seg_edge_base(x, y, W, H);
      const int32_t i = y * W + x;
      if (x < W - 1) a[e] = i, b[e++] = i + 1;
      if (y < H - 1) a[e] = i, b[e++] = i + W;
      if (x < W - 1 && y < H - 1) a[e] = i, b[e++] = i + W + 1;
      if (x < W - 1 && y > 0) a[e] = i, b[e++] = i - W + 1;
    }
}

namespace {

// union-find over the pixels; the threshold of a set lives at its root
struct Forest {
  std::vector<int32_t> parent, size;
  explicit Forest(size_t n) : parent(n), size(n, 1) {
    for (size_t i = 0; i < n; ++i) parent[i] = (int32_t)i;
  }
  int32_t find(int32_t x) {
    while (parent[x] != x) {
      parent[x] = parent[parent[x]];
      x = parent[x];
    }
    return x;
  }
  int32_t join(int32_t a, int32_t b) {  // roots; returns the new root
    if (size[a] < size[b]) std::swap(a, b);
    parent[b] = a;
    size[a] += size[b];
    return a;
  }
};

}  // namespace

// The merge pass over edges given in sorted order (order[i] = edge index,
// ea/eb/w indexed by edge), then the small-component merge in the same
// order, then labels numbered by each set's smallest pixel.  The partition
// does not depend on the forest's union rule: a threshold is only read at
// the current root of its set.
uint32_t seg_merge(uint32_t n_pixels, uint64_t n_edges, const uint32_t* order, const int32_t* ea,
                   const int32_t* eb, const float* w, float k, float min_size, int32_t* labels) {
  Forest f(n_pixels);
  std::vector<float> thr(n_pixels, k / (float)1);  // THRESHOLD(1, k)
  for (uint64_t i = 0; i < n_edges; ++i) {
    const uint32_t e = order[i];
    const float we = w[e];
    const int32_t a = f.find(ea[e]), b = f.find(eb[e]);
    if (a == b || !(we <= thr[a] && we <= thr[b])) continue;
    const int32_t r = f.join(a, b);
    thr[r] = we + k / (float)f.size[r];
  }
  for (uint64_t i = 0; i < n_edges; ++i) {
    const uint32_t e = order[i];
    const int32_t a = f.find(ea[e]), b = f.find(eb[e]);
    if (a != b && ((float)f.size[a] < min_size || (float)f.size[b] < min_size)) f.join(a, b);
  }
  std::vector<int32_t> id(n_pixels, -1);
  uint32_t next = 0;
  for (uint32_t v = 0; v < n_pixels; ++v) {
    const int32_t r = f.find((int32_t)v);
    if (id[r] < 0) id[r] = (int32_t)next++;
    labels[v] = id[r];
  }
  return next;
}

// ---- GPU graph + sort ------------------------------------------------------

size_t seg_workspace_bytes(int32_t W, int32_t H) {
  const size_t n = (size_t)W * H;
  const uint64_t E = seg_num_edges(W, H);
  const size_t nblk = (size_t)((E + kRsTile - 1) / kRsTile);
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  return al(3 * n) + al(2 * n) + al(4 * n) + 2 * al(12 * n) + 2 * al(8 * E) + 3 * al(4 * E) +
         al(4 * 256 * (nblk ? nblk : 1)) + al(4 * 256) + al(16) + al(4 * n) + al(4 * (n / 1024 + 2));
}

void seg_ws_inputs(void* ws, int32_t W, int32_t H, uint8_t** hsv, uint16_t** depth, float** sal) {
  const size_t n = (size_t)W * H;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  char* p = static_cast<char*>(ws);
  *hsv = (uint8_t*)p;
  p += al(3 * n);
  *depth = (uint16_t*)p;
  p += al(2 * n);
  *sal = (float*)p;
}

namespace {

// Device buffers of the graph stage after the sort.
struct SegGraphDev {
  uint64_t* sorted;  // keys in ascending order (edge index in the low 32 bits)
  uint64_t* spare;   // the sort's other key buffer (free after the sort)
  float* w;          // weights in edge order
  int32_t* ea;
  int32_t* eb;
  uint32_t* misc;    // [0] depth min, [1] depth max, [2] error bits, [3] zero-weight edges
  float* tmp;        // 12 n bytes, free after the smoothing
  int32_t* lab;      // n labels
  uint32_t* lblk;    // the label numbering's block counts (n / 1024 + 2)
};

// Upload (or take the inputs already in their slots), smooth, weigh and sort.
cudaError_t seg_graph_device(const uint8_t* hsv_host[3], const uint16_t* depth_host, const float* sal_host,
                             int32_t W, int32_t H, const float* mask, int len, float kdv, float kdc, float kx,
                             float ks, void* ws, int sms, cudaStream_t st, SegGraphDev* out) {
  const size_t n = (size_t)W * H;
  const uint64_t E = seg_num_edges(W, H);
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  char* p = static_cast<char*>(ws);
  uint8_t* d_hsv = (uint8_t*)p;
  p += al(3 * n);
  uint16_t* d_depth = (uint16_t*)p;
  p += al(2 * n);
  float* d_sal = (float*)p;
  p += al(4 * n);
  float* d_tmp = (float*)p;
  p += al(12 * n);
  float* d_sm = (float*)p;
  p += al(12 * n);
  uint64_t* d_k0 = (uint64_t*)p;
  p += al(8 * E);
  uint64_t* d_k1 = (uint64_t*)p;
  p += al(8 * E);
  float* d_w = (float*)p;
  p += al(4 * E);
  int32_t* d_ea = (int32_t*)p;
  p += al(4 * E);
  int32_t* d_eb = (int32_t*)p;
  p += al(4 * E);
  const uint32_t nblk = (uint32_t)((E + kRsTile - 1) / kRsTile);
  uint32_t* d_hist = (uint32_t*)p;
  p += al(4 * 256 * (nblk ? nblk : 1));
  uint32_t* d_tot = (uint32_t*)p;
  p += al(4 * 256);
  uint32_t* d_misc = (uint32_t*)p;
  p += al(16);
  int32_t* d_lab = (int32_t*)p;
  p += al(4 * n);
  uint32_t* d_lblk = (uint32_t*)p;

  cudaError_t e;
  if (hsv_host) {
    for (int c = 0; c < 3; ++c)
      if ((e = cudaMemcpyAsync(d_hsv + c * n, hsv_host[c], n, cudaMemcpyHostToDevice, st)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(d_depth, depth_host, 2 * n, cudaMemcpyHostToDevice, st)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(d_sal, sal_host, 4 * n, cudaMemcpyHostToDevice, st)) != cudaSuccess) return e;
    const uint32_t misc[4] = {depth_host[0], depth_host[0], 0u, 0u};
    if ((e = cudaMemcpyAsync(d_misc, misc, sizeof(misc), cudaMemcpyHostToDevice, st)) != cudaSuccess) return e;
  } else {
    // the inputs are already in their slots (written by the stages before)
    seg_misc_init_kernel<<<1, 1, 0, st>>>(d_depth, d_misc);
  }

  SegConst c{};
  for (int i = 0; i < len; ++i) c.mask[i] = mask[i];
  c.len = len;
  c.W = W;
  c.H = H;
  c.kdv = kdv;
  c.kdc = kdc;
  c.kx = kx;
  c.ks = ks;
  seg_rows_kernel<<<grid_for(3 * n, 256, sms), 256, 0, st>>>(d_hsv, d_tmp, c);
  seg_cols_kernel<<<grid_for(3 * n, 256, sms), 256, 0, st>>>(d_tmp, d_sm, c);
  if (n > 1) seg_range_kernel<<<grid_for(n - 1, 256, sms), 256, 0, st>>>(d_depth, n - 1, d_misc);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  uint64_t* src = d_k0;
  uint64_t* dst = d_k1;
  if (E > 0) {
    seg_edges_kernel<<<grid_for(n, 256, sms), 256, 0, st>>>(d_sm, d_depth, d_sal, d_misc, c, E, d_k0, d_w,
                                                            d_ea, d_eb, d_misc + 2);
    // key bits: the edge index in the low bit_length(E - 1) bits, the
    // weight's order bits in the high 32
    const int idx_bits = bit_length(E - 1);
    for (int shift = 0; shift < 64; shift += 8) {
      if (shift < 32 && shift >= idx_bits) continue;  // all keys share these digits
      rs_hist_kernel<<<nblk, kRsThreads, 0, st>>>(src, (uint32_t)E, shift, d_hist, nblk);
      rs_rowscan_kernel<<<kRsThreads, kRsThreads, 0, st>>>(d_hist, nblk, d_tot);
      rs_scatter_kernel<<<nblk, kRsThreads, 0, st>>>(src, dst, (uint32_t)E, shift, d_hist, d_tot, nblk,
                                                     d_misc + 2);
      std::swap(src, dst);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  *out = SegGraphDev{src, dst, d_w, d_ea, d_eb, d_misc, d_tmp, d_lab, d_lblk};
  return cudaSuccess;
}

// The sorted edges from position `first` (*first_at when first_at is not
// null) packed for the host: (first end << 2 | direction) and the weight,
// in sorted order.  Directions: 0 right, 1 down, 2 down-right, 3 up-right
// (the second end is first + 1, W, W + 1, 1 - W).
__global__ void seg_pack_kernel(const uint64_t* __restrict__ sorted, const int32_t* __restrict__ ea,
                                const int32_t* __restrict__ eb, const float* __restrict__ w, uint32_t E,
                                int32_t W, const uint32_t* first_at, uint32_t* __restrict__ pk,
                                float* __restrict__ pw) {
  const uint32_t first = first_at ? *first_at : 0u;
  for (size_t i = first + blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < E;
       i += (size_t)gridDim.x * blockDim.x) {
    const uint32_t e = (uint32_t)(sorted[i] & 0xFFFFFFFFull);
    const int32_t a = ea[e], d = eb[e] - a;
    const uint32_t code = d == 1 ? 0u : d == W ? 1u : d == W + 1 ? 2u : 3u;
    pk[i - first] = ((uint32_t)a << 2) | code;
    pw[i - first] = w[e];
  }
}

// ---- the zero-weight edges: connected components -------------------------
//
// segment_graph's pass starts with singletons whose threshold is k / 1.  The
// sorted edges begin with the weight-0 ones, and with k >= 0 every set
// admits weight 0 (k / |C| >= 0, and a set merged at weight 0 has threshold
// 0 + k / |C|).  So the pass over them joins exactly the connected
// components of the weight-0 edges, whatever their order, and leaves each
// component with threshold k / |C| (its last join sets it at its final
// size).  The GPU builds that forest; the host starts its pass after those
// edges, and its small-component pass skips them too (their ends are in one
// set from then on).

// z = the number of weight-0 edges (sorted keys whose order bits are those
// of +0), or 0 when k < 0
__global__ void seg_zero_count_kernel(const uint64_t* __restrict__ sorted, uint32_t E, int enabled, uint32_t* z) {
  const uint32_t zb = 0x80000000u;  // order bits of +0
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < E; i += (size_t)gridDim.x * blockDim.x) {
    const bool here = (uint32_t)(sorted[i] >> 32) == zb;
    const bool next = i + 1 < E && (uint32_t)(sorted[i + 1] >> 32) == zb;
    if (enabled && here && !next) *z = (uint32_t)(i + 1);  // the one boundary
  }
}

// A set's size and threshold side by side (one cache line holds both, the
// host reads them together).
struct SetState {
  int32_t size;
  float thr;
};

__global__ void seg_forest_init_kernel(int32_t* __restrict__ parent, SetState* __restrict__ state, uint32_t n) {
  for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < n; v += (size_t)gridDim.x * blockDim.x) {
    parent[v] = (int32_t)v;
    state[v].size = 0;
  }
}

// root of x, halving the path (only non-root entries are rewritten here;
// roots change only by the hooking CAS)
__device__ __forceinline__ int32_t seg_root(volatile int32_t* parent, int32_t x) {
  while (true) {
    const int32_t p = parent[x];
    if (p == x) return x;
    const int32_t g = parent[p];
    if (g != p) parent[x] = g;
    x = p;
  }
}

// join the ends of each weight-0 edge: the larger root is hooked under the
// smaller by CAS (a failed CAS means another thread hooked it: retry from
// its new root), so each component's root ends as its smallest pixel
__global__ void seg_zero_link_kernel(const uint64_t* __restrict__ sorted, const int32_t* __restrict__ ea,
                                     const int32_t* __restrict__ eb, const uint32_t* z, int32_t* parent) {
  const uint32_t nz = *z;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nz; i += (size_t)gridDim.x * blockDim.x) {
    const uint32_t e = (uint32_t)(sorted[i] & 0xFFFFFFFFull);
    int32_t a = ea[e], b = eb[e];
    while (true) {
      a = seg_root(parent, a);
      b = seg_root(parent, b);
      if (a == b) break;
      if (a > b) {
        const int32_t t = a;
        a = b;
        b = t;
      }
      if (atomicCAS(parent + b, b, a) == b) break;
    }
  }
}

__global__ void seg_forest_flatten_kernel(int32_t* parent, SetState* __restrict__ state, uint32_t n) {
  for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < n; v += (size_t)gridDim.x * blockDim.x) {
    const int32_t r = seg_root(parent, (int32_t)v);
    parent[v] = r;
    atomicAdd(&state[r].size, 1);
  }
}

// ---- the small-component pass's candidate edges -------------------------
//
// After segment_graph's pass, an edge can join its ends in the
// small-component pass only if, at that pass's start, they lie in different
// sets and one of them is smaller than min_size: sets only grow and only
// merge, so every other edge finds its ends in one set, or both sets large,
// whatever the pass did before it.  The GPU lists those edges in sorted
// order from the forest the host's first pass left (uploaded), and the host
// runs the pass over the list alone.

constexpr int kCandThreads = 1024;

__global__ void seg_forest_roots_kernel(int32_t* parent, uint32_t n) {
  for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < n; v += (size_t)gridDim.x * blockDim.x)
    parent[v] = seg_root(parent, (int32_t)v);
}

__device__ __forceinline__ bool seg_is_candidate(uint32_t pk, int32_t W, const int32_t* __restrict__ root,
                                                 const SetState* __restrict__ st, float min_size) {
  const int32_t a0 = (int32_t)(pk >> 2);
  const uint32_t d = pk & 3u;
  const int32_t b0 = a0 + (d == 0u ? 1 : d == 1u ? W : d == 2u ? W + 1 : 1 - W);
  const int32_t ra = root[a0], rb = root[b0];
  return ra != rb && ((float)st[ra].size < min_size || (float)st[rb].size < min_size);
}

// candidates per block of kCandThreads packed edges
__global__ void __launch_bounds__(kCandThreads) seg_cand_count_kernel(const uint32_t* __restrict__ pk, uint32_t E2,
                                                                      int32_t W, const int32_t* __restrict__ root,
                                                                      const SetState* __restrict__ st,
                                                                      float min_size, uint32_t* __restrict__ blk) {
  const size_t i = (size_t)blockIdx.x * kCandThreads + threadIdx.x;
  const bool c = i < E2 && seg_is_candidate(pk[i], W, root, st, min_size);
  const int cnt = __syncthreads_count(c);
  if (threadIdx.x == 0) blk[blockIdx.x] = (uint32_t)cnt;
}

// exclusive prefix of the block counts, in place; the total into blk[nb]
__global__ void __launch_bounds__(kCandThreads) seg_cand_scan_kernel(uint32_t* blk, uint32_t nb) {
  __shared__ uint32_t part[kCandThreads];
  const uint32_t per = (nb + kCandThreads - 1) / kCandThreads;
  const uint32_t lo = threadIdx.x * per, hi = min(lo + per, nb);
  uint32_t s = 0;
  for (uint32_t i = lo; i < hi; ++i) s += blk[i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int off = 1; off < kCandThreads; off <<= 1) {
    const uint32_t v = threadIdx.x >= (unsigned)off ? part[threadIdx.x - off] : 0u;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  uint32_t run = threadIdx.x ? part[threadIdx.x - 1] : 0u;
  for (uint32_t i = lo; i < hi; ++i) {
    const uint32_t v = blk[i];
    blk[i] = run;
    run += v;
  }
  if (threadIdx.x == kCandThreads - 1) blk[nb] = part[kCandThreads - 1];
}

// the candidates, in sorted order
__global__ void __launch_bounds__(kCandThreads) seg_cand_scatter_kernel(const uint32_t* __restrict__ pk, uint32_t E2,
                                                                        int32_t W, const int32_t* __restrict__ root,
                                                                        const SetState* __restrict__ st,
                                                                        float min_size, const uint32_t* __restrict__ blk,
                                                                        uint32_t* __restrict__ out) {
  __shared__ uint32_t wbase[kCandThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const size_t i = (size_t)blockIdx.x * kCandThreads + threadIdx.x;
  const uint32_t v = i < E2 ? pk[i] : 0u;
  const bool c = i < E2 && seg_is_candidate(v, W, root, st, min_size);
  const unsigned bal = __ballot_sync(0xffffffffu, c);
  if (lane == 0) wbase[warp] = (uint32_t)__popc(bal);
  __syncthreads();
  if (warp == 0) {  // exclusive scan of the warps' counts
    const uint32_t cnt = lane < kCandThreads / 32 ? wbase[lane] : 0u;
    uint32_t x = cnt;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane < kCandThreads / 32) wbase[lane] = x - cnt;
  }
  __syncthreads();
  if (c) out[blk[blockIdx.x] + wbase[warp] + (uint32_t)__popc(bal & ((1u << lane) - 1u))] = v;
}

// ---- labels numbered by each set's smallest pixel (collectSets' order) ----

__global__ void seg_minpix_init_kernel(int32_t* __restrict__ minpix, uint32_t n) {
  for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < n; v += (size_t)gridDim.x * blockDim.x)
    minpix[v] = INT32_MAX;
}

// each set's smallest pixel; a warp's lanes of one set leave the atomic to
// the lowest of them (pixels rise with the lane), so a large set costs one
// atomic per warp, not one per pixel
__global__ void seg_minpix_kernel(const int32_t* __restrict__ root, int32_t* minpix, uint32_t n) {
  const int lane = threadIdx.x & 31;
  for (size_t v0 = blockIdx.x * (size_t)blockDim.x + (threadIdx.x & ~31u); v0 < n;
       v0 += (size_t)gridDim.x * blockDim.x) {  // whole warps
    const size_t v = v0 + lane;
    const int32_t r = v < n ? root[v] : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, r);
    if (v < n && (peers & ((1u << lane) - 1u)) == 0u) atomicMin(minpix + r, (int32_t)v);
  }
}

// first pixels (each set's smallest) per block of kCandThreads pixels
__global__ void __launch_bounds__(kCandThreads) seg_first_count_kernel(const int32_t* __restrict__ root,
                                                                       const int32_t* __restrict__ minpix,
                                                                       uint32_t n, uint32_t* __restrict__ blk) {
  const size_t v = (size_t)blockIdx.x * kCandThreads + threadIdx.x;
  const bool f = v < n && minpix[root[v]] == (int32_t)v;
  const int cnt = __syncthreads_count(f);
  if (threadIdx.x == 0) blk[blockIdx.x] = (uint32_t)cnt;
}

// a set's number, at its first pixel: the first pixels before it
__global__ void __launch_bounds__(kCandThreads) seg_first_number_kernel(const int32_t* __restrict__ root,
                                                                        const int32_t* __restrict__ minpix,
                                                                        uint32_t n, const uint32_t* __restrict__ blk,
                                                                        int32_t* __restrict__ number) {
  __shared__ uint32_t wbase[kCandThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const size_t v = (size_t)blockIdx.x * kCandThreads + threadIdx.x;
  const bool f = v < n && minpix[root[v]] == (int32_t)v;
  const unsigned bal = __ballot_sync(0xffffffffu, f);
  if (lane == 0) wbase[warp] = (uint32_t)__popc(bal);
  __syncthreads();
  if (warp == 0) {
    const uint32_t cnt = lane < kCandThreads / 32 ? wbase[lane] : 0u;
    uint32_t x = cnt;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane < kCandThreads / 32) wbase[lane] = x - cnt;
  }
  __syncthreads();
  if (f) number[v] = (int32_t)(blk[blockIdx.x] + wbase[warp] + (uint32_t)__popc(bal & ((1u << lane) - 1u)));
}

__global__ void seg_labels_kernel(const int32_t* __restrict__ root, const int32_t* __restrict__ minpix,
                                  const int32_t* __restrict__ number, uint32_t n, int32_t* __restrict__ labels) {
  for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < n; v += (size_t)gridDim.x * blockDim.x)
    labels[v] = number[minpix[root[v]]];
}

// the roots' thresholds: 0 + k / |C| = k / |C| (singletons: k / 1)
__global__ void seg_forest_thr_kernel(const int32_t* __restrict__ parent, float k, uint32_t n,
                                      SetState* __restrict__ state) {
  for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < n; v += (size_t)gridDim.x * blockDim.x)
    state[v].thr = parent[v] == (int32_t)v ? __fdiv_rn(k, (float)state[v].size) : 0.0f;
}

}  // namespace

cudaError_t seg_graph_sorted(const uint8_t* hsv_host[3], const uint16_t* depth_host, const float* sal_host,
                             int32_t W, int32_t H, const float* mask, int len, float kdv, float kdc, float kx,
                             float ks, void* ws, int sms, cudaStream_t st, uint32_t* order_host,
                             int32_t* ea_host, int32_t* eb_host, float* w_host, uint32_t* err_host) {
  const uint64_t E = seg_num_edges(W, H);
  SegGraphDev g;
  cudaError_t e = seg_graph_device(hsv_host, depth_host, sal_host, W, H, mask, len, kdv, kdc, kx, ks, ws, sms, st, &g);
  if (e != cudaSuccess) return e;
  if (E > 0) {
    // the sorted order: the low 32 bits of each key; copy keys back whole
    std::vector<uint64_t> keys(E);
    if ((e = cudaMemcpyAsync(keys.data(), g.sorted, 8 * E, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(ea_host, g.ea, 4 * E, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(eb_host, g.eb, 4 * E, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(w_host, g.w, 4 * E, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(err_host, g.misc + 2, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    for (uint64_t i = 0; i < E; ++i) order_host[i] = (uint32_t)(keys[i] & 0xFFFFFFFFull);
  } else {
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    *err_host = 0;
  }
  return cudaSuccess;
}

// pinned layout: 64 bytes of words ([0] error bits, [1] zero-weight edges,
// [2] small-pass candidates, [3] sets, [8] the front stage's error word),
// the packed edges and their weights,
// then the forest after the zero-weight edges: parent, (size, threshold)
size_t seg_merge_pinned_bytes(int32_t W, int32_t H) {
  return 64 + 8 * (size_t)seg_num_edges(W, H) + 12 * (size_t)W * H;
}

namespace {

// The host's part of the merge, on the forest the GPU left after the
// weight-0 edges (parent, size and threshold at the roots, in pinned
// memory): segment_graph's pass over the remaining sorted edges, chunk by
// chunk as their copies land, then the small-component pass, then labels
// numbered by smallest pixel.  A threshold is only read at the current root
// of its set, so the partition does not depend on the union rule.
struct PinnedForest {
  int32_t* parent;
  SetState* st;
  int32_t find(int32_t x) {
    while (parent[x] != x) {
      parent[x] = parent[parent[x]];
      x = parent[x];
    }
    return x;
  }
  int32_t join(int32_t a, int32_t b) {  // roots; returns the new root
    if (st[a].size < st[b].size) std::swap(a, b);
    parent[b] = a;
    st[a].size += st[b].size;
    return a;
  }
};

// how far ahead (in edges) the host brings the ends' parent entries into
// cache, in both passes (on the GB300's Grace cores: 10-20% off the passes)
constexpr uint64_t kMergePrefetch = 16;

}  // namespace

// The graph stage with the merge passes streamed: the GPU sorts the edges,
// joins the weight-0 ones (their connected components), packs the rest
// (8 bytes each), and they come back in n_chunks copies into pinned host
// memory after the forest; the host runs segment_graph's pass over each
// chunk as soon as its copy has landed, then the small-component pass and
// the labels.  Same partition and numbering as seg_merge over the same
// sorted order.
cudaError_t seg_graph_merge(const uint8_t* hsv_host[3], const uint16_t* depth_host, const float* sal_host,
                            int32_t W, int32_t H, const float* mask, int len, float kdv, float kdc, float kx,
                            float ks, void* ws, int sms, cudaStream_t st, void* pinned, const cudaEvent_t* ev,
                            int n_chunks, float k, float min_size, int32_t* labels, uint32_t* n_sets,
                            uint32_t* err_host, int32_t* labels_dev) {
  const uint64_t E = seg_num_edges(W, H);
  const uint32_t n = (uint32_t)((size_t)W * H);
  SegGraphDev g;
  cudaError_t e = seg_graph_device(hsv_host, depth_host, sal_host, W, H, mask, len, kdv, kdc, kx, ks, ws, sms, st, &g);
  if (e != cudaSuccess) return e;
  uint32_t* h_words = reinterpret_cast<uint32_t*>(pinned);
  uint32_t* h_pk = reinterpret_cast<uint32_t*>(static_cast<char*>(pinned) + 64);
  float* h_pw = reinterpret_cast<float*>(h_pk + E);
  int32_t* h_par = reinterpret_cast<int32_t*>(h_pw + E);
  int32_t* d_par = reinterpret_cast<int32_t*>(g.tmp);  // the 12 n bytes of scratch: parent, then (size, threshold)
  SetState* d_state = reinterpret_cast<SetState*>(d_par + n);
  uint32_t* d_z = g.misc + 3;
  // the forest after the weight-0 edges, and the remaining edges packed
  if (E > 0) {
    seg_zero_count_kernel<<<grid_for(E, 256, sms), 256, 0, st>>>(g.sorted, (uint32_t)E, k >= 0.0f ? 1 : 0, d_z);
    if ((e = cudaMemcpyAsync(h_words, g.misc + 2, 8, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    if ((e = cudaEventRecord(ev[0], st)) != cudaSuccess) return e;
  }
  seg_forest_init_kernel<<<grid_for(n, 256, sms), 256, 0, st>>>(d_par, d_state, n);
  if (E > 0) seg_zero_link_kernel<<<grid_for(E, 256, sms), 256, 0, st>>>(g.sorted, g.ea, g.eb, d_z, d_par);
  seg_forest_flatten_kernel<<<grid_for(n, 256, sms), 256, 0, st>>>(d_par, d_state, n);
  seg_forest_thr_kernel<<<grid_for(n, 256, sms), 256, 0, st>>>(d_par, k, n, d_state);
  uint32_t* d_pk = reinterpret_cast<uint32_t*>(g.spare);
  float* d_pw = reinterpret_cast<float*>(d_pk + E);
  if (E > 0)
    seg_pack_kernel<<<grid_for(E, 256, sms), 256, 0, st>>>(g.sorted, g.ea, g.eb, g.w, (uint32_t)E, W, d_z, d_pk,
                                                           d_pw);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  uint64_t E2 = 0;  // edges after the weight-0 ones
  if (E > 0) {
    if ((e = cudaEventSynchronize(ev[0])) != cudaSuccess) return e;
    *err_host = h_words[0];
    if (*err_host) {  // let the caller report it; finish the work first
      if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
      return cudaSuccess;
    }
    E2 = E - h_words[1];
  } else {
    *err_host = 0;
  }
  SetState* h_state = reinterpret_cast<SetState*>(h_par + n);
  if ((e = cudaMemcpyAsync(h_par, d_par, 12 * (size_t)n, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
  const int chunks = E2 > 0 ? n_chunks : 0;
  for (int c = 0; c < chunks; ++c) {
    const uint64_t c0 = E2 * c / n_chunks, c1 = E2 * (c + 1) / n_chunks;
    if (c1 > c0) {
      if ((e = cudaMemcpyAsync(h_pk + c0, d_pk + c0, 4 * (c1 - c0), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return e;
      if ((e = cudaMemcpyAsync(h_pw + c0, d_pw + c0, 4 * (c1 - c0), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return e;
    }
    if ((e = cudaEventRecord(ev[c], st)) != cudaSuccess) return e;
  }
  if (chunks == 0 && (e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  const int32_t dstep[4] = {1, W, W + 1, 1 - W};
  PinnedForest f{h_par, h_state};
  for (int c = 0; c < chunks; ++c) {
    const uint64_t c0 = E2 * c / n_chunks, c1 = E2 * (c + 1) / n_chunks;
    if ((e = cudaEventSynchronize(ev[c])) != cudaSuccess) return e;  // chunk 0's event follows the forest too
    for (uint64_t i = c0; i < c1; ++i) {
      if (i + kMergePrefetch < c1) {  // within the chunk that has landed
        const uint32_t q = h_pk[i + kMergePrefetch];
        const int32_t qa = (int32_t)(q >> 2);
        __builtin_prefetch(h_par + qa, 1);
        __builtin_prefetch(h_par + qa + dstep[q & 3u], 1);
      }
      const uint32_t pk = h_pk[i];
      const int32_t a0 = (int32_t)(pk >> 2), b0 = a0 + dstep[pk & 3u];
      const float we = h_pw[i];
      const int32_t a = f.find(a0), b = f.find(b0);
      if (a == b || !(we <= f.st[a].thr && we <= f.st[b].thr)) continue;
      const int32_t r = f.join(a, b);
      f.st[r].thr = we + k / (float)f.st[r].size;
    }
  }
  // the small-component pass over the candidate edges, which the GPU lists
  // from the forest the first pass left
  uint64_t nc = 0;  // candidates
  if (E2 > 0) {
    const uint32_t nb = (uint32_t)((E2 + kCandThreads - 1) / kCandThreads);
    uint32_t* d_cand = reinterpret_cast<uint32_t*>(g.sorted);  // free after the packing: 8 E bytes
    // the block counts (E2 / 1024 + 2 <= n words) in the labels' buffer,
    // which the labels take only later
    uint32_t* d_blk = reinterpret_cast<uint32_t*>(g.lab);
    if ((e = cudaMemcpyAsync(d_par, h_par, 12 * (size_t)n, cudaMemcpyHostToDevice, st)) != cudaSuccess) return e;
    seg_forest_roots_kernel<<<grid_for(n, 256, sms), 256, 0, st>>>(d_par, n);
    seg_cand_count_kernel<<<nb, kCandThreads, 0, st>>>(d_pk, (uint32_t)E2, W, d_par, d_state, min_size, d_blk);
    seg_cand_scan_kernel<<<1, kCandThreads, 0, st>>>(d_blk, nb);
    seg_cand_scatter_kernel<<<nb, kCandThreads, 0, st>>>(d_pk, (uint32_t)E2, W, d_par, d_state, min_size, d_blk,
                                                          d_cand);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(h_words + 2, d_blk + nb, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    nc = h_words[2];
    if (nc > E2) return cudaErrorUnknown;  // cannot happen: at most every edge
    // the list lands where the packed edges were (the host is done with them)
    if (nc > 0 && (e = cudaMemcpyAsync(h_pk, d_cand, 4 * nc, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  }
  for (uint64_t i = 0; i < nc; ++i) {
    if (i + kMergePrefetch < nc) {
      const uint32_t q = h_pk[i + kMergePrefetch];
      const int32_t qa = (int32_t)(q >> 2);
      __builtin_prefetch(h_par + qa);
      __builtin_prefetch(h_par + qa + dstep[q & 3u]);
    }
    const uint32_t pk = h_pk[i];
    const int32_t a0 = (int32_t)(pk >> 2), b0 = a0 + dstep[pk & 3u];
    const int32_t a = f.find(a0), b = f.find(b0);
    if (a != b && ((float)f.st[a].size < min_size || (float)f.st[b].size < min_size)) f.join(a, b);
  }
  // the labels on the GPU, from the final forest: roots, each set's
  // smallest pixel, the sets numbered in the order of those pixels
  {
    int32_t* d_minpix = reinterpret_cast<int32_t*>(d_state);  // the records' 8 n bytes are free now
    int32_t* d_number = d_minpix + n;
    int32_t* d_lab = labels_dev ? labels_dev : g.lab;
    uint32_t* d_blk = g.lblk;
    const uint32_t nb = (n + kCandThreads - 1) / kCandThreads;
    if ((e = cudaMemcpyAsync(d_par, h_par, 4 * (size_t)n, cudaMemcpyHostToDevice, st)) != cudaSuccess) return e;
    seg_forest_roots_kernel<<<grid_for(n, 256, sms), 256, 0, st>>>(d_par, n);
    seg_minpix_init_kernel<<<grid_for(n, 256, sms), 256, 0, st>>>(d_minpix, n);
    seg_minpix_kernel<<<grid_for(n, 256, sms), 256, 0, st>>>(d_par, d_minpix, n);
    seg_first_count_kernel<<<nb, kCandThreads, 0, st>>>(d_par, d_minpix, n, d_blk);
    seg_cand_scan_kernel<<<1, kCandThreads, 0, st>>>(d_blk, nb);
    seg_first_number_kernel<<<nb, kCandThreads, 0, st>>>(d_par, d_minpix, n, d_blk, d_number);
    seg_labels_kernel<<<grid_for(n, 256, sms), 256, 0, st>>>(d_par, d_minpix, d_number, n, d_lab);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(labels, d_lab, 4 * (size_t)n, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(h_words + 3, d_blk + nb, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    *n_sets = h_words[3];
  }
  return cudaSuccess;
}

}  // namespace qpso
