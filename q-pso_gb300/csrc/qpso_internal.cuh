// qpso_internal.cuh -- device-resident instance layout shared by the kernels
// (qpso_kernels.cu) and the host runtime (qpso_api.cu).
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "meshlets.h"
#include "qpso.h"
#include "qpso_device.cuh"

namespace qpso {

// Error bits reported through Instance::err.
enum : uint32_t {
  kErrBound = 1u << 0,     // a face wrote outside its conservative tile bound
  kErrTimeout = 1u << 1,   // a bounded inter-CTA wait gave up
  kErrArg = 1u << 2,       // bad launch arguments detected on the device
};

// One solve instance as the kernels see it (one cluster x mesh x swarm).
// Particle state is SoA [7][P] (index p + d*P), like main.cu:1389-1465.
struct Instance {
  const float* mesh;        // loadOBJ3 layout, 9*F floats (main.h:620-679)
  uint32_t F;
  const MeshletHdr* mlets;  // meshlets of the same faces (the fused kernels read these)
  const unsigned char* mlet_blob;
  const float4* mlet_box;   // per meshlet: object-space lo, hi (2 float4)
  uint32_t n_mlets;
  float mesh_lo[3], mesh_hi[3];
  const uint16_t* obs;      // cluster-masked observed depth (mm), width*height
  const int32_t* sat;       // (height+1) x (width+1) counts of obs != 0
  Camera cam;
  SolveParams prm;
  float* pos;
  float* vel;
  float* pbest;
  float* pbest_fit;         // [P]
  float* fit;               // [P] fitness of the current iteration
  float* gbest;             // [8]: fitness, pose[7]
  uint32_t* done;           // CTAs finished in the current iteration
  uint32_t* err;            // error bits
  unsigned long long* stats;  // [0] raster pixel writes, [1] tile passes
  unsigned long long* argkey;  // smallest (fitness bits << 32 | particle) of the iteration
  float* trace;             // optional [iterations][8] gbest after each iteration
  uint32_t chunks;          // CTAs (work items) per iteration
  uint32_t ppb;             // particles per work item
  uint32_t cur_iter;        // serving: next iteration to run (advanced by the last CTA)
};

// Launch-shape knobs chosen by the tuner.
struct TileConfig {
  int threads;      // CTA size
  int tile_px;      // int32 depth tile capacity (pixels); a multiple of 8
  int ppb;          // particles per work item
};

// Per-instance preparation job: mask the frame to the cluster and build
// the summed-area table of observed pixels.
struct PrepDesc {
  const uint16_t* depth;
  const int32_t* labels;    // nullable: depth is already masked
  int32_t label;
  int32_t width, height;
  uint16_t* obs;
  int32_t* sat;
};

// Entry of the batched kernel's work queue: iteration `iter` of instance
// `inst`.  CTAs claim its chunks through `next` once `ready` is set; the CTA
// that completes the iteration appends the instance's next iteration.
struct QEntry {
  uint32_t inst;
  uint32_t iter;
  uint32_t next;   // chunks claimed so far
  uint32_t ready;  // set (after inst and iter) when the entry may be claimed
};

// Head and tail of the batched kernel's work queue.
struct QCtl {
  uint32_t head;   // first entry with unclaimed chunks
  uint32_t tail;   // next free entry
  uint32_t total;  // entries: the instances' iterations
  uint32_t pad;
};

struct BatchArgs {
  Instance* inst;           // device array of instances
  QEntry* queue;            // [total]: iteration 0 of every instance, most expensive first, then appended
  QCtl* qctl;
  uint32_t* err;            // batch-level error bits (zeroed)
  unsigned long long timeout_ns;  // limit of one wait for work
};

// Host-side launch wrappers (defined in qpso_kernels.cu).
cudaError_t launch_prep(const PrepDesc* jobs, int n, int max_w, int max_h, cudaStream_t st);
cudaError_t launch_mesh_aabb(const float* mesh, uint32_t F, float* out, cudaStream_t st);
// `var`: the fused-kernel variant the launch needs, the largest over its
// solves: 0 = REF raster and fp32 projection only, 1 = the EDGE raster too
// (some solve is in QPSO_RASTER_EDGE mode), 2 = the reference projection too
// (some frame uses QPSO_PROJ_REF_ACCV).  `vcap`: the largest meshlet
// (vertices) of the launch's meshes, which sizes the per-warp vertex caches.
cudaError_t launch_step(const Instance* inst, uint32_t iter, uint32_t chunks, const TileConfig& cfg,
                        cudaStream_t st, int var, int vcap);
cudaError_t launch_batch(const BatchArgs& args, int grid, const TileConfig& cfg, cudaStream_t st, int var,
                         int vcap);
cudaError_t batch_max_grid(const TileConfig& cfg, int var, int vcap, int* blocks_per_sm);
int tile_for_occupancy(int threads, int ppb, int vcap, int per_sm, bool batched, int var);
cudaError_t launch_score(const Instance* inst, const float* poses, uint32_t n, float* fit_out,
                         const TileConfig& cfg, int grid, cudaStream_t st);
cudaError_t launch_score_mlets(const Instance* inst, const float* poses, uint32_t n, float* fit_out,
                               const TileConfig& cfg, int grid, cudaStream_t st, int var, int vcap);
// Dynamic shared memory of the fused kernels; vcap: vertex cache slots per
// warp, the largest meshlet of the launch's meshes (meshlet_cap()).
size_t fused_smem_bytes(int threads, int ppb, int tile_px, int vcap);
// qpso_refine's pattern search, one copy for the host and the device: every
// float operation is +, -, *, / or sqrt in a fixed order (the device build
// contracts nothing, the host unit is compiled without contraction), so the
// oracle replays it bit for bit.
//
// splitmix64 (Steele, Lea and Flood; the public-domain generator Vigna
// recommends for seeding).  Draw n (0-based) of a stream seeded with s is
// splitmix64_out(s + (n + 1) * kSplitmixGamma): any draw can be reached
// directly.
constexpr uint64_t kSplitmixGamma = 0x9E3779B97F4A7C15ull;
__host__ __device__ inline uint64_t splitmix64_out(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
// a uniform float in [-1, 1): 24 random bits, exact in float
__host__ __device__ inline float uniform_pm1(uint64_t& state) {
  state += kSplitmixGamma;
  const float u = (float)(splitmix64_out(state) >> 40) * 5.9604644775390625e-8f;  // 2^-24
  return u * 2.0f - 1.0f;
}
// q <- normalise(dq * q), dq = (1, hx, hy, hz), then the top hemisphere
__host__ __device__ inline void rotate_small(float q[4], float hx, float hy, float hz) {
  const float a0 = 1.0f, a1 = hx, a2 = hy, a3 = hz;
  const float b0 = q[0], b1 = q[1], b2 = q[2], b3 = q[3];
  float r[4];
  r[0] = a0 * b0 - a1 * b1 - a2 * b2 - a3 * b3;
  r[1] = a0 * b1 + a1 * b0 + a2 * b3 - a3 * b2;
  r[2] = a0 * b2 - a1 * b3 + a2 * b0 + a3 * b1;
  r[3] = a0 * b3 + a1 * b2 - a2 * b1 + a3 * b0;
  const float n = sqrtf(r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + r[3] * r[3]);
  const float sgn = r[0] < 0.0f ? -1.0f : 1.0f;
  for (int k = 0; k < 4; ++k) q[k] = sgn * (r[k] / n);
}
// Candidate i of a round (K per round): the pose stepped by +-step_t along
// one axis (i < 6), rotated by about +-step_r about one axis (i < 12), or
// moved at random within the steps, from draw `draw0` of the stream on.
__host__ __device__ inline void refine_candidate(const float pose[7], uint32_t i, float step_t, float step_r,
                                                 uint64_t rng_seed, uint64_t draw0, float c[7]) {
  for (int k = 0; k < 7; ++k) c[k] = pose[k];
  if (i < 6) {
    c[i / 2] = c[i / 2] + ((i & 1) ? -step_t : step_t);
  } else if (i < 12) {
    float h[3] = {0.0f, 0.0f, 0.0f};
    h[(i - 6) / 2] = ((i & 1) ? -step_r : step_r) * 0.5f;
    rotate_small(c + 3, h[0], h[1], h[2]);
  } else {
    uint64_t state = rng_seed + draw0 * kSplitmixGamma;
    for (int k = 0; k < 3; ++k) c[k] = c[k] + uniform_pm1(state) * step_t;
    float h[3];
    for (int k = 0; k < 3; ++k) h[k] = uniform_pm1(state) * step_r * 0.5f;
    rotate_small(c + 3, h[0], h[1], h[2]);
  }
}
// The search's state in device memory: the current pose, its fitness, the
// two steps, the stream's seed and the round.
struct RefineState {
  float pose[7];
  float fit;
  float step_t, step_r;
  uint32_t round, K;
  uint64_t rng_seed;
};
// one round: K candidates around the state's pose; then the first smallest
// fitness replaces the pose when it is lower, else both steps halve
cudaError_t launch_refine_gen(const RefineState* st, float* cand, uint32_t K, cudaStream_t s);
cudaError_t launch_refine_pick(RefineState* st, const float* cand, const float* fits, uint32_t K, cudaStream_t s);

cudaError_t launch_render_window(const Instance* inst, const float* pose, int32_t x0, int32_t y0,
                                 int32_t w, int32_t h, int32_t* out, int32_t* box, int threads,
                                 cudaStream_t st);
cudaError_t launch_queue_probe(QCtl* qctl, QEntry* queue, uint32_t* err, uint32_t grid,
                               unsigned long long timeout_ns, cudaStream_t st);
// Serving epoch: the dataflow queue of the batched kernel over the active
// requests (args.inst = the slot records), request i running its
// iterations up to end_iter[i] (device array), one cooperative launch.
cudaError_t epoch_max_grid(const TileConfig& cfg, int var, int vcap, int* blocks_per_sm);
cudaError_t launch_epoch(const BatchArgs& args, const uint32_t* end_iter, int grid, const TileConfig& cfg,
                         cudaStream_t st, int var, int vcap);
cudaError_t launch_noalloc_init(const Instance& I, const PrepDesc& J, Instance* di, PrepDesc* dj,
                                cudaStream_t st);
cudaError_t launch_copy_flags(const uint32_t* src, uint32_t* dst, cudaStream_t st);
size_t smem_ctl_bytes();
// Per-label accumulators of a label map (cluster records).
struct ClusterAcc {
  unsigned long long sum_z, sum_xz, sum_yz;
  uint32_t n, nz;
  int32_t minx, maxx, miny, maxy;
};
cudaError_t launch_label_max(const int32_t* labels, uint32_t n, int32_t* out, cudaStream_t st);
cudaError_t launch_cluster_stats(const uint16_t* depth, const int32_t* labels, int32_t W, int32_t H,
                                 ClusterAcc* acc, int32_t nlab, cudaStream_t st);
// Float depth image of one pose with the arithmetic of the reference's host
// render (RenderCPU); out: width*height floats on the device.
cudaError_t launch_host_render(const float* mesh, uint32_t F, const float pose[7], const Camera& cam,
                               float* out, cudaStream_t st);

// Graph stage of the segmentation (qpso_segment.cu).  seg_num_edges: edges
// of the W x H pixel graph; seg_gauss_mask: the smoothing mask (length, or
// -1 above capacity); seg_edge_ends: every edge's ends in the reference's
// order; seg_merge: the merge passes over edges in the given order and the
// labels numbered by each set's smallest pixel (returns the set count);
// seg_graph_sorted: upload, smoothing, depth range, edge weights and the
// radix sort on the GPU, then the sorted order, the edges' ends and weights
// (in edge order) and the kernels' error bits back on the host
// (1 and 4: an index out of range, 2: a NaN weight).
uint64_t seg_num_edges(int32_t W, int32_t H);
int seg_gauss_mask(float sigma, float* mask, int capacity);
void seg_edge_ends(int32_t W, int32_t H, int32_t* a, int32_t* b);
uint32_t seg_merge(uint32_t n_pixels, uint64_t n_edges, const uint32_t* order, const int32_t* ea,
                   const int32_t* eb, const float* w, float k, float min_size, int32_t* labels);
size_t seg_workspace_bytes(int32_t W, int32_t H);
cudaError_t seg_graph_sorted(const uint8_t* hsv_host[3], const uint16_t* depth_host, const float* sal_host,
                             int32_t W, int32_t H, const float* mask, int len, float kdv, float kdc, float kx,
                             float ks, void* ws, int sms, cudaStream_t st, uint32_t* order_host,
                             int32_t* ea_host, int32_t* eb_host, float* w_host, uint32_t* err_host);

// The stages around the graph stage (qpso_seg_front.cu): colour
// conversions, depth smoothing, inpainting and Canny saliency, from host
// BGR and raw depth to device planes in the graph stage's input slots.
struct SegFrontArgs {
  const uint8_t* bgr_host;   // W x H x 3, B G R
  const uint16_t* depth_host;
  int32_t W, H;
  float beta, gamma;
  int32_t radius;            // inpainting radius (shrunk map, px)
  float canny_low, canny_high;
  int32_t dth, plus_d, point_3d;
  float g_angle, l_angle;
  float fx, fy, cx, cy;
  uint8_t* hsv_out;          // device: H, S, V planes (3 W H)
  uint16_t* inpainted_out;   // device: W H
  float* saliency_out;       // device: W H
  uint8_t* gray_host;        // optional host copies
  uint16_t* smoothed_host;
  uint8_t* edges_host;
  uint32_t* err_pinned;      // optional pinned word: nonzero when the inpainting fill's grid barrier expired
};
int seg_gauss_taps(int ksize, int32_t* taps);
size_t seg_front_workspace_bytes(int32_t W, int32_t H, int32_t radius);
cudaError_t seg_front_run(const SegFrontArgs& a, void* ws, int sms, size_t smem_optin, cudaStream_t st);

// Per-set moments of a label map for the cluster filter (PostSegmFilter).
struct SetMoments {
  unsigned long long n, sx, sy, sxx, syy, sxy, nz, sz, suz, svz, nzero, vb[3];
  int32_t minx, maxx, miny, maxy;
};
cudaError_t launch_set_moments(const int32_t* labels, const uint16_t* inp, const uint8_t* v8, int32_t W, int32_t H,
                               int32_t n_sets, SetMoments* acc, int sms, cudaStream_t st);
// The graph stage with the merge passes streamed over packed sorted edges
// copied back in n_chunks pieces (pinned: seg_merge_pinned_bytes; ev:
// n_chunks events); labels numbered by smallest pixel, into host memory
// and, when labels_dev is not null, into that device buffer too.
size_t seg_merge_pinned_bytes(int32_t W, int32_t H);
cudaError_t seg_graph_merge(const uint8_t* hsv_host[3], const uint16_t* depth_host, const float* sal_host,
                            int32_t W, int32_t H, const float* mask, int len, float kdv, float kdc, float kx,
                            float ks, void* ws, int sms, cudaStream_t st, void* pinned, const cudaEvent_t* ev,
                            int n_chunks, float k, float min_size, int32_t* labels, uint32_t* n_sets,
                            uint32_t* err_host, int32_t* labels_dev);
// the graph stage's device input slots inside its workspace
void seg_ws_inputs(void* ws, int32_t W, int32_t H, uint8_t** hsv, uint16_t** depth, float** sal);
// PostSegmFilter's record of one set from its moments (host).
void seg_cluster_record(const SetMoments& m, int32_t label, const qpso_seg_front_params& fp, qpso_seg_cluster* r);

}  // namespace qpso
