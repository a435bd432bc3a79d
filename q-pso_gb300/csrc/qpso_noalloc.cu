// qpso_noalloc.cu -- pose scoring that allocates nothing.
//
// Some callers cannot let a library call cudaMalloc: a host application that
// owns all device memory through its own pool or caching allocator with a
// fixed budget (a foreign cudaMalloc breaks its accounting and can fail when
// the pool holds the memory), or a real-time control loop (grasping, visual
// servoing) where cudaMalloc's implicit device synchronisation and
// unbounded latency are not acceptable in the loop.  qpso_score_poses_noalloc
// serves them: the caller passes device pointers it already owns for the
// inputs and the outputs, and every intermediate buffer (the cluster-masked
// observed depth, its summed-area table, the instance record and its
// counters) lives in one file-scope device array of fixed size, so the call
// makes no allocation, no host<->device copy and no synchronisation.
//
// Limits and sharing: the array holds kNoallocScratchBytes (4 MiB), enough
// for frames up to about 690,000 pixels (640x480 and 960x720 fit); larger
// frames are rejected with QPSO_ERR_ARG.  Every GPU that loads the library
// holds the array until the process exits.  All calls on a device share it
// and it keeps the last call's contents, so each call rewrites every word it
// reads (records, counters, masked depth, summed-area table) before use, and
// two calls whose work overlaps on the GPU (different streams, or different
// host threads) race on it: serialise them on one stream.
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <cstring>

#include "qpso.h"
#include "qpso_checks.h"
#include "qpso_internal.cuh"

using namespace qpso;

namespace {

constexpr size_t kNoallocScratchBytes = 4u << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

// Device address of g_noalloc_scratch in the current device's context.  In
// host code the symbol name is only a host-side stand-in, so the address
// comes from cudaGetSymbolAddress with the device current.  It is looked up
// on every call (a host-side table lookup, no device work): a cached address
// would outlive the module it points into after cudaDeviceReset or a switch
// to another context on the same device.
cudaError_t scratch_address(unsigned char** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return e;
  *out = static_cast<unsigned char*>(p);
  return cudaSuccess;
}

size_t up256(size_t x) { return (x + 255) / 256 * 256; }

struct Header {
  float gbest[8];
  uint32_t done;
  uint32_t err;
  unsigned long long stats[2];
};

}  // namespace

extern "C" qpso_status qpso_score_poses_noalloc(const float* d_mesh_soa, uint32_t num_faces,
                                                const uint16_t* d_depth_mm, const int32_t* d_labels,
                                                const qpso_camera* cam, const qpso_solve_desc* desc,
                                                const float* d_poses, uint32_t n, float* d_fit_out,
                                                uint32_t* d_flags_out, void* stream) {
  if (!d_mesh_soa || num_faces == 0 || !d_depth_mm || !cam || !desc || !d_poses || !d_fit_out ||
      n == 0)
    return QPSO_ERR_ARG;
  // the same checks as qpso_frame_upload (camera) and qpso_score_poses (cluster fields)
  if (camera_error(*cam) || cluster_error(*desc, cam->width, cam->height)) return QPSO_ERR_ARG;
  if (desc->cluster_label >= 0 && !d_labels) return QPSO_ERR_ARG;
  const size_t w = (size_t)cam->width, h = (size_t)cam->height;
  // scratch layout: instance | prep job | header | masked depth | table
  const size_t o_inst = 0;
  const size_t o_prep = up256(o_inst + sizeof(Instance));
  const size_t o_hdr = up256(o_prep + sizeof(PrepDesc));
  const size_t o_obs = up256(o_hdr + sizeof(Header));
  const size_t o_sat = up256(o_obs + w * h * sizeof(uint16_t));
  const size_t need = o_sat + (w + 1) * (h + 1) * sizeof(int32_t);
  if (need > kNoallocScratchBytes) return QPSO_ERR_ARG;  // frame too large for the fixed scratch

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return QPSO_ERR_CUDA;
  unsigned char* base = nullptr;
  if (scratch_address(&base) != cudaSuccess) return QPSO_ERR_CUDA;
  cudaStream_t st = static_cast<cudaStream_t>(stream);

  Instance I;
  std::memset(&I, 0, sizeof(I));
  I.mesh = d_mesh_soa;
  I.F = num_faces;
  I.obs = reinterpret_cast<const uint16_t*>(base + o_obs);
  I.sat = reinterpret_cast<const int32_t*>(base + o_sat);
  I.cam = Camera{cam->fx, cam->fy, cam->cx, cam->cy, cam->width, cam->height, cam->projection};
  SolveParams& p = I.prm;
  p.c1 = desc->c1;
  p.c2 = desc->c2;
  p.w = desc->w;
  p.vdot = desc->vdot;
  p.ang_lo = desc->ang_lo;
  p.ang_hi = desc->ang_hi;
  for (int k = 0; k < 4; ++k) p.qinit[k] = desc->qinit[k];
  for (int k = 0; k < 3; ++k) {
    p.t_lo[k] = desc->t_lo[k];
    p.t_hi[k] = desc->t_hi[k];
  }
  p.cl_min_x = desc->cl_min_x;
  p.cl_max_x = desc->cl_max_x;
  p.cl_min_y = desc->cl_min_y;
  p.cl_max_y = desc->cl_max_y;
  p.num_points = desc->num_points;
  p.num_particles = n;
  p.iterations = 1;
  p.seed = desc->seed;
  p.stream = desc->stream;
  p.raster_mode = desc->raster_mode;
  I.gbest = reinterpret_cast<float*>(base + o_hdr + offsetof(Header, gbest));
  I.done = reinterpret_cast<uint32_t*>(base + o_hdr + offsetof(Header, done));
  I.err = reinterpret_cast<uint32_t*>(base + o_hdr + offsetof(Header, err));
  I.stats = reinterpret_cast<unsigned long long*>(base + o_hdr + offsetof(Header, stats));
  I.chunks = n;
  I.ppb = 1;
  PrepDesc J;
  J.depth = d_depth_mm;
  J.labels = desc->cluster_label >= 0 ? d_labels : nullptr;
  J.label = desc->cluster_label;
  J.width = cam->width;
  J.height = cam->height;
  J.obs = reinterpret_cast<uint16_t*>(base + o_obs);
  J.sat = reinterpret_cast<int32_t*>(base + o_sat);

  static_assert(offsetof(Instance, mesh_hi) == offsetof(Instance, mesh_lo) + 3 * sizeof(float),
                "mesh box must be 6 consecutive floats");
  Instance* di = reinterpret_cast<Instance*>(base + o_inst);
  PrepDesc* dj = reinterpret_cast<PrepDesc*>(base + o_prep);
  float* dbox = reinterpret_cast<float*>(base + o_inst + offsetof(Instance, mesh_lo));
  const uint32_t* derr = reinterpret_cast<const uint32_t*>(base + o_hdr + offsetof(Header, err));
  const TileConfig cfg{256, 16384, 1};
  int nsm = 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return QPSO_ERR_CUDA;
  cudaError_t e = launch_noalloc_init(I, J, di, dj, st);
  if (e == cudaSuccess) e = launch_mesh_aabb(d_mesh_soa, num_faces, dbox, st);
  if (e == cudaSuccess) e = launch_prep(dj, 1, cam->width, cam->height, st);
  if (e == cudaSuccess) {
    const int grid = (int)(n < (uint32_t)nsm * 4 ? n : (uint32_t)nsm * 4);
    e = launch_score(di, d_poses, n, d_fit_out, cfg, grid, st);
  }
  if (e == cudaSuccess && d_flags_out) e = launch_copy_flags(derr, d_flags_out, st);
  return e == cudaSuccess ? QPSO_OK : QPSO_ERR_CUDA;
}
