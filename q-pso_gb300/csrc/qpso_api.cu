// qpso_api.cu -- host runtime behind the C ABI of include/qpso.h.
//
// The reference's host program (main.cu:1301-1780) allocates a 1.26 GB
// per-particle render buffer, 16 streams and ~2k launches per iteration.
// This runtime keeps meshes and frames resident behind integer ids, lays
// every solve's state out in one grow-only device workspace, stages its
// metadata through one pinned buffer (one H2D copy, one D2H copy per solve)
// and runs the fused kernels of qpso_kernels.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <thread>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "meshlets.h"
#include "qpso.h"
#include "qpso_checks.h"
#include "qpso_internal.cuh"

using namespace qpso;

namespace {

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

struct MeshObj {
  float* d = nullptr;
  uint32_t F = 0;
  float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  MeshletHdr* mlets = nullptr;       // device
  unsigned char* blob = nullptr;     // device
  uint32_t n_mlets = 0;
  size_t box_off = 0;                // per-meshlet boxes, bytes into blob
  int mlet_cap = kMletVerts;         // meshlet size (faces, vertices) of this mesh
};

struct FrameObj {
  uint16_t* depth = nullptr;
  int32_t* labels = nullptr;
  qpso_camera cam{};
};

struct Buf {
  void* p = nullptr;
  size_t cap = 0;
};

// Offsets of one solve batch inside the device workspace and the pinned
// staging buffer.  The metadata block (instances, headers, prep jobs, the
// work queue's first entries and its head/tail) is contiguous so that one
// copy uploads it.
struct Header {  // per instance, 64 bytes: result + counters read back once
  float gbest[8];
  uint32_t done;
  uint32_t err;
  unsigned long long stats[2];
  unsigned long long argkey;  // the iteration's smallest (fitness bits, particle) key; all ones between iterations
};
static_assert(sizeof(Header) == 64, "header layout");

struct Layout {
  // qinit / qctl: the batched kernel's first queue entries and head/tail
  // (uploaded with the metadata); queue: its whole work queue (device only)
  size_t inst = 0, hdr = 0, prep = 0, qinit = 0, qctl = 0, berr = 0, meta_end = 0, queue = 0;
  size_t total = 0;
  std::vector<size_t> obs, sat, pos, vel, pbest, pbf, fit, trace;
};

}  // namespace

struct qpso_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  int num_sms = 0;
  int smem_optin = 0;
  std::string err;
  std::unordered_map<uint32_t, MeshObj> meshes;
  std::unordered_map<uint32_t, FrameObj> frames;
  uint32_t next_id = 1;
  TileConfig plain{256, 16384, 1};
  TileConfig batch{256, 16384, 1};
  Buf ws;    // device workspace
  Buf pin;   // pinned host staging
  // batched-launch graph cache
  cudaGraphExec_t gexec = nullptr;
  std::vector<uint64_t> gkey;
  // device-time accounting
  bool profiling = false;
  std::vector<cudaEvent_t> ev;   // pool of timing events
  cudaEvent_t gev[2] = {nullptr, nullptr};  // around the batched kernel in the graph
  qpso_profile prof{};
  cudaEvent_t timers[64] = {};
  Buf scrub;
  // segmentation: pinned landing buffer of the sorted edges and the events
  // that mark its chunks
  Buf segpin;
  cudaEvent_t seg_ev[8] = {};
  std::mutex mu;
};

namespace {

qpso_status fail(qpso_context* ctx, qpso_status st, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return st;
}

qpso_status cuda_fail(qpso_context* ctx, cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  return fail(ctx, e == cudaErrorMemoryAllocation ? QPSO_ERR_NOMEM : QPSO_ERR_CUDA, m);
}

#define QPSO_CUDA(ctx, call)                                  \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return cuda_fail((ctx), e_, #call); \
  } while (0)

qpso_status ensure_ws(qpso_context* ctx, size_t bytes) {
  if (bytes <= ctx->ws.cap) return QPSO_OK;
  if (ctx->ws.p) {
    QPSO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    cudaFree(ctx->ws.p);
    ctx->ws.p = nullptr;
    ctx->ws.cap = 0;
  }
  const size_t cap = align_up(bytes + bytes / 4, 1 << 20);
  QPSO_CUDA(ctx, cudaMalloc(&ctx->ws.p, cap));
  ctx->ws.cap = cap;
  return QPSO_OK;
}

qpso_status ensure_pin(qpso_context* ctx, size_t bytes) {
  if (bytes <= ctx->pin.cap) return QPSO_OK;
  if (ctx->pin.p) {
    QPSO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    cudaFreeHost(ctx->pin.p);
    ctx->pin.p = nullptr;
    ctx->pin.cap = 0;
  }
  const size_t cap = align_up(bytes + bytes / 4, 1 << 16);
  QPSO_CUDA(ctx, cudaMallocHost(&ctx->pin.p, cap));
  ctx->pin.cap = cap;
  return QPSO_OK;
}

constexpr int kSegChunks = 8;

// pinned buffer and chunk events of the streamed segmentation merge
qpso_status ensure_segpin(qpso_context* ctx, size_t bytes) {
  for (int i = 0; i < kSegChunks; ++i)
    if (!ctx->seg_ev[i]) QPSO_CUDA(ctx, cudaEventCreateWithFlags(&ctx->seg_ev[i], cudaEventDisableTiming));
  if (bytes <= ctx->segpin.cap) return QPSO_OK;
  if (ctx->segpin.p) {
    QPSO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    cudaFreeHost(ctx->segpin.p);
    ctx->segpin.p = nullptr;
    ctx->segpin.cap = 0;
  }
  const size_t cap = align_up(bytes, 1 << 16);
  QPSO_CUDA(ctx, cudaMallocHost(&ctx->segpin.p, cap));
  ctx->segpin.cap = cap;
  return QPSO_OK;
}

qpso_status ensure_events(qpso_context* ctx, size_t n) {
  while (ctx->ev.size() < n) {
    cudaEvent_t e;
    QPSO_CUDA(ctx, cudaEventCreate(&e));
    ctx->ev.push_back(e);
  }
  return QPSO_OK;
}

// Sum the device time between event pairs (2i, 2i+1), i < pairs.
double event_pairs_ms(qpso_context* ctx, size_t pairs) {
  double ms = 0.0;
  for (size_t i = 0; i < pairs; ++i) {
    float t = 0.f;
    if (cudaEventElapsedTime(&t, ctx->ev[2 * i], ctx->ev[2 * i + 1]) == cudaSuccess) ms += t;
  }
  return ms;
}

// A launch shape is valid when its shared memory fits a CTA for meshlets of
// vcap vertices (set_launch_config checks the smallest, 64; a launch checks
// its meshes' own with fits_smem).
bool valid_cfg(const qpso_launch_config& c, int smem_optin, int vcap = 64) {
  return c.threads >= 32 && c.threads <= 1024 && c.threads % 32 == 0 && c.tile_px >= 64 &&
         c.tile_px % 8 == 0 && c.ppb >= 1 && c.ppb <= 16 && c.threads >= 8 * c.ppb &&
         fused_smem_bytes(c.threads, c.ppb, c.tile_px, vcap) <= (size_t)smem_optin;
}

int launch_vcap(const std::vector<const MeshObj*>& ms) {
  int v = 64;
  for (const MeshObj* m : ms) v = std::max(v, m->mlet_cap);
  return v;
}

// The launch shape a launch uses: the installed one, or, when meshes above
// 16384 faces (128-vertex meshlets, larger vertex caches) push its shared
// memory past the CTA limit, the same shape with the tile halved (then the
// threads halved) until it fits.  Results do not depend on the shape; the
// particles per work item stay, so work items and chunks do too.
bool shrink_cfg(TileConfig& cfg, int vcap, int smem_optin) {
  while (fused_smem_bytes(cfg.threads, cfg.ppb, cfg.tile_px, vcap) > (size_t)smem_optin) {
    if (cfg.tile_px >= 2 * 1024) {
      cfg.tile_px = cfg.tile_px / 16 * 8;
    } else if (cfg.threads / 2 >= std::max(32, 8 * cfg.ppb) && cfg.threads % 64 == 0) {
      cfg.threads /= 2;
    } else {
      return false;
    }
  }
  return true;
}

qpso_status fit_cfg(qpso_context* ctx, TileConfig& cfg, int vcap) {
  if (!shrink_cfg(cfg, vcap, ctx->smem_optin))
    return fail(ctx, QPSO_ERR_ARG, "launch config cannot fit the meshes' vertex caches");
  return QPSO_OK;
}

// The fused-kernel variant a solve needs (the launch takes the largest):
// 2 for a frame in the reference projection, 1 for the EDGE raster, else 0.
int kernel_variant(const qpso_solve_desc& d, const qpso_camera& c) {
  if (c.projection == QPSO_PROJ_REF_ACCV) return 2;
  return d.raster_mode == QPSO_RASTER_EDGE ? 1 : 0;
}

bool projection_ok(const qpso_camera* cam) {
  return cam->projection == QPSO_PROJ_FP32 || cam->projection == QPSO_PROJ_REF_ACCV;
}

// The intrinsics a camera projects with: its fields, or the reference's
// ACCV values (main.h:30-33).
void camera_intrinsics(const qpso_camera& c, double k[4]) {
  if (c.projection == QPSO_PROJ_REF_ACCV) {
    k[0] = 572.41140;
    k[1] = 573.57043;
    k[2] = 325.26110;
    k[3] = 242.04899;
  } else {
    k[0] = c.fx;
    k[1] = c.fy;
    k[2] = c.cx;
    k[3] = c.cy;
  }
}

qpso_status check_desc(qpso_context* ctx, const qpso_solve_desc& d, const MeshObj** m,
                       const FrameObj** f) {
  auto mi = ctx->meshes.find(d.mesh_id);
  if (mi == ctx->meshes.end()) return fail(ctx, QPSO_ERR_NOT_FOUND, "unknown mesh id");
  auto fi = ctx->frames.find(d.frame_id);
  if (fi == ctx->frames.end()) return fail(ctx, QPSO_ERR_NOT_FOUND, "unknown frame id");
  if (d.num_particles == 0 || d.num_particles > (1u << 20))
    return fail(ctx, QPSO_ERR_ARG, "num_particles must be in [1, 2^20]");
  if (d.iterations == 0 || d.iterations > (1u << 20))
    return fail(ctx, QPSO_ERR_ARG, "iterations must be in [1, 2^20]");
  const qpso_camera& c = fi->second.cam;
  if (const char* why = cluster_error(d, c.width, c.height)) return fail(ctx, QPSO_ERR_ARG, why);
  if (d.cluster_label >= 0 && fi->second.labels == nullptr)
    return fail(ctx, QPSO_ERR_ARG, "frame has no label map");
  for (int k = 0; k < 3; ++k)
    if (!(d.t_lo[k] <= d.t_hi[k])) return fail(ctx, QPSO_ERR_ARG, "t_lo must be <= t_hi");
  *m = &mi->second;
  *f = &fi->second;
  return QPSO_OK;
}

SolveParams to_params(const qpso_solve_desc& d) {
  SolveParams p;
  p.c1 = d.c1;
  p.c2 = d.c2;
  p.w = d.w;
  p.vdot = d.vdot;
  p.ang_lo = d.ang_lo;
  p.ang_hi = d.ang_hi;
  for (int k = 0; k < 4; ++k) p.qinit[k] = d.qinit[k];
  for (int k = 0; k < 3; ++k) {
    p.t_lo[k] = d.t_lo[k];
    p.t_hi[k] = d.t_hi[k];
  }
  p.cl_min_x = d.cl_min_x;
  p.cl_max_x = d.cl_max_x;
  p.cl_min_y = d.cl_min_y;
  p.cl_max_y = d.cl_max_y;
  p.num_points = d.num_points;
  p.num_particles = d.num_particles;
  p.iterations = d.iterations;
  p.seed = d.seed;
  p.stream = d.stream;
  p.raster_mode = d.raster_mode;
  return p;
}

Layout make_layout(const std::vector<const qpso_solve_desc*>& ds,
                   const std::vector<const FrameObj*>& frames, uint32_t q_entries, bool trace) {
  Layout L;
  const size_t n = ds.size();
  size_t o = 0;
  L.inst = o;
  o = align_up(o + n * sizeof(Instance), 256);
  L.hdr = o;
  o = align_up(o + n * sizeof(Header), 256);
  L.prep = o;
  o = align_up(o + n * sizeof(PrepDesc), 256);
  L.qinit = o;
  o = align_up(o + (q_entries ? n : 0) * sizeof(QEntry), 256);
  L.qctl = o;
  o = align_up(o + sizeof(QCtl), 256);
  L.berr = o;
  o = align_up(o + sizeof(uint32_t), 256);
  L.meta_end = o;
  L.queue = o;
  o = align_up(o + (size_t)q_entries * sizeof(QEntry), 256);
  for (size_t i = 0; i < n; ++i) {
    const qpso_camera& c = frames[i]->cam;
    const size_t P = ds[i]->num_particles;
    L.obs.push_back(o);
    o = align_up(o + (size_t)c.width * c.height * sizeof(uint16_t), 256);
    L.sat.push_back(o);
    o = align_up(o + (size_t)(c.width + 1) * (c.height + 1) * sizeof(int32_t), 256);
    L.pos.push_back(o);
    o = align_up(o + 7 * P * sizeof(float), 256);
    L.vel.push_back(o);
    o = align_up(o + 7 * P * sizeof(float), 256);
    L.pbest.push_back(o);
    o = align_up(o + 7 * P * sizeof(float), 256);
    L.pbf.push_back(o);
    o = align_up(o + P * sizeof(float), 256);
    L.fit.push_back(o);
    o = align_up(o + P * sizeof(float), 256);
    L.trace.push_back(o);
    if (trace) o = align_up(o + (size_t)ds[i]->iterations * 8 * sizeof(float), 256);
  }
  L.total = o;
  return L;
}

// Fill the pinned metadata block for a batch laid out by L.
void fill_meta(qpso_context* ctx, const Layout& L, const std::vector<const qpso_solve_desc*>& ds,
               const std::vector<const MeshObj*>& meshes, const std::vector<const FrameObj*>& frames,
               uint32_t ppb, bool trace) {
  char* h = static_cast<char*>(ctx->pin.p);
  char* d = static_cast<char*>(ctx->ws.p);
  std::memset(h, 0, L.meta_end);
  Instance* hi = reinterpret_cast<Instance*>(h + L.inst);
  Header* hh = reinterpret_cast<Header*>(h + L.hdr);
  PrepDesc* hp = reinterpret_cast<PrepDesc*>(h + L.prep);
  for (size_t i = 0; i < ds.size(); ++i) {
    const qpso_solve_desc& s = *ds[i];
    const MeshObj& m = *meshes[i];
    const FrameObj& f = *frames[i];
    Instance& I = hi[i];
    I.mesh = m.d;
    I.F = m.F;
    I.mlets = m.mlets;
    I.mlet_blob = m.blob;
    I.mlet_box = reinterpret_cast<const float4*>(m.blob + m.box_off);
    I.n_mlets = m.n_mlets;
    for (int k = 0; k < 3; ++k) {
      I.mesh_lo[k] = m.lo[k];
      I.mesh_hi[k] = m.hi[k];
    }
    I.obs = reinterpret_cast<const uint16_t*>(d + L.obs[i]);
    I.sat = reinterpret_cast<const int32_t*>(d + L.sat[i]);
    I.cam = Camera{f.cam.fx, f.cam.fy, f.cam.cx, f.cam.cy, f.cam.width, f.cam.height, f.cam.projection};
    I.prm = to_params(s);
    I.pos = reinterpret_cast<float*>(d + L.pos[i]);
    I.vel = reinterpret_cast<float*>(d + L.vel[i]);
    I.pbest = reinterpret_cast<float*>(d + L.pbest[i]);
    I.pbest_fit = reinterpret_cast<float*>(d + L.pbf[i]);
    I.fit = reinterpret_cast<float*>(d + L.fit[i]);
    Header* dh = reinterpret_cast<Header*>(d + L.hdr) + i;
    I.gbest = dh->gbest;
    I.done = &dh->done;
    I.err = &dh->err;
    I.stats = dh->stats;
    I.argkey = &dh->argkey;
    I.trace = trace ? reinterpret_cast<float*>(d + L.trace[i]) : nullptr;
    I.ppb = ppb;
    I.chunks = (s.num_particles + ppb - 1) / ppb;
    hh[i].gbest[0] = kBestInit;
    hh[i].argkey = ~0ull;
    PrepDesc& p = hp[i];
    p.depth = f.depth;
    p.labels = (s.cluster_label >= 0) ? f.labels : nullptr;
    p.label = s.cluster_label;
    p.width = f.cam.width;
    p.height = f.cam.height;
    p.obs = reinterpret_cast<uint16_t*>(d + L.obs[i]);
    p.sat = reinterpret_cast<int32_t*>(d + L.sat[i]);
  }
}

qpso_status gather_descs(qpso_context* ctx, const qpso_solve_desc* descs, uint32_t n,
                         std::vector<const qpso_solve_desc*>& ds, std::vector<const MeshObj*>& ms,
                         std::vector<const FrameObj*>& fs) {
  for (uint32_t i = 0; i < n; ++i) {
    const MeshObj* m;
    const FrameObj* f;
    qpso_status st = check_desc(ctx, descs[i], &m, &f);
    if (st != QPSO_OK) return st;
    ds.push_back(&descs[i]);
    ms.push_back(m);
    fs.push_back(f);
  }
  return QPSO_OK;
}

void read_result(const Header& h, qpso_result* r) {
  r->fit = h.gbest[0];
  for (int k = 0; k < 7; ++k) r->pose[k] = h.gbest[1 + k];
  r->flags = h.err;
  r->reserved = 0;
  r->raster_writes = h.stats[0];
  r->tile_passes = h.stats[1];
}

}  // namespace

// ===========================================================================
extern "C" {

const char* qpso_version(void) { return "qpso-gb300 0.1 (sm_103a)"; }

qpso_status qpso_create(int device, qpso_context** out) {
  if (!out) return QPSO_ERR_ARG;
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || device < 0 || device >= n) return QPSO_ERR_CUDA;
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return QPSO_ERR_CUDA;
  qpso_context* ctx = new (std::nothrow) qpso_context();
  if (!ctx) return QPSO_ERR_NOMEM;
  ctx->device = device;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return QPSO_ERR_CUDA;
  }
  if (prop.major * 10 + prop.minor < 100) {
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return QPSO_ERR_CUDA;  // the kernels are built for sm_103a only
  }
  ctx->num_sms = prop.multiProcessorCount;
  ctx->smem_optin = (int)prop.sharedMemPerBlockOptin - (int)smem_ctl_bytes() - 1024;
  ctx->plain = TileConfig{256, 8192, 1};
  ctx->batch = TileConfig{256, 8192, 1};
  *out = ctx;
  return QPSO_OK;
}

void qpso_destroy(qpso_context* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (auto& kv : ctx->meshes) {
    cudaFree(kv.second.d);
    cudaFree(kv.second.mlets);
    cudaFree(kv.second.blob);
  }
  for (auto& kv : ctx->frames) {
    cudaFree(kv.second.depth);
    cudaFree(kv.second.labels);
  }
  if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
  for (cudaEvent_t e : ctx->ev) cudaEventDestroy(e);
  for (cudaEvent_t e : ctx->timers)
    if (e) cudaEventDestroy(e);
  if (ctx->scrub.p) cudaFree(ctx->scrub.p);
  for (cudaEvent_t e : ctx->gev)
    if (e) cudaEventDestroy(e);
  if (ctx->ws.p) cudaFree(ctx->ws.p);
  if (ctx->pin.p) cudaFreeHost(ctx->pin.p);
  if (ctx->segpin.p) cudaFreeHost(ctx->segpin.p);
  for (cudaEvent_t e : ctx->seg_ev)
    if (e) cudaEventDestroy(e);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
}

const char* qpso_last_error(const qpso_context* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

qpso_status qpso_mesh_upload(qpso_context* ctx, const float* soa, uint32_t F, uint32_t* mesh_id) {
  if (!ctx || !soa || !mesh_id || F == 0 || F > (1u << 26)) return fail(ctx, QPSO_ERR_ARG, "bad mesh");
  for (size_t i = 0; i < 9 * (size_t)F; ++i)
    if (!std::isfinite(soa[i])) return fail(ctx, QPSO_ERR_ARG, "mesh has a non-finite coordinate");
  cudaSetDevice(ctx->device);
  std::vector<MeshletHdr> hdr;
  std::vector<unsigned char> blob;
  size_t box_off = 0;
  const int cap = meshlet_cap(F);
  build_meshlets(soa, F, hdr, blob, &box_off, cap);
  MeshObj m;
  m.F = F;
  m.n_mlets = (uint32_t)hdr.size();
  m.mlet_cap = cap;
  m.box_off = box_off;
  QPSO_CUDA(ctx, cudaMalloc(&m.d, 9 * (size_t)F * sizeof(float) + 32));
  cudaError_t e = cudaMalloc(&m.mlets, hdr.size() * sizeof(MeshletHdr));
  if (e == cudaSuccess) e = cudaMalloc(&m.blob, blob.size());
  float* dbox = m.d + 9 * (size_t)F;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(m.d, soa, 9 * (size_t)F * sizeof(float), cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(m.mlets, hdr.data(), hdr.size() * sizeof(MeshletHdr), cudaMemcpyHostToDevice,
                        ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(m.blob, blob.data(), blob.size(), cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = launch_mesh_aabb(m.d, F, dbox, ctx->stream);
  float box[6];
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(box, dbox, sizeof(box), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    cudaFree(m.d);
    if (m.mlets) cudaFree(m.mlets);
    if (m.blob) cudaFree(m.blob);
    return cuda_fail(ctx, e, "mesh upload");
  }
  for (int k = 0; k < 3; ++k) {
    m.lo[k] = box[k];
    m.hi[k] = box[3 + k];
  }
  std::lock_guard<std::mutex> g(ctx->mu);
  *mesh_id = ctx->next_id++;
  ctx->meshes[*mesh_id] = m;
  return QPSO_OK;
}

qpso_status qpso_mesh_release(qpso_context* ctx, uint32_t id) {
  if (!ctx) return QPSO_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  auto it = ctx->meshes.find(id);
  if (it == ctx->meshes.end()) return fail(ctx, QPSO_ERR_NOT_FOUND, "unknown mesh id");
  cudaStreamSynchronize(ctx->stream);
  cudaFree(it->second.d);
  cudaFree(it->second.mlets);
  cudaFree(it->second.blob);
  ctx->meshes.erase(it);
  return QPSO_OK;
}

qpso_status qpso_frame_upload(qpso_context* ctx, const uint16_t* depth, const int32_t* labels,
                              const qpso_camera* cam, uint32_t* frame_id) {
  if (!ctx || !depth || !cam || !frame_id) return fail(ctx, QPSO_ERR_ARG, "null argument");
  if (const char* why = camera_error(*cam)) return fail(ctx, QPSO_ERR_ARG, why);
  cudaSetDevice(ctx->device);
  FrameObj f;
  f.cam = *cam;
  const size_t npx = (size_t)cam->width * cam->height;
  QPSO_CUDA(ctx, cudaMalloc(&f.depth, npx * sizeof(uint16_t)));
  cudaError_t e = cudaMemcpyAsync(f.depth, depth, npx * sizeof(uint16_t), cudaMemcpyHostToDevice,
                                  ctx->stream);
  if (e == cudaSuccess && labels) {
    e = cudaMalloc(&f.labels, npx * sizeof(int32_t));
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(f.labels, labels, npx * sizeof(int32_t), cudaMemcpyHostToDevice,
                          ctx->stream);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    cudaFree(f.depth);
    if (f.labels) cudaFree(f.labels);
    return cuda_fail(ctx, e, "frame upload");
  }
  std::lock_guard<std::mutex> g(ctx->mu);
  *frame_id = ctx->next_id++;
  ctx->frames[*frame_id] = f;
  return QPSO_OK;
}

qpso_status qpso_frame_release(qpso_context* ctx, uint32_t id) {
  if (!ctx) return QPSO_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  auto it = ctx->frames.find(id);
  if (it == ctx->frames.end()) return fail(ctx, QPSO_ERR_NOT_FOUND, "unknown frame id");
  cudaStreamSynchronize(ctx->stream);
  cudaFree(it->second.depth);
  if (it->second.labels) cudaFree(it->second.labels);
  ctx->frames.erase(it);
  return QPSO_OK;
}

qpso_status qpso_frame_update(qpso_context* ctx, uint32_t id, const uint16_t* depth,
                              const int32_t* labels) {
  if (!ctx || !depth) return fail(ctx, QPSO_ERR_ARG, "null argument");
  auto it = ctx->frames.find(id);
  if (it == ctx->frames.end()) return fail(ctx, QPSO_ERR_NOT_FOUND, "unknown frame id");
  FrameObj& f = it->second;
  if (labels && !f.labels) return fail(ctx, QPSO_ERR_ARG, "frame was uploaded without labels");
  cudaSetDevice(ctx->device);
  const size_t npx = (size_t)f.cam.width * f.cam.height;
  QPSO_CUDA(ctx, cudaMemcpyAsync(f.depth, depth, npx * 2, cudaMemcpyHostToDevice, ctx->stream));
  if (labels)
    QPSO_CUDA(ctx, cudaMemcpyAsync(f.labels, labels, npx * 4, cudaMemcpyHostToDevice, ctx->stream));
  QPSO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return QPSO_OK;
}

void* qpso_host_alloc(uint64_t bytes) {
  void* p = nullptr;
  if (bytes == 0 || cudaMallocHost(&p, bytes) != cudaSuccess) return nullptr;
  return p;
}

void qpso_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

void* qpso_get_stream(const qpso_context* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

qpso_status qpso_set_profiling(qpso_context* ctx, int enable) {
  if (!ctx) return QPSO_ERR_ARG;
  ctx->profiling = enable != 0;
  return QPSO_OK;
}

qpso_status qpso_get_profile(qpso_context* ctx, qpso_profile* out, int reset) {
  if (!ctx || !out) return QPSO_ERR_ARG;
  *out = ctx->prof;
  if (reset) ctx->prof = qpso_profile{};
  return QPSO_OK;
}

qpso_status qpso_timer_record(qpso_context* ctx, uint32_t slot) {
  if (!ctx || slot >= 64) return fail(ctx, QPSO_ERR_ARG, "timer slot must be < 64");
  cudaSetDevice(ctx->device);
  if (!ctx->timers[slot]) QPSO_CUDA(ctx, cudaEventCreate(&ctx->timers[slot]));
  QPSO_CUDA(ctx, cudaEventRecord(ctx->timers[slot], ctx->stream));
  return QPSO_OK;
}

qpso_status qpso_timer_elapsed(qpso_context* ctx, uint32_t a, uint32_t b, float* ms) {
  if (!ctx || !ms || a >= 64 || b >= 64 || !ctx->timers[a] || !ctx->timers[b])
    return fail(ctx, QPSO_ERR_ARG, "timer slots not recorded");
  QPSO_CUDA(ctx, cudaEventSynchronize(ctx->timers[b]));
  QPSO_CUDA(ctx, cudaEventElapsedTime(ms, ctx->timers[a], ctx->timers[b]));
  return QPSO_OK;
}

qpso_status qpso_scrub_l2(qpso_context* ctx, uint64_t bytes) {
  if (!ctx || bytes == 0 || bytes > (8ull << 30)) return fail(ctx, QPSO_ERR_ARG, "scrub size");
  cudaSetDevice(ctx->device);
  if (ctx->scrub.cap < bytes) {
    if (ctx->scrub.p) {
      QPSO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      cudaFree(ctx->scrub.p);
      ctx->scrub.p = nullptr;
      ctx->scrub.cap = 0;
    }
    QPSO_CUDA(ctx, cudaMalloc(&ctx->scrub.p, bytes));
    ctx->scrub.cap = bytes;
  }
  static uint8_t flip = 0;
  flip ^= 0x5a;
  QPSO_CUDA(ctx, cudaMemsetAsync(ctx->scrub.p, flip, bytes, ctx->stream));
  return QPSO_OK;
}

void qpso_solve_desc_init(qpso_solve_desc* d) {
  if (!d) return;
  std::memset(d, 0, sizeof(*d));
  d->cluster_label = -1;
  d->num_particles = 1024;  // Nparticle_, main.h:84
  d->iterations = 20;       // max_steps_, main.h:99
  d->c1 = 1.0f;             // c1_, main.h:104
  d->c2 = 1.0f;             // c2_, main.h:105
  d->w = 0.3;               // psoW_, main.h:106
  d->vdot = 3.0f;           // vdot_, main.h:126
  d->ang_lo = -10.0f;       // aminX_, main.h:118
  d->ang_hi = 10.0f;        // amaxX_, main.h:119
  d->qinit[0] = 0.7071f;    // main.cu:130
  d->qinit[1] = 0.7071f;
  d->qinit[2] = 0.0f;
  d->qinit[3] = 0.0f;
}

void qpso_box_from_centroid(const float c_mm[3], float bound, float bound_z, float lo[3],
                            float hi[3]) {
  for (int k = 0; k < 3; ++k) {
    const float c = c_mm[k] * 0.001f;
    const float b = (k == 2) ? bound_z : bound;
    lo[k] = c - b;
    hi[k] = c + b;
  }
}

qpso_status qpso_set_launch_config(qpso_context* ctx, const qpso_launch_config* plain,
                                   const qpso_launch_config* batch) {
  if (!ctx) return QPSO_ERR_ARG;
  if (plain && !valid_cfg(*plain, ctx->smem_optin)) return fail(ctx, QPSO_ERR_ARG, "bad plain launch config");
  if (batch && !valid_cfg(*batch, ctx->smem_optin)) return fail(ctx, QPSO_ERR_ARG, "bad batch launch config");
  if (plain) ctx->plain = TileConfig{plain->threads, plain->tile_px, plain->ppb};
  if (batch) ctx->batch = TileConfig{batch->threads, batch->tile_px, batch->ppb};
  return QPSO_OK;
}

qpso_status qpso_get_launch_config(const qpso_context* ctx, qpso_launch_config* plain,
                                   qpso_launch_config* batch) {
  if (!ctx) return QPSO_ERR_ARG;
  if (plain) *plain = qpso_launch_config{ctx->plain.threads, ctx->plain.tile_px, ctx->plain.ppb};
  if (batch) *batch = qpso_launch_config{ctx->batch.threads, ctx->batch.tile_px, ctx->batch.ppb};
  return QPSO_OK;
}

qpso_status qpso_solve_traced(qpso_context* ctx, const qpso_solve_desc* desc, qpso_result* result,
                              float* trace, float* pos, float* vel, float* pbest, float* pbest_fit) {
  if (!ctx || !desc || !result) return fail(ctx, QPSO_ERR_ARG, "null argument");
  cudaSetDevice(ctx->device);
  std::vector<const qpso_solve_desc*> ds;
  std::vector<const MeshObj*> ms;
  std::vector<const FrameObj*> fs;
  qpso_status st = gather_descs(ctx, desc, 1, ds, ms, fs);
  if (st != QPSO_OK) return st;
  TileConfig cfg = ctx->plain;
  const int vcap = launch_vcap(ms);
  if ((st = fit_cfg(ctx, cfg, vcap)) != QPSO_OK) return st;
  const bool want_trace = trace != nullptr;
  Layout L = make_layout(ds, fs, 0, want_trace);
  if ((st = ensure_ws(ctx, L.total)) != QPSO_OK) return st;
  if ((st = ensure_pin(ctx, L.meta_end)) != QPSO_OK) return st;
  fill_meta(ctx, L, ds, ms, fs, (uint32_t)cfg.ppb, want_trace);
  char* d = static_cast<char*>(ctx->ws.p);
  char* h = static_cast<char*>(ctx->pin.p);
  cudaStream_t s = ctx->stream;
  QPSO_CUDA(ctx, cudaMemcpyAsync(d, h, L.meta_end, cudaMemcpyHostToDevice, s));
  QPSO_CUDA(ctx, launch_prep(reinterpret_cast<PrepDesc*>(d + L.prep), 1, fs[0]->cam.width,
                             fs[0]->cam.height, s));
  const Instance* dinst = reinterpret_cast<const Instance*>(d + L.inst);
  const uint32_t chunks = (desc->num_particles + cfg.ppb - 1) / cfg.ppb;
  const bool prof = ctx->profiling;
  if (prof && (st = ensure_events(ctx, 2 * (size_t)desc->iterations)) != QPSO_OK) return st;
  for (uint32_t it = 0; it < desc->iterations; ++it) {
    if (prof) QPSO_CUDA(ctx, cudaEventRecord(ctx->ev[2 * it], s));
    QPSO_CUDA(ctx, launch_step(dinst, it, chunks, cfg, s, kernel_variant(*desc, fs[0]->cam), vcap));
    if (prof) QPSO_CUDA(ctx, cudaEventRecord(ctx->ev[2 * it + 1], s));
  }
  QPSO_CUDA(ctx, cudaMemcpyAsync(h + L.hdr, d + L.hdr, sizeof(Header), cudaMemcpyDeviceToHost, s));
  const size_t P = desc->num_particles;
  if (trace)
    QPSO_CUDA(ctx, cudaMemcpyAsync(trace, d + L.trace[0], desc->iterations * 8 * sizeof(float),
                                   cudaMemcpyDeviceToHost, s));
  if (pos) QPSO_CUDA(ctx, cudaMemcpyAsync(pos, d + L.pos[0], 7 * P * 4, cudaMemcpyDeviceToHost, s));
  if (vel) QPSO_CUDA(ctx, cudaMemcpyAsync(vel, d + L.vel[0], 7 * P * 4, cudaMemcpyDeviceToHost, s));
  if (pbest)
    QPSO_CUDA(ctx, cudaMemcpyAsync(pbest, d + L.pbest[0], 7 * P * 4, cudaMemcpyDeviceToHost, s));
  if (pbest_fit)
    QPSO_CUDA(ctx, cudaMemcpyAsync(pbest_fit, d + L.pbf[0], P * 4, cudaMemcpyDeviceToHost, s));
  QPSO_CUDA(ctx, cudaStreamSynchronize(s));
  if (prof) {
    ctx->prof.step_launches += desc->iterations;
    ctx->prof.step_ms += event_pairs_ms(ctx, desc->iterations);
    ctx->prof.prep_launches += 2;
  }
  const Header& hd = *reinterpret_cast<const Header*>(h + L.hdr);
  read_result(hd, result);
  if (hd.err & kErrBound) return fail(ctx, QPSO_ERR_INTERNAL, "raster bound violated");
  return QPSO_OK;
}

qpso_status qpso_solve(qpso_context* ctx, const qpso_solve_desc* desc, qpso_result* result) {
  return qpso_solve_traced(ctx, desc, result, nullptr, nullptr, nullptr, nullptr, nullptr);
}

qpso_status qpso_solve_batch(qpso_context* ctx, const qpso_solve_desc* descs, uint32_t n,
                             qpso_result* results) {
  if (!ctx || !descs || !results || n == 0) return fail(ctx, QPSO_ERR_ARG, "bad batch arguments");
  cudaSetDevice(ctx->device);
  std::vector<const qpso_solve_desc*> ds;
  std::vector<const MeshObj*> ms;
  std::vector<const FrameObj*> fs;
  qpso_status st = gather_descs(ctx, descs, n, ds, ms, fs);
  if (st != QPSO_OK) return st;
  TileConfig cfg = ctx->batch;
  // instances, most expensive first
  std::vector<uint32_t> order(n);
  std::vector<double> cost(n);
  uint32_t max_iters = 0, max_w = 0, max_h = 0;
  int var = 0;
  for (uint32_t i = 0; i < n; ++i) {
    order[i] = i;
    var = std::max(var, kernel_variant(*ds[i], fs[i]->cam));
    const double area = (double)(ds[i]->cl_max_x - ds[i]->cl_min_x) * (ds[i]->cl_max_y - ds[i]->cl_min_y);
    cost[i] = (double)ms[i]->F * 3.0 + area;
    max_iters = std::max(max_iters, ds[i]->iterations);
    max_w = std::max(max_w, (uint32_t)fs[i]->cam.width);
    max_h = std::max(max_h, (uint32_t)fs[i]->cam.height);
  }
  std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return cost[a] > cost[b]; });
  // the work queue: one entry per (instance, iteration), iteration 0 of
  // every instance first, most expensive first
  size_t all_chunks = 0;
  uint64_t q_entries = 0;
  for (uint32_t i = 0; i < n; ++i) {
    all_chunks += (ds[i]->num_particles + cfg.ppb - 1) / cfg.ppb;
    q_entries += ds[i]->iterations;
  }
  if (q_entries > 0xffffffffull) return fail(ctx, QPSO_ERR_ARG, "too many iterations in one batch");
  Layout L = make_layout(ds, fs, (uint32_t)q_entries, false);
  if ((st = ensure_ws(ctx, L.total)) != QPSO_OK) return st;
  if ((st = ensure_pin(ctx, L.meta_end)) != QPSO_OK) return st;
  int per_sm = 0;
  const int vcap = launch_vcap(ms);
  if ((st = fit_cfg(ctx, cfg, vcap)) != QPSO_OK) return st;
  QPSO_CUDA(ctx, batch_max_grid(cfg, var, vcap, &per_sm));
  if (per_sm <= 0) return fail(ctx, QPSO_ERR_ARG, "batch launch config does not fit on an SM");
  const int grid = (int)std::min<size_t>(all_chunks, (size_t)per_sm * ctx->num_sms);
  // wait before touching pinned staging that an earlier graph may read
  QPSO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  fill_meta(ctx, L, ds, ms, fs, (uint32_t)cfg.ppb, false);
  char* d = static_cast<char*>(ctx->ws.p);
  char* h = static_cast<char*>(ctx->pin.p);
  {
    QEntry* qi = reinterpret_cast<QEntry*>(h + L.qinit);
    for (uint32_t k = 0; k < n; ++k) qi[k] = QEntry{order[k], 0u, 0u, 1u};
    *reinterpret_cast<QCtl*>(h + L.qctl) = QCtl{0u, n, (uint32_t)q_entries, 0u};  // iteration 0 queued
  }
  cudaStream_t s = ctx->stream;
  if (!ctx->gev[0]) {
    QPSO_CUDA(ctx, cudaEventCreate(&ctx->gev[0]));
    QPSO_CUDA(ctx, cudaEventCreate(&ctx->gev[1]));
  }
  std::vector<uint64_t> key = {(uint64_t)(uintptr_t)d, (uint64_t)(uintptr_t)h, L.total, L.meta_end,
                               n, q_entries, max_iters, (uint64_t)grid, (uint64_t)cfg.threads,
                               (uint64_t)cfg.tile_px, (uint64_t)cfg.ppb, max_w, max_h, (uint64_t)var,
                               (uint64_t)vcap};
  if (!ctx->gexec || key != ctx->gkey) {
    if (ctx->gexec) {
      cudaGraphExecDestroy(ctx->gexec);
      ctx->gexec = nullptr;
    }
    BatchArgs A;
    A.inst = reinterpret_cast<Instance*>(d + L.inst);
    A.queue = reinterpret_cast<QEntry*>(d + L.queue);
    A.qctl = reinterpret_cast<QCtl*>(d + L.qctl);
    A.err = reinterpret_cast<uint32_t*>(d + L.berr);
    A.timeout_ns = 20ull * 1000 * 1000 * 1000;  // 20 s per wait for work
    cudaGraph_t graph;
    QPSO_CUDA(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaMemcpyAsync(d, h, L.meta_end, cudaMemcpyHostToDevice, s);
    // every replay starts from an empty queue holding iteration 0 of each instance
    if (e == cudaSuccess) e = cudaMemsetAsync(d + L.queue, 0, (size_t)q_entries * sizeof(QEntry), s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d + L.queue, d + L.qinit, n * sizeof(QEntry), cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess)
      e = launch_prep(reinterpret_cast<PrepDesc*>(d + L.prep), (int)n, (int)max_w, (int)max_h, s);
    if (e == cudaSuccess) e = launch_batch(A, grid, cfg, s, var, vcap);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h + L.hdr, d + L.hdr, n * sizeof(Header), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h + L.berr, d + L.berr, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    cudaError_t e2 = cudaStreamEndCapture(s, &graph);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "batch capture");
    if (e2 != cudaSuccess) return cuda_fail(ctx, e2, "batch capture end");
    e = cudaGraphInstantiate(&ctx->gexec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      ctx->gexec = nullptr;
      return cuda_fail(ctx, e, "graph instantiate");
    }
    ctx->gkey = key;
  }
  // device time of the replayed graph: metadata upload, preparation, the
  // persistent kernel and the result read-back (the kernel dominates)
  if (ctx->profiling) QPSO_CUDA(ctx, cudaEventRecord(ctx->gev[0], s));
  QPSO_CUDA(ctx, cudaGraphLaunch(ctx->gexec, s));
  if (ctx->profiling) QPSO_CUDA(ctx, cudaEventRecord(ctx->gev[1], s));
  QPSO_CUDA(ctx, cudaStreamSynchronize(s));
  if (ctx->profiling) {
    float t = 0.f;
    if (cudaEventElapsedTime(&t, ctx->gev[0], ctx->gev[1]) == cudaSuccess) ctx->prof.batch_ms += t;
    ctx->prof.batch_launches += 1;
    ctx->prof.prep_launches += 2;
  }
  const Header* hh = reinterpret_cast<const Header*>(h + L.hdr);
  bool bad = false;
  for (uint32_t i = 0; i < n; ++i) {
    read_result(hh[i], &results[i]);
    bad = bad || (hh[i].err & kErrBound);
  }
  const uint32_t berr = *reinterpret_cast<const uint32_t*>(h + L.berr);
  if (berr & kErrTimeout) return fail(ctx, QPSO_ERR_TIMEOUT, "batch wait for work timed out");
  if (bad) return fail(ctx, QPSO_ERR_INTERNAL, "raster bound violated");
  return QPSO_OK;
}

qpso_status qpso_autotune(qpso_context* ctx, const qpso_solve_desc* descs, uint32_t n, int batched,
                          uint32_t tune_iters, qpso_launch_config* best, float* best_ms) {
  if (!ctx || !descs || n == 0 || tune_iters == 0) return fail(ctx, QPSO_ERR_ARG, "bad autotune arguments");
  std::vector<qpso_solve_desc> ds(descs, descs + n);
  int var = 0;
  int vcap = 64;
  for (auto& d : ds) {
    d.iterations = std::min(d.iterations, tune_iters);
    auto fi = ctx->frames.find(d.frame_id);
    if (fi != ctx->frames.end()) var = std::max(var, kernel_variant(d, fi->second.cam));
    auto mi = ctx->meshes.find(d.mesh_id);
    if (mi != ctx->meshes.end()) vcap = std::max(vcap, mi->second.mlet_cap);
  }
  const TileConfig saved = batched ? ctx->batch : ctx->plain;
  TileConfig win = saved;
  float win_ms = 3.0e38f;
  std::vector<qpso_result> res(n);
  qpso_status st = QPSO_OK;
  if (!ctx->timers[0]) QPSO_CUDA(ctx, cudaEventCreate(&ctx->timers[0]));
  if (!ctx->timers[1]) QPSO_CUDA(ctx, cudaEventCreate(&ctx->timers[1]));
  const int threads[] = {128, 256, 512};
  const int ppbs[] = {1, 2, 4};
  for (int th : threads)
    for (int pb : ppbs) {
      // fixed sizes, and the largest tile that keeps two CTAs on an SM
      std::vector<int> tiles = {4096, 8192, 16384, 32768, 49152};
      const int t2 = tile_for_occupancy(th, pb, vcap, 2, batched != 0, var);
      if (t2 > 0 && std::find(tiles.begin(), tiles.end(), t2) == tiles.end()) tiles.push_back(t2);
      for (int tp : tiles) {
        const qpso_launch_config c{th, tp, pb};
        if (!valid_cfg(c, ctx->smem_optin, vcap)) continue;
        const TileConfig tc{th, tp, pb};
        if (batched) {
          int per_sm = 0;
          if (batch_max_grid(tc, var, vcap, &per_sm) != cudaSuccess || per_sm <= 0) continue;
          ctx->batch = tc;
        } else {
          ctx->plain = tc;
        }
        float ms = 3.0e38f;
        for (int rep = 0; rep < 3 && st == QPSO_OK; ++rep) {  // rep 0 warms up (graph capture)
          float t = 0.f;
          QPSO_CUDA(ctx, cudaEventRecord(ctx->timers[0], ctx->stream));
          if (batched) {
            st = qpso_solve_batch(ctx, ds.data(), n, res.data());
          } else {
            for (uint32_t i = 0; i < n && st == QPSO_OK; ++i) st = qpso_solve(ctx, &ds[i], &res[i]);
          }
          QPSO_CUDA(ctx, cudaEventRecord(ctx->timers[1], ctx->stream));
          QPSO_CUDA(ctx, cudaEventSynchronize(ctx->timers[1]));
          QPSO_CUDA(ctx, cudaEventElapsedTime(&t, ctx->timers[0], ctx->timers[1]));
          if (rep > 0) ms = std::min(ms, t);  // best of the two timed runs
        }
        if (st != QPSO_OK) {
          if (batched) ctx->batch = saved; else ctx->plain = saved;
          return st;
        }
        if (ms < win_ms) {
          win_ms = ms;
          win = tc;
        }
      }
    }
  if (batched) ctx->batch = win; else ctx->plain = win;
  if (best) *best = qpso_launch_config{win.threads, win.tile_px, win.ppb};
  if (best_ms) *best_ms = win_ms;
  return QPSO_OK;
}

qpso_status qpso_score_poses(qpso_context* ctx, const qpso_solve_desc* desc, const float* poses,
                             uint32_t n, float* fit_out) {
  if (!ctx || !desc || !poses || !fit_out || n == 0) return fail(ctx, QPSO_ERR_ARG, "null argument");
  cudaSetDevice(ctx->device);
  std::vector<const qpso_solve_desc*> ds;
  std::vector<const MeshObj*> ms;
  std::vector<const FrameObj*> fs;
  qpso_status st = gather_descs(ctx, desc, 1, ds, ms, fs);
  if (st != QPSO_OK) return st;
  Layout L = make_layout(ds, fs, 0, false);
  const size_t pose_off = align_up(L.total, 256);
  const size_t fit_off = align_up(pose_off + (size_t)n * 7 * sizeof(float), 256);
  const size_t total = align_up(fit_off + (size_t)n * sizeof(float), 256);
  if ((st = ensure_ws(ctx, total)) != QPSO_OK) return st;
  if ((st = ensure_pin(ctx, L.meta_end)) != QPSO_OK) return st;
  QPSO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  TileConfig cfg = ctx->plain;
  const int vcap = launch_vcap(ms);
  if ((st = fit_cfg(ctx, cfg, vcap)) != QPSO_OK) return st;
  fill_meta(ctx, L, ds, ms, fs, (uint32_t)cfg.ppb, false);
  char* d = static_cast<char*>(ctx->ws.p);
  char* h = static_cast<char*>(ctx->pin.p);
  cudaStream_t s = ctx->stream;
  QPSO_CUDA(ctx, cudaMemcpyAsync(d, h, L.meta_end, cudaMemcpyHostToDevice, s));
  QPSO_CUDA(ctx, launch_prep(reinterpret_cast<PrepDesc*>(d + L.prep), 1, fs[0]->cam.width,
                             fs[0]->cam.height, s));
  QPSO_CUDA(ctx, cudaMemcpyAsync(d + pose_off, poses, (size_t)n * 7 * sizeof(float),
                                 cudaMemcpyHostToDevice, s));
  const uint32_t groups = (n + cfg.ppb - 1) / cfg.ppb;
  const int grid = (int)std::min<uint32_t>(groups, (uint32_t)ctx->num_sms * 4);
  QPSO_CUDA(ctx, launch_score_mlets(reinterpret_cast<const Instance*>(d + L.inst),
                                    reinterpret_cast<const float*>(d + pose_off), n,
                                    reinterpret_cast<float*>(d + fit_off), cfg, grid, s,
                                    kernel_variant(*desc, fs[0]->cam), vcap));
  QPSO_CUDA(ctx, cudaMemcpyAsync(fit_out, d + fit_off, (size_t)n * sizeof(float),
                                 cudaMemcpyDeviceToHost, s));
  QPSO_CUDA(ctx, cudaMemcpyAsync(h + L.hdr, d + L.hdr, sizeof(Header), cudaMemcpyDeviceToHost, s));
  QPSO_CUDA(ctx, cudaStreamSynchronize(s));
  const Header& hd = *reinterpret_cast<const Header*>(h + L.hdr);
  if (hd.err & kErrBound) return fail(ctx, QPSO_ERR_INTERNAL, "raster bound violated");
  return QPSO_OK;
}

void qpso_refine_params_init(qpso_refine_params* p) {
  if (!p) return;
  p->rounds = 32;
  p->candidates = 128;
  p->step_t = 0.03f;
  p->step_rot = 0.5f;
  p->raster_mode = QPSO_RASTER_EDGE;
}

}  // extern "C"

namespace {

}  // namespace

extern "C" {

qpso_status qpso_refine(qpso_context* ctx, const qpso_solve_desc* desc, const qpso_refine_params* prm,
                        const float pose_in[7], float pose_out[7], float* fit_out) {
  if (!ctx || !desc || !prm || !pose_in || !pose_out || !fit_out) return fail(ctx, QPSO_ERR_ARG, "null argument");
  if (prm->candidates < 12 || prm->candidates > 4096 || prm->rounds > 4096 || !(prm->step_t >= 0.0f) ||
      !(prm->step_rot >= 0.0f) || !std::isfinite(prm->step_t) || !std::isfinite(prm->step_rot) ||
      (prm->raster_mode != QPSO_RASTER_REF && prm->raster_mode != QPSO_RASTER_EDGE))
    return fail(ctx, QPSO_ERR_ARG, "bad refinement parameters");
  for (int k = 0; k < 7; ++k)
    if (!std::isfinite(pose_in[k])) return fail(ctx, QPSO_ERR_ARG, "non-finite pose");
  qpso_solve_desc d = *desc;
  d.raster_mode = prm->raster_mode;
  cudaSetDevice(ctx->device);
  std::vector<const qpso_solve_desc*> ds;
  std::vector<const MeshObj*> ms;
  std::vector<const FrameObj*> fs;
  qpso_status st = gather_descs(ctx, &d, 1, ds, ms, fs);
  if (st != QPSO_OK) return st;
  // the whole search runs on the device: the instance and its summed-area
  // table are prepared once, each round generates its candidates, scores
  // them with the solver's render and fitness and keeps the best, and the
  // host waits once at the end
  const uint32_t K = prm->candidates;
  Layout L = make_layout(ds, fs, 0, false);
  const size_t state_off = align_up(L.total, 256);
  const size_t cand_off = align_up(state_off + sizeof(RefineState), 256);
  const size_t fit_off = align_up(cand_off + (size_t)K * 7 * sizeof(float), 256);
  const size_t total = align_up(fit_off + (size_t)K * sizeof(float), 256);
  if ((st = ensure_ws(ctx, total)) != QPSO_OK) return st;
  // the state's host copy sits after the metadata in the pinned buffer
  const size_t hstate_off = align_up(std::max<size_t>(L.meta_end, L.hdr + sizeof(Header)), 256);
  if ((st = ensure_pin(ctx, hstate_off + sizeof(RefineState))) != QPSO_OK) return st;
  QPSO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  TileConfig cfg = ctx->plain;
  const int vcap = launch_vcap(ms);
  if ((st = fit_cfg(ctx, cfg, vcap)) != QPSO_OK) return st;
  fill_meta(ctx, L, ds, ms, fs, (uint32_t)cfg.ppb, false);
  char* dw = static_cast<char*>(ctx->ws.p);
  char* hp = static_cast<char*>(ctx->pin.p);
  RefineState* hs = reinterpret_cast<RefineState*>(hp + hstate_off);
  std::memset(hs, 0, sizeof(RefineState));
  for (int k = 0; k < 7; ++k) hs->pose[k] = pose_in[k];
  rotate_small(hs->pose + 3, 0.0f, 0.0f, 0.0f);  // normalised, top hemisphere
  hs->step_t = prm->step_t;
  hs->step_r = prm->step_rot;
  hs->K = K;
  hs->rng_seed = desc->seed ^ ((uint64_t)desc->stream << 32) ^ 0x5245464E45ull;
  RefineState* dst = reinterpret_cast<RefineState*>(dw + state_off);
  float* dcand = reinterpret_cast<float*>(dw + cand_off);
  float* dfit = reinterpret_cast<float*>(dw + fit_off);
  const Instance* dinst = reinterpret_cast<const Instance*>(dw + L.inst);
  const int var = kernel_variant(d, fs[0]->cam);
  cudaStream_t s = ctx->stream;
  QPSO_CUDA(ctx, cudaMemcpyAsync(dw, hp, L.meta_end, cudaMemcpyHostToDevice, s));
  QPSO_CUDA(ctx, cudaMemcpyAsync(dst, hs, sizeof(RefineState), cudaMemcpyHostToDevice, s));
  QPSO_CUDA(ctx, launch_prep(reinterpret_cast<PrepDesc*>(dw + L.prep), 1, fs[0]->cam.width, fs[0]->cam.height,
                             s));
  // the starting pose's fitness, straight into the state
  QPSO_CUDA(ctx, launch_score_mlets(dinst, dst->pose, 1, &dst->fit, cfg, 1, s, var, vcap));
  const uint32_t groups = (K + cfg.ppb - 1) / cfg.ppb;
  const int grid = (int)std::min<uint32_t>(groups, (uint32_t)ctx->num_sms * 4);
  for (uint32_t r = 0; r < prm->rounds; ++r) {
    QPSO_CUDA(ctx, launch_refine_gen(dst, dcand, K, s));
    QPSO_CUDA(ctx, launch_score_mlets(dinst, dcand, K, dfit, cfg, grid, s, var, vcap));
    QPSO_CUDA(ctx, launch_refine_pick(dst, dcand, dfit, K, s));
  }
  QPSO_CUDA(ctx, cudaMemcpyAsync(hs, dst, sizeof(RefineState), cudaMemcpyDeviceToHost, s));
  QPSO_CUDA(ctx, cudaMemcpyAsync(hp + L.hdr, dw + L.hdr, sizeof(Header), cudaMemcpyDeviceToHost, s));
  QPSO_CUDA(ctx, cudaStreamSynchronize(s));
  const Header& hd = *reinterpret_cast<const Header*>(hp + L.hdr);
  if (hd.err & kErrBound) return fail(ctx, QPSO_ERR_INTERNAL, "raster bound violated");
  for (int k = 0; k < 7; ++k) pose_out[k] = hs->pose[k];
  *fit_out = hs->fit;
  return QPSO_OK;
}

qpso_status qpso_render(qpso_context* ctx, uint32_t mesh_id, const qpso_camera* cam,
                        const float pose[7], int32_t x0, int32_t y0, int32_t w, int32_t h,
                        int32_t* depth_out, int32_t box_out[4]) {
  if (!ctx || !cam || !pose || !depth_out || !box_out || w <= 0 || h <= 0 || w % 4 != 0 || !projection_ok(cam))
    return fail(ctx, QPSO_ERR_ARG, "bad render arguments (w must be a positive multiple of 4)");
  if ((size_t)w * h * 4 > (size_t)ctx->smem_optin)
    return fail(ctx, QPSO_ERR_ARG, "render window exceeds one CTA's shared memory");
  auto mi = ctx->meshes.find(mesh_id);
  if (mi == ctx->meshes.end()) return fail(ctx, QPSO_ERR_NOT_FOUND, "unknown mesh id");
  cudaSetDevice(ctx->device);
  const MeshObj& m = mi->second;
  const size_t inst_off = 0, pose_off = 256, box_off = 512, out_off = 1024;
  const size_t total = out_off + (size_t)w * h * 4;
  qpso_status st;
  if ((st = ensure_ws(ctx, total)) != QPSO_OK) return st;
  if ((st = ensure_pin(ctx, 1024)) != QPSO_OK) return st;
  QPSO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  char* d = static_cast<char*>(ctx->ws.p);
  char* hp = static_cast<char*>(ctx->pin.p);
  std::memset(hp, 0, 1024);
  Instance& I = *reinterpret_cast<Instance*>(hp + inst_off);
  I.mesh = m.d;
  I.F = m.F;
  for (int k = 0; k < 3; ++k) {
    I.mesh_lo[k] = m.lo[k];
    I.mesh_hi[k] = m.hi[k];
  }
  I.cam = Camera{cam->fx, cam->fy, cam->cx, cam->cy, cam->width, cam->height, cam->projection};
  std::memcpy(hp + pose_off, pose, 7 * sizeof(float));
  cudaStream_t s = ctx->stream;
  QPSO_CUDA(ctx, cudaMemcpyAsync(d, hp, 1024, cudaMemcpyHostToDevice, s));
  QPSO_CUDA(ctx, launch_render_window(reinterpret_cast<const Instance*>(d + inst_off),
                                      reinterpret_cast<const float*>(d + pose_off), x0, y0, w, h,
                                      reinterpret_cast<int32_t*>(d + out_off),
                                      reinterpret_cast<int32_t*>(d + box_off), 256, s));
  QPSO_CUDA(ctx, cudaMemcpyAsync(depth_out, d + out_off, (size_t)w * h * 4, cudaMemcpyDeviceToHost, s));
  QPSO_CUDA(ctx, cudaMemcpyAsync(box_out, d + box_off, 16, cudaMemcpyDeviceToHost, s));
  QPSO_CUDA(ctx, cudaStreamSynchronize(s));
  return QPSO_OK;
}

qpso_status qpso_frame_clusters(qpso_context* ctx, uint32_t frame_id, qpso_cluster* out, uint32_t capacity,
                                uint32_t* n_clusters) {
  if (!ctx || !n_clusters) return fail(ctx, QPSO_ERR_ARG, "bad cluster arguments");
  auto fi = ctx->frames.find(frame_id);
  if (fi == ctx->frames.end()) return fail(ctx, QPSO_ERR_NOT_FOUND, "unknown frame id");
  const FrameObj& f = fi->second;
  if (!f.labels) return fail(ctx, QPSO_ERR_ARG, "frame has no label map");
  cudaSetDevice(ctx->device);
  const int32_t W = f.cam.width, H = f.cam.height;
  qpso_status st;
  if ((st = ensure_ws(ctx, 256 + 65536 * sizeof(ClusterAcc))) != QPSO_OK) return st;
  QPSO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  char* d = static_cast<char*>(ctx->ws.p);
  int32_t maxl = -1;
  QPSO_CUDA(ctx, launch_label_max(f.labels, (uint32_t)W * (uint32_t)H, reinterpret_cast<int32_t*>(d),
                                  ctx->stream));
  QPSO_CUDA(ctx, cudaMemcpyAsync(&maxl, d, 4, cudaMemcpyDeviceToHost, ctx->stream));
  QPSO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (maxl > 65535) return fail(ctx, QPSO_ERR_ARG, "label above 65535");
  std::vector<ClusterAcc> acc((size_t)(maxl + 1));
  if (maxl >= 0) {
    ClusterAcc* da = reinterpret_cast<ClusterAcc*>(d + 256);
    QPSO_CUDA(ctx, launch_cluster_stats(f.depth, f.labels, W, H, da, maxl + 1, ctx->stream));
    QPSO_CUDA(ctx, cudaMemcpyAsync(acc.data(), da, acc.size() * sizeof(ClusterAcc), cudaMemcpyDeviceToHost,
                                   ctx->stream));
    QPSO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  uint32_t n = 0;
  for (int32_t l = 0; l <= maxl; ++l) {
    const ClusterAcc& a = acc[(size_t)l];
    if (a.n == 0) continue;
    if (out && n < capacity) {
      qpso_cluster& c = out[n];
      c.label = l;
      c.num_points = a.n;
      c.min_x = a.minx;
      c.max_x = a.maxx;
      c.min_y = a.miny;
      c.max_y = a.maxy;
      c.depth_points = a.nz;
      if (a.nz) {
        const double sz = (double)a.sum_z;
        double k[4];
        camera_intrinsics(f.cam, k);
        c.centroid_mm[0] = (float)(((double)a.sum_xz - k[2] * sz) / (k[0] * a.nz));
        c.centroid_mm[1] = (float)(((double)a.sum_yz - k[3] * sz) / (k[1] * a.nz));
        c.centroid_mm[2] = (float)(sz / a.nz);
      } else {
        c.centroid_mm[0] = c.centroid_mm[1] = c.centroid_mm[2] = 0.f;
      }
    }
    ++n;
  }
  *n_clusters = n;
  if (out && n > capacity) return fail(ctx, QPSO_ERR_ARG, "more clusters than capacity");
  return QPSO_OK;
}

qpso_status qpso_render_depth_f32(qpso_context* ctx, uint32_t mesh_id, const qpso_camera* cam,
                                  const float pose[7], float* depth_out) {
  if (!ctx || !cam || !pose || !depth_out || cam->width <= 0 || cam->height <= 0 ||
      (int64_t)cam->width * cam->height > (1 << 26) || !projection_ok(cam))
    return fail(ctx, QPSO_ERR_ARG, "bad render arguments");
  auto mi = ctx->meshes.find(mesh_id);
  if (mi == ctx->meshes.end()) return fail(ctx, QPSO_ERR_NOT_FOUND, "unknown mesh id");
  cudaSetDevice(ctx->device);
  const size_t bytes = (size_t)cam->width * cam->height * sizeof(float);
  qpso_status st;
  if ((st = ensure_ws(ctx, bytes)) != QPSO_OK) return st;
  QPSO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  float* d = static_cast<float*>(ctx->ws.p);
  const Camera c{cam->fx, cam->fy, cam->cx, cam->cy, cam->width, cam->height, cam->projection};
  QPSO_CUDA(ctx, launch_host_render(mi->second.d, mi->second.F, pose, c, d, ctx->stream));
  QPSO_CUDA(ctx, cudaMemcpyAsync(depth_out, d, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  QPSO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return QPSO_OK;
}

qpso_status qpso_barrier_selftest(qpso_context* ctx, uint64_t timeout_ns, uint32_t* err_bits) {
  if (!ctx || !err_bits || timeout_ns == 0 || timeout_ns > 10ull * 1000 * 1000 * 1000)
    return fail(ctx, QPSO_ERR_ARG, "timeout must be in (0, 10 s]");
  cudaSetDevice(ctx->device);
  qpso_status st;
  if ((st = ensure_ws(ctx, 256)) != QPSO_OK) return st;
  if ((st = ensure_pin(ctx, 16)) != QPSO_OK) return st;
  QPSO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  char* d = static_cast<char*>(ctx->ws.p);
  cudaStream_t s = ctx->stream;
  // a queue of one entry that is never appended (ready stays 0): both CTAs'
  // claims must wait out the limit
  QCtl* qc = reinterpret_cast<QCtl*>(d);
  QEntry* q = reinterpret_cast<QEntry*>(d + 64);
  uint32_t* err = reinterpret_cast<uint32_t*>(d + 128);
  QPSO_CUDA(ctx, cudaMemsetAsync(d, 0, 256, s));
  const uint32_t total = 1u;
  QPSO_CUDA(ctx, cudaMemcpyAsync(&qc->total, &total, sizeof(total), cudaMemcpyHostToDevice, s));
  QPSO_CUDA(ctx, launch_queue_probe(qc, q, err, 2, timeout_ns, s));
  QPSO_CUDA(ctx, cudaMemcpyAsync(ctx->pin.p, err, 4, cudaMemcpyDeviceToHost, s));
  QPSO_CUDA(ctx, cudaStreamSynchronize(s));
  *err_bits = *static_cast<uint32_t*>(ctx->pin.p);
  return (*err_bits & kErrTimeout) ? QPSO_ERR_TIMEOUT : QPSO_OK;
}

// ---- segmentation: the graph stage of GraphCannySeg ----

void qpso_seg_params_init(qpso_seg_params* p) {
  if (!p) return;
  p->sigma = 0.8f;
  p->k = (float)50 / 10000.f;
  p->min_size = 500.0f;
  p->kx = (float)2000 / 1000.f;
  p->ky = (float)30 / 1000.f;
  p->ks = (float)49 / 1000.f;
  p->kdv = 4.5f;
  p->kdc = 0.1f;
}

uint64_t qpso_segment_num_edges(uint32_t width, uint32_t height) {
  if (width == 0 || height == 0 || (uint64_t)width * height > (1u << 26)) return 0;
  return seg_num_edges((int32_t)width, (int32_t)height);
}

qpso_status qpso_segment_edge_ends(uint32_t width, uint32_t height, int32_t* a, int32_t* b) {
  if (!a || !b || width == 0 || height == 0 || (uint64_t)width * height > (1u << 26)) return QPSO_ERR_ARG;
  seg_edge_ends((int32_t)width, (int32_t)height, a, b);
  return QPSO_OK;
}

int32_t qpso_segment_gauss_mask(float sigma, float* mask, int32_t capacity) {
  if (!mask || capacity <= 0 || std::isnan(sigma)) return -1;
  return seg_gauss_mask(sigma, mask, capacity);
}

}  // extern "C"

namespace {

bool seg_params_ok(const qpso_seg_params* p) {
  float m[32];
  return p && std::isfinite(p->sigma) && std::isfinite(p->k) && std::isfinite(p->min_size) &&
         std::isfinite(p->kx) && std::isfinite(p->ks) && std::isfinite(p->kdv) && std::isfinite(p->kdc) &&
         seg_gauss_mask(p->sigma, m, 32) > 0;
}

}  // namespace

extern "C" {

qpso_status qpso_segment_edges(uint32_t width, uint32_t height, const float* weights, const qpso_seg_params* prm,
                               int32_t* labels, uint32_t* n_clusters) {
  if (!weights || !labels || !n_clusters || !seg_params_ok(prm) || width == 0 || height == 0 ||
      (uint64_t)width * height > (1u << 26))
    return QPSO_ERR_ARG;
  const int32_t W = (int32_t)width, H = (int32_t)height;
  const uint64_t E = seg_num_edges(W, H);
  for (uint64_t e = 0; e < E; ++e)
    if (std::isnan(weights[e])) return QPSO_ERR_ARG;
  std::vector<int32_t> ea(E), eb(E);
  seg_edge_ends(W, H, ea.data(), eb.data());
  // ascending weight, equal weights by edge index
  std::vector<uint32_t> order(E);
  for (uint64_t e = 0; e < E; ++e) order[e] = (uint32_t)e;
  std::stable_sort(order.begin(), order.end(), [&](uint32_t i, uint32_t j) { return weights[i] < weights[j]; });
  *n_clusters = seg_merge((uint32_t)(W * H), E, order.data(), ea.data(), eb.data(), weights, prm->k,
                          prm->min_size, labels);
  return QPSO_OK;
}

qpso_status qpso_segment_planes(qpso_context* ctx, const uint8_t* h, const uint8_t* s, const uint8_t* v,
                                const uint16_t* depth_mm, const float* saliency, uint32_t width, uint32_t height,
                                const qpso_seg_params* prm, int32_t* labels, float* edge_weights,
                                uint32_t* n_clusters) {
  if (!ctx || !h || !s || !v || !depth_mm || !saliency || !labels || !n_clusters || width == 0 || height == 0 ||
      (uint64_t)width * height > (1u << 26))
    return fail(ctx, QPSO_ERR_ARG, "bad segmentation arguments");
  if (!seg_params_ok(prm)) return fail(ctx, QPSO_ERR_ARG, "bad segmentation parameters (sigma above 7.75?)");
  const int32_t W = (int32_t)width, H = (int32_t)height;
  const uint64_t E = seg_num_edges(W, H);
  float mask[32];
  const int len = seg_gauss_mask(prm->sigma, mask, 32);
  cudaSetDevice(ctx->device);
  qpso_status st;
  if ((st = ensure_ws(ctx, seg_workspace_bytes(W, H))) != QPSO_OK) return st;
  QPSO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (!edge_weights) {
    if ((st = ensure_segpin(ctx, seg_merge_pinned_bytes(W, H))) != QPSO_OK) return st;
    const uint8_t* hsv[3] = {h, s, v};
    uint32_t err = 0;
    QPSO_CUDA(ctx, seg_graph_merge(hsv, depth_mm, saliency, W, H, mask, len, prm->kdv, prm->kdc, prm->kx, prm->ks,
                                   ctx->ws.p, ctx->num_sms, ctx->stream, ctx->segpin.p, ctx->seg_ev, kSegChunks,
                                   prm->k, prm->min_size, labels, n_clusters, &err, nullptr));
    if (err & 5u) return fail(ctx, QPSO_ERR_INTERNAL, "segmentation graph: index out of range");
    if (err & 2u)
      return fail(ctx, QPSO_ERR_ARG, "segmentation graph: NaN edge weight (depth range zero, or NaN saliency)");
    return QPSO_OK;
  }
  std::vector<uint32_t> order(E);
  std::vector<int32_t> ea(E), eb(E);
  std::vector<float> w(E);
  uint32_t err = 0;
  const uint8_t* hsv[3] = {h, s, v};
  QPSO_CUDA(ctx, seg_graph_sorted(hsv, depth_mm, saliency, W, H, mask, len, prm->kdv, prm->kdc, prm->kx, prm->ks,
                                  ctx->ws.p, ctx->num_sms, ctx->stream, order.data(), ea.data(), eb.data(),
                                  w.data(), &err));
  if (err & 5u) return fail(ctx, QPSO_ERR_INTERNAL, "segmentation graph: index out of range");
  if (err & 2u)
    return fail(ctx, QPSO_ERR_ARG, "segmentation graph: NaN edge weight (depth range zero, or NaN saliency)");
  if (edge_weights) std::memcpy(edge_weights, w.data(), sizeof(float) * E);
  *n_clusters = seg_merge((uint32_t)(W * H), E, order.data(), ea.data(), eb.data(), w.data(), prm->k,
                          prm->min_size, labels);
  return QPSO_OK;
}

void qpso_seg_front_params_init(qpso_seg_front_params* p) {
  if (!p) return;
  p->beta = 2000.0f;
  p->gamma = 18000.0f;
  p->inpaint_radius = 20;
  p->canny_low = (float)50 / 1000.f;
  p->canny_high = (float)75 / 1000.f;
  p->dth = 30;
  p->plus_d = 7;
  p->point_3d = 5;
  // ((float)angle) * deg2rad with deg2rad = M_PI / 180.0f (GraphCannySeg.h:39): double arithmetic
  p->g_angle = (float)((double)148.0f * 3.14159265358979323846 / 180.0);
  p->l_angle = (float)((double)151.0f * 3.14159265358979323846 / 180.0);
  p->fx = 572.41140f;
  p->fy = 573.57043f;
  p->cx = 325.26110f;
  p->cy = 242.04899f;
  p->far_obj_z = 1500.0f;
  p->max_ecc = 0.978f;
  p->max_l1 = 13800.0f;
  p->max_l2 = 1950.0f;
}

}  // extern "C"

namespace {

bool front_params_ok(const qpso_seg_front_params* f) {
  return f && std::isfinite(f->beta) && std::isfinite(f->gamma) && f->inpaint_radius >= 1 &&
         f->inpaint_radius <= 64 && std::isfinite(f->canny_low) && std::isfinite(f->canny_high) && f->dth >= 0 &&
         f->plus_d >= 1 && f->point_3d >= 1 && f->plus_d <= 64 && f->point_3d <= 64 && std::isfinite(f->g_angle) &&
         std::isfinite(f->l_angle) && std::isfinite(f->fx) && f->fx != 0.0f && std::isfinite(f->fy) &&
         f->fy != 0.0f && std::isfinite(f->cx) && std::isfinite(f->cy) && std::isfinite(f->far_obj_z) &&
         std::isfinite(f->max_ecc) && std::isfinite(f->max_l1) && std::isfinite(f->max_l2);
}

// capacity of the per-set moment table: after the small-component merge
// every set holds at least min_size pixels, unless the frame is one set
size_t max_sets(size_t n, float min_size) {
  if (!(min_size >= 1.0f)) return n;
  const size_t m = (size_t)((double)n / (double)min_size) + 1;
  return m < n ? m : n;
}

// Per-set moments on the GPU and the cluster records on the host.  labels,
// inpainted depth and value plane are device pointers; moments has room
// for n_sets records.
qpso_status cluster_records(qpso_context* ctx, const int32_t* d_labels, const uint16_t* d_inp, const uint8_t* d_v,
                            int32_t W, int32_t H, uint32_t n_sets, SetMoments* d_mom,
                            const qpso_seg_front_params* fp, int keep_all, qpso_seg_cluster* out,
                            uint32_t capacity, uint32_t* n_out) {
  std::vector<SetMoments> mom(n_sets);
  QPSO_CUDA(ctx, launch_set_moments(d_labels, d_inp, d_v, W, H, (int32_t)n_sets, d_mom, ctx->num_sms, ctx->stream));
  if (n_sets)
    QPSO_CUDA(ctx, cudaMemcpyAsync(mom.data(), d_mom, n_sets * sizeof(SetMoments), cudaMemcpyDeviceToHost,
                                   ctx->stream));
  QPSO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  uint32_t k = 0;
  for (uint32_t i = 0; i < n_sets; ++i) {
    if (mom[i].n == 0) continue;
    qpso_seg_cluster r;
    seg_cluster_record(mom[i], (int32_t)i, *fp, &r);
    if (!keep_all && !r.kept) continue;
    if (out && k < capacity) out[k] = r;
    ++k;
  }
  *n_out = k;
  return QPSO_OK;
}

}  // namespace

extern "C" {

qpso_status qpso_segment_rgbd(qpso_context* ctx, const uint8_t* bgr, const uint16_t* depth_mm, uint32_t width,
                              uint32_t height, const qpso_seg_params* prm, const qpso_seg_front_params* fp,
                              int32_t* labels, uint32_t* n_sets, qpso_seg_cluster* clusters, uint32_t capacity,
                              uint32_t* n_clusters, const qpso_seg_frame_out* planes) {
  if (!ctx || !bgr || !depth_mm || !labels || !n_sets || !n_clusters || width < 3 || height < 3 ||
      (uint64_t)width * height > (1u << 26))
    return fail(ctx, QPSO_ERR_ARG, "bad segmentation arguments");
  if (!seg_params_ok(prm)) return fail(ctx, QPSO_ERR_ARG, "bad segmentation parameters (sigma above 7.75?)");
  if (!front_params_ok(fp)) return fail(ctx, QPSO_ERR_ARG, "bad front-stage segmentation parameters");
  const int32_t W = (int32_t)width, H = (int32_t)height;
  const size_t n = (size_t)W * H;
  const uint64_t E = seg_num_edges(W, H);
  float mask[32];
  const int len = seg_gauss_mask(prm->sigma, mask, 32);
  cudaSetDevice(ctx->device);
  const size_t graph_bytes = align_up(seg_workspace_bytes(W, H), 256);
  const size_t front_bytes = align_up(seg_front_workspace_bytes(W, H, fp->inpaint_radius), 256);
  const size_t label_bytes = align_up(n * sizeof(int32_t), 256);
  const size_t mom_bytes = align_up(max_sets(n, prm->min_size) * sizeof(SetMoments), 256);
  qpso_status st;
  if ((st = ensure_ws(ctx, graph_bytes + front_bytes + label_bytes + mom_bytes)) != QPSO_OK) return st;
  QPSO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  char* base = static_cast<char*>(ctx->ws.p);
  char* front_ws = base + graph_bytes;
  int32_t* d_labels = reinterpret_cast<int32_t*>(front_ws + front_bytes);
  SetMoments* d_mom = reinterpret_cast<SetMoments*>(front_ws + front_bytes + label_bytes);
  uint8_t* d_hsv = nullptr;
  uint16_t* d_depth = nullptr;
  float* d_sal = nullptr;
  seg_ws_inputs(base, W, H, &d_hsv, &d_depth, &d_sal);
  SegFrontArgs a{};
  a.bgr_host = bgr;
  a.depth_host = depth_mm;
  a.W = W;
  a.H = H;
  a.beta = fp->beta;
  a.gamma = fp->gamma;
  a.radius = fp->inpaint_radius;
  a.canny_low = fp->canny_low;
  a.canny_high = fp->canny_high;
  a.dth = fp->dth;
  a.plus_d = fp->plus_d;
  a.point_3d = fp->point_3d;
  a.g_angle = fp->g_angle;
  a.l_angle = fp->l_angle;
  a.fx = fp->fx;
  a.fy = fp->fy;
  a.cx = fp->cx;
  a.cy = fp->cy;
  a.hsv_out = d_hsv;
  a.inpainted_out = d_depth;
  a.saliency_out = d_sal;
  if (planes) {
    a.gray_host = planes->gray;
    a.smoothed_host = planes->smoothed;
    a.edges_host = planes->edges;
  }
  if ((st = ensure_segpin(ctx, seg_merge_pinned_bytes(W, H))) != QPSO_OK) return st;
  uint32_t* front_err = reinterpret_cast<uint32_t*>(static_cast<char*>(ctx->segpin.p) + 32);
  *front_err = 0u;
  a.err_pinned = front_err;
  QPSO_CUDA(ctx, seg_front_run(a, front_ws, ctx->num_sms, (size_t)ctx->smem_optin, ctx->stream));
  if (planes) {
    uint8_t* hp[3] = {planes->h, planes->s, planes->v};
    for (int c = 0; c < 3; ++c)
      if (hp[c]) QPSO_CUDA(ctx, cudaMemcpyAsync(hp[c], d_hsv + c * n, n, cudaMemcpyDeviceToHost, ctx->stream));
    if (planes->inpainted)
      QPSO_CUDA(ctx, cudaMemcpyAsync(planes->inpainted, d_depth, 2 * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (planes->saliency)
      QPSO_CUDA(ctx, cudaMemcpyAsync(planes->saliency, d_sal, 4 * n, cudaMemcpyDeviceToHost, ctx->stream));
  }
  uint32_t err = 0, ns = 0;
  QPSO_CUDA(ctx, seg_graph_merge(nullptr, nullptr, nullptr, W, H, mask, len, prm->kdv, prm->kdc, prm->kx, prm->ks,
                                 base, ctx->num_sms, ctx->stream, ctx->segpin.p, ctx->seg_ev, kSegChunks, prm->k,
                                 prm->min_size, labels, &ns, &err, d_labels));
  // the front's error word was copied before the graph stage, which has
  // synchronised with the stream since
  if (*front_err) return fail(ctx, QPSO_ERR_TIMEOUT, "segmentation: the inpainting fill's grid barrier timed out");
  if (err & 5u) return fail(ctx, QPSO_ERR_INTERNAL, "segmentation graph: index out of range");
  if (err & 2u) return fail(ctx, QPSO_ERR_ARG, "segmentation graph: NaN edge weight (flat inpainted depth?)");
  *n_sets = ns;
  if ((size_t)ns * sizeof(SetMoments) > mom_bytes)
    return fail(ctx, QPSO_ERR_INTERNAL, "segmentation: more sets than the small-component merge allows");
  // the merge left the labels in d_labels as well
  return cluster_records(ctx, d_labels, d_depth, d_hsv + 2 * n, W, H, ns, d_mom, fp, 0, clusters, capacity,
                         n_clusters);
}

qpso_status qpso_segment_clusters(qpso_context* ctx, const int32_t* labels, uint32_t n_sets,
                                  const uint16_t* inpainted_mm, const uint8_t* v_plane, uint32_t width,
                                  uint32_t height, const qpso_seg_front_params* fp, int keep_all,
                                  qpso_seg_cluster* out, uint32_t capacity, uint32_t* n_out) {
  if (!ctx || !labels || !inpainted_mm || !v_plane || !n_out || width == 0 || height == 0 ||
      (uint64_t)width * height > (1u << 26) || n_sets > width * height)
    return fail(ctx, QPSO_ERR_ARG, "bad cluster-filter arguments");
  if (!front_params_ok(fp)) return fail(ctx, QPSO_ERR_ARG, "bad front-stage segmentation parameters");
  const int32_t W = (int32_t)width, H = (int32_t)height;
  const size_t n = (size_t)W * H;
  cudaSetDevice(ctx->device);
  const size_t lb = align_up(4 * n, 256), zb = align_up(2 * n, 256), vb = align_up(n, 256);
  qpso_status st;
  if ((st = ensure_ws(ctx, lb + zb + vb + align_up((size_t)n_sets * sizeof(SetMoments), 256) + 256)) != QPSO_OK)
    return st;
  QPSO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  char* base = static_cast<char*>(ctx->ws.p);
  int32_t* d_lab = reinterpret_cast<int32_t*>(base);
  uint16_t* d_z = reinterpret_cast<uint16_t*>(base + lb);
  uint8_t* d_v = reinterpret_cast<uint8_t*>(base + lb + zb);
  SetMoments* d_mom = reinterpret_cast<SetMoments*>(base + lb + zb + vb);
  QPSO_CUDA(ctx, cudaMemcpyAsync(d_lab, labels, 4 * n, cudaMemcpyHostToDevice, ctx->stream));
  QPSO_CUDA(ctx, cudaMemcpyAsync(d_z, inpainted_mm, 2 * n, cudaMemcpyHostToDevice, ctx->stream));
  QPSO_CUDA(ctx, cudaMemcpyAsync(d_v, v_plane, n, cudaMemcpyHostToDevice, ctx->stream));
  return cluster_records(ctx, d_lab, d_z, d_v, W, H, n_sets, d_mom, fp, keep_all, out, capacity, n_out);
}

}  // extern "C"

// ===========================================================================
// Serving: continuous batching of solve requests.

namespace {

using Clock = std::chrono::steady_clock;

struct ServerReq {
  qpso_solve_desc desc;
  Clock::time_point t_submit, t_done;
  int state = 0;  // 0 queued, 1 active, 2 done, 3 failed
  qpso_status status = QPSO_OK;
  qpso_result result{};
  int slot = -1;
  void* dmem = nullptr;
  size_t bytes = 0;
  uint32_t remaining = 0;
  int vcap = 64;  // meshlet size of its mesh
  double cost = 0.0;  // render cost of one particle, for the order of work items
  int var = 0;  // fused-kernel variant it needs (kernel_variant)
};

size_t request_bytes(const qpso_solve_desc& d, const qpso_camera& c) {
  const size_t P = d.num_particles;
  return align_up((size_t)c.width * c.height * 2, 256) +
         align_up((size_t)(c.width + 1) * (c.height + 1) * 4, 256) + 3 * align_up(7 * P * 4, 256) +
         2 * align_up(P * 4, 256);
}

}  // namespace

struct qpso_server {
  qpso_context* ctx = nullptr;
  cudaStream_t stream = nullptr;
  cudaMemPool_t pool = nullptr;
  qpso_server_config cfg{};
  TileConfig tc{};
  std::thread th;
  std::mutex mu;
  std::condition_variable cv, cv_done;
  bool stop = false;
  std::deque<uint64_t> queue;
  std::unordered_map<uint64_t, ServerReq> reqs;
  uint64_t next_id = 1;
  // device slots
  Instance* d_slots = nullptr;
  Header* d_hdr = nullptr;
  PrepDesc* d_prep = nullptr;
  // an epoch's dataflow queue: at most iters_per_epoch entries per slot
  QEntry* d_queue = nullptr;
  QCtl* d_qctl = nullptr;
  uint32_t* d_end = nullptr;     // per slot: the epoch's last iteration + 1
  uint32_t* d_berr = nullptr;
  Instance* h_slots = nullptr;  // pinned staging
  Header* h_hdr = nullptr;
  PrepDesc* h_prep = nullptr;
  QEntry* h_qinit = nullptr;    // the epoch's first entries, one per active slot
  QCtl* h_qctl = nullptr;
  uint32_t* h_end = nullptr;
  uint32_t* h_berr = nullptr;
  std::vector<int> free_slots;
  std::vector<uint64_t> slot_req;
  qpso_server_stats st{};
  std::string err;
};

namespace {

void server_fail_all(qpso_server* s, qpso_status code, const std::string& why) {
  std::lock_guard<std::mutex> g(s->mu);
  for (auto& kv : s->reqs)
    if (kv.second.state < 2) {
      kv.second.state = 3;
      kv.second.status = code;
      kv.second.t_done = Clock::now();
      s->st.failed++;
    }
  s->queue.clear();
  s->err = why;
  s->cv_done.notify_all();
}

void server_loop(qpso_server* s) {
  qpso_context* ctx = s->ctx;
  cudaSetDevice(ctx->device);
  const uint32_t S = s->cfg.max_slots;
  std::vector<int> active;  // slots in use
  for (;;) {
    std::vector<int> admitted;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv.wait(lk, [&] { return s->stop || !s->queue.empty() || !active.empty(); });
      if (s->stop && s->queue.empty() && active.empty()) break;
      // admission: free slots and memory budget, first come first served
      while (!s->queue.empty() && !s->free_slots.empty()) {
        const uint64_t rid = s->queue.front();
        ServerReq& r = s->reqs[rid];
        const FrameObj* f = nullptr;
        const MeshObj* m = nullptr;
        {
          std::lock_guard<std::mutex> g(ctx->mu);
          auto fi = ctx->frames.find(r.desc.frame_id);
          auto mi = ctx->meshes.find(r.desc.mesh_id);
          if (fi != ctx->frames.end()) f = &fi->second;
          if (mi != ctx->meshes.end()) m = &mi->second;
        }
        if (!f || !m) {
          r.state = 3;
          r.status = QPSO_ERR_NOT_FOUND;
          r.t_done = Clock::now();
          s->st.failed++;
          s->queue.pop_front();
          s->cv_done.notify_all();
          continue;
        }
        const size_t need = request_bytes(r.desc, f->cam);
        if (s->st.bytes_in_use + need > s->st.budget_bytes) break;  // wait for memory
        void* mem = nullptr;
        if (cudaMallocFromPoolAsync(&mem, need, s->pool, s->stream) != cudaSuccess) break;
        const int slot = s->free_slots.back();
        s->free_slots.pop_back();
        s->queue.pop_front();
        r.slot = slot;
        r.dmem = mem;
        r.bytes = need;
        r.state = 1;
        r.remaining = r.desc.iterations;
        r.vcap = m->mlet_cap;
        r.cost = (double)m->F * 3.0 + (double)(r.desc.cl_max_x - r.desc.cl_min_x) *
                                          (double)(r.desc.cl_max_y - r.desc.cl_min_y);
        r.var = kernel_variant(r.desc, f->cam);
        s->slot_req[slot] = rid;
        s->st.bytes_in_use += need;
        s->st.peak_bytes = std::max(s->st.peak_bytes, s->st.bytes_in_use);
        s->st.admitted++;
        // instance record of the slot
        char* d = static_cast<char*>(mem);
        Instance& I = s->h_slots[slot];
        std::memset(&I, 0, sizeof(I));
        I.mesh = m->d;
        I.F = m->F;
        I.mlets = m->mlets;
        I.mlet_blob = m->blob;
        I.mlet_box = reinterpret_cast<const float4*>(m->blob + m->box_off);
        I.n_mlets = m->n_mlets;
        for (int k = 0; k < 3; ++k) {
          I.mesh_lo[k] = m->lo[k];
          I.mesh_hi[k] = m->hi[k];
        }
        const qpso_camera& c = f->cam;
        const size_t P = r.desc.num_particles;
        size_t o = 0;
        I.obs = reinterpret_cast<const uint16_t*>(d + o);
        uint16_t* obs = reinterpret_cast<uint16_t*>(d + o);
        o += align_up((size_t)c.width * c.height * 2, 256);
        I.sat = reinterpret_cast<const int32_t*>(d + o);
        int32_t* sat = reinterpret_cast<int32_t*>(d + o);
        o += align_up((size_t)(c.width + 1) * (c.height + 1) * 4, 256);
        I.pos = reinterpret_cast<float*>(d + o);
        o += align_up(7 * P * 4, 256);
        I.vel = reinterpret_cast<float*>(d + o);
        o += align_up(7 * P * 4, 256);
        I.pbest = reinterpret_cast<float*>(d + o);
        o += align_up(7 * P * 4, 256);
        I.pbest_fit = reinterpret_cast<float*>(d + o);
        o += align_up(P * 4, 256);
        I.fit = reinterpret_cast<float*>(d + o);
        I.cam = Camera{c.fx, c.fy, c.cx, c.cy, c.width, c.height, c.projection};
        I.prm = to_params(r.desc);
        Header* dh = s->d_hdr + slot;
        I.gbest = dh->gbest;
        I.done = &dh->done;
        I.err = &dh->err;
        I.stats = dh->stats;
        I.argkey = &dh->argkey;
        I.trace = nullptr;
        I.ppb = (uint32_t)s->tc.ppb;
        I.chunks = (uint32_t)((P + s->tc.ppb - 1) / s->tc.ppb);
        I.cur_iter = 0;
        Header& hh = s->h_hdr[slot];
        std::memset(&hh, 0, sizeof(hh));
        hh.gbest[0] = kBestInit;
        hh.argkey = ~0ull;
        PrepDesc& pj = s->h_prep[admitted.size()];
        pj.depth = f->depth;
        pj.labels = r.desc.cluster_label >= 0 ? f->labels : nullptr;
        pj.label = r.desc.cluster_label;
        pj.width = c.width;
        pj.height = c.height;
        pj.obs = obs;
        pj.sat = sat;
        admitted.push_back(slot);
      }
      s->st.pending = (uint32_t)s->queue.size();
    }
    cudaError_t e = cudaSuccess;
    int max_w = 0, max_h = 0;
    for (size_t i = 0; i < admitted.size(); ++i) {
      const int slot = admitted[i];
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->d_slots + slot, s->h_slots + slot, sizeof(Instance), cudaMemcpyHostToDevice,
                            s->stream);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->d_hdr + slot, s->h_hdr + slot, sizeof(Header), cudaMemcpyHostToDevice,
                            s->stream);
      max_w = std::max(max_w, s->h_prep[i].width);
      max_h = std::max(max_h, s->h_prep[i].height);
      active.push_back(slot);
    }
    if (!admitted.empty()) {
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->d_prep, s->h_prep, admitted.size() * sizeof(PrepDesc), cudaMemcpyHostToDevice,
                            s->stream);
      if (e == cudaSuccess) e = launch_prep(s->d_prep, (int)admitted.size(), max_w, max_h, s->stream);
    }
    if (active.empty()) {
      if (e != cudaSuccess) server_fail_all(s, QPSO_ERR_CUDA, cudaGetErrorString(e));
      continue;
    }
    // the epoch: every active request advances by up to iters_per_epoch
    // iterations, each at its own pace, in one launch of the dataflow
    // queue; the queue starts with the requests' current iterations, the
    // most expensive requests first so that no large render starts last
    const uint32_t E = s->cfg.iters_per_epoch;
    int var = 0;
    int vcap = 64;
    uint32_t n_init = 0, total = 0;
    uint64_t all_chunks = 0;
    std::vector<uint32_t> ran(S, 0);
    {
      std::lock_guard<std::mutex> g(s->mu);
      std::vector<int> order(active);
      std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return s->reqs[s->slot_req[a]].cost > s->reqs[s->slot_req[b]].cost;
      });
      for (int slot : order) {
        const ServerReq& r = s->reqs[s->slot_req[slot]];
        var = std::max(var, r.var);
        vcap = std::max(vcap, r.vcap);
        const uint32_t start = r.desc.iterations - r.remaining;
        const uint32_t end = start + std::min(E, r.remaining);
        ran[slot] = end - start;
        s->h_end[slot] = end;
        s->h_qinit[n_init++] = QEntry{(uint32_t)slot, start, 0u, 1u};
        total += end - start;
        all_chunks += s->h_slots[slot].chunks;
      }
    }
    *s->h_qctl = QCtl{0u, n_init, total, 0u};
    *s->h_berr = 0u;
    TileConfig tc = s->tc;  // fits every vcap (checked at submit)
    shrink_cfg(tc, vcap, s->ctx->smem_optin);
    int per_sm = 0;
    if (e == cudaSuccess) e = epoch_max_grid(tc, var, vcap, &per_sm);
    if (e == cudaSuccess && per_sm <= 0) e = cudaErrorInvalidConfiguration;
    const int grid = (int)std::min<uint64_t>(all_chunks, (uint64_t)std::max(per_sm, 1) * s->ctx->num_sms);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(s->d_end, s->h_end, S * sizeof(uint32_t), cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->d_queue, 0, (size_t)total * sizeof(QEntry), s->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(s->d_queue, s->h_qinit, n_init * sizeof(QEntry), cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->d_qctl, s->h_qctl, sizeof(QCtl), cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(s->d_berr, s->h_berr, sizeof(uint32_t), cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) {
      BatchArgs A;
      A.inst = s->d_slots;
      A.queue = s->d_queue;
      A.qctl = s->d_qctl;
      A.err = s->d_berr;
      A.timeout_ns = 20ull * 1000 * 1000 * 1000;  // 20 s per wait for work
      e = launch_epoch(A, s->d_end, grid, tc, s->stream, var, vcap);
    }
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(s->h_hdr, s->d_hdr, S * sizeof(Header), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(s->h_berr, s->d_berr, sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess && *s->h_berr != 0u) {
      server_fail_all(s, QPSO_ERR_TIMEOUT, "serving epoch: a bounded wait for work expired");
      active.clear();
      continue;
    }
    if (e != cudaSuccess) {
      server_fail_all(s, QPSO_ERR_CUDA, cudaGetErrorString(e));
      active.clear();
      continue;
    }
    std::lock_guard<std::mutex> g(s->mu);
    s->st.epochs++;
    s->st.launches += 1;
    std::vector<int> still;
    for (int slot : active) {
      ServerReq& r = s->reqs[s->slot_req[slot]];
      r.remaining -= ran[slot];
      if (r.remaining > 0) {
        still.push_back(slot);
        continue;
      }
      read_result(s->h_hdr[slot], &r.result);
      r.status = (s->h_hdr[slot].err & kErrBound) ? QPSO_ERR_INTERNAL : QPSO_OK;
      r.state = 2;
      r.t_done = Clock::now();
      cudaFreeAsync(r.dmem, s->stream);
      s->st.bytes_in_use -= r.bytes;
      s->st.completed++;
      s->free_slots.push_back(slot);
    }
    active.swap(still);
    s->st.active = (uint32_t)active.size();
    s->st.peak_active = std::max(s->st.peak_active, s->st.active);
    s->cv_done.notify_all();
  }
}

}  // namespace

extern "C" {

qpso_status qpso_server_start(qpso_context* ctx, const qpso_server_config* cfg, qpso_server** out) {
  if (!ctx || !cfg || !out || cfg->max_slots == 0 || cfg->max_slots > 65536 || cfg->iters_per_epoch == 0)
    return fail(ctx, QPSO_ERR_ARG, "bad server config");
  cudaSetDevice(ctx->device);
  qpso_server* s = new (std::nothrow) qpso_server();
  if (!s) return QPSO_ERR_NOMEM;
  s->ctx = ctx;
  s->cfg = *cfg;
  s->tc = ctx->batch;
  const uint32_t S = cfg->max_slots;
  const size_t max_entries = (size_t)S * cfg->iters_per_epoch;
  cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = ctx->device;
  if (e == cudaSuccess) e = cudaMemPoolCreate(&s->pool, &props);
  if (e == cudaSuccess) {
    uint64_t keep = UINT64_MAX;
    e = cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  if (e == cudaSuccess) e = cudaMalloc(&s->d_slots, S * sizeof(Instance));
  if (e == cudaSuccess) e = cudaMalloc(&s->d_hdr, S * sizeof(Header));
  if (e == cudaSuccess) e = cudaMalloc(&s->d_prep, S * sizeof(PrepDesc));
  if (e == cudaSuccess) e = cudaMalloc(&s->d_queue, max_entries * sizeof(QEntry));
  if (e == cudaSuccess) e = cudaMalloc(&s->d_qctl, sizeof(QCtl));
  if (e == cudaSuccess) e = cudaMalloc(&s->d_end, S * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&s->d_berr, sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMallocHost(&s->h_slots, S * sizeof(Instance));
  if (e == cudaSuccess) e = cudaMallocHost(&s->h_hdr, S * sizeof(Header));
  if (e == cudaSuccess) e = cudaMallocHost(&s->h_prep, S * sizeof(PrepDesc));
  if (e == cudaSuccess) e = cudaMallocHost(&s->h_qinit, S * sizeof(QEntry));
  if (e == cudaSuccess) e = cudaMallocHost(&s->h_qctl, sizeof(QCtl));
  if (e == cudaSuccess) e = cudaMallocHost(&s->h_end, S * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMallocHost(&s->h_berr, sizeof(uint32_t));
  size_t free_b = 0, total_b = 0;
  if (e == cudaSuccess) e = cudaMemGetInfo(&free_b, &total_b);
  if (e != cudaSuccess) {
    qpso_server_stop(s);
    return cuda_fail(ctx, e, "server start");
  }
  s->st.budget_bytes = cfg->hbm_budget_bytes ? cfg->hbm_budget_bytes : free_b / 2;
  s->free_slots.reserve(S);
  for (int i = (int)S - 1; i >= 0; --i) s->free_slots.push_back(i);
  s->slot_req.assign(S, 0);
  s->th = std::thread(server_loop, s);
  *out = s;
  return QPSO_OK;
}

qpso_status qpso_server_submit(qpso_server* s, const qpso_solve_desc* desc, uint64_t* id) {
  if (!s || !desc || !id) return QPSO_ERR_ARG;
  const MeshObj* m;
  const FrameObj* f;
  qpso_status st;
  {
    std::lock_guard<std::mutex> g(s->ctx->mu);
    st = check_desc(s->ctx, *desc, &m, &f);
  }
  if (st != QPSO_OK) return st;
  TileConfig fit = s->tc;
  if (!shrink_cfg(fit, m->mlet_cap, s->ctx->smem_optin))
    return fail(s->ctx, QPSO_ERR_ARG, "the server's launch config cannot fit this mesh's vertex caches");
  if (request_bytes(*desc, f->cam) > s->st.budget_bytes) return QPSO_ERR_BUSY;
  std::lock_guard<std::mutex> g(s->mu);
  if (s->stop) return QPSO_ERR_BUSY;
  ServerReq r;
  r.desc = *desc;
  r.t_submit = Clock::now();
  *id = s->next_id++;
  s->reqs.emplace(*id, r);
  s->queue.push_back(*id);
  s->st.submitted++;
  s->st.pending = (uint32_t)s->queue.size();
  s->cv.notify_one();
  return QPSO_OK;
}

static void fill_done(const ServerReq& r, qpso_result* res, double* lat) {
  if (res) *res = r.result;
  if (lat) *lat = std::chrono::duration<double, std::milli>(r.t_done - r.t_submit).count();
}

qpso_status qpso_server_poll(qpso_server* s, uint64_t id, int* done, qpso_result* res, double* lat) {
  if (!s || !done) return QPSO_ERR_ARG;
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return QPSO_ERR_NOT_FOUND;
  *done = it->second.state >= 2;
  if (*done) {
    fill_done(it->second, res, lat);
    const qpso_status st = it->second.status;
    s->reqs.erase(it);
    return st;
  }
  return QPSO_OK;
}

qpso_status qpso_server_wait(qpso_server* s, uint64_t id, uint64_t timeout_ms, qpso_result* res,
                             double* lat) {
  if (!s) return QPSO_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return QPSO_ERR_NOT_FOUND;
  const bool ok = s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms),
                                      [&] { return it->second.state >= 2; });
  if (!ok) return QPSO_ERR_TIMEOUT;
  fill_done(it->second, res, lat);
  const qpso_status st = it->second.status;
  s->reqs.erase(it);
  return st;
}

qpso_status qpso_server_stats_get(qpso_server* s, qpso_server_stats* out) {
  if (!s || !out) return QPSO_ERR_ARG;
  std::lock_guard<std::mutex> g(s->mu);
  *out = s->st;
  return QPSO_OK;
}

qpso_status qpso_server_stop(qpso_server* s) {
  if (!s) return QPSO_ERR_ARG;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
    s->cv.notify_all();
  }
  if (s->th.joinable()) s->th.join();
  cudaSetDevice(s->ctx->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  for (auto& kv : s->reqs)
    if (kv.second.dmem && kv.second.state == 1) cudaFreeAsync(kv.second.dmem, s->stream);
  if (s->stream) cudaStreamSynchronize(s->stream);
  cudaFree(s->d_slots);
  cudaFree(s->d_hdr);
  cudaFree(s->d_prep);
  cudaFree(s->d_queue);
  cudaFree(s->d_qctl);
  cudaFree(s->d_end);
  cudaFree(s->d_berr);
  cudaFreeHost(s->h_slots);
  cudaFreeHost(s->h_hdr);
  cudaFreeHost(s->h_prep);
  cudaFreeHost(s->h_qinit);
  cudaFreeHost(s->h_qctl);
  cudaFreeHost(s->h_end);
  cudaFreeHost(s->h_berr);
  if (s->pool) cudaMemPoolDestroy(s->pool);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return QPSO_OK;
}

}  // extern "C"
