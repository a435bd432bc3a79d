/*
 * ref_gpu.cu -- host harness for the reference's CUDA kernels rebuilt for
 * sm_103a (see ref_gpu.h).  TEST INFRASTRUCTURE ONLY.
 *
 * Everything here is this project's code: the kernels come from a cubin
 * compiled from the reference's own sources, loaded with the driver API and
 * found by their plain names (the recipe gives them C linkage).  The launch
 * sequence and shapes follow the reference's main() (main.cu:1389-1727).
 */
#include "ref_gpu.h"

#include <cuda.h>
#include <cuda_runtime.h>
#include <thrust/device_ptr.h>
#include <thrust/execution_policy.h>
#include <thrust/extrema.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

namespace {

constexpr int kStreams = 16;            // NumStreams, main.h:130
constexpr size_t kRxC = (size_t)RG_ROWS * RG_COLS;
constexpr int kThreads = 512;           // fxptThsPerBlock, main.h:162
constexpr int kMinBlocks = 6;           // fxptBlocks, main.h:161
constexpr int kAabbSlots = 64;          // _2warpSize_: per-particle block slots of d_AABB
constexpr float kBestInit = 1.0e10f;    // max_best_fit_, main.h:99
constexpr double kMargin = 8.0;         // px kept free inside the image by the in-frame check
constexpr double kMinZ = 0.05;          // m

// QPSOParams_t as main.h:182-204 lays it out (__align__(16), 64 bytes).
struct RefParams {
    float c1, c2;
    float x_lo[3], x_hi[3];
    uint32_t num_point_segmented_cluster;
    uint32_t num_verts, num_faces;
    int32_t aabb_min_x, aabb_max_x, aabb_min_y, aabb_max_y;
    uint32_t pad;
};
static_assert(sizeof(RefParams) == 64, "QPSOParams_t layout");

}  // namespace

struct rg_ctx {
    CUmodule mod = nullptr;
    CUfunction k_init = nullptr, k_render = nullptr, k_aabb = nullptr, k_fit = nullptr,
               k_best = nullptr, k_update = nullptr, k_fill = nullptr;
    CUdeviceptr params = 0;
    cudaStream_t streams[kStreams] = {};
    uint32_t faces = 0;
    int blocks = kMinBlocks;
    float obj_lo[3] = {0, 0, 0}, obj_hi[3] = {0, 0, 0};  // object-space box of the mesh
    bool scene = false, table = false;
    uint32_t cursor_max = 0;  // largest table cursor any particle holds
    float *obj = nullptr;
    int *depth = nullptr, *kinect = nullptr;
    int32_t *aabb = nullptr, *final_aabb = nullptr;
    float *pos = nullptr, *vel = nullptr, *pos_b = nullptr, *fit = nullptr, *pbest_fit = nullptr;
    float *best_fit = nullptr, *best_pose = nullptr, *pos_nb = nullptr, *rand = nullptr;
    unsigned *rand_idx = nullptr;
    std::string err;
};

namespace {

int fail(rg_ctx *c, int code, const std::string &msg)
{
    if (c) c->err = msg;
    return code;
}

#define RG_RT(c, call)                                                                          \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess) return fail(c, RG_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
    } while (0)
#define RG_DRV(c, call)                                                                         \
    do {                                                                                        \
        CUresult r_ = (call);                                                                   \
        if (r_ != CUDA_SUCCESS) {                                                               \
            const char *s_ = nullptr;                                                           \
            cuGetErrorString(r_, &s_);                                                          \
            return fail(c, RG_ERR_CUDA, std::string(#call ": ") + (s_ ? s_ : "?"));            \
        }                                                                                       \
    } while (0)

// d_AABB as main.cu:1500-1518 initialises it: every block slot of every
// particle holds the empty box (50000, -1, 50000, -1).
int reset_aabb(rg_ctx *c)
{
    std::vector<int32_t> h((size_t)RG_NPARTICLE * 4 * kAabbSlots);
    for (size_t p = 0; p < RG_NPARTICLE; ++p)
        for (int l = 0; l < kAabbSlots; ++l) {
            const size_t i = p * 4 * kAabbSlots + l;
            h[i] = 50000;
            h[i + 64] = -1;
            h[i + 128] = 50000;
            h[i + 192] = -1;
        }
    RG_RT(c, cudaMemcpy(c->aabb, h.data(), h.size() * 4, cudaMemcpyHostToDevice));
    return RG_OK;
}

int fill_depth(rg_ctx *c)
{
    int *d = c->depth;
    void *args[] = {&d};
    // FillTheDepthBufferMaxValKernel<<<(80,60),(8,8)>>>, main.cu:1576-1594
    RG_DRV(c, cuLaunchKernel(c->k_fill, RG_COLS / 8, RG_ROWS / 8, 1, 8, 8, 1, 0, 0, args, nullptr));
    RG_RT(c, cudaDeviceSynchronize());
    return RG_OK;
}

// Every pose of particles 0..n-1 keeps its mesh inside the image: the eight
// corners of the object box, rotated (v + q0 t + u x t, t = 2 u x v, the
// reference's formula, main.h:349-369), translated and projected with the
// reference's ACCV intrinsics (main.h:30-33), lie >= kMinZ in front of the
// camera and kMargin px inside the image.
int check_in_frame(rg_ctx *c, uint32_t n)
{
    std::vector<float> pos((size_t)7 * RG_NPARTICLE);
    RG_RT(c, cudaMemcpy(pos.data(), c->pos, pos.size() * 4, cudaMemcpyDeviceToHost));
    for (uint32_t p = 0; p < n; ++p) {
        double s[7];
        for (int d = 0; d < 7; ++d) s[d] = pos[p + (size_t)d * RG_NPARTICLE];
        for (int k = 0; k < 8; ++k) {
            const double v[3] = {(k & 1) ? c->obj_hi[0] : c->obj_lo[0], (k & 2) ? c->obj_hi[1] : c->obj_lo[1],
                                 (k & 4) ? c->obj_hi[2] : c->obj_lo[2]};
            const double u[3] = {s[4], s[5], s[6]};
            const double t[3] = {2 * (u[1] * v[2] - u[2] * v[1]), 2 * (u[2] * v[0] - u[0] * v[2]),
                                 2 * (u[0] * v[1] - u[1] * v[0])};
            const double w[3] = {v[0] + s[3] * t[0] + (u[1] * t[2] - u[2] * t[1]) + s[0],
                                 v[1] + s[3] * t[1] + (u[2] * t[0] - u[0] * t[2]) + s[1],
                                 v[2] + s[3] * t[2] + (u[0] * t[1] - u[1] * t[0]) + s[2]};
            if (!(w[2] >= kMinZ)) return fail(c, RG_OUT_OF_FRAME, "pose behind or too near the camera");
            const double x = 325.26110 + 572.41140 * (w[0] / w[2]);
            const double y = 242.04899 + 573.57043 * (w[1] / w[2]);
            if (!(x >= kMargin && x <= RG_COLS - kMargin && y >= kMargin && y <= RG_ROWS - kMargin))
                return fail(c, RG_OUT_OF_FRAME, "pose of particle " + std::to_string(p) + " leaves the image");
        }
    }
    return RG_OK;
}

int launch_renders(rg_ctx *c, uint32_t n)
{
    for (uint32_t p = 0; p < n; ++p) {
        float *obj = c->obj, *pos = c->pos;
        int *depth = c->depth;
        int32_t *aabb = c->aabb;
        uint32_t offset = (uint32_t)(p * kRxC), pidx = p;
        void *args[] = {&obj, &depth, &offset, &pos, &pidx, &aabb};
        RG_DRV(c, cuLaunchKernel(c->k_render, c->blocks, 1, 1, kThreads, 1, 1, 0,
                                 (CUstream)c->streams[p % kStreams], args, nullptr));
    }
    RG_RT(c, cudaDeviceSynchronize());
    return RG_OK;
}

int launch_aabb(rg_ctx *c)
{
    int32_t *aabb = c->aabb, *fin = c->final_aabb;
    void *args[] = {&aabb, &fin};
    RG_DRV(c, cuLaunchKernel(c->k_aabb, RG_NPARTICLE, 1, 1, 256, 1, 1, 0, 0, args, nullptr));
    RG_RT(c, cudaDeviceSynchronize());
    return RG_OK;
}

int launch_fitness(rg_ctx *c, uint32_t n)
{
    for (uint32_t p = 0; p < n; ++p) {
        int *depth = c->depth, *kin = c->kinect;
        int32_t *fin = c->final_aabb;
        float *fit = c->fit;
        uint32_t offset = (uint32_t)(p * kRxC), pidx = p;
        void *args[] = {&depth, &offset, &pidx, &fin, &fit, &kin};
        RG_DRV(c, cuLaunchKernel(c->k_fit, 1, 1, 1, 1024, 1, 1, 0, (CUstream)c->streams[p % kStreams], args,
                                 nullptr));
    }
    RG_RT(c, cudaDeviceSynchronize());
    return RG_OK;
}

// main.cu:1691-1727, with the two host reads of the solution in between
int best_and_update(rg_ctx *c, float *best_fit_host)
{
    if (c->cursor_max + 12 > RG_RAND_STRIDE) return fail(c, RG_ERR_ARG, "uniform table exhausted");
    thrust::device_ptr<float> f(c->fit);
    thrust::device_ptr<float> m = thrust::min_element(thrust::device, f, f + RG_NPARTICLE);
    int best = (int)(m - f);
    float *d_min = thrust::raw_pointer_cast(m);
    {
        float *fit = c->fit, *pbf = c->pbest_fit, *nb = c->pos_nb, *pos = c->pos, *vel = c->vel,
              *pb = c->pos_b, *bf = c->best_fit, *bp = c->best_pose;
        void *args[] = {&fit, &pbf, &nb, &pos, &vel, &pb, &bf, &bp, &d_min, &best};
        RG_DRV(c, cuLaunchKernel(c->k_best, 8, 1, 1, 128, 1, 1, 0, 0, args, nullptr));
        RG_RT(c, cudaDeviceSynchronize());
    }
    float h_fit = 0.f, h_pose[7];
    RG_RT(c, cudaMemcpy(&h_fit, c->best_fit, 4, cudaMemcpyDeviceToHost));
    RG_RT(c, cudaMemcpy(h_pose, c->best_pose, 28, cudaMemcpyDeviceToHost));
    if (best_fit_host) *best_fit_host = h_fit;
    {
        float *bp = c->best_pose, *rnd = c->rand, *pos = c->pos, *vel = c->vel, *pb = c->pos_b;
        unsigned *ri = c->rand_idx;
        void *args[] = {&bp, &rnd, &pos, &vel, &pb, &ri};
        RG_DRV(c, cuLaunchKernel(c->k_update, 8, 1, 1, 128, 1, 1, 0, 0, args, nullptr));
        RG_RT(c, cudaDeviceSynchronize());
    }
    c->cursor_max += 12;
    return RG_OK;
}

}  // namespace

extern "C" {

int rg_open(const char *cubin_path, rg_ctx **out)
{
    if (!cubin_path || !out) return RG_ERR_ARG;
    *out = nullptr;
    rg_ctx *c = new rg_ctx();
    *out = c;
    RG_RT(c, cudaFree(0));  // primary context, current on this thread
    RG_DRV(c, cuModuleLoad(&c->mod, cubin_path));
    struct { CUfunction *f; const char *name; } fns[] = {
        {&c->k_init, "InitQPSO"},
        {&c->k_render, "RenderFixedPointKernelAABB"},
        {&c->k_aabb, "ComputeAABBFinalReductionKernel"},
        {&c->k_fit, "ComputeFitnessKernel"},
        {&c->k_best, "UpdatePersonalAndGlobalBest"},
        {&c->k_update, "UpdateParticlesEquationKernel"},
        {&c->k_fill, "FillTheDepthBufferMaxValKernel"},
    };
    for (auto &f : fns) RG_DRV(c, cuModuleGetFunction(f.f, c->mod, f.name));
    size_t bytes = 0;
    RG_DRV(c, cuModuleGetGlobal(&c->params, &bytes, c->mod, "d_qpso_params"));
    if (bytes != sizeof(RefParams)) return fail(c, RG_ERR_ARG, "d_qpso_params is not 64 bytes");
    for (auto &s : c->streams) RG_RT(c, cudaStreamCreate(&s));
    RG_RT(c, cudaMalloc(&c->depth, (size_t)RG_NPARTICLE * kRxC * 4));
    RG_RT(c, cudaMalloc(&c->kinect, kRxC * 4));
    RG_RT(c, cudaMalloc(&c->aabb, (size_t)RG_NPARTICLE * 4 * kAabbSlots * 4));
    RG_RT(c, cudaMalloc(&c->final_aabb, (size_t)RG_NPARTICLE * 32 * 4));
    RG_RT(c, cudaMemset(c->final_aabb, 0, (size_t)RG_NPARTICLE * 32 * 4));
    float **st[] = {&c->pos, &c->vel, &c->pos_b};
    for (auto s : st) {
        RG_RT(c, cudaMalloc(s, (size_t)7 * RG_NPARTICLE * 4));
        RG_RT(c, cudaMemset(*s, 0, (size_t)7 * RG_NPARTICLE * 4));
    }
    RG_RT(c, cudaMalloc(&c->fit, RG_NPARTICLE * 4));
    RG_RT(c, cudaMemset(c->fit, 0, RG_NPARTICLE * 4));
    RG_RT(c, cudaMalloc(&c->pbest_fit, RG_NPARTICLE * 4));
    RG_RT(c, cudaMalloc(&c->best_fit, 4));
    RG_RT(c, cudaMalloc(&c->best_pose, 28));
    RG_RT(c, cudaMalloc(&c->pos_nb, 28));
    RG_RT(c, cudaMemset(c->pos_nb, 0, 28));
    RG_RT(c, cudaMalloc(&c->rand, (size_t)RG_RAND_STRIDE * RG_NPARTICLE * 4));
    RG_RT(c, cudaMemset(c->rand, 0, (size_t)RG_RAND_STRIDE * RG_NPARTICLE * 4));
    RG_RT(c, cudaMalloc(&c->rand_idx, RG_NPARTICLE * 4));
    RG_RT(c, cudaMemset(c->rand_idx, 0, RG_NPARTICLE * 4));
    return RG_OK;
}

void rg_close(rg_ctx *c)
{
    if (!c) return;
    cudaDeviceSynchronize();
    for (auto s : c->streams)
        if (s) cudaStreamDestroy(s);
    void *bufs[] = {c->obj, c->depth, c->kinect, c->aabb, c->final_aabb, c->pos, c->vel, c->pos_b,
                    c->fit, c->pbest_fit, c->best_fit, c->best_pose, c->pos_nb, c->rand, c->rand_idx};
    for (void *b : bufs)
        if (b) cudaFree(b);
    if (c->mod) cuModuleUnload(c->mod);
    delete c;
}

const char *rg_last_error(const rg_ctx *c) { return c ? c->err.c_str() : "null context"; }

int rg_set_scene(rg_ctx *c, const float *mesh, uint32_t F, const int32_t *depth, const rg_params *prm)
{
    if (!c || !mesh || !depth || !prm) return fail(c, RG_ERR_ARG, "null argument");
    if (F == 0 || F > (uint32_t)kAabbSlots * kThreads) return fail(c, RG_ERR_ARG, "faces must be in [1, 32768]");
    if (prm->aabb_min_x < 0 || prm->aabb_min_y < 0 || prm->aabb_max_x > RG_COLS - 1 ||
        prm->aabb_max_y > RG_ROWS - 1 || prm->aabb_min_x > prm->aabb_max_x || prm->aabb_min_y > prm->aabb_max_y)
        return fail(c, RG_ERR_ARG, "cluster box must lie inside the image");
    if (prm->num_points == 0) return fail(c, RG_ERR_ARG, "num_points must be positive");
    for (int d = 0; d < 3; ++d) {
        float lo = mesh[(size_t)d * 3 * F], hi = lo;
        for (size_t i = 0; i < (size_t)3 * F; ++i) {
            const float v = mesh[(size_t)d * 3 * F + i];
            if (!std::isfinite(v)) return fail(c, RG_ERR_ARG, "mesh coordinates must be finite");
            lo = std::min(lo, v);
            hi = std::max(hi, v);
        }
        c->obj_lo[d] = lo;
        c->obj_hi[d] = hi;
    }
    if (c->obj) cudaFree(c->obj);
    c->obj = nullptr;
    RG_RT(c, cudaMalloc(&c->obj, (size_t)9 * F * 4));
    RG_RT(c, cudaMemcpy(c->obj, mesh, (size_t)9 * F * 4, cudaMemcpyHostToDevice));
    RG_RT(c, cudaMemcpy(c->kinect, depth, kRxC * 4, cudaMemcpyHostToDevice));
    RefParams p;
    std::memset(&p, 0, sizeof(p));
    p.c1 = 1.0f;
    p.c2 = 1.0f;
    for (int d = 0; d < 3; ++d) {
        p.x_lo[d] = prm->x_lo[d];
        p.x_hi[d] = prm->x_hi[d];
    }
    p.num_point_segmented_cluster = prm->num_points;
    p.num_verts = 3 * F;
    p.num_faces = F;
    p.aabb_min_x = prm->aabb_min_x;
    p.aabb_max_x = prm->aabb_max_x;
    p.aabb_min_y = prm->aabb_min_y;
    p.aabb_max_y = prm->aabb_max_y;
    RG_DRV(c, cuMemcpyHtoD(c->params, &p, sizeof(p)));
    c->faces = F;
    c->blocks = std::max<int>(kMinBlocks, (int)((F + kThreads - 1) / kThreads));
    int st = reset_aabb(c);
    if (st != RG_OK) return st;
    c->scene = true;
    return RG_OK;
}

int rg_set_rand_table(rg_ctx *c, const float *table)
{
    if (!c || !table) return fail(c, RG_ERR_ARG, "null argument");
    RG_RT(c, cudaMemcpy(c->rand, table, (size_t)RG_RAND_STRIDE * RG_NPARTICLE * 4, cudaMemcpyHostToDevice));
    c->table = true;
    return RG_OK;
}

int rg_init(rg_ctx *c)
{
    if (!c || !c->scene || !c->table) return fail(c, RG_ERR_ARG, "scene and table first");
    float *nb = c->pos_nb, *rnd = c->rand, *pos = c->pos, *vel = c->vel, *pb = c->pos_b;
    unsigned *ri = c->rand_idx;
    void *args[] = {&nb, &rnd, &pos, &vel, &pb, &ri};
    RG_DRV(c, cuLaunchKernel(c->k_init, 8, 1, 1, 128, 1, 1, 0, 0, args, nullptr));
    RG_RT(c, cudaDeviceSynchronize());
    c->cursor_max = 12;
    return RG_OK;
}

int rg_get_state(rg_ctx *c, float *pos, float *vel, float *pbest, float *fit, float *pbest_fit,
                 float *best_fit, float *best_pose, uint32_t *cursor)
{
    if (!c) return RG_ERR_ARG;
    const size_t S = (size_t)7 * RG_NPARTICLE * 4;
    if (pos) RG_RT(c, cudaMemcpy(pos, c->pos, S, cudaMemcpyDeviceToHost));
    if (vel) RG_RT(c, cudaMemcpy(vel, c->vel, S, cudaMemcpyDeviceToHost));
    if (pbest) RG_RT(c, cudaMemcpy(pbest, c->pos_b, S, cudaMemcpyDeviceToHost));
    if (fit) RG_RT(c, cudaMemcpy(fit, c->fit, RG_NPARTICLE * 4, cudaMemcpyDeviceToHost));
    if (pbest_fit) RG_RT(c, cudaMemcpy(pbest_fit, c->pbest_fit, RG_NPARTICLE * 4, cudaMemcpyDeviceToHost));
    if (best_fit) RG_RT(c, cudaMemcpy(best_fit, c->best_fit, 4, cudaMemcpyDeviceToHost));
    if (best_pose) RG_RT(c, cudaMemcpy(best_pose, c->best_pose, 28, cudaMemcpyDeviceToHost));
    if (cursor) RG_RT(c, cudaMemcpy(cursor, c->rand_idx, RG_NPARTICLE * 4, cudaMemcpyDeviceToHost));
    return RG_OK;
}

int rg_set_state(rg_ctx *c, const float *pos, const float *vel, const float *pbest, const float *fit,
                 const float *pbest_fit, const float *best_fit, const float *best_pose, const uint32_t *cursor)
{
    if (!c) return RG_ERR_ARG;
    const size_t S = (size_t)7 * RG_NPARTICLE * 4;
    if (cursor) {
        uint32_t mx = 0;
        for (int p = 0; p < RG_NPARTICLE; ++p) mx = std::max(mx, cursor[p]);
        if (mx > RG_RAND_STRIDE) return fail(c, RG_ERR_ARG, "cursor beyond the uniform table");
        c->cursor_max = mx;
        RG_RT(c, cudaMemcpy(c->rand_idx, cursor, RG_NPARTICLE * 4, cudaMemcpyHostToDevice));
    }
    if (pos) RG_RT(c, cudaMemcpy(c->pos, pos, S, cudaMemcpyHostToDevice));
    if (vel) RG_RT(c, cudaMemcpy(c->vel, vel, S, cudaMemcpyHostToDevice));
    if (pbest) RG_RT(c, cudaMemcpy(c->pos_b, pbest, S, cudaMemcpyHostToDevice));
    if (fit) RG_RT(c, cudaMemcpy(c->fit, fit, RG_NPARTICLE * 4, cudaMemcpyHostToDevice));
    if (pbest_fit) RG_RT(c, cudaMemcpy(c->pbest_fit, pbest_fit, RG_NPARTICLE * 4, cudaMemcpyHostToDevice));
    if (best_fit) RG_RT(c, cudaMemcpy(c->best_fit, best_fit, 4, cudaMemcpyHostToDevice));
    if (best_pose) RG_RT(c, cudaMemcpy(c->best_pose, best_pose, 28, cudaMemcpyHostToDevice));
    return RG_OK;
}

int rg_render_score(rg_ctx *c, uint32_t n, int32_t *depth_out, int32_t *aabb_out)
{
    if (!c || !c->scene) return fail(c, RG_ERR_ARG, "scene first");
    if (n == 0 || n > RG_NPARTICLE) return fail(c, RG_ERR_ARG, "n must be in [1, 1024]");
    int st = check_in_frame(c, n);
    if (st != RG_OK) return st;
    if ((st = fill_depth(c)) != RG_OK) return st;
    if ((st = launch_renders(c, n)) != RG_OK) return st;
    if (depth_out) RG_RT(c, cudaMemcpy(depth_out, c->depth, (size_t)n * kRxC * 4, cudaMemcpyDeviceToHost));
    if ((st = launch_aabb(c)) != RG_OK) return st;
    if (aabb_out) {
        std::vector<int32_t> fin((size_t)RG_NPARTICLE * 32);
        RG_RT(c, cudaMemcpy(fin.data(), c->final_aabb, fin.size() * 4, cudaMemcpyDeviceToHost));
        for (uint32_t p = 0; p < n; ++p)
            for (int k = 0; k < 4; ++k) aabb_out[4 * p + k] = fin[(size_t)p * 32 + k];
    }
    return launch_fitness(c, n);
}

int rg_best_and_update(rg_ctx *c)
{
    if (!c || !c->scene || !c->table) return fail(c, RG_ERR_ARG, "scene and table first");
    return best_and_update(c, nullptr);
}

int rg_solve(rg_ctx *c, uint32_t iterations, float *fit_trace, double *ms, uint32_t *done)
{
    if (!c || !c->scene || !c->table) return fail(c, RG_ERR_ARG, "scene and table first");
    if (iterations == 0 || 12 * (iterations + 1) > RG_RAND_STRIDE)
        return fail(c, RG_ERR_ARG, "iterations must be in [1, 41]");
    if (ms) *ms = 0.0;
    if (done) *done = 0;
    // the reference's initial values (main.cu:1389-1470)
    std::vector<float> pbf(RG_NPARTICLE, kBestInit), zero7(7, 0.f);
    const float bf = kBestInit;
    int st = rg_set_state(c, nullptr, nullptr, nullptr, nullptr, pbf.data(), &bf, zero7.data(), nullptr);
    if (st != RG_OK) return st;
    if ((st = fill_depth(c)) != RG_OK) return st;
    if ((st = rg_init(c)) != RG_OK) return st;
    for (uint32_t it = 0; it < iterations; ++it) {
        if ((st = check_in_frame(c, RG_NPARTICLE)) != RG_OK) return st;
        const auto t0 = std::chrono::steady_clock::now();
        if ((st = launch_renders(c, RG_NPARTICLE)) != RG_OK) return st;
        if ((st = launch_aabb(c)) != RG_OK) return st;
        if ((st = launch_fitness(c, RG_NPARTICLE)) != RG_OK) return st;
        float best = 0.f;
        if ((st = best_and_update(c, &best)) != RG_OK) return st;
        const auto t1 = std::chrono::steady_clock::now();
        if (ms) *ms += std::chrono::duration<double, std::milli>(t1 - t0).count();
        if (fit_trace) fit_trace[it] = best;
        if (done) *done = it + 1;
    }
    return RG_OK;
}

}  // extern "C"
