/*
 * ref_gpu.h -- host harness for the reference's own CUDA kernels, rebuilt
 * for sm_103a from main.h and main.cu:72-1195 (oracle/build.py writes
 * oracle/_ref/ref_kernels_{ieee,fast}.cubin where the reference sources
 * are present).
 *
 * TEST INFRASTRUCTURE ONLY: a parity reference and a measured baseline, never the
 * product.  The harness is this project's code; it loads the kernels with
 * the CUDA driver API and drives them the way the reference's main() does
 * (main.cu:1389-1727): Nparticle_ = 1024 particles in [7][1024] state
 * arrays, one 640x480 int32 depth buffer per particle, renders on 16
 * streams, thrust::min_element, the best update and the particle update.
 *
 * The reference's raster and fitness do not clip (main.h:1442,
 * main.cu:628-640): a pose whose mesh leaves the image writes outside its
 * depth buffer.  So before every render launch the harness projects the
 * mesh's object-space box corners for every pose to be rendered and
 * refuses (RG_OUT_OF_FRAME, nothing launched) unless every corner lies at
 * least 5 cm in front of the camera and 8 px inside the image; the
 * projected box bounds every face's raster rectangle, and the margin covers
 * the host/device rounding difference and the rectangle's rounding up.
 */
#ifndef QPSO_REF_GPU_H
#define QPSO_REF_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RG_OK 0
#define RG_ERR_CUDA 1
#define RG_ERR_ARG 2
#define RG_OUT_OF_FRAME 3

#define RG_NPARTICLE 1024 /* Nparticle_, main.h:84 */
#define RG_RAND_STRIDE 512 /* strideDimRandGem_, main.h:83: uniforms per particle */
#define RG_ROWS 480
#define RG_COLS 640

typedef struct rg_ctx rg_ctx;

/* QPSOParams_t (main.h:182-204) fields the kernels read. */
typedef struct {
    float x_lo[3], x_hi[3];    /* translation box, metres */
    uint32_t num_points;       /* num_point_SegmentedCluster */
    int32_t aabb_min_x, aabb_max_x, aabb_min_y, aabb_max_y; /* cluster box, inside the image */
} rg_params;

/* Load a cubin (ieee or fast build) on the current device. */
int rg_open(const char *cubin_path, rg_ctx **out);
void rg_close(rg_ctx *ctx);
const char *rg_last_error(const rg_ctx *ctx);

/* Mesh in the loadOBJ3 layout (36*F bytes, F <= 32768), the cluster-masked
 * observed depth widened to int32 (640x480, main.cu:1548-1557) and the
 * per-solve constants.  The render grid is max(6, ceil(F/512)) blocks of
 * 512 threads: the reference's 6x512 (main.cu:1639) up to 3072 faces. */
int rg_set_scene(rg_ctx *ctx, const float *mesh_soa, uint32_t num_faces, const int32_t *depth,
                 const rg_params *prm);

/* The 512x1024 uniform table d_randGen (main.cu:1337-1387), entry
 * j*1024 + p = draw j of particle p. */
int rg_set_rand_table(rg_ctx *ctx, const float *table);

/* InitQPSO<<<8,128>>> (main.cu:1601): fills the state from the table. */
int rg_init(rg_ctx *ctx);

/* State arrays, [7][1024] SoA, plus per-particle fitness, personal-best
 * fitness, the solution's best fitness and pose, and the table cursors.
 * NULL pointers are skipped. */
int rg_get_state(rg_ctx *ctx, float *pos, float *vel, float *pbest, float *fit, float *pbest_fit,
                 float *best_fit, float *best_pose, uint32_t *cursor);
int rg_set_state(rg_ctx *ctx, const float *pos, const float *vel, const float *pbest,
                 const float *fit, const float *pbest_fit, const float *best_fit,
                 const float *best_pose, const uint32_t *cursor);

/* Render and score particles 0..n-1 at their current poses: the render
 * launches on 16 streams, ComputeAABBFinalReductionKernel, and one
 * ComputeFitnessKernel<<<1,1024>>> per particle (main.cu:1620-1680).
 * depth_out (n*640*480, may be NULL) receives the depth buffers as the
 * render left them, aabb_out (n*4, may be NULL) the render boxes; the
 * fitness lands in the state's fit array. */
int rg_render_score(rg_ctx *ctx, uint32_t n, int32_t *depth_out, int32_t *aabb_out);

/* thrust::min_element over the 1024 fitnesses, UpdatePersonalAndGlobalBest
 * and UpdateParticlesEquationKernel (main.cu:1691-1727). */
int rg_best_and_update(rg_ctx *ctx);

/* The reference's solve loop: InitQPSO, then `iterations` (<= 41, the
 * table's 512 draws per particle) of render, score, best update and
 * particle update over all 1024 particles, as main.cu:1601-1727 runs them.
 * Host wall time of the iterations' GPU work, each bracketed by device
 * synchronisations like the reference's, goes to *ms (the in-frame check
 * between iterations is not counted).  Stops early with RG_OUT_OF_FRAME
 * when a pose would leave the image; *done = iterations completed. */
int rg_solve(rg_ctx *ctx, uint32_t iterations, float *fit_trace, double *ms, uint32_t *done);

#ifdef __cplusplus
}
#endif
#endif
