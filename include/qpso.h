/*
 * qpso.h -- C ABI of the GB300-native Q-PSO pose solver.
 *
 * The reference (morpheus1820/Q-PSO) is one executable with no library API;
 * its in-process boundary is the set of kernels and buffers that main()
 * drives (main.cu:1301-1780).  Each entry point below names the reference
 * code it replaces.  Conventions: plain C types only; the caller owns host
 * memory, which is copied during the call; the library owns device objects
 * behind integer ids; every function returns a qpso_status; no exception
 * crosses the boundary; a context is not thread-safe except the
 * qpso_server_* calls, which lock internally.
 */
#ifndef QPSO_H
#define QPSO_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct qpso_context qpso_context;
typedef int32_t qpso_status;

#define QPSO_OK 0
#define QPSO_ERR_ARG 1        /* invalid argument */
#define QPSO_ERR_NOMEM 2      /* device or host allocation failed */
#define QPSO_ERR_CUDA 3       /* a CUDA call failed; see qpso_last_error */
#define QPSO_ERR_TIMEOUT 4    /* a bounded device-side wait expired */
#define QPSO_ERR_BUSY 5       /* admission refused: not enough free memory / slots */
#define QPSO_ERR_NOT_FOUND 6  /* unknown mesh, frame or request id */
#define QPSO_ERR_INTERNAL 7   /* a device-side consistency check failed */

/* Pinhole camera.  The reference hard-codes the ACCV intrinsics as double
 * macros FX/FY/CX/CY and a 640x480 frame (main.h:30-33, 128-129). */
typedef struct {
    float fx, fy, cx, cy;
    int32_t width, height;
    /* QPSO_PROJ_FP32 (0): u = cx + fx * (x/z) as one fp32 fused multiply-add
     * with the fields above.  QPSO_PROJ_REF_ACCV (1): the reference's own
     * projection, with the ACCV intrinsics compiled into its kernels and
     * host renderer (main.h:30-33) evaluated in double, u = (float)(CX + FX *
     * (double)(x/z)) (main.h:537-539, 1849-1851); fx..cy are ignored.  Its
     * renders equal the reference's kernels' bit for bit. */
    int32_t projection;
} qpso_camera;

#define QPSO_PROJ_FP32 0
#define QPSO_PROJ_REF_ACCV 1

/* One pose solve: QPSOParams_t (main.h:182-204) plus the compile-time
 * constants of main.h:83-136 as run-time fields.  Defaults from
 * qpso_solve_desc_init equal the reference's values. */
typedef struct {
    uint32_t mesh_id;
    uint32_t frame_id;
    int32_t cluster_label;     /* frame label selecting the cluster; -1: depth already masked */
    int32_t cl_min_x, cl_max_x, cl_min_y, cl_max_y; /* cluster AABB, max exclusive (cv::Rect tl/br) */
    uint32_t num_points;       /* num_point_SegmentedCluster */
    float t_lo[3], t_hi[3];    /* translation box x_lo/x_hi (main.cu:1318-1323), metres */
    uint32_t num_particles;    /* Nparticle_ (main.h:84) */
    uint32_t iterations;       /* max_steps_ (main.h:99) */
    float c1, c2;              /* c1_, c2_ */
    double w;                  /* psoW_ */
    float vdot;                /* vdot_ */
    float ang_lo, ang_hi;      /* aminX_ .. amaxZ_ */
    float qinit[4];            /* InitQPSO qinit (main.cu:128-132) */
    uint64_t seed;             /* Philox key (replaces the GSL mt19937 table) */
    uint32_t stream;           /* Philox stream id of this solve */
    uint32_t raster_mode;      /* QPSO_RASTER_REF (default) or QPSO_RASTER_EDGE */
} qpso_solve_desc;

/* Raster modes of a solve.  REF: what the reference computes
 * (renderFixedPointAABB, main.h:1306-1491): every pixel of a front face's
 * bounding rectangle, because its inside mask (main.h:1440) is never
 * applied (the guard of main.h:1473 tests a bit the mask never has).  EDGE:
 * that mask applied, only pixels whose three biased edge functions are all
 * > 0 (top-left fill convention, watertight across shared edges); no
 * counterpart in what the reference runs.  The render AABB of the fitness
 * window takes every face rectangle in both modes; raster_writes counts
 * rectangle pixels in REF mode and covered pixels in EDGE mode. */
#define QPSO_RASTER_REF 0
#define QPSO_RASTER_EDGE 1

typedef struct {
    float fit;                 /* d_solution_best_fit */
    float pose[7];             /* d_solution_best_pose: tx,ty,tz (m), q0..q3 */
    uint32_t flags;            /* device error bits (0 = clean) */
    uint32_t reserved;
    uint64_t raster_writes;    /* pixel writes issued by the rasteriser */
    uint64_t tile_passes;      /* shared-memory tile passes (1 per particle-render when it fits) */
} qpso_result;

typedef struct {
    int32_t threads;           /* CTA size, multiple of 32, <= 1024 */
    int32_t tile_px;           /* int32 depth-tile capacity in pixels, multiple of 8 */
    int32_t ppb;               /* particles per work item, 1..16 */
} qpso_launch_config;

const char *qpso_version(void);

/* Context on one GPU (replaces the set-up of main.cu:1301-1574). */
qpso_status qpso_create(int device, qpso_context **out);
void qpso_destroy(qpso_context *ctx);
const char *qpso_last_error(const qpso_context *ctx);

/* Mesh in the loadOBJ3 layout (main.h:620-679): 9*num_faces floats,
 * [x(v0)|x(v1)|x(v2)|y(v0)|y(v1)|y(v2)|z(v0)|z(v1)|z(v2)], metres.
 * Replaces loadOBJ3 + cudaMemcpy of d_obj_model (main.cu:1366-1373). */
qpso_status qpso_mesh_upload(qpso_context *ctx, const float *soa_xyz, uint32_t num_faces,
                             uint32_t *mesh_id);
qpso_status qpso_mesh_release(qpso_context *ctx, uint32_t mesh_id);

/* Depth frame (uint16 mm, row-major width*height) with an optional int32
 * label map (cluster ids).  Replaces the d_depth_kinect upload of the
 * cluster-masked depth (main.cu:1548-1557). */
qpso_status qpso_frame_upload(qpso_context *ctx, const uint16_t *depth_mm, const int32_t *labels,
                              const qpso_camera *cam, uint32_t *frame_id);
qpso_status qpso_frame_release(qpso_context *ctx, uint32_t frame_id);

/* One cluster of a frame's label map, with the fields of the segmentation's
 * SegResults record (GraphCannySeg.h:594-618) that the solve reads: the
 * pixel count (num_points), the bounding rectangle (rect_aabb_, max
 * exclusive) and the centroid of the back-projected pixels that have depth
 * (centroid3D, compute3DCentroid GraphCannySeg.h:2569-2597:
 * X = (u - cx) z / fx, Y = (v - cy) z / fy, Z = z, in mm).  The sums are
 * exact integers here.
 *
 * The reference's records are built from collectSets lists
 * (GraphCannySeg.cpp:305-352), which hold one pixel of the cluster twice
 * (the first pixel's union-find parent).  So its SegResults.num_points, the
 * fitness's num_point_SegmentedCluster, is this num_points + 1, and its
 * centroid counts that one pixel twice (which pixel a label map does not
 * say).  To reproduce the reference's fitness from a label map, fill
 * qpso_solve_desc.num_points with num_points + 1, as qpso_main does. */
typedef struct {
    int32_t label;
    uint32_t num_points;
    int32_t min_x, max_x, min_y, max_y;
    uint32_t depth_points;     /* pixels of the cluster with depth > 0 */
    float centroid_mm[3];      /* 0,0,0 when no pixel has depth */
} qpso_cluster;

/* The cluster records of every label >= 0 of a resident frame's label map
 * (computed on the GPU), ordered by label; labels without pixels are
 * skipped.  With out == NULL only *n_clusters is set.  The frame needs a
 * label map; labels above 65535 are refused. */
qpso_status qpso_frame_clusters(qpso_context *ctx, uint32_t frame_id, qpso_cluster *out,
                                uint32_t capacity, uint32_t *n_clusters);

/* Overwrite a resident frame's depth (and labels, if it has a label map)
 * in place, without allocating: the per-frame input of a serving loop.
 * Same role as qpso_frame_upload for a frame that is already resident. */
qpso_status qpso_frame_update(qpso_context *ctx, uint32_t frame_id, const uint16_t *depth_mm,
                              const int32_t *labels);

/* Page-locked host buffers for fast uploads (cudaMallocHost).  No
 * counterpart in the reference, which copies from pageable memory. */
void *qpso_host_alloc(uint64_t bytes);
void qpso_host_free(void *ptr);

/* The CUDA stream (cudaStream_t) every call of this context runs on. */
void *qpso_get_stream(const qpso_context *ctx);

/* Device-time accounting of the solver kernels with CUDA events on the
 * context stream (off by default).  No counterpart in the reference, whose
 * timers are host gettimeofday (myTimer.h). */
typedef struct {
    uint64_t step_launches;    /* fused per-iteration kernels (plain path) */
    double step_ms;            /* their summed device time */
    uint64_t batch_launches;   /* persistent batched kernels */
    double batch_ms;
    uint64_t prep_launches;    /* mask / summed-area-table kernels */
} qpso_profile;
qpso_status qpso_set_profiling(qpso_context *ctx, int enable);
qpso_status qpso_get_profile(qpso_context *ctx, qpso_profile *out, int reset);

/* CUDA events on the context stream for timing whole calls on the device:
 * record slot (0..63); elapsed waits for slot b and returns b - a in ms. */
qpso_status qpso_timer_record(qpso_context *ctx, uint32_t slot);
qpso_status qpso_timer_elapsed(qpso_context *ctx, uint32_t a, uint32_t b, float *ms);
/* Write `bytes` of scratch device memory on the context stream so that the
 * next call starts with a cold L2 (benchmark hygiene). */
qpso_status qpso_scrub_l2(qpso_context *ctx, uint64_t bytes);

/* Reference defaults (main.h:83-136, main.cu:128-132). */
void qpso_solve_desc_init(qpso_solve_desc *desc);
/* Translation box from a cluster centroid in mm (main.cu:1285-1323):
 * c = centroid*0.001f; lo = c - bound; hi = c + bound (bound_z for z). */
void qpso_box_from_centroid(const float centroid_mm[3], float bound, float bound_z,
                            float t_lo[3], float t_hi[3]);

/* Launch shapes of the plain and batched paths.  A shape is accepted when
 * its shared memory fits a CTA with the vertex caches of meshes of up to
 * 16384 faces; a launch over a larger mesh (128-vertex meshlets) that would
 * not fit halves the tile, then the threads, until it does.  Results do not
 * depend on the launch shape. */
qpso_status qpso_set_launch_config(qpso_context *ctx, const qpso_launch_config *plain,
                                   const qpso_launch_config *batch);
qpso_status qpso_get_launch_config(const qpso_context *ctx, qpso_launch_config *plain,
                                   qpso_launch_config *batch);

/* Autotuner (no counterpart in the reference, whose launch shape is the
 * fixed 6x512 / 1x1024 of main.cu:1639,1674).  Times a short run (at most
 * tune_iters iterations) of the given solves for every valid candidate
 * (threads 128/256/512, tile 4K..48K px, 1/2/4 particles per work item)
 * on the plain path (batched = 0) or the batched path (batched = 1),
 * installs the fastest in the context and returns it.  Results do not
 * depend on the launch shape, only the speed does. */
qpso_status qpso_autotune(qpso_context *ctx, const qpso_solve_desc *descs, uint32_t n, int batched,
                          uint32_t tune_iters, qpso_launch_config *best, float *best_ms);

/* Plain solve: one fused launch per PSO iteration.  Replaces the host loop
 * main.cu:1601-1727 (InitQPSO, then per iteration 1024 render launches,
 * the AABB kernel, 1024 fitness launches, thrust::min_element,
 * UpdatePersonalAndGlobalBest, UpdateParticlesEquationKernel). */
qpso_status qpso_solve(qpso_context *ctx, const qpso_solve_desc *desc, qpso_result *result);

/* Plain solve that also returns the gbest trace (iterations x 8 floats:
 * fit, pose) and the final SoA state [7][P] (each pointer may be NULL). */
qpso_status qpso_solve_traced(qpso_context *ctx, const qpso_solve_desc *desc, qpso_result *result,
                              float *trace, float *pos, float *vel, float *pbest, float *pbest_fit);

/* Batched solve: every iteration of all n solves in one persistent
 * cooperative launch (replayed from a CUDA graph when the shape repeats),
 * scheduled as a queue of (solve, iteration) entries: a solve's next
 * iteration starts as soon as its own previous one completes.  Results are
 * bit-identical to n calls of qpso_solve. */
qpso_status qpso_solve_batch(qpso_context *ctx, const qpso_solve_desc *descs, uint32_t n,
                             qpso_result *results);

/* Score explicit poses (n x 7 floats) for the cluster/mesh of desc without
 * touching PSO state: RenderFixedPointKernelAABB +
 * ComputeAABBFinalReductionKernel + ComputeFitnessKernel (main.cu:305-764)
 * for arbitrary poses. */
qpso_status qpso_score_poses(qpso_context *ctx, const qpso_solve_desc *desc, const float *poses,
                             uint32_t n, float *fit_out);

/* Pose scoring that allocates nothing (no counterpart in the reference).
 * For callers that cannot let a library call cudaMalloc: applications whose
 * device memory is owned by their own pool or caching allocator with a fixed
 * budget, and real-time loops where cudaMalloc's implicit synchronisation
 * and latency are not acceptable.  Same results as qpso_score_poses.
 * Inputs and outputs are device pointers the caller owns: the mesh
 * (loadOBJ3 layout, 9*num_faces floats), the depth frame (uint16 mm,
 * cam->width*cam->height) and, when desc->cluster_label >= 0, its int32
 * label map; n poses (n x 7 floats); fit_out (n floats); flags_out
 * (optional, one uint32 of device error bits).  From desc the cluster
 * fields (label, AABB, num_points) and raster_mode are read and checked as
 * qpso_score_poses checks them, and the camera as qpso_frame_upload checks
 * it; the PSO constants are copied but play no part in a score; mesh_id
 * and frame_id are ignored.  Work is queued on `stream` (a cudaStream_t,
 * NULL for the legacy default stream) on the current device; results are
 * ready when the stream is synchronised.  Intermediate buffers live in one
 * 4 MiB device array fixed at load time (held by every GPU that loads the
 * library until exit): frames above about 690,000 pixels (640x480 and
 * 960x720 fit) are rejected with QPSO_ERR_ARG.  Every call looks up that
 * array's device address in the current context (cudaGetSymbolAddress), so
 * the address stays right after cudaDeviceReset.  The first call on a
 * device also sets the scoring kernel's shared-memory limit
 * (cudaFuncSetAttribute, 64 KB for its 16384-pixel tile): make one warm-up
 * call per device before any stream capture.  All calls on a device share
 * the array and leave their contents in it; calls that overlap on the GPU
 * race, so issue them on one stream. */
qpso_status qpso_score_poses_noalloc(const float *d_mesh_soa, uint32_t num_faces,
                                     const uint16_t *d_depth_mm, const int32_t *d_labels,
                                     const qpso_camera *cam, const qpso_solve_desc *desc,
                                     const float *d_poses, uint32_t n, float *d_fit_out,
                                     uint32_t *d_flags_out, void *stream);

/* Local refinement of a solved pose (no counterpart in the reference, whose
 * answer is the PSO's global best, main.cu:1736-1757).  A deterministic
 * pattern search around pose_in: each round scores `candidates` poses with
 * the solver's render and fitness in `raster_mode` (default
 * QPSO_RASTER_EDGE, the rasteriser's real triangle coverage): a step of
 * +-step_t (m) along each axis, a rotation of about +-step_rot (rad) about
 * each axis, and the rest random within those steps (a splitmix64 stream
 * seeded by desc->seed and desc->stream); the best candidate replaces the
 * pose when its fitness is lower, else both steps halve.  Rotations use
 * dq = (1, a/2) renormalised, so every float operation is +, -, *, / or
 * sqrt: the oracle replays the search bit for bit.  desc names the mesh,
 * frame and cluster; its PSO fields and raster_mode are not read.
 * pose_out and *fit_out receive the refined pose and its fitness in
 * raster_mode; the solve's own result, the reference-parity trajectory,
 * is untouched.  The rounds run on the device, queued without waits; the
 * call returns when the last one ends. */
typedef struct {
    uint32_t rounds;          /* 32 */
    uint32_t candidates;      /* 128, at least 12 (the axis steps) */
    float step_t;             /* 0.03 m */
    float step_rot;           /* 0.5 rad */
    uint32_t raster_mode;     /* QPSO_RASTER_EDGE */
} qpso_refine_params;
void qpso_refine_params_init(qpso_refine_params *p);
qpso_status qpso_refine(qpso_context *ctx, const qpso_solve_desc *desc, const qpso_refine_params *prm,
                        const float pose_in[7], float pose_out[7], float *fit_out);

/* Render one pose of a mesh with the solver's rasteriser (renderFixedPointAABB,
 * main.h:1306-1491) into a window [x0,x0+w) x [y0,y0+h) of the raster
 * domain (int32 mm, 60000 where nothing was drawn) and return the render
 * AABB {minx,maxx,miny,maxy}: the depth the fitness of that pose saw. */
qpso_status qpso_render(qpso_context *ctx, uint32_t mesh_id, const qpso_camera *cam,
                        const float pose[7], int32_t x0, int32_t y0, int32_t w, int32_t h,
                        int32_t *depth_out, int32_t box_out[4]);

/* The depth image the reference writes for the best pose
 * (results/<rgb>-<N>-best.csv, main.cu:1758-1762): RenderCPU
 * (main.h:2012-2043) on the GPU, i.e. its own rasteriser CPUfixedPointRender
 * (main.h:1857-1991; iround vertex snapping, float depth, background 60000)
 * after the solver's projection.  depth_out receives width*height floats,
 * row-major.  Writes outside the image are dropped (the reference indexes
 * y*640+x unclipped). */
qpso_status qpso_render_depth_f32(qpso_context *ctx, uint32_t mesh_id, const qpso_camera *cam,
                                  const float pose[7], float *depth_out);

/* ---- input formats (host only: no context, no GPU) ----
 * Wavefront OBJ text into the loadOBJ3 layout (main.h:620-679, which reads
 * it through assimp): `v` vertices and `f` faces with 1-based or negative
 * indices and optional /t/n parts; polygons become triangle fans from their
 * first corner.  With soa_out == NULL only *num_faces is set; otherwise
 * soa_out holds 9*capacity_faces floats.  QPSO_ERR_NOT_FOUND when the file
 * cannot be read, QPSO_ERR_ARG when it is malformed or too large. */
qpso_status qpso_obj_load(const char *path, float *soa_out, uint32_t capacity_faces,
                          uint32_t *num_faces);

/* A uint16 image: the ACCV binary depth format of loadDepth (main.cu:35-64:
 * int32 rows, int32 cols, rows*cols uint16, row-major, host byte order) or a
 * greyscale PNG of 16 or 8 bits (not interlaced), told apart by the PNG
 * signature.  With out == NULL only the size is set. */
qpso_status qpso_image_u16_load(const char *path, uint16_t *out, uint64_t capacity_px,
                                uint32_t *width, uint32_t *height);

/* A colour image as 8-bit B, G, R (the channel order cv::imread gives the
 * reference, main.cu:1238): a PNG (grey, RGB, grey + alpha or RGBA, 8 or
 * 16 bits, not interlaced; alpha dropped, 16-bit samples keep their high
 * byte) or a binary PPM (P6, maxval 255), told apart by the PNG signature.
 * out receives width*height*3 bytes (capacity_px pixels); with out == NULL
 * only the size is set. */
qpso_status qpso_image_bgr8_load(const char *path, uint8_t *out, uint64_t capacity_px, uint32_t *width,
                                 uint32_t *height);

/* A B, G, R image written as a baseline JPEG (ITU-T T.81; 4:4:4 YCbCr,
 * the Annex K tables, quality 1..100 scaled as the IJG software does), the
 * format of the cluster images the reference's main writes with
 * cv::imwrite (main.cu:1262-1272, default quality 95).  QPSO_ERR_ARG for
 * bad arguments (a side above 65535), QPSO_ERR_NOT_FOUND when the file
 * cannot be written. */
qpso_status qpso_image_jpeg_write(const char *path, const uint8_t *bgr, uint32_t width, uint32_t height,
                                  int32_t quality);

/* ---- serving: continuous batching of solve requests ----
 * No counterpart in the reference (one solve per process).  A scheduler
 * thread admits submitted requests into free slots while the slot count and
 * the HBM budget allow (their swarm state, masked depth and summed-area
 * table are allocated on admission from the server's own memory pool and
 * stay resident until the request completes), and runs epochs: each epoch
 * is one persistent launch of the batched solve's dataflow queue in which
 * every active request advances by up to iters_per_epoch iterations, each
 * at its own pace (a request waits only for its own previous iteration);
 * finished requests leave and queued ones join between epochs.  Meshes and frames are the context's resident objects
 * and must stay uploaded while requests use them.  A request reads its
 * frame's depth and labels when it is admitted (its masked copy is made
 * then): a qpso_frame_update issued while it is still queued is what it
 * sees, one issued after its admission is not.  A request's result is
 * bit-identical to qpso_solve of the same descriptor, whatever else runs. */
typedef struct qpso_server qpso_server;
typedef struct {
    uint32_t max_slots;        /* requests on the GPU at once (>= 1) */
    uint64_t hbm_budget_bytes; /* request memory cap; 0 = half of free HBM at start */
    uint32_t iters_per_epoch;  /* iterations a request advances per scheduling epoch (>= 1) */
} qpso_server_config;
typedef struct {
    uint64_t submitted, admitted, completed, failed;
    uint32_t pending, active, peak_active;
    uint64_t bytes_in_use, peak_bytes, budget_bytes;
    uint64_t epochs, launches;  /* launches: one per epoch */
} qpso_server_stats;
qpso_status qpso_server_start(qpso_context *ctx, const qpso_server_config *cfg, qpso_server **out);
/* Queue a request; QPSO_ERR_BUSY if it could never fit the budget. */
qpso_status qpso_server_submit(qpso_server *srv, const qpso_solve_desc *desc, uint64_t *request_id);
/* Non-blocking query; *done = 1 once finished (result and latency set).
 * A finished request's result is handed out once (by poll or wait); its id
 * is unknown afterwards. */
qpso_status qpso_server_poll(qpso_server *srv, uint64_t request_id, int *done, qpso_result *result,
                             double *latency_ms);
/* Block until the request finishes or timeout_ms passes (QPSO_ERR_TIMEOUT). */
qpso_status qpso_server_wait(qpso_server *srv, uint64_t request_id, uint64_t timeout_ms,
                             qpso_result *result, double *latency_ms);
qpso_status qpso_server_stats_get(qpso_server *srv, qpso_server_stats *out);
/* Finish every queued and active request, then stop the scheduler. */
qpso_status qpso_server_stop(qpso_server *srv);

/* Checks the bounded device wait of the batched kernel: CTAs waiting for
 * work from a queue whose next entry is never appended must give up after
 * timeout_ns and report QPSO_ERR_TIMEOUT.  No counterpart in the reference
 * (which has no device waits). */
qpso_status qpso_barrier_selftest(qpso_context *ctx, uint64_t timeout_ns, uint32_t *err_bits);

/* ---- segmentation: the graph stage of GraphCannySeg ----
 * The reference segments the colour-and-depth frame before the solve
 * (GraphCannySeg<hsv>::run, GraphCannySeg.cpp:1438-1459).  Its graph stage
 * (segment_image, GraphCannySeg.cpp:1053-1250) takes an HSV image, the
 * inpainted depth and a saliency map, builds the pixel graph with edges
 * to (x+1, y), (x, y+1), (x+1, y+1) and (x+1, y-1), weighs them (diff,
 * GraphCannySeg.h:2051-2288), merges with segment_graph
 * (GraphCannySeg.cpp:1301-1373) and the small-component pass
 * (GraphCannySeg.cpp:1243-1248), and numbers the sets by their smallest
 * pixel (collectSets, GraphCannySeg.cpp:305-352).  The stages before it
 * (HSV conversion, inpainting, Canny saliency) and the cluster filter
 * after it (PostSegmFilter) are OpenCV's or call it and are not here.
 *
 * Equal weights: the reference's std::sort leaves their order to the C++
 * library; here they are ordered by edge index. */
typedef struct {
    float sigma;      /* 0.8: Gaussian smoothing of each HSV plane (main.h:65) */
    float k;          /* 50 / 10000: merge threshold constant (main.h:58, main.cu:1214) */
    float min_size;   /* 500: smaller components are merged (main.h:64) */
    float kx, ky, ks; /* 2000, 30, 49 / 1000: weight mix (main.h:59-61); ky is not read */
    float kdv, kdc;   /* 4.5, 0.1: HSV distance weights (main.h:62-63) */
} qpso_seg_params;

/* The reference main's values above. */
void qpso_seg_params_init(qpso_seg_params *p);

/* Edges of the width x height pixel graph, (W-1)(4H-3) + H-1 for
 * W, H >= 1; 0 for an empty or oversized (above 2^26 pixels) image. */
uint64_t qpso_segment_num_edges(uint32_t width, uint32_t height);

/* Every edge's ends (pixel indices y*W+x) in the reference's edge order
 * (GraphCannySeg.cpp:1174-1210): per pixel in row-major order, right,
 * down, down-right, up-right where inside.  Host only. */
qpso_status qpso_segment_edge_ends(uint32_t width, uint32_t height, int32_t *a, int32_t *b);

/* The smoothing mask (make_fgauss + normalize, GraphCannySeg.h:462-476):
 * writes ceil(4 sigma) + 1 taps and returns their count, or -1 above
 * capacity or for a NaN sigma.  Host only. */
int32_t qpso_segment_gauss_mask(float sigma, float *mask, int32_t capacity);

/* The merge passes over given edge weights (one per edge, in the order of
 * qpso_segment_edge_ends): sorted ascending with ties by edge index, then
 * segment_graph with prm->k and the small-component merge with
 * prm->min_size.  labels (width*height) receives each pixel's set, sets
 * numbered by their smallest pixel; *n_clusters the set count.  NaN
 * weights are refused.  Host only. */
qpso_status qpso_segment_edges(uint32_t width, uint32_t height, const float *weights,
                               const qpso_seg_params *prm, int32_t *labels, uint32_t *n_clusters);

/* The whole graph stage.  h, s, v: 8-bit planes (H in 0..180, OpenCV's
 * 8-bit HSV), depth_mm: the inpainted depth, saliency: one float per
 * pixel, all width*height row-major on the host.  The GPU smooths the
 * planes, normalises the depth by the range of every pixel but the last
 * (the reference's ranges end at the last pixel's address), weighs every
 * edge and radix-sorts them; the merge passes run on the host as in
 * qpso_segment_edges.  edge_weights (optional, qpso_segment_num_edges
 * floats) receives the weights in edge order.  The weight calls CUDA's cos
 * and log2f where the reference calls the C library's: weights agree to an
 * ulp or so.  QPSO_ERR_ARG for a NaN weight (all pixels but the last at one
 * depth, or a NaN saliency) or sigma above 7.75. */
qpso_status qpso_segment_planes(qpso_context *ctx, const uint8_t *h, const uint8_t *s, const uint8_t *v,
                                const uint16_t *depth_mm, const float *saliency, uint32_t width,
                                uint32_t height, const qpso_seg_params *prm, int32_t *labels,
                                float *edge_weights, uint32_t *n_clusters);

/* ---- segmentation: the stages around the graph stage ----
 * GraphCannySeg<hsv>::run (GraphCannySeg.cpp:1438-1459) from the colour
 * image and the raw depth: dynamicDepthSmoothing (GraphCannySeg.cpp:426-634),
 * inpaintDepth (GraphCannySeg.h:1164-1230), myCannyWithOri2
 * (GraphCannySeg.cpp:638-1050), the HSV conversion of segment_image, the
 * graph stage above, and PostSegmFilter (GraphCannySeg.h:1639-1873), which
 * keeps the sets that can be objects and gives them the order the
 * reference's cluster index N counts in (main.cu:1253-1269).  The
 * reference runs the stages before and after the graph with OpenCV 2.4;
 * here they are GPU kernels restating the published algorithms (colour
 * conversion, separable Gaussian, Scharr, exact Euclidean distance
 * transform, summed-area tables, Telea's fast-marching inpainting,
 * bilinear resizing, PCA of the pixel coordinates), with exact integer or
 * fixed-order float arithmetic; OpenCV's own rounding is not reproduced. */
typedef struct {
    float beta;               /* 2000: dynamicDepthSmoothing(2000.f) (GraphCannySeg.cpp:1441) */
    float gamma;              /* 18000: its depth-change threshold (default argument) */
    int32_t inpaint_radius;   /* 20: cv::inpaint radius in inpaintDepth (GraphCannySeg.h:1186) */
    float canny_low, canny_high; /* Lcanny / 1000, Hcanny / 1000 = 0.05, 0.075 (main.h:75-76) */
    int32_t dth, plus_d, point_3d; /* 30 mm, 7 px, 5 px: the depth test (main.h:70-72) */
    float g_angle, l_angle;   /* 148 and 151 degrees in radians (main.h:73-74) */
    float fx, fy, cx, cy;     /* k_vec, the ACCV intrinsics (main.h:51-56) */
    float far_obj_z;          /* 1500 mm: farther centroids are dropped (main.h:77) */
    float max_ecc, max_l1, max_l2; /* 0.978, 13800, 1950: PCA limits (main.h:66-68) */
} qpso_seg_front_params;

/* The reference main's values above. */
void qpso_seg_front_params_init(qpso_seg_front_params *p);

/* One set of a label map: the SegResults fields the solve reads
 * (GraphCannySeg.h:594-618) and what PostSegmFilter tests. */
typedef struct {
    int32_t label;            /* the set's number in the label map */
    uint32_t num_points;      /* SegResults.num_points = pixels + 1 (collectSets lists one pixel twice) */
    uint32_t pixels;
    int32_t min_x, max_x, min_y, max_y; /* rect_aabb_ (cv::boundingRect), max exclusive */
    float centroid_mm[3];     /* centroid3D of the pixels with inpainted depth (compute3DCentroid) */
    float nan_ratio;          /* pixels without depth / num_points (dropped at >= 0.3) */
    float dark_ratio;         /* pixels in the first 3 of 32 value bins / num_points (dropped at >= 0.3) */
    double eig[2];            /* PCA eigenvalues of the pixel coordinates (computePCA) */
    double eccentricity;      /* sqrt(1 - eig[1] / eig[0]) */
    int32_t far;              /* centroid farther than far_obj_z */
    int32_t kept;             /* passes every filter */
} qpso_seg_cluster;

/* Optional host copies of the intermediate planes (each W x H; any may be
 * NULL): the 8-bit HSV planes and grey image, the smoothed and the
 * inpainted depth (mm), the saliency map and the Canny edge map (0 / 255)
 * after the depth test. */
typedef struct {
    uint8_t *h, *s, *v, *gray;
    uint16_t *smoothed, *inpainted;
    float *saliency;
    uint8_t *edges;
} qpso_seg_frame_out;

/* Segment one frame from its colour image (bgr: width x height x 3, B G R)
 * and raw depth (uint16 mm).  labels (width x height) receives every
 * pixel's set, numbered by smallest pixel, *n_sets the set count;
 * clusters (capacity records; may be NULL) the kept sets in the
 * reference's order (vecSegResults), *n_clusters their count.  The solve
 * of cluster N reads the inpainted depth (planes->inpainted) masked to it
 * (SegResults.clusterDepth). */
qpso_status qpso_segment_rgbd(qpso_context *ctx, const uint8_t *bgr, const uint16_t *depth_mm,
                              uint32_t width, uint32_t height, const qpso_seg_params *prm,
                              const qpso_seg_front_params *fp, int32_t *labels, uint32_t *n_sets,
                              qpso_seg_cluster *clusters, uint32_t capacity, uint32_t *n_clusters,
                              const qpso_seg_frame_out *planes);

/* PostSegmFilter over a given label map (labels 0..n_sets-1, -1 none),
 * its inpainted depth and its HSV value plane, all on the host: per-set
 * moments on the GPU, the filter on the host.  With keep_all != 0 every
 * set's record is returned (kept says which pass), else only the kept
 * ones, in label order. */
qpso_status qpso_segment_clusters(qpso_context *ctx, const int32_t *labels, uint32_t n_sets,
                                  const uint16_t *inpainted_mm, const uint8_t *v_plane, uint32_t width,
                                  uint32_t height, const qpso_seg_front_params *fp, int keep_all,
                                  qpso_seg_cluster *out, uint32_t capacity, uint32_t *n_out);

#ifdef __cplusplus
}
#endif
#endif /* QPSO_H */
