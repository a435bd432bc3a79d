/*
 * qpso_oracle.h -- scalar CPU restatement of the Q-PSO pose-solve hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle for the CUDA path in
 * q-pso_gb300/csrc: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline arm may load it.  The product path never calls it and has no CPU
 * fallback.
 *
 * Parity status: pinned.  The reference ships no tests, fixtures or golden
 * vectors.  The quaternion helpers, the vertex rotation and the fixed-point
 * rasteriser of the reference's main.h are compiled from the reference
 * sources by oracle/ref_pin (stub headers for OpenCV/assimp, one emulated
 * thread) and their outputs are committed as tests/golden fixtures; this
 * restatement is checked against them.  The reference's whole program
 * cannot be built (OpenCV 2.4, GSL and a missing header), but its kernels
 * can: oracle/build.py compiles main.h and main.cu:72-1195 for the GPU, and
 * tests/test_gpu_ref_kernels.py checks this restatement's raster, fitness,
 * init, best update and particle update against them on identical inputs.
 * Only GSL's random stream stays unpinned (Philox replaces it).
 * The segmentation's graph stage (GraphCannySeg's smoothing, depth
 * normalisation, edge weights, segment_graph, small-component merge and
 * collectSets) is compiled from the reference sources by oracle/build.py
 * (build_seg_pin) and pinned the same way (tests/golden/ref_seg*.npz).
 *
 * Arithmetic contract shared with the CUDA kernels (both sides must agree
 * bit for bit):
 *   - every float expression is evaluated in source order with one IEEE
 *     rounding per operation (no contraction: gcc -ffp-contract=off, nvcc
 *     --fmad=false), except the projection u = cx + fx*(x/z), which the
 *     reference evaluates in double (its intrinsics are double macros) and
 *     which both sides evaluate as one fp32 fused multiply-add;
 *   - int32 edge arithmetic wraps modulo 2^32, right shifts are arithmetic,
 *     float->int conversion rounds half to even and saturates (NaN -> 0),
 *     exactly like cvt.rni.s32.f32;
 *   - sin, cos and acos are this project's own fp32 series
 *     (qo_sinf/qo_cosf/qo_acosf), not libm or CUDA's;
 *   - random numbers come from Philox4x32-10 (Salmon et al., SC'11).
 */
#ifndef QPSO_ORACLE_H
#define QPSO_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QO_NDIM 7
#define QO_DEPTH_BG 60000         /* maxVal_depthBufferInt, main.h:157 */
#define QO_AABB_INIT_MIN 50000    /* max_AABB_, main.h:159 */
#define QO_AABB_INIT_MAX (-1)     /* min_AABB_, main.h:160 */
#define QO_GUARD 1024             /* raster domain = image grown by this many px per side */

typedef struct {
    float fx, fy, cx, cy;
    int32_t width, height;
    /* QO_PROJ_FP32: u = fmaf(fx, x/z, cx) with the fields above (the
     * kernels' contract).  QO_PROJ_REF_ACCV: the reference's own
     * expression with its compiled-in double ACCV intrinsics (main.h:30-33),
     * u = (float)(CX + FX * (double)(x/z)), fx..cy ignored; used to check
     * the reference's kernels rebuilt for the GPU. */
    int32_t proj;
} qo_camera;

#define QO_PROJ_FP32 0
#define QO_PROJ_REF_ACCV 1

/* Per-solve constants: QPSOParams_t (main.h:182-204) plus the compile-time
 * macros of main.h:83-136 that this project makes runtime parameters. */
typedef struct {
    float c1, c2;                 /* c1_, c2_ (main.h:104-105) */
    double w;                     /* psoW_ 0.3 (main.h:106), applied in double */
    float vdot;                   /* vdot_ 3 (main.h:126) */
    float ang_lo, ang_hi;         /* aminX_/amaxX_ -10/10 (main.h:118-123) */
    float qinit[4];               /* InitQPSO qinit (main.cu:128-132) */
    float t_lo[3], t_hi[3];       /* x_lo, x_hi (main.cu:1318-1323) */
    int32_t cl_min_x, cl_max_x, cl_min_y, cl_max_y; /* cluster AABB, br() exclusive */
    uint32_t num_points;          /* num_point_SegmentedCluster */
    uint32_t num_particles;
    uint32_t iterations;
    uint64_t seed;
    uint32_t stream;              /* Philox stream id of this solve instance */
    uint32_t raster_mode;         /* QO_RASTER_REF (0) or QO_RASTER_EDGE (1) */
} qo_params;

/* Raster modes.  REF: what the reference computes, every pixel of a front
 * face's bounding rectangle (its inside mask is never applied).  EDGE: the
 * inside test the reference's mask encodes (main.h:1440), pixels with all
 * three biased edge functions > 0 (top-left fill convention). */
#define QO_RASTER_REF 0
#define QO_RASTER_EDGE 1

typedef struct {
    uint32_t n_rendered;          /* sNrenderedPointsWarpBallot total */
    uint32_t n_no_obs;            /* sNumRenderedDepthWoutValid3dClusterPixel */
    uint32_t n_seg_rendered;      /* rendered pixels with observed depth */
    uint32_t n_seg_not_rendered;  /* sNumSegDepthWoutValid3dModelPixel */
    uint64_t sq_lo, sq_hi;        /* sum of (z_r - z_k)^2 in mm^2, 128 bit */
    int32_t r_min_x, r_max_x, r_min_y, r_max_y;   /* render AABB */
    int32_t w_min_x, w_max_x, w_min_y, w_max_y;   /* fitness window */
    int32_t partial_len;          /* pixels visited on row w_max_y */
    float fit;
} qo_score;

/* ---- RNG ---- */
void qo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
float qo_uniform(uint64_t seed, uint32_t stream, uint32_t particle, uint32_t draw);

/* ---- math ---- */
double qo_sin(double x);
double qo_cos(double x);
double qo_acos(double x);
float qo_sinf(float x);
float qo_cosf(float x);
float qo_acosf(float x);

/* ---- quaternion helpers (7-float PSO state vectors) ---- */
void qo_quat_prod(const float *p, const float *q, float *out);
void qo_quat_prod_conj(const float *p, const float *q, float *out);
void qo_normalize_quat(float *s);
void qo_cast_top_half(float *q4);
void qo_quat_kinematics(float *s, const float *w);
void qo_quat_kinematics_init(const float *qinit7, float *s, const float *w);
void qo_rotate(const float *s, const float v[3], float out[3]);
void qo_project(const float *s, const float v[3], const qo_camera *cam, float out[3]);

/* ---- raster ---- */
/* z-buffer over the raster domain [-QO_GUARD, width+QO_GUARD) x
 * [-QO_GUARD, height+QO_GUARD), row-major, initialised to QO_DEPTH_BG. */
int32_t qo_domain_w(const qo_camera *cam);
int32_t qo_domain_h(const qo_camera *cam);
void qo_zbuf_reset(int32_t *zbuf, const qo_camera *cam);
/* Rasterise one face given its three projected vertices (u, v, z_mm).
 * Updates the render AABB in box[4] = {minx,maxx,miny,maxy}.  Returns the
 * number of pixel writes issued inside the domain. */
int64_t qo_raster_face(const float v1[3], const float v2[3], const float v3[3],
                       const qo_camera *cam, int32_t *zbuf, int32_t box[4]);
/* Render a whole mesh (loadOBJ3 SoA layout, 9*F floats) at pose s. */
int64_t qo_render(const float *mesh, uint32_t num_faces, const float *s,
                  const qo_camera *cam, int32_t *zbuf, int32_t box[4]);
/* The same with a raster mode; in EDGE mode the returned count is the
 * number of covered pixels written. */
int64_t qo_raster_face_mode(const float v1[3], const float v2[3], const float v3[3],
                            const qo_camera *cam, int32_t *zbuf, int32_t box[4], uint32_t mode);
int64_t qo_render_mode(const float *mesh, uint32_t num_faces, const float *s,
                       const qo_camera *cam, int32_t *zbuf, int32_t box[4], uint32_t mode);

/* The reference's host render of the best pose (RenderCPU): iround snapping,
 * float depth, the image only (width*height floats, row-major, filled with
 * the background 60000 first). */
void qo_raster_face_cpu(const float v1[3], const float v2[3], const float v3[3],
                        const qo_camera *cam, float *depth);
void qo_render_cpu(const float *mesh, uint32_t num_faces, const float *s,
                   const qo_camera *cam, float *depth);

/* ---- fitness ---- */
void qo_score_zbuf(const int32_t *zbuf, const int32_t box[4], const uint16_t *obs,
                   const qo_camera *cam, const qo_params *prm, qo_score *out);
float qo_fitness_from_counts(uint32_t n_seg_not_rendered, uint32_t n_rendered,
                             uint32_t n_no_obs, uint64_t sq_lo, uint64_t sq_hi,
                             uint32_t num_points);
double qo_fitness_fp64(const qo_score *sc, uint32_t num_points);

/* ---- PSO ---- */
void qo_init_particle(const qo_params *prm, uint32_t p, float *pos, float *vel, float *pbest);
void qo_update_particle(const qo_params *prm, uint32_t p, uint32_t iter,
                        float *pos, float *vel, const float *pbest, const float *gbest);

/* Full solve.  Arrays are SoA [7][P] (index p + d*P) like main.cu:1389-1465.
 * trace_gbest (optional) receives iterations x 8 floats (fit, pose[7]) after
 * each best update; trace_fit (optional) receives iterations x P fitness. */
typedef struct {
    float gbest_fit;
    float gbest[QO_NDIM];
    uint64_t raster_writes;
} qo_result;

int qo_solve(const float *mesh, uint32_t num_faces, const uint16_t *obs,
             const qo_camera *cam, const qo_params *prm,
             float *pos, float *vel, float *pbest, float *pbest_fit,
             qo_result *res, float *trace_gbest, float *trace_fit);

int qo_solve_mt(const float *mesh, uint32_t num_faces, const uint16_t *obs,
                const qo_camera *cam, const qo_params *prm,
                float *pos, float *vel, float *pbest, float *pbest_fit,
                qo_result *res, float *trace_gbest, float *trace_fit, int threads);

void qo_default_params(qo_params *prm);

/* ---- segmentation core (the producer of the clusters) ----
 * The disjoint-set forest, segment_graph and the small-component merge of
 * the reference's graph segmentation (GraphCannySeg.cpp:231-272,
 * 1301-1373, 1243-1248), and the listing of its sets that numbers the
 * clusters (collectSets, GraphCannySeg.cpp:305-352).  Pinned against
 * those functions compiled from the reference sources (oracle/ref_pin,
 * build_seg_pin) and against fixtures frozen from them. */
typedef struct {
    float w;
    int32_t a, b;
} qo_edge;

/* Sorts the edges by weight in place (ascending; ties keep their input
 * order, where the reference's unstable std::sort leaves the order of equal
 * weights to the C++ library: DEVIATION) unless presorted != 0, merges
 * with threshold k / |C| (segment_graph), then, when merge != 0, joins the
 * ends of every edge, in the same order, whose components differ and one of
 * which is smaller than min_size.  Then lists the sets as collectSets does:
 * one list per set in the order of the set's smallest pixel index, each
 * [first pixel, its parent, the rest of the set's circular list], so a set
 * of n pixels gives a list of n + 1 entries.
 *
 * offsets receives n_lists + 1 entries (capacity n_vertices + 1), points
 * the lists' pixel indices (capacity 2 * n_vertices).  *num_sets receives
 * the forest's set count.  Returns n_lists, or -1 on bad arguments
 * (non-positive n_vertices, an edge end out of range, a NaN weight). */
int32_t qo_segment_graph(int32_t n_vertices, int32_t n_edges, qo_edge *edges, int32_t presorted,
                         float k, float min_size, int32_t merge, int32_t *offsets, int32_t *points,
                         int32_t *num_sets);

/* The pixel graph of segment_image (GraphCannySeg.cpp:1053-1250) for an
 * HSV image, its inpainted depth and its saliency, with the constants the
 * reference's main passes (main.h:58-65, main.cu:1214-1217). */
typedef struct {
    float sigma;      /* 0.8, Gaussian smoothing of each HSV plane */
    float k;          /* 50 / 10000, segment_graph threshold constant */
    float min_size;   /* 500, small-component merge */
    float kx, ky, ks; /* 2000, 30, 49 / 1000: weight mix (ky is unread) */
    float kdv, kdc;   /* 4.5, 0.1: HSV distance weights */
} qo_seg_params;

void qo_seg_default_params(qo_seg_params *sp);

/* smooth (GraphCannySeg.h:423-489): the mask exp(-(i/sigma)^2 / 2),
 * i < ceil(4 sigma) + 1, normalised to unit sum over both sides; a pass
 * along the rows then one along the columns, edges clamped. */
int32_t qo_gauss_mask(float sigma, float *mask, int32_t capacity);
int32_t qo_smooth(const float *src, int32_t W, int32_t H, float sigma, float *dst);

/* the depth mapped to [0, 1] by the minimum and maximum of every pixel
 * but the last (GraphCannySeg.cpp:1105-1127: the ranges end at the last
 * pixel's address) */
void qo_depth_norm(const uint16_t *depth, int32_t W, int32_t H, float *out);

/* the weight of the edge from pivot (x1, y1) to neighbour (x2, y2): the
 * HSV + depth + saliency branch of diff (GraphCannySeg.h:2051-2288) over
 * smoothed planes (H in 0..180, S and V in 0..255), normalised depth and
 * saliency */
float qo_edge_weight(const float *sh, const float *ss, const float *sv, const float *dnorm,
                     const float *sal, int32_t W, int32_t x1, int32_t y1, int32_t x2, int32_t y2,
                     const qo_seg_params *sp);

/* the edges in the reference's order: per pixel in row-major order, to
 * (x+1, y), (x, y+1), (x+1, y+1), (x+1, y-1) where inside
 * (GraphCannySeg.cpp:1174-1210); capacity 4 W H; returns the count */
int32_t qo_graph_edges(const float *sh, const float *ss, const float *sv, const float *dnorm,
                       const float *sal, int32_t W, int32_t H, const qo_seg_params *sp, qo_edge *out);

/* End to end from 8-bit HSV planes, uint16 depth (mm) and saliency: the
 * planes as floats, smoothed, the depth normalised, the graph, then
 * qo_segment_graph with k and min_size (merge on).  Returns n_lists, or -1
 * (bad sizes, or a NaN weight: a depth image whose pixels but the last are
 * all equal). */
int32_t qo_segment_planes(const uint8_t *h8, const uint8_t *s8, const uint8_t *v8,
                          const uint16_t *depth, const float *sal, int32_t W, int32_t H,
                          const qo_seg_params *sp, int32_t *offsets, int32_t *points,
                          int32_t *num_sets);

/* ---- the stages around the graph segmentation (qpso_seg_front.c) ----
 * GraphCannySeg<hsv>::run (GraphCannySeg.cpp:1438-1459) before and after
 * segment_image, restated from the published algorithms OpenCV implements;
 * unpinned against OpenCV (absent here).  See qpso_seg_front.c. */
typedef struct {
    float beta, gamma;          /* dynamicDepthSmoothing(2000), gamma 18000 */
    int32_t inpaint_radius;     /* 20: cv::inpaint radius (GraphCannySeg.h:1186) */
    float canny_low, canny_high;/* Lcanny / 1000, Hcanny / 1000 (main.h:75-76, main.cu:1220-1221) */
    int32_t dth, plus_d, point_3d; /* 30, 7, 5 (main.h:70-72) */
    float g_angle, l_angle;     /* 148 and 151 degrees in radians (main.h:73-74) */
    float fx, fy, cx, cy;       /* k_vec (main.h:51-56): the ACCV intrinsics */
    float far_obj_z;            /* 1500 mm (main.h:77) */
    float max_ecc, max_l1, max_l2; /* 0.978, 13800, 1950 (main.h:66-68) */
} qo_seg_front_params;

void qo_seg_front_default_params(qo_seg_front_params *fp);

void qo_bgr_to_hsv_gray(const uint8_t *bgr, int32_t n, uint8_t *h, uint8_t *s, uint8_t *v,
                        uint8_t *gray);
float qo_smooth_alfa(void);
/* out: smoothed depth; c_out (optional): the depth-change map (0/1);
 * r_out (optional): the smoothing radius map R before rounding */
int32_t qo_depth_smooth(const uint16_t *d, int32_t W, int32_t H, float beta, float gamma,
                        uint16_t *out, uint8_t *c_out, float *r_out);
void qo_resize_bilinear_u8(const uint8_t *src, int32_t sw, int32_t sh, uint8_t *dst, int32_t dw, int32_t dh);
float qo_eikonal2(float a, float b);
/* arrival times of the masked pixels; Jacobi iterations used, or -1 */
int32_t qo_telea_times(const uint8_t *mask, int32_t w, int32_t h, float *T);
/* inpaints img where mask != 0 in place; returns the pixels filled */
int32_t qo_telea(uint8_t *img, const uint8_t *mask, int32_t w, int32_t h, int32_t radius);
/* small_out (optional, capacity (W/5 + 1) (H/5 + 1)): the shrunk 8-bit map after inpainting */
int32_t qo_inpaint_depth(const uint16_t *sm, int32_t W, int32_t H, int32_t radius, uint16_t *out,
                         uint8_t *small_out, int32_t *small_w, int32_t *small_h);
int32_t qo_gauss_taps(int32_t ksize, int32_t *taps);
void qo_blur_u8(const uint8_t *src, int32_t W, int32_t H, int32_t ksize, uint8_t *dst);
int32_t qo_orient_bin(int32_t x, int32_t y);
float qo_angle3(const float p1[3], const float p0[3], const float p2[3]);
/* sal: the saliency map; edges_out (optional): the 0/255 edge map after
 * the depth test, before the 7x7 blur */
int32_t qo_canny_saliency(const uint8_t *gray, const uint16_t *inp, int32_t W, int32_t H,
                          const qo_seg_front_params *fp, float *sal, uint8_t *edges_out);

/* One set of the label map with the fields of SegResults the solve reads
 * and the quantities PostSegmFilter tests. */
typedef struct {
    int32_t label;
    uint32_t num_points;        /* n + 1: the length of the reference's list */
    uint32_t pixels;            /* n */
    int32_t min_x, max_x, min_y, max_y; /* boundingRect, max exclusive */
    float centroid_mm[3];
    float nan_ratio, dark_ratio;
    double eig[2];
    double eccentricity;
    int32_t far, kept;
} qo_seg_cluster;

void qo_seg_cluster_stats(int64_t n, int64_t sx, int64_t sy, int64_t sxx, int64_t syy, int64_t sxy,
                          int64_t nz, int64_t sz, int64_t suz, int64_t svz, int64_t nzero, const int64_t vb[3],
                          const qo_seg_front_params *fp, qo_seg_cluster *r);
/* labels: 0..n_sets-1 (sets numbered by smallest pixel), -1 none; out:
 * capacity n_sets; the kept records (every record with keep_all != 0) in
 * label order; returns their count */
int32_t qo_seg_clusters(const int32_t *labels, int32_t n_sets, const uint16_t *inp, const uint8_t *v8,
                        int32_t W, int32_t H, const qo_seg_front_params *fp, qo_seg_cluster *out,
                        int32_t keep_all);

#ifdef __cplusplus
}
#endif
#endif
