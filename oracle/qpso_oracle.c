/*
 * qpso_oracle.c -- scalar CPU restatement of the Q-PSO pose-solve hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle; see qpso_oracle.h for the parity
 * status and the arithmetic contract).  Build with -ffp-contract=off.
 *
 * Every function cites the reference file:line it restates.  Where the
 * reference is racy, undefined or launch-shape dependent, the restatement
 * fixes one deterministic meaning; each such point is marked DEVIATION.
 */
#include "qpso_oracle.h"

#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* Philox4x32-10, Salmon, Moraes, Dror, Shaw, "Parallel random numbers:
 * as easy as 1, 2, 3", SC'11.  Replaces the GSL mt19937 table of
 * main.cu:1337-1352 (capped at 512 draws per particle). */
void qo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Draw number `draw` of particle `particle` in stream `stream`: counter
 * (draw/4, particle, stream, 0), key (seed lo, seed hi), lane draw%4,
 * top 24 bits scaled to [0, 1). */
float qo_uniform(uint64_t seed, uint32_t stream, uint32_t particle, uint32_t draw)
{
    uint32_t ctr[4] = {draw >> 2, particle, stream, 0u};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t o[4];
    qo_philox4x32_10(ctr, key, o);
    return (float)(o[draw & 3u] >> 8) * 0x1p-24f;
}

/* ------------------------------------------------------------------ */
/* sin/cos/acos.  The reference calls CUDA's cosf/sinf/acosf under
 * -use_fast_math (main.h:287-294, 391-399; main.cu:946,970); those differ
 * between CUDA and libm, so both sides of this project use the same series
 * instead.  The double forms (Cody-Waite reduction by pi/2 in three 30-bit
 * parts, Taylor polynomials on [-pi/4, pi/4], truncation < 1e-19; acos via
 * asin's Taylor series on [0, 1/2] and acos(x) = 2 asin(sqrt((1-x)/2))
 * above 1/2) serve as the reference and as the fallback of the fp32 forms
 * below for arguments beyond 4096. */
static const double QO_PIO2_1 = 1.5707963276654482;
static const double QO_PIO2_2 = -8.705515692000731e-10;
static const double QO_PIO2_3 = -3.50343439808993e-19;
static const double QO_2OPI = 0.6366197723675814;
static const double QO_PI = 3.141592653589793;
static const double QO_PIO2 = 1.5707963267948966;

static double qo_sin_kernel(double r)
{
    double r2 = r * r;
    double p = 2.8114572543455206e-15;
    p = p * r2 + -7.647163731819816e-13;
    p = p * r2 + 1.6059043836821613e-10;
    p = p * r2 + -2.505210838544172e-08;
    p = p * r2 + 2.7557319223985893e-06;
    p = p * r2 + -0.0001984126984126984;
    p = p * r2 + 0.008333333333333333;
    p = p * r2 + -0.16666666666666666;
    return r + r * (r2 * p);
}

static double qo_cos_kernel(double r)
{
    double r2 = r * r;
    double p = -1.5619206968586225e-16;
    p = p * r2 + 4.779477332387385e-14;
    p = p * r2 + -1.1470745597729725e-11;
    p = p * r2 + 2.08767569878681e-09;
    p = p * r2 + -2.755731922398589e-07;
    p = p * r2 + 2.48015873015873e-05;
    p = p * r2 + -0.001388888888888889;
    p = p * r2 + 0.041666666666666664;
    p = p * r2 + -0.5;
    return 1.0 + r2 * p;
}

/* Reduce x to r in [-pi/4, pi/4] and quadrant q = k mod 4. */
static double qo_reduce(double x, int *q)
{
    double ax = fabs(x);
    if (ax > 1.0e6) {
        /* outside any argument this solver produces; fmod is exact on both
         * sides, so the result is still deterministic */
        x = fmod(x, 2.0 * QO_PI);
    }
    double k = rint(x * QO_2OPI);
    double r = x - k * QO_PIO2_1;
    r = r - k * QO_PIO2_2;
    r = r - k * QO_PIO2_3;
    long long ki = (long long)k;
    *q = (int)(ki & 3);
    return r;
}

double qo_sin(double x)
{
    if (x != x || isinf(x)) return x - x;
    int q;
    double r = qo_reduce(x, &q);
    switch (q) {
    case 0: return qo_sin_kernel(r);
    case 1: return qo_cos_kernel(r);
    case 2: return -qo_sin_kernel(r);
    default: return -qo_cos_kernel(r);
    }
}

double qo_cos(double x)
{
    if (x != x || isinf(x)) return x - x;
    int q;
    double r = qo_reduce(x, &q);
    switch (q) {
    case 0: return qo_cos_kernel(r);
    case 1: return -qo_sin_kernel(r);
    case 2: return -qo_cos_kernel(r);
    default: return qo_sin_kernel(r);
    }
}

static const double QO_ASIN_C[27] = {
    0.16666666666666666, 0.075, 0.044642857142857144, 0.030381944444444444,
    0.022372159090909092, 0.017352764423076924, 0.01396484375,
    0.011551800896139705, 0.009761609529194078, 0.008390335809616815,
    0.0073125258735988454, 0.006447210311889649, 0.005740037670841924,
    0.005153309682319905, 0.004660143486915096, 0.004240907093679363,
    0.003880964558837669, 0.0035692053938259347, 0.003297059503473485,
    0.0030578216492580306, 0.002846178401108942, 0.00265787063820729,
    0.0024894486782468836, 0.002338091892111975, 0.0022014739737101384,
    0.0020776610325181676, 0.0019650336162772837};

/* asin on [-1/2, 1/2] */
static double qo_asin_kernel(double x)
{
    double x2 = x * x;
    double p = QO_ASIN_C[26];
    for (int i = 25; i >= 0; --i) p = p * x2 + QO_ASIN_C[i];
    return x + x * (x2 * p);
}

double qo_acos(double x)
{
    if (x != x) return x;
    if (x > 1.0) x = 1.0;
    if (x < -1.0) x = -1.0;
    if (x > 0.5) return 2.0 * qo_asin_kernel(sqrt((1.0 - x) * 0.5));
    if (x < -0.5) return QO_PI - 2.0 * qo_asin_kernel(sqrt((1.0 + x) * 0.5));
    return QO_PIO2 - qo_asin_kernel(x);
}

/* fp32 forms used by the PSO step: Cody-Waite reduction by pi/2 split in
 * three parts of 12, 12 and 24 bits (k*P1 and k*P2 exact for |x| <= 4096,
 * larger arguments fall back to the double routines), Taylor polynomials
 * on [-pi/4, pi/4] (truncation < 7e-12), asin's Taylor series to x^23 on
 * [0, 1/2] (truncation < 5e-10), all in fp32 with one rounding per
 * operation.  GB300's fp64 pipe is narrow, so the step stays in fp32. */
static const float QF_P1 = 1.57080078125f;
static const float QF_P2 = -4.453584551811218e-06f;
static const float QF_P3 = -8.705515752716053e-10f;
static const float QF_2OPI = 0.6366197466850281f;
static const float QF_PI = 3.1415927410125732f;
static const float QF_PIO2 = 1.5707963705062866f;

static float qf_sin_kernel(float r)
{
    const float r2 = r * r;
    float p = -2.5052107943679403e-08f;
    p = p * r2 + 2.7557318844628753e-06f;
    p = p * r2 + -0.00019841270113829523f;
    p = p * r2 + 0.008333333767950535f;
    p = p * r2 + -0.1666666716337204f;
    return r + r * (r2 * p);
}

static float qf_cos_kernel(float r)
{
    const float r2 = r * r;
    float p = 2.0876755879584152e-09f;
    p = p * r2 + -2.755731998149713e-07f;
    p = p * r2 + 2.4801587642286904e-05f;
    p = p * r2 + -0.0013888889225199819f;
    p = p * r2 + 0.0416666679084301f;
    p = p * r2 + -0.5f;
    return 1.0f + r2 * p;
}

static float qf_reduce(float x, int *q)
{
    const float k = rintf(x * QF_2OPI);
    float r = x - k * QF_P1;
    r = r - k * QF_P2;
    r = r - k * QF_P3;
    *q = (int)((long)k & 3);
    return r;
}

float qo_sinf(float x)
{
    if (x != x || isinf(x)) return x - x;
    if (fabsf(x) > 4096.0f) return (float)qo_sin((double)x);
    int q;
    const float r = qf_reduce(x, &q);
    switch (q) {
    case 0: return qf_sin_kernel(r);
    case 1: return qf_cos_kernel(r);
    case 2: return -qf_sin_kernel(r);
    default: return -qf_cos_kernel(r);
    }
}

float qo_cosf(float x)
{
    if (x != x || isinf(x)) return x - x;
    if (fabsf(x) > 4096.0f) return (float)qo_cos((double)x);
    int q;
    const float r = qf_reduce(x, &q);
    switch (q) {
    case 0: return qf_cos_kernel(r);
    case 1: return -qf_sin_kernel(r);
    case 2: return -qf_cos_kernel(r);
    default: return qf_sin_kernel(r);
    }
}

static const float QF_ASIN_C[11] = {
    0.1666666716337204f, 0.07500000298023224f, 0.0446428582072258f, 0.0303819440305233f,
    0.022372158244252205f, 0.017352763563394547f, 0.013964843936264515f, 0.01155180111527443f,
    0.009761609137058258f, 0.008390335366129875f, 0.007312525995075703f};

static float qf_asin_kernel(float x)
{
    const float x2 = x * x;
    float p = QF_ASIN_C[10];
    for (int i = 9; i >= 0; --i) p = p * x2 + QF_ASIN_C[i];
    return x + x * (x2 * p);
}

/* acos with the argument clamped to [-1, 1] (DEVIATION: the reference's
 * acosf of a dot product that rounds to 1 + ulp is NaN). */
float qo_acosf(float x)
{
    if (x != x) return x;
    if (x > 1.0f) x = 1.0f;
    if (x < -1.0f) x = -1.0f;
    if (x > 0.5f) return 2.0f * qf_asin_kernel(sqrtf((1.0f - x) * 0.5f));
    if (x < -0.5f) return QF_PI - 2.0f * qf_asin_kernel(sqrtf((1.0f + x) * 0.5f));
    return QF_PIO2 - qf_asin_kernel(x);
}

/* ------------------------------------------------------------------ */
/* Quaternion helpers.  State vectors are [tx,ty,tz,q0,q1,q2,q3]
 * (main.h:88-94). */
#define TX 0
#define TY 1
#define TZ 2
#define Q0 3
#define Q1 4
#define Q2 5
#define Q3 6
#define QO_MIN_NORM 1.0e-7f /* MIN_NORM_, main.h:95 */

/* QuatProd_pqPSOstateVect, main.h:248-254 (p, q are 7-vectors) */
void qo_quat_prod(const float *p, const float *q, float *o)
{
    o[0] = p[Q0] * q[Q0] - p[Q1] * q[Q1] - p[Q2] * q[Q2] - p[Q3] * q[Q3];
    o[1] = p[Q1] * q[Q0] + p[Q0] * q[Q1] + p[Q2] * q[Q3] - p[Q3] * q[Q2];
    o[2] = p[Q2] * q[Q0] + p[Q0] * q[Q2] + p[Q3] * q[Q1] - p[Q1] * q[Q3];
    o[3] = p[Q3] * q[Q0] + p[Q0] * q[Q3] + p[Q1] * q[Q2] - p[Q2] * q[Q1];
}

/* QuatProd_pq_1PSOstateVect, main.h:256-264: p * conj(q) */
void qo_quat_prod_conj(const float *p, const float *q, float *o)
{
    o[0] = p[Q0] * q[Q0] + p[Q1] * q[Q1] + p[Q2] * q[Q2] + p[Q3] * q[Q3];
    o[1] = p[Q1] * q[Q0] - p[Q0] * q[Q1] - p[Q2] * q[Q3] + p[Q3] * q[Q2];
    o[2] = p[Q2] * q[Q0] - p[Q0] * q[Q2] - p[Q3] * q[Q1] + p[Q1] * q[Q3];
    o[3] = p[Q3] * q[Q0] - p[Q0] * q[Q3] - p[Q1] * q[Q2] + p[Q2] * q[Q1];
}

/* NormalizeQuaternionPSOstateVect, main.h:209-221 (__frcp_rn == 1/x) */
void qo_normalize_quat(float *s)
{
    const float den = sqrtf(s[Q0] * s[Q0] + s[Q1] * s[Q1] + s[Q2] * s[Q2] + s[Q3] * s[Q3]);
    if (den > QO_MIN_NORM) {
        const float r = 1.0f / den;
        s[Q0] = s[Q0] * r;
        s[Q1] = s[Q1] * r;
        s[Q2] = s[Q2] * r;
        s[Q3] = s[Q3] * r;
    }
}

/* Cast2TopHalfHypersphere, main.h:236-246 (4-vector) */
void qo_cast_top_half(float *q)
{
    if (q[0] < 0.0f) {
        q[0] = -q[0]; q[1] = -q[1]; q[2] = -q[2]; q[3] = -q[3];
    }
}

static void qo_cast_top_half_state(float *s) /* main.h:223-234 */
{
    if (s[Q0] < 0.0f) {
        s[Q0] = -s[Q0]; s[Q1] = -s[Q1]; s[Q2] = -s[Q2]; s[Q3] = -s[Q3];
    }
}

/* Exponential-map step shared by QuatKinematicsPSOStateVectWithInit
 * (main.h:266-307) and QuatKinematicsPSOStateVect (main.h:373-413):
 * q <- cos(|w Ts|/2) q0 + 1/2 sinc (q0 (x) (0, w Ts)), renormalised and cast
 * to the top half.  mTs_ = 0.5 (main.h:96) scales exactly. */
static void qo_kinematics(const float *q_from, float *s, const float *w)
{
    float wt[7] = {0, 0, 0, 0, 0, 0, 0};
    wt[Q1] = w[Q1] * 0.5f;
    wt[Q2] = w[Q2] * 0.5f;
    wt[Q3] = w[Q3] * 0.5f;
    const float nrm = sqrtf(wt[Q1] * wt[Q1] + wt[Q2] * wt[Q2] + wt[Q3] * wt[Q3]);
    const float dom = nrm * 0.5f;
    const float cosw = qo_cosf(dom);
    float sinw;
    if (dom < QO_MIN_NORM) {
        sinw = 1.0f;
    } else {
        const float r = 1.0f / dom;
        sinw = qo_sinf(dom) * r;
    }
    float qxw[4];
    qo_quat_prod(q_from, wt, qxw);
    float qn[4];
    for (int i = 0; i < 4; ++i) qn[i] = cosw * q_from[Q0 + i] + 0.5f * sinw * qxw[i];
    for (int i = 0; i < 4; ++i) s[Q0 + i] = qn[i];
    qo_normalize_quat(s);
    qo_cast_top_half_state(s);
}

void qo_quat_kinematics(float *s, const float *w)
{
    float from[7];
    memcpy(from, s, sizeof(from));
    qo_kinematics(from, s, w);
}

void qo_quat_kinematics_init(const float *qinit7, float *s, const float *w)
{
    qo_kinematics(qinit7, s, w);
}

/* quatVectRotationPSOstateVect, main.h:328-347: t = 2 q.xyz x v;
 * v' = v + q.w t + q.xyz x t (cross product as in main.h:309-326). */
void qo_rotate(const float *s, const float v[3], float o[3])
{
    float t[3], k[3];
    t[0] = s[Q2] * v[2] - s[Q3] * v[1];
    t[1] = -(s[Q1] * v[2] - s[Q3] * v[0]);
    t[2] = s[Q1] * v[1] - s[Q2] * v[0];
    t[0] = 2.0f * t[0]; t[1] = 2.0f * t[1]; t[2] = 2.0f * t[2];
    k[0] = s[Q2] * t[2] - s[Q3] * t[1];
    k[1] = -(s[Q1] * t[2] - s[Q3] * t[0]);
    k[2] = s[Q1] * t[1] - s[Q2] * t[0];
    o[0] = v[0] + s[Q0] * t[0] + k[0];
    o[1] = v[1] + s[Q0] * t[1] + k[1];
    o[2] = v[2] + s[Q0] * t[2] + k[2];
}

/* projectModelPointsToPixels(const float*, const float4&, float4&),
 * main.h:513-545: rotate, translate, u = cx + fx x/z, v = cy + fy y/z with
 * x/z = x * rcp_rn(z), z in mm.  DEVIATION: the reference's intrinsics are
 * double macros, so it evaluates cx + fx*(x/z) in double; this library takes
 * fp32 intrinsics at run time and evaluates it as one fp32 fma. */
void qo_project(const float *s, const float v[3], const qo_camera *cam, float o[3])
{
    float p[3];
    qo_rotate(s, v, p);
    p[0] = p[0] + s[TX];
    p[1] = p[1] + s[TY];
    p[2] = p[2] + s[TZ];
    const float rz = 1.0f / p[2];
    if (cam->proj == QO_PROJ_REF_ACCV) {
        /* main.h:537-539 with FX, FY, CX, CY of main.h:30-33 */
        o[0] = (float)(325.26110 + 572.41140 * (double)(p[0] * rz));
        o[1] = (float)(242.04899 + 573.57043 * (double)(p[1] * rz));
    } else {
        o[0] = fmaf(cam->fx, p[0] * rz, cam->cx);
        o[1] = fmaf(cam->fy, p[1] * rz, cam->cy);
    }
    o[2] = 1000.0f * p[2];
}

/* ------------------------------------------------------------------ */
/* Fixed-point raster.  Integer helpers give the wrap-around, arithmetic
 * shift and saturating round-to-nearest-even conversion that the reference
 * gets from CUDA (int32 arithmetic, >> on int, __float2int_rn). */
static inline int32_t w_add(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
static inline int32_t w_sub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
static inline int32_t w_mul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }
static inline int32_t w_shl(int32_t a, int s) { return (int32_t)((uint32_t)a << s); }
static inline int32_t asr(int32_t a, int s) { return a >> s; } /* gcc: arithmetic */
static inline int32_t imin(int32_t a, int32_t b) { return a < b ? a : b; }
static inline int32_t imax(int32_t a, int32_t b) { return a > b ? a : b; }

static inline int32_t f2i_rn(float f)
{
    if (f != f) return 0;
    if (f >= 2147483648.0f) return INT32_MAX;
    if (f <= -2147483648.0f) return INT32_MIN;
    return (int32_t)nearbyintf(f); /* default rounding mode: half to even */
}

int32_t qo_domain_w(const qo_camera *cam) { return cam->width + 2 * QO_GUARD; }
int32_t qo_domain_h(const qo_camera *cam) { return cam->height + 2 * QO_GUARD; }

void qo_zbuf_reset(int32_t *zbuf, const qo_camera *cam)
{
    size_t n = (size_t)qo_domain_w(cam) * (size_t)qo_domain_h(cam);
    for (size_t i = 0; i < n; ++i) zbuf[i] = QO_DEPTH_BG;
}

/* renderFixedPointAABB, main.h:1306-1491, for one face.
 *
 * Quirks kept exactly: the inside test is a no-op (the mask of main.h:1440
 * is 0 or 1 and the guard of main.h:1473 tests its sign bit), so every pixel
 * of the face's integer bounding rectangle is written; depth is
 * z1 + cx2*(z2-z1)/A + cx3*(z3-z1)/A with cx = (E+15)>>8 (main.h:1421-1448).
 * The render AABB takes every face, culled or not, before culling
 * (main.h:1348-1359 then 1371-1378), and starts from 50000 / -1.
 *
 * DEVIATION: writes outside the raster domain (the image grown by QO_GUARD
 * px) are dropped.  The reference writes every pixel through the linear
 * index y*640+x with no clipping (main.h:1442), which aliases columns
 * outside [0,640) into neighbouring rows and rows outside [0,480) into other
 * particles' buffers or past the allocation. */
int64_t qo_raster_face(const float v1[3], const float v2[3], const float v3[3],
                       const qo_camera *cam, int32_t *zbuf, int32_t box[4])
{
    return qo_raster_face_mode(v1, v2, v3, cam, zbuf, box, QO_RASTER_REF);
}

/* EDGE mode (not what the reference runs): the reference computes the
 * inside mask (CX1 > 0) & (CX2 > 0) & (CX3 > 0) from the biased edge
 * functions (main.h:1440) but its guard tests the mask's sign bit
 * (main.h:1473), which is never set.  EDGE applies the mask: only covered
 * pixels, with the top-left fill convention of the +1 bias
 * (main.h:1393-1401), are written and counted. */
int64_t qo_raster_face_mode(const float v1[3], const float v2[3], const float v3[3],
                            const qo_camera *cam, int32_t *zbuf, int32_t box[4], uint32_t mode)
{
    const int32_t Y1 = f2i_rn(16.0f * v1[1]);
    const int32_t Y2 = f2i_rn(16.0f * v2[1]);
    const int32_t Y3 = f2i_rn(16.0f * v3[1]);
    const int32_t X1 = f2i_rn(16.0f * v1[0]);
    const int32_t X2 = f2i_rn(16.0f * v2[0]);
    const int32_t X3 = f2i_rn(16.0f * v3[0]);

    const int32_t minx = asr(w_add(imin(imin(X1, X2), X3), 0xF), 4);
    const int32_t maxx = asr(w_add(imax(imax(X1, X2), X3), 0xF), 4);
    const int32_t miny = asr(w_add(imin(imin(Y1, Y2), Y3), 0xF), 4);
    const int32_t maxy = asr(w_add(imax(imax(Y1, Y2), Y3), 0xF), 4);

    box[0] = imin(box[0], minx);
    box[1] = imax(box[1], maxx);
    box[2] = imin(box[2], miny);
    box[3] = imax(box[3], maxy);

    const int32_t DX12 = w_sub(X1, X2), DX23 = w_sub(X2, X3), DX31 = w_sub(X3, X1);
    const int32_t DY12 = w_sub(Y1, Y2), DY23 = w_sub(Y2, Y3), DY31 = w_sub(Y3, Y1);

    const int32_t tri_area = w_sub(w_mul(DX12, DY31), w_mul(DX31, DY12));
    if (tri_area <= 0) return 0;
    if (w_sub(maxx, minx) <= 0 || w_sub(maxy, miny) <= 0) return 0;

    const float rA = 1.0f / (float)tri_area; /* overA_ == 1 (main.h:155) */

    const int32_t FDX12 = w_shl(DX12, 4), FDX23 = w_shl(DX23, 4), FDX31 = w_shl(DX31, 4);
    const int32_t FDY12 = w_shl(DY12, 4), FDY23 = w_shl(DY23, 4), FDY31 = w_shl(DY31, 4);

    int32_t C1 = w_sub(w_mul(DY12, X1), w_mul(DX12, Y1));
    int32_t C2 = w_sub(w_mul(DY23, X2), w_mul(DX23, Y2));
    int32_t C3 = w_sub(w_mul(DY31, X3), w_mul(DX31, Y3));
    C1 = w_add(C1, (DY12 < 0 || (DY12 == 0 && DX12 > 0)) ? 1 : 0);
    C2 = w_add(C2, (DY23 < 0 || (DY23 == 0 && DX23 > 0)) ? 1 : 0);
    C3 = w_add(C3, (DY31 < 0 || (DY31 == 0 && DX31 > 0)) ? 1 : 0);

    const int32_t MINY = w_shl(miny, 4), MINX = w_shl(minx, 4);
    const int32_t CY1 = w_sub(w_add(C1, w_mul(DX12, MINY)), w_mul(DY12, MINX));
    const int32_t CY2 = w_sub(w_add(C2, w_mul(DX23, MINY)), w_mul(DY23, MINX));
    const int32_t CY3 = w_sub(w_add(C3, w_mul(DX31, MINY)), w_mul(DY31, MINX));

    const float z1 = v1[2];
    const float z2 = (v2[2] - v1[2]) * rA;
    const float z3 = (v3[2] - v1[2]) * rA;

    /* loop bounds: [minx, maxx) x [miny, maxy), clipped to the domain; the
     * true extents are < 2^31 because the wrapped differences are > 0 */
    const int64_t dx0 = -QO_GUARD, dx1 = (int64_t)cam->width + QO_GUARD;
    const int64_t dy0 = -QO_GUARD, dy1 = (int64_t)cam->height + QO_GUARD;
    const int64_t ext_x = (int64_t)(uint32_t)w_sub(maxx, minx);
    const int64_t ext_y = (int64_t)(uint32_t)w_sub(maxy, miny);
    int64_t xa = minx, xb = (int64_t)minx + ext_x;
    int64_t ya = miny, yb = (int64_t)miny + ext_y;
    if (xa < dx0) xa = dx0;
    if (xb > dx1) xb = dx1;
    if (ya < dy0) ya = dy0;
    if (yb > dy1) yb = dy1;
    if (xa >= xb || ya >= yb) return 0;

    const int32_t dw = qo_domain_w(cam);
    int64_t writes = 0;
    for (int64_t y = ya; y < yb; ++y) {
        const int32_t ry = (int32_t)(y - (int64_t)miny); /* rows since miny */
        for (int64_t x = xa; x < xb; ++x) {
            const int32_t rx = (int32_t)(x - (int64_t)minx);
            const int32_t CX2 = w_sub(w_add(CY2, w_mul(ry, FDX23)), w_mul(rx, FDY23));
            const int32_t CX3 = w_sub(w_add(CY3, w_mul(ry, FDX31)), w_mul(rx, FDY31));
            if (mode == QO_RASTER_EDGE) {
                const int32_t CX1 = w_sub(w_add(CY1, w_mul(ry, FDX12)), w_mul(rx, FDY12));
                if (!(CX1 > 0 && CX2 > 0 && CX3 > 0)) continue;
            }
            const int32_t cx2 = asr(w_add(CX2, 0xF), 8);
            const int32_t cx3 = asr(w_add(CX3, 0xF), 8);
            float depth = z1;
            depth = depth + (float)cx2 * z2;
            depth = depth + (float)cx3 * z3;
            const int32_t d = f2i_rn(depth);
            int32_t *px = &zbuf[(size_t)(y + QO_GUARD) * (size_t)dw + (size_t)(x + QO_GUARD)];
            if (d < *px) *px = d;
            ++writes;
        }
    }
    return writes;
}

/* RenderFixedPointKernelAABB, main.cu:305-419: one face per thread, vertices
 * read from the loadOBJ3 SoA layout (main.h:620-679, index f + j*F + c*3F). */
int64_t qo_render(const float *mesh, uint32_t F, const float *s, const qo_camera *cam,
                  int32_t *zbuf, int32_t box[4])
{
    return qo_render_mode(mesh, F, s, cam, zbuf, box, QO_RASTER_REF);
}

int64_t qo_render_mode(const float *mesh, uint32_t F, const float *s, const qo_camera *cam,
                       int32_t *zbuf, int32_t box[4], uint32_t mode)
{
    box[0] = QO_AABB_INIT_MIN; box[1] = QO_AABB_INIT_MAX;
    box[2] = QO_AABB_INIT_MIN; box[3] = QO_AABB_INIT_MAX;
    int64_t writes = 0;
    for (uint32_t f = 0; f < F; ++f) {
        float v[3][3], uvz[3][3];
        for (int j = 0; j < 3; ++j) {
            v[j][0] = mesh[f + (size_t)j * F];
            v[j][1] = mesh[f + 3 * (size_t)F + (size_t)j * F];
            v[j][2] = mesh[f + 6 * (size_t)F + (size_t)j * F];
            qo_project(s, v[j], cam, uvz[j]);
        }
        writes += qo_raster_face_mode(uvz[0], uvz[1], uvz[2], cam, zbuf, box, mode);
    }
    return writes;
}

/* ------------------------------------------------------------------ */
/* RenderCPU, main.h:2012-2043: the reference's host render of the best pose
 * (written to results/<rgb>-<N>-best.csv).  Its projection,
 * projectModelPointsToPixelsCPU (main.h:1823-1855), is the same arithmetic
 * as the kernels' (qo_project).  Its rasteriser CPUfixedPointRender
 * (main.h:1857-1991) differs from the GPU one in two places, kept exactly:
 * vertices snap with iround(v) = (int)(v + 0.5f) (main.h:1808-1811),
 * truncating toward zero, and depth stays a float compared with `<` in a
 * float buffer that starts at 60000 (main.h:156).  The inside test is the
 * same no-op, so the face's whole bounding rectangle is written.
 *
 * iround of a value outside the int range, which is undefined in C, is
 * taken as saturating (NaN -> 0).  DEVIATION: writes are clipped to the
 * image; the reference indexes y*640+x unclipped into a 640x480 stack array
 * (main.h:1962), aliasing columns into neighbouring rows and writing past
 * the array for rows outside the image. */
static inline int32_t iround_ref(float v)
{
    const float t = v + 0.5f;
    if (t != t) return 0;
    if (t >= 2147483648.0f) return INT32_MAX;
    if (t <= -2147483648.0f) return INT32_MIN;
    return (int32_t)t; /* truncation toward zero */
}

void qo_raster_face_cpu(const float v1[3], const float v2[3], const float v3[3],
                        const qo_camera *cam, float *depth)
{
    const int32_t Y1 = iround_ref(16.0f * v1[1]);
    const int32_t Y2 = iround_ref(16.0f * v2[1]);
    const int32_t Y3 = iround_ref(16.0f * v3[1]);
    const int32_t X1 = iround_ref(16.0f * v1[0]);
    const int32_t X2 = iround_ref(16.0f * v2[0]);
    const int32_t X3 = iround_ref(16.0f * v3[0]);

    const int32_t DX12 = w_sub(X1, X2), DX23 = w_sub(X2, X3), DX31 = w_sub(X3, X1);
    const int32_t DY12 = w_sub(Y1, Y2), DY23 = w_sub(Y2, Y3), DY31 = w_sub(Y3, Y1);
    const int32_t tri_area = w_sub(w_mul(DX12, DY31), w_mul(DX31, DY12));
    if (tri_area <= 0) return;
    const float rA = 1.0f / (float)tri_area; /* overA_ / float(triArea), overA_ == 1 */

    const int32_t FDX23 = w_shl(DX23, 4), FDX31 = w_shl(DX31, 4);
    const int32_t FDY23 = w_shl(DY23, 4), FDY31 = w_shl(DY31, 4);
    const int32_t minx = asr(w_add(imin(imin(X1, X2), X3), 0xF), 4);
    const int32_t maxx = asr(w_add(imax(imax(X1, X2), X3), 0xF), 4);
    const int32_t miny = asr(w_add(imin(imin(Y1, Y2), Y3), 0xF), 4);
    const int32_t maxy = asr(w_add(imax(imax(Y1, Y2), Y3), 0xF), 4);
    if (w_sub(maxx, minx) <= 0 || w_sub(maxy, miny) <= 0) return;

    int32_t C2 = w_sub(w_mul(DY23, X2), w_mul(DX23, Y2));
    int32_t C3 = w_sub(w_mul(DY31, X3), w_mul(DX31, Y3));
    C2 = w_add(C2, (DY23 < 0 || (DY23 == 0 && DX23 > 0)) ? 1 : 0);
    C3 = w_add(C3, (DY31 < 0 || (DY31 == 0 && DX31 > 0)) ? 1 : 0);
    const int32_t MINY = w_shl(miny, 4), MINX = w_shl(minx, 4);
    const int32_t CY2 = w_sub(w_add(C2, w_mul(DX23, MINY)), w_mul(DY23, MINX));
    const int32_t CY3 = w_sub(w_add(C3, w_mul(DX31, MINY)), w_mul(DY31, MINX));
    const float z1 = v1[2];
    const float z2 = (v2[2] - v1[2]) * rA;
    const float z3 = (v3[2] - v1[2]) * rA;

    const int64_t ext_x = (int64_t)(uint32_t)w_sub(maxx, minx);
    const int64_t ext_y = (int64_t)(uint32_t)w_sub(maxy, miny);
    int64_t xa = minx, xb = (int64_t)minx + ext_x;
    int64_t ya = miny, yb = (int64_t)miny + ext_y;
    if (xa < 0) xa = 0;
    if (xb > cam->width) xb = cam->width;
    if (ya < 0) ya = 0;
    if (yb > cam->height) yb = cam->height;
    for (int64_t y = ya; y < yb; ++y) {
        const int32_t ry = (int32_t)(y - (int64_t)miny);
        for (int64_t x = xa; x < xb; ++x) {
            const int32_t rx = (int32_t)(x - (int64_t)minx);
            const int32_t CX2 = w_sub(w_add(CY2, w_mul(ry, FDX23)), w_mul(rx, FDY23));
            const int32_t CX3 = w_sub(w_add(CY3, w_mul(ry, FDX31)), w_mul(rx, FDY31));
            const int32_t cx2 = asr(w_add(CX2, 0xF), 8);
            const int32_t cx3 = asr(w_add(CX3, 0xF), 8);
            float d = z1;
            d = d + (float)cx2 * z2;
            d = d + (float)cx3 * z3;
            float *px = &depth[(size_t)y * (size_t)cam->width + (size_t)x];
            if (d < *px) *px = d;
        }
    }
}

void qo_render_cpu(const float *mesh, uint32_t F, const float *s, const qo_camera *cam,
                   float *depth)
{
    const size_t n = (size_t)cam->width * (size_t)cam->height;
    for (size_t i = 0; i < n; ++i) depth[i] = (float)QO_DEPTH_BG;
    for (uint32_t f = 0; f < F; ++f) {
        float v[3][3], uvz[3][3];
        for (int j = 0; j < 3; ++j) {
            v[j][0] = mesh[f + (size_t)j * F];
            v[j][1] = mesh[f + 3 * (size_t)F + (size_t)j * F];
            v[j][2] = mesh[f + 6 * (size_t)F + (size_t)j * F];
            qo_project(s, v[j], cam, uvz[j]);
        }
        qo_raster_face_cpu(uvz[0], uvz[1], uvz[2], cam, depth);
    }
}

/* ------------------------------------------------------------------ */
/* ComputeFitnessKernel, main.cu:550-764.
 *
 * Window = union of the render AABB and the cluster AABB (main.cu:596-622);
 * the reference walks t = 0 .. ceil(Area/1024)*1024-1 with x = t % W,
 * y = t / W and keeps y <= maxY (main.cu:624-640), so it visits the rows
 * [minY, maxY) fully plus the first min(W, pad) pixels of row maxY, where
 * pad = ceil(Area/1024)*1024 - Area.  That tail is kept.
 *
 * DEVIATION: the reference computes y with a float reciprocal of W
 * (main.cu:628), which for 137 of the first 1024 widths puts some x = 0
 * pixels on the previous row: those pixels are visited twice by racing
 * threads and their neighbours never, and the never-visited pixels are not
 * reset, so their depth leaks into the particle's next render.  This build
 * visits each window pixel exactly once.  The reference also converts Area
 * to float (exact below 2^24 px) and overflows int32 for windows above
 * 2^31 px; here Area is an exact 64-bit integer.
 *
 * Observed depth outside the image reads as 0.  The rendered depth of a
 * pixel outside the raster domain is the background value. */
void qo_score_zbuf(const int32_t *zbuf, const int32_t box[4], const uint16_t *obs,
                   const qo_camera *cam, const qo_params *prm, qo_score *out)
{
    memset(out, 0, sizeof(*out));
    out->r_min_x = box[0]; out->r_max_x = box[1];
    out->r_min_y = box[2]; out->r_max_y = box[3];
    const int32_t minX = imin(box[0], prm->cl_min_x);
    const int32_t maxX = imax(box[1], prm->cl_max_x);
    const int32_t minY = imin(box[2], prm->cl_min_y);
    const int32_t maxY = imax(box[3], prm->cl_max_y);
    out->w_min_x = minX; out->w_max_x = maxX; out->w_min_y = minY; out->w_max_y = maxY;
    const int64_t W = (int64_t)maxX - minX, H = (int64_t)maxY - minY;
    int64_t L = 0;
    if (W > 0 && H > 0) {
        const int64_t area = W * H;
        const int64_t pad = (1024 - area % 1024) % 1024;
        L = pad < W ? pad : W;
    }
    out->partial_len = (int32_t)L;
    if (W <= 0 || H <= 0) {
        out->fit = qo_fitness_from_counts(0, 0, 0, 0, 0, prm->num_points);
        return;
    }
    const int32_t dw = qo_domain_w(cam);
    uint32_t nR = 0, nNo = 0, nSegR = 0, nSNR = 0;
    uint64_t lo = 0, hi = 0;
    /* Visited pixels outside the raster domain have neither a rendered nor
     * an observed depth and add nothing, so the walk is clipped to it. */
    const int64_t cx0 = -QO_GUARD, cx1 = (int64_t)cam->width + QO_GUARD;
    const int64_t cy0 = -QO_GUARD, cy1 = (int64_t)cam->height + QO_GUARD;
    for (int64_t y = (minY > cy0 ? minY : cy0); y <= maxY && y < cy1; ++y) {
        int64_t xe = (y < maxY) ? (int64_t)maxX : (int64_t)minX + L;
        if (xe > cx1) xe = cx1;
        for (int64_t x = (minX > cx0 ? minX : cx0); x < xe; ++x) {
            int32_t zr = QO_DEPTH_BG;
            if (x >= -QO_GUARD && x < cam->width + QO_GUARD &&
                y >= -QO_GUARD && y < cam->height + QO_GUARD)
                zr = zbuf[(size_t)(y + QO_GUARD) * (size_t)dw + (size_t)(x + QO_GUARD)];
            int32_t zk = 0;
            if (x >= 0 && x < cam->width && y >= 0 && y < cam->height)
                zk = obs[(size_t)y * (size_t)cam->width + (size_t)x];
            if (zk != 0 && zr == QO_DEPTH_BG) ++nSNR;
            if (zr != QO_DEPTH_BG) {
                ++nR;
                if (zk == 0) {
                    ++nNo;
                } else {
                    const int32_t d = w_sub(zr, zk);
                    const uint64_t sq = (uint64_t)((int64_t)d * (int64_t)d);
                    lo += sq;
                    if (lo < sq) ++hi;
                    ++nSegR;
                }
            }
        }
    }
    out->n_rendered = nR;
    out->n_no_obs = nNo;
    out->n_seg_rendered = nSegR;
    out->n_seg_not_rendered = nSNR;
    out->sq_lo = lo;
    out->sq_hi = hi;
    out->fit = qo_fitness_from_counts(nSNR, nR, nNo, lo, hi, prm->num_points);
}

/* main.cu:743-760.  The reference sums float((zr-zk)*0.001)^2 in float;
 * here the sum of squares is an exact integer (mm^2), converted once.
 * DEVIATION: with no rendered pixel the reference computes 0 * rcp(0) =
 * NaN; here the fitness is +inf (never a best, as NaN never was). */
float qo_fitness_from_counts(uint32_t nSNR, uint32_t nR, uint32_t nNo, uint64_t lo,
                             uint64_t hi, uint32_t num_points)
{
    if (nR == 0) return INFINITY;
    const double S = (hi != 0) ? (double)hi * 18446744073709551616.0 + (double)lo : (double)lo;
    const float ratio = (float)nSNR * (1.0f / (float)num_points);
    const float rR = 1.0f / (float)nR;
    const float ratioT = (float)nNo * rR;
    const float zerr = (float)(S * 1.0e-6) * rR;
    return (float)((double)(ratio + ratioT) * 0.05 + (double)zerr);
}

/* FP64 recomputation of the fitness from the integer counts, for the
 * 1e-5 relative agreement check. */
double qo_fitness_fp64(const qo_score *sc, uint32_t num_points)
{
    if (sc->n_rendered == 0) return INFINITY;
    const double S = (double)sc->sq_hi * 18446744073709551616.0 + (double)sc->sq_lo;
    return 0.05 * ((double)sc->n_seg_not_rendered / (double)num_points +
                   (double)sc->n_no_obs / (double)sc->n_rendered) +
           S * 1.0e-6 / (double)sc->n_rendered;
}

/* ------------------------------------------------------------------ */
/* InitQPSO, main.cu:72-198.  Draws 0..11 of the particle's stream. */
void qo_init_particle(const qo_params *prm, uint32_t p, float *pos, float *vel, float *pb)
{
    const uint32_t P = prm->num_particles;
    uint32_t k = 0;
#define U() qo_uniform(prm->seed, prm->stream, p, k++)
    float s[7], v[7];
    for (int d = 0; d < 3; ++d) {
        s[d] = prm->t_lo[d] + (prm->t_hi[d] - prm->t_lo[d]) * U();
        v[d] = -prm->vdot + (2.0f * prm->vdot) * U();
    }
    float qinit[7] = {0.f, 0.f, 0.f, prm->qinit[0], prm->qinit[1], prm->qinit[2], prm->qinit[3]};
    float wpert[7] = {0, 0, 0, 0, 0, 0, 0};
    const float span = prm->ang_hi - prm->ang_lo;
    wpert[Q1] = prm->ang_lo + span * U();
    wpert[Q2] = prm->ang_lo + span * U();
    wpert[Q3] = prm->ang_lo + span * U();
    qo_quat_kinematics_init(qinit, s, wpert);
    v[Q0] = 0.0f;
    v[Q1] = prm->ang_lo + span * U();
    v[Q2] = prm->ang_lo + span * U();
    v[Q3] = prm->ang_lo + span * U();
#undef U
    for (int d = 0; d < 7; ++d) {
        pos[p + (size_t)d * P] = s[d];
        vel[p + (size_t)d * P] = v[d];
        pb[p + (size_t)d * P] = s[d];
    }
}

/* UpdateParticlesEquationKernel, main.cu:858-1060.  Iteration `iter` (>= 1)
 * uses draws 12*iter .. 12*iter+11. */
void qo_update_particle(const qo_params *prm, uint32_t p, uint32_t iter, float *pos,
                        float *vel, const float *pbv, const float *gb)
{
    const uint32_t P = prm->num_particles;
    uint32_t k = 12u * iter;
#define U() qo_uniform(prm->seed, prm->stream, p, k++)
    float s[7], v[7], b[7], g[7];
    for (int d = 0; d < 7; ++d) {
        s[d] = pos[p + (size_t)d * P];
        v[d] = vel[p + (size_t)d * P];
        b[d] = pbv[p + (size_t)d * P];
        g[d] = gb[d];
    }
    for (int d = 0; d < 3; ++d) {
        const float r1 = prm->c1 * U();
        const float r2 = prm->c2 * U();
        const float iV = (float)(prm->w * (double)v[d]);
        const float cV = r1 * (b[d] - s[d]);
        const float sV = r2 * (g[d] - s[d]);
        v[d] = iV + cV + sV;
        s[d] = s[d] + v[d];
        if (s[d] < prm->t_lo[d]) {
            s[d] = prm->t_lo[d];
            v[d] = 0.0f;
        } else if (s[d] > prm->t_hi[d]) {
            s[d] = prm->t_hi[d];
            v[d] = 0.0f;
        }
    }
    float qc[4], qs[4], wc[3] = {0, 0, 0}, ws[3] = {0, 0, 0};
    qo_quat_prod_conj(b, s, qc);
    qo_cast_top_half(qc);
    const float nc = sqrtf(qc[1] * qc[1] + qc[2] * qc[2] + qc[3] * qc[3]);
    if (nc > QO_MIN_NORM) {
        const float rn = 1.0f / nc;
        const float a = 2.0f * qo_acosf(qc[0]) * rn;
        wc[0] = qc[1] * a; wc[1] = qc[2] * a; wc[2] = qc[3] * a;
    }
    qo_quat_prod_conj(g, s, qs);
    qo_cast_top_half(qs);
    const float ns = sqrtf(qs[1] * qs[1] + qs[2] * qs[2] + qs[3] * qs[3]);
    if (ns > QO_MIN_NORM) {
        const float rn = 1.0f / ns;
        const float a = 2.0f * qo_acosf(qs[0]) * rn;
        ws[0] = qs[1] * a; ws[1] = qs[2] * a; ws[2] = qs[3] * a;
    }
    v[Q0] = 0.0f;
    for (int i = 1; i < 4; ++i) {
        const float r1 = prm->c1 * U();
        const float r2 = prm->c2 * U();
        const float iW = (float)(prm->w * (double)v[Q0 + i]);
        const float cW = r1 * wc[i - 1];
        const float sW = r2 * ws[i - 1];
        v[Q0 + i] = iW + cW + sW;
    }
#undef U
    qo_quat_kinematics(s, v);
    for (int d = 0; d < 7; ++d) {
        pos[p + (size_t)d * P] = s[d];
        vel[p + (size_t)d * P] = v[d];
    }
}

/* ------------------------------------------------------------------ */
void qo_default_params(qo_params *prm)
{
    memset(prm, 0, sizeof(*prm));
    prm->c1 = 1.0f;
    prm->c2 = 1.0f;
    prm->w = 0.3;
    prm->vdot = 3.0f;
    prm->ang_lo = -10.0f;
    prm->ang_hi = 10.0f;
    prm->qinit[0] = 0.7071f; prm->qinit[1] = 0.7071f; prm->qinit[2] = 0.f; prm->qinit[3] = 0.f;
    prm->num_particles = 64;
    prm->iterations = 50;
}

/* Multi-threaded form of qo_solve: particles are rendered and scored in
 * parallel (one z-buffer per thread); every result is identical. */
int qo_solve_mt(const float *mesh, uint32_t F, const uint16_t *obs, const qo_camera *cam,
                const qo_params *prm, float *pos, float *vel, float *pbest, float *pbest_fit,
                qo_result *res, float *trace_gbest, float *trace_fit, int threads)
{
    const uint32_t P = prm->num_particles;
    if (P == 0 || F == 0 || prm->num_points == 0) return -1;
    if (threads < 1) threads = 1;
    if ((uint32_t)threads > P) threads = (int)P;
    const size_t dn = (size_t)qo_domain_w(cam) * (size_t)qo_domain_h(cam);
    int32_t **zb = (int32_t **)calloc((size_t)threads, sizeof(int32_t *));
    float *fit = (float *)malloc(P * sizeof(float));
    int ok = zb && fit;
    for (int t = 0; ok && t < threads; ++t) {
        zb[t] = (int32_t *)malloc(dn * sizeof(int32_t));
        if (!zb[t]) ok = 0; else qo_zbuf_reset(zb[t], cam);
    }
    if (!ok) {
        if (zb) for (int t = 0; t < threads; ++t) free(zb[t]);
        free(zb); free(fit);
        return -2;
    }
    const int32_t dw = qo_domain_w(cam);

    float gfit = 1.0e10f; /* max_best_fit_, main.h:100 */
    float g[7] = {0, 0, 0, 0, 0, 0, 0};
    uint64_t writes = 0;
    for (uint32_t p = 0; p < P; ++p) {
        qo_init_particle(prm, p, pos, vel, pbest);
        pbest_fit[p] = 1.0e10f;
    }
    for (uint32_t it = 0; it < prm->iterations; ++it) {
        if (it > 0) {
#pragma omp parallel for num_threads(threads) schedule(static)
            for (int64_t p = 0; p < (int64_t)P; ++p)
                qo_update_particle(prm, (uint32_t)p, it, pos, vel, pbest, g);
        }
        uint64_t wsum = 0;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1) reduction(+ : wsum)
        for (int64_t pp = 0; pp < (int64_t)P; ++pp) {
#ifdef _OPENMP
            int32_t *zbuf = zb[omp_get_thread_num()];
#else
            int32_t *zbuf = zb[0];
#endif
            const uint32_t p = (uint32_t)pp;
            float s[7];
            for (int d = 0; d < 7; ++d) s[d] = pos[p + (size_t)d * P];
            int32_t box[4];
            wsum += (uint64_t)qo_render_mode(mesh, F, s, cam, zbuf, box, prm->raster_mode);
            qo_score sc;
            qo_score_zbuf(zbuf, box, obs, cam, prm, &sc);
            fit[p] = sc.fit;
            /* reset the touched part of the z-buffer (the reference's fitness
             * kernel resets the pixels it visits) */
            int64_t x0 = box[0], x1 = box[1], y0 = box[2], y1 = box[3];
            if (x0 < -QO_GUARD) x0 = -QO_GUARD;
            if (y0 < -QO_GUARD) y0 = -QO_GUARD;
            if (x1 > cam->width + QO_GUARD) x1 = cam->width + QO_GUARD;
            if (y1 > cam->height + QO_GUARD) y1 = cam->height + QO_GUARD;
            for (int64_t y = y0; y < y1; ++y)
                for (int64_t x = x0; x < x1; ++x)
                    zbuf[(size_t)(y + QO_GUARD) * (size_t)dw + (size_t)(x + QO_GUARD)] = QO_DEPTH_BG;
        }
        writes += wsum;
        uint32_t best = 0;
        for (uint32_t p = 0; p < P; ++p) {
            if (fit[p] < pbest_fit[p]) {
                pbest_fit[p] = fit[p];
                for (int d = 0; d < 7; ++d) pbest[p + (size_t)d * P] = pos[p + (size_t)d * P];
            }
            if (fit[p] < fit[best]) best = p;
        }
        if (fit[best] < gfit) {
            gfit = fit[best];
            for (int d = 0; d < 7; ++d) g[d] = pos[best + (size_t)d * P];
        }
        if (trace_gbest) {
            trace_gbest[(size_t)it * 8] = gfit;
            for (int d = 0; d < 7; ++d) trace_gbest[(size_t)it * 8 + 1 + d] = g[d];
        }
        if (trace_fit)
            for (uint32_t p = 0; p < P; ++p) trace_fit[(size_t)it * P + p] = fit[p];
    }
    res->gbest_fit = gfit;
    for (int d = 0; d < 7; ++d) res->gbest[d] = g[d];
    res->raster_writes = writes;
    for (int t = 0; t < threads; ++t) free(zb[t]);
    free(zb);
    free(fit);
    return 0;
}

/* Host loop main.cu:1601-1727: init, then per iteration render + score every
 * particle, personal/global best update (main.cu:768-855, argmin with the
 * first minimum like thrust::min_element), then the particle update. */
int qo_solve(const float *mesh, uint32_t F, const uint16_t *obs, const qo_camera *cam,
             const qo_params *prm, float *pos, float *vel, float *pbest, float *pbest_fit,
             qo_result *res, float *trace_gbest, float *trace_fit)
{
    return qo_solve_mt(mesh, F, obs, cam, prm, pos, vel, pbest, pbest_fit, res, trace_gbest,
                       trace_fit, 1);
}

/* ------------------------------------------------------------------------
 * Segmentation core: disjoint-set forest (GraphCannySeg.cpp:231-272),
 * segment_graph (GraphCannySeg.cpp:1301-1373), the small-component merge
 * (GraphCannySeg.cpp:1243-1248) and the set listing that numbers the
 * clusters (collectSets, GraphCannySeg.cpp:305-352).
 * ------------------------------------------------------------------------ */

typedef struct {
    int32_t *parent, *rank, *size, *link;
    int32_t count;
} qo_forest;

/* find: walk to the root, then point x (only x) at it -- the reference's
 * one-step compression (GraphCannySeg.cpp:247-253).  Which node a set's
 * first pixel points at decides the duplicated entry of its list. */
static int32_t qo_forest_find(qo_forest *f, int32_t x)
{
    int32_t r = x;
    while (f->parent[r] != r) r = f->parent[r];
    f->parent[x] = r;
    return r;
}

/* join of two roots (GraphCannySeg.cpp:255-272): splice the circular member
 * lists, then union by rank with y winning ties (y's rank grows). */
static void qo_forest_join(qo_forest *f, int32_t x, int32_t y)
{
    const int32_t t = f->link[y];
    f->link[y] = f->link[x];
    f->link[x] = t;
    if (f->rank[x] > f->rank[y]) {
        f->parent[y] = x;
        f->size[x] += f->size[y];
    } else {
        f->parent[x] = y;
        f->size[y] += f->size[x];
        if (f->rank[x] == f->rank[y]) f->rank[y] += 1;
    }
    f->count -= 1;
}

static _Thread_local const qo_edge *qo_sort_base;  /* qsort passes no context */

/* ascending weight; equal weights by input position (a total order, so
 * qsort's lack of stability does not matter) */
static int qo_edge_order(const void *pa, const void *pb)
{
    const int32_t i = *(const int32_t *)pa, j = *(const int32_t *)pb;
    const float wi = qo_sort_base[i].w, wj = qo_sort_base[j].w;
    if (wi < wj) return -1;
    if (wj < wi) return 1;
    return (i > j) - (i < j);
}

int32_t qo_segment_graph(int32_t n_vertices, int32_t n_edges, qo_edge *edges, int32_t presorted,
                         float k, float min_size, int32_t merge, int32_t *offsets, int32_t *points,
                         int32_t *num_sets)
{
    if (n_vertices <= 0 || n_edges < 0) return -1;
    for (int32_t e = 0; e < n_edges; ++e)
        if (edges[e].a < 0 || edges[e].a >= n_vertices || edges[e].b < 0 || edges[e].b >= n_vertices ||
            edges[e].w != edges[e].w)
            return -1;

    if (!presorted && n_edges > 1) {
        /* DEVIATION: ties keep their input order; the reference's std::sort
         * (GraphCannySeg.cpp:1303) leaves the order of equal weights to the
         * C++ library's introsort. */
        int32_t *ord = (int32_t *)malloc((size_t)n_edges * sizeof(int32_t));
        qo_edge *tmp = (qo_edge *)malloc((size_t)n_edges * sizeof(qo_edge));
        if (!ord || !tmp) {
            free(ord);
            free(tmp);
            return -1;
        }
        for (int32_t e = 0; e < n_edges; ++e) ord[e] = e;
        qo_sort_base = edges;
        qsort(ord, (size_t)n_edges, sizeof(int32_t), qo_edge_order);
        for (int32_t e = 0; e < n_edges; ++e) tmp[e] = edges[ord[e]];
        memcpy(edges, tmp, (size_t)n_edges * sizeof(qo_edge));
        free(ord);
        free(tmp);
    }

    const size_t n = (size_t)n_vertices;
    qo_forest f;
    f.parent = (int32_t *)malloc(4 * n * sizeof(int32_t));
    float *thr = (float *)malloc(n * sizeof(float));
    uint8_t *listed = (uint8_t *)calloc(n, 1);
    if (!f.parent || !thr || !listed) {
        free(f.parent);
        free(thr);
        free(listed);
        return -1;
    }
    f.rank = f.parent + n;
    f.size = f.parent + 2 * n;
    f.link = f.parent + 3 * n;
    f.count = n_vertices;
    for (int32_t v = 0; v < n_vertices; ++v) {
        f.parent[v] = v;
        f.rank[v] = 0;
        f.size[v] = 1;
        f.link[v] = v;
        thr[v] = k / (float)1;  /* THRESHOLD(1, k) = k / |C| with |C| = 1 */
    }

    /* Kruskal-like pass: merge when the edge is no heavier than both
     * components' thresholds, then the merged root's threshold becomes
     * w + k / |C| (segment_graph). */
    for (int32_t e = 0; e < n_edges; ++e) {
        const float w = edges[e].w;
        int32_t a = qo_forest_find(&f, edges[e].a);
        const int32_t b = qo_forest_find(&f, edges[e].b);
        if (a == b || !(w <= thr[a] && w <= thr[b])) continue;
        qo_forest_join(&f, a, b);
        a = qo_forest_find(&f, a);
        thr[a] = w + k / (float)f.size[a];
    }

    /* small components: the same sorted edges once more; min_size is a
     * float and the comparison is int < float, as in the reference */
    if (merge) {
        for (int32_t e = 0; e < n_edges; ++e) {
            const int32_t a = qo_forest_find(&f, edges[e].a);
            const int32_t b = qo_forest_find(&f, edges[e].b);
            if (a != b && ((float)f.size[a] < min_size || (float)f.size[b] < min_size))
                qo_forest_join(&f, a, b);
        }
    }
    *num_sets = f.count;

    /* collectSets: sets in the order of their smallest pixel; each list is
     * that pixel, its parent pointer (not find(): whatever node the forest
     * left it pointing at, possibly the pixel itself), then the circular
     * list from the pixel onward -- which visits the parent again. */
    int32_t lists = 0, np = 0;
    offsets[0] = 0;
    for (int32_t v = 0; v < n_vertices; ++v) {
        if (listed[v]) continue;
        points[np++] = v;
        listed[v] = 1;
        const int32_t p = f.parent[v];
        points[np++] = p;
        listed[p] = 1;
        for (int32_t x = f.link[v]; x != v; x = f.link[x]) {
            listed[x] = 1;
            points[np++] = x;
        }
        offsets[++lists] = np;
    }
    free(f.parent);
    free(thr);
    free(listed);
    return lists;
}

/* ------------------------------------------------------------------------
 * Pixel graph: Gaussian smoothing (GraphCannySeg.h:423-489), depth
 * normalisation (GraphCannySeg.cpp:1105-1127), edge weight (the HSV +
 * depth + saliency branch of diff, GraphCannySeg.h:2051-2288), the edge
 * loop (GraphCannySeg.cpp:1174-1210).  The reference's float/double mix is
 * kept operation by operation; cos, exp and log2f are the C library's, as
 * the reference calls them.
 * ------------------------------------------------------------------------ */

void qo_seg_default_params(qo_seg_params *sp)
{
    sp->sigma = 0.8f;
    sp->k = (float)50 / 10000.f;
    sp->min_size = 500.0f;
    sp->kx = (float)2000 / 1000.f;
    sp->ky = (float)30 / 1000.f;
    sp->ks = (float)49 / 1000.f;
    sp->kdv = 4.5f;
    sp->kdc = 0.1f;
}

int32_t qo_gauss_mask(float sigma, float *mask, int32_t capacity)
{
    if (sigma < 0.01f) sigma = 0.01f;
    /* sigma * WIDTH is a double product (WIDTH is 4.0) */
    const int32_t len = (int32_t)ceil((double)sigma * 4.0) + 1;
    if (len > capacity) return -1;
    for (int32_t i = 0; i < len; ++i) {
        const float q = (float)i / sigma;
        const float q2 = q * q;
        mask[i] = (float)exp(-0.5 * (double)q2);
    }
    float sum = 0.0f;
    for (int32_t i = 1; i < len; ++i) sum += fabsf(mask[i]);
    sum = 2.0f * sum + fabsf(mask[0]);
    for (int32_t i = 0; i < len; ++i) mask[i] /= sum;
    return len;
}

/* one pass along the rows of a w x h plane, written transposed (h x w) */
static void qo_convolve_rows_t(const float *src, int32_t w, int32_t h, const float *mask,
                               int32_t len, float *dst_t)
{
    for (int32_t y = 0; y < h; ++y) {
        const float *row = src + (size_t)y * w;
        for (int32_t x = 0; x < w; ++x) {
            float sum = mask[0] * row[x];
            for (int32_t i = 1; i < len; ++i) {
                const int32_t xl = x - i > 0 ? x - i : 0;
                const int32_t xr = x + i < w - 1 ? x + i : w - 1;
                sum += mask[i] * (row[xl] + row[xr]);
            }
            dst_t[(size_t)x * h + y] = sum;
        }
    }
}

int32_t qo_smooth(const float *src, int32_t W, int32_t H, float sigma, float *dst)
{
    float mask[256];
    const int32_t len = qo_gauss_mask(sigma, mask, 256);
    if (len < 0 || W <= 0 || H <= 0) return -1;
    float *tmp = (float *)malloc((size_t)W * H * sizeof(float));
    if (!tmp) return -1;
    qo_convolve_rows_t(src, W, H, mask, len, tmp);  /* tmp: H wide, W high */
    qo_convolve_rows_t(tmp, H, W, mask, len, dst);  /* back to W x H */
    free(tmp);
    return 0;
}

void qo_depth_norm(const uint16_t *depth, int32_t W, int32_t H, float *out)
{
    const size_t n = (size_t)W * H;
    /* std::max_element/min_element over [first, last pixel): the last
     * pixel is not in the range; with one pixel the empty range yields it */
    uint16_t mx = depth[0], mn = depth[0];
    if (n > 1) {
        for (size_t i = 1; i + 1 < n; ++i) {
            if (depth[i] > mx) mx = depth[i];
            if (depth[i] < mn) mn = depth[i];
        }
    }
    const float fmn = (float)mn, fmx = (float)mx;
    for (size_t i = 0; i < n; ++i) {
        const float d = (float)depth[i];
        /* mapminmax(d, min, max, 0, 1) = (1 - 0) * (d - min) / (max - min) + 0 */
        out[i] = (1.0f - 0.0f) * (d - fmn) / (fmx - fmn) + 0.0f;
    }
}

float qo_edge_weight(const float *sh, const float *ss, const float *sv, const float *dnorm,
                     const float *sal, int32_t W, int32_t x1, int32_t y1, int32_t x2, int32_t y2,
                     const qo_seg_params *sp)
{
    const size_t p = (size_t)y1 * W + x1, q = (size_t)y2 * W + x2;
    const float c_map = 1.f / 255.f;
    const float h1 = sh[q] * 2.0f, s1 = ss[q] * c_map, v1 = sv[q] * c_map;
    const float h2 = sh[p] * 2.0f, s2 = ss[p] * c_map, v2 = sv[p] * c_map;
    const float z_pivot = dnorm[p], z_current = dnorm[q];

    const float delta_v = sp->kdv * fabsf(v1 - v2);
    const float delta_h = fabsf(h1 - h2);
    const float theta = delta_h < 180 ? delta_h : 360 - delta_h;
    /* theta * M_PI / 180.0f is a double expression, so is everything the
     * cosine touches; the product rounds to float once, at the assignment */
    const double ang = (double)theta * 3.14159265358979323846 / 180.0;  /* M_PI */
    const double chord = (double)(s1 * s1 + s2 * s2) - (double)(2.0f * s1 * s2) * cos(ang);
    const float delta_c = (float)((double)sp->kdc * sqrt(chord));
    float dist_hsv = sqrtf(delta_v * delta_v + delta_c * delta_c);
    if (isnan(dist_hsv) || isinf(dist_hsv)) dist_hsv = 0.0f;
    if (v1 < 0.03f) dist_hsv = 0.01f;
    dist_hsv /= sqrtf(sp->kdv * sp->kdv + sp->kdc * sp->kdc);

    const float ds = sal[p];
    const float delta_depth = fabsf(z_pivot - z_current);
    return (sp->kx * delta_depth * log2f(1.0f + dist_hsv) + sp->ks * ds) / (sp->kx + sp->ks);
}

int32_t qo_graph_edges(const float *sh, const float *ss, const float *sv, const float *dnorm,
                       const float *sal, int32_t W, int32_t H, const qo_seg_params *sp, qo_edge *out)
{
    int32_t n = 0;
    for (int32_t y = 0; y < H; ++y)
        for (int32_t x = 0; x < W; ++x) {
            const int32_t i = y * W + x;
            if (x < W - 1) {
                out[n].a = i;
                out[n].b = i + 1;
                out[n++].w = qo_edge_weight(sh, ss, sv, dnorm, sal, W, x, y, x + 1, y, sp);
            }
            if (y < H - 1) {
                out[n].a = i;
                out[n].b = i + W;
                out[n++].w = qo_edge_weight(sh, ss, sv, dnorm, sal, W, x, y, x, y + 1, sp);
            }
            if (x < W - 1 && y < H - 1) {
                out[n].a = i;
                out[n].b = i + W + 1;
                out[n++].w = qo_edge_weight(sh, ss, sv, dnorm, sal, W, x, y, x + 1, y + 1, sp);
            }
            if (x < W - 1 && y > 0) {
                out[n].a = i;
                out[n].b = i - W + 1;
                out[n++].w = qo_edge_weight(sh, ss, sv, dnorm, sal, W, x, y, x + 1, y - 1, sp);
            }
        }
    return n;
}

int32_t qo_segment_planes(const uint8_t *h8, const uint8_t *s8, const uint8_t *v8,
                          const uint16_t *depth, const float *sal, int32_t W, int32_t H,
                          const qo_seg_params *sp, int32_t *offsets, int32_t *points,
                          int32_t *num_sets)
{
    if (W <= 0 || H <= 0) return -1;
    const size_t n = (size_t)W * H;
    float *buf = (float *)malloc(7 * n * sizeof(float));
    qo_edge *edges = (qo_edge *)malloc(4 * n * sizeof(qo_edge));
    if (!buf || !edges) {
        free(buf);
        free(edges);
        return -1;
    }
    float *hf = buf, *sf = buf + n, *vf = buf + 2 * n;
    float *sh = buf + 3 * n, *ss = buf + 4 * n, *sv = buf + 5 * n, *dn = buf + 6 * n;
    for (size_t i = 0; i < n; ++i) {
        hf[i] = (float)h8[i];
        sf[i] = (float)s8[i];
        vf[i] = (float)v8[i];
    }
    int32_t r = -1;
    if (qo_smooth(hf, W, H, sp->sigma, sh) == 0 && qo_smooth(sf, W, H, sp->sigma, ss) == 0 &&
        qo_smooth(vf, W, H, sp->sigma, sv) == 0) {
        qo_depth_norm(depth, W, H, dn);
        const int32_t m = qo_graph_edges(sh, ss, sv, dn, sal, W, H, sp, edges);
        r = qo_segment_graph(W * H, m, edges, 0, sp->k, sp->min_size, 1, offsets, points, num_sets);
    }
    free(buf);
    free(edges);
    return r;
}
