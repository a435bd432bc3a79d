// qpso_device.cuh -- device-side math of the Q-PSO pose solve on sm_103a.
//
// Arithmetic contract (shared with the scalar restatement the tests check
// against; compiled with --fmad=false so that every float expression is one
// IEEE rounding per operation in source order):
//   * the projection u = cx + fx*(x/z) is one fp32 fma (the reference
//     evaluates it in double because its intrinsics are double macros,
//     main.h:30-33,538-540);
//   * int32 edge arithmetic wraps modulo 2^32 (done in uint32), right shifts
//     are arithmetic, float->int is cvt.rni (half-even, saturating);
//   * sin, cos and acos are this project's fp32 series, not CUDA's math
//     library (the reference's fast-math cosf/sinf/acosf differ from any
//     host libm);
//   * random numbers are Philox4x32-10 (Salmon et al., SC'11) keyed by
//     (seed) with counter (draw/4, particle, stream, 0).
#pragma once

#include <cstdint>

namespace qpso {

constexpr int kNdim = 7;
constexpr int kTX = 0, kTY = 1, kTZ = 2, kQ0 = 3, kQ1 = 4, kQ2 = 5, kQ3 = 6;
constexpr int32_t kDepthBg = 60000;        // maxVal_depthBufferInt, main.h:157
constexpr int32_t kAabbInitMin = 50000;    // max_AABB_, main.h:159
constexpr int32_t kAabbInitMax = -1;       // min_AABB_, main.h:160
constexpr int32_t kGuard = 1024;           // raster domain = image grown by this per side
constexpr float kMinNorm = 1.0e-7f;        // MIN_NORM_, main.h:95
constexpr float kBestInit = 1.0e10f;       // max_best_fit_, main.h:100

// ------------------------------------------------------------------------
// Philox4x32-10
__device__ __forceinline__ void philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                              uint32_t k0, uint32_t k1, uint32_t out[4]) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    const uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
    const uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

// Twelve uniforms of one particle's draw group g (draws 12g .. 12g+11):
// three Philox blocks, 24-bit mantissa in [0, 1).
__device__ __forceinline__ void draw_group(uint64_t seed, uint32_t stream, uint32_t particle,
                                           uint32_t g, float u[12]) {
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    uint32_t o[4];
    philox4x32_10(3u * g + b, particle, stream, 0u, (uint32_t)seed, (uint32_t)(seed >> 32), o);
#pragma unroll
    for (int l = 0; l < 4; ++l) u[4 * b + l] = (float)(o[l] >> 8) * 0x1p-24f;
  }
}

// ------------------------------------------------------------------------
// sin/cos/acos: Cody-Waite reduction by pi/2 (three 30-bit parts) and
// Taylor polynomials on [-pi/4, pi/4]; acos through asin's Taylor series on
// [0, 1/2] and acos(x) = 2 asin(sqrt((1-x)/2)) above 1/2.
__device__ __forceinline__ double sin_kernel(double r) {
  const double r2 = r * r;
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

__device__ __forceinline__ double cos_kernel(double r) {
  const double r2 = r * r;
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

__device__ __forceinline__ double reduce_pio2(double x, int* q) {
  if (fabs(x) > 1.0e6) x = fmod(x, 2.0 * 3.141592653589793);
  const double k = rint(x * 0.6366197723675814);
  double r = x - k * 1.5707963276654482;
  r = r - k * -8.705515692000731e-10;
  r = r - k * -3.50343439808993e-19;
  *q = (int)((long long)k & 3);
  return r;
}

__device__ __forceinline__ double dsin(double x) {
  if (x != x || isinf(x)) return x - x;
  int q;
  const double r = reduce_pio2(x, &q);
  switch (q) {
    case 0: return sin_kernel(r);
    case 1: return cos_kernel(r);
    case 2: return -sin_kernel(r);
    default: return -cos_kernel(r);
  }
}

__device__ __forceinline__ double dcos(double x) {
  if (x != x || isinf(x)) return x - x;
  int q;
  const double r = reduce_pio2(x, &q);
  switch (q) {
    case 0: return cos_kernel(r);
    case 1: return -sin_kernel(r);
    case 2: return -cos_kernel(r);
    default: return sin_kernel(r);
  }
}

__device__ __forceinline__ double asin_kernel(double x) {
  const double c[27] = {
      0.16666666666666666,   0.075,                 0.044642857142857144,  0.030381944444444444,
      0.022372159090909092,  0.017352764423076924,  0.01396484375,         0.011551800896139705,
      0.009761609529194078,  0.008390335809616815,  0.0073125258735988454, 0.006447210311889649,
      0.005740037670841924,  0.005153309682319905,  0.004660143486915096,  0.004240907093679363,
      0.003880964558837669,  0.0035692053938259347, 0.003297059503473485,  0.0030578216492580306,
      0.002846178401108942,  0.00265787063820729,   0.0024894486782468836, 0.002338091892111975,
      0.0022014739737101384, 0.0020776610325181676, 0.0019650336162772837};
  const double x2 = x * x;
  double p = c[26];
#pragma unroll
  for (int i = 25; i >= 0; --i) p = p * x2 + c[i];
  return x + x * (x2 * p);
}

// acos with its argument clamped to [-1, 1].  The reference's acosf of a
// dot product that rounds to 1 + ulp returns NaN and kills the particle.
__device__ __forceinline__ double dacos(double x) {
  if (x != x) return x;
  if (x > 1.0) x = 1.0;
  if (x < -1.0) x = -1.0;
  if (x > 0.5) return 2.0 * asin_kernel(sqrt((1.0 - x) * 0.5));
  if (x < -0.5) return 3.141592653589793 - 2.0 * asin_kernel(sqrt((1.0 + x) * 0.5));
  return 1.5707963267948966 - asin_kernel(x);
}

// fp32 forms used by the PSO step (the double forms above are their
// fallback beyond |x| = 4096): Cody-Waite reduction with pi/2 split in 12 +
// 12 + 24 bits, Taylor polynomials on [-pi/4, pi/4], asin's Taylor series
// to x^23 on [0, 1/2].  GB300's fp64 pipe is narrow, so the step stays fp32.
__device__ __forceinline__ float fsin_kernel(float r) {
  const float r2 = r * r;
  float p = -2.5052107943679403e-08f;
  p = p * r2 + 2.7557318844628753e-06f;
  p = p * r2 + -0.00019841270113829523f;
  p = p * r2 + 0.008333333767950535f;
  p = p * r2 + -0.1666666716337204f;
  return r + r * (r2 * p);
}

__device__ __forceinline__ float fcos_kernel(float r) {
  const float r2 = r * r;
  float p = 2.0876755879584152e-09f;
  p = p * r2 + -2.755731998149713e-07f;
  p = p * r2 + 2.4801587642286904e-05f;
  p = p * r2 + -0.0013888889225199819f;
  p = p * r2 + 0.0416666679084301f;
  p = p * r2 + -0.5f;
  return 1.0f + r2 * p;
}

__device__ __forceinline__ float freduce(float x, int* q) {
  const float k = rintf(x * 0.6366197466850281f);
  float r = x - k * 1.57080078125f;
  r = r - k * -4.453584551811218e-06f;
  r = r - k * -8.705515752716053e-10f;
  *q = (int)((long long)k & 3);
  return r;
}

__device__ __forceinline__ float fsin(float x) {
  if (x != x || isinf(x)) return x - x;
  if (fabsf(x) > 4096.0f) return (float)dsin((double)x);
  int q;
  const float r = freduce(x, &q);
  switch (q) {
    case 0: return fsin_kernel(r);
    case 1: return fcos_kernel(r);
    case 2: return -fsin_kernel(r);
    default: return -fcos_kernel(r);
  }
}

__device__ __forceinline__ float fcos(float x) {
  if (x != x || isinf(x)) return x - x;
  if (fabsf(x) > 4096.0f) return (float)dcos((double)x);
  int q;
  const float r = freduce(x, &q);
  switch (q) {
    case 0: return fcos_kernel(r);
    case 1: return -fsin_kernel(r);
    case 2: return -fcos_kernel(r);
    default: return fsin_kernel(r);
  }
}

__device__ __forceinline__ float fasin_kernel(float x) {
  const float c[11] = {0.1666666716337204f,   0.07500000298023224f,  0.0446428582072258f,
                       0.0303819440305233f,   0.022372158244252205f, 0.017352763563394547f,
                       0.013964843936264515f, 0.01155180111527443f,  0.009761609137058258f,
                       0.008390335366129875f, 0.007312525995075703f};
  const float x2 = x * x;
  float p = c[10];
#pragma unroll
  for (int i = 9; i >= 0; --i) p = p * x2 + c[i];
  return x + x * (x2 * p);
}

// acos with its argument clamped to [-1, 1] (the reference's acosf of a
// dot product that rounds to 1 + ulp is NaN and kills the particle).
__device__ __forceinline__ float facos(float x) {
  if (x != x) return x;
  if (x > 1.0f) x = 1.0f;
  if (x < -1.0f) x = -1.0f;
  if (x > 0.5f) return 2.0f * fasin_kernel(sqrtf((1.0f - x) * 0.5f));
  if (x < -0.5f) return 3.1415927410125732f - 2.0f * fasin_kernel(sqrtf((1.0f + x) * 0.5f));
  return 1.5707963705062866f - fasin_kernel(x);
}

// ------------------------------------------------------------------------
// Quaternion algebra on 7-float state vectors [tx,ty,tz,q0,q1,q2,q3].

// QuatProd_pqPSOstateVect, main.h:248-254
__device__ __forceinline__ void quat_prod(const float* p, const float* q, float* o) {
  o[0] = p[kQ0] * q[kQ0] - p[kQ1] * q[kQ1] - p[kQ2] * q[kQ2] - p[kQ3] * q[kQ3];
  o[1] = p[kQ1] * q[kQ0] + p[kQ0] * q[kQ1] + p[kQ2] * q[kQ3] - p[kQ3] * q[kQ2];
  o[2] = p[kQ2] * q[kQ0] + p[kQ0] * q[kQ2] + p[kQ3] * q[kQ1] - p[kQ1] * q[kQ3];
  o[3] = p[kQ3] * q[kQ0] + p[kQ0] * q[kQ3] + p[kQ1] * q[kQ2] - p[kQ2] * q[kQ1];
}

// QuatProd_pq_1PSOstateVect, main.h:256-264: p * conj(q)
__device__ __forceinline__ void quat_prod_conj(const float* p, const float* q, float* o) {
  o[0] = p[kQ0] * q[kQ0] + p[kQ1] * q[kQ1] + p[kQ2] * q[kQ2] + p[kQ3] * q[kQ3];
  o[1] = p[kQ1] * q[kQ0] - p[kQ0] * q[kQ1] - p[kQ2] * q[kQ3] + p[kQ3] * q[kQ2];
  o[2] = p[kQ2] * q[kQ0] - p[kQ0] * q[kQ2] - p[kQ3] * q[kQ1] + p[kQ1] * q[kQ3];
  o[3] = p[kQ3] * q[kQ0] - p[kQ0] * q[kQ3] - p[kQ1] * q[kQ2] + p[kQ2] * q[kQ1];
}

// NormalizeQuaternionPSOstateVect, main.h:209-221
__device__ __forceinline__ void normalize_quat(float* s) {
  const float den = sqrtf(s[kQ0] * s[kQ0] + s[kQ1] * s[kQ1] + s[kQ2] * s[kQ2] + s[kQ3] * s[kQ3]);
  if (den > kMinNorm) {
    const float r = 1.0f / den;
    s[kQ0] = s[kQ0] * r;
    s[kQ1] = s[kQ1] * r;
    s[kQ2] = s[kQ2] * r;
    s[kQ3] = s[kQ3] * r;
  }
}

// Cast2TopHalfHypersphere, main.h:236-246
__device__ __forceinline__ void cast_top_half(float* q) {
  if (q[0] < 0.0f) {
    q[0] = -q[0];
    q[1] = -q[1];
    q[2] = -q[2];
    q[3] = -q[3];
  }
}

// Exponential-map step of QuatKinematicsPSOStateVect(WithInit),
// main.h:266-307 / 373-413; mTs_ = 0.5 (main.h:96) scales exactly.
__device__ __forceinline__ void kinematics(const float* from, float* s, const float* w) {
  float wt[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  wt[kQ1] = w[kQ1] * 0.5f;
  wt[kQ2] = w[kQ2] * 0.5f;
  wt[kQ3] = w[kQ3] * 0.5f;
  const float nrm = sqrtf(wt[kQ1] * wt[kQ1] + wt[kQ2] * wt[kQ2] + wt[kQ3] * wt[kQ3]);
  const float dom = nrm * 0.5f;
  const float cosw = fcos(dom);
  float sinw;
  if (dom < kMinNorm) {
    sinw = 1.0f;
  } else {
    const float r = 1.0f / dom;
    sinw = fsin(dom) * r;
  }
  float qxw[4];
  quat_prod(from, wt, qxw);
  float qn[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) qn[i] = cosw * from[kQ0 + i] + 0.5f * sinw * qxw[i];
#pragma unroll
  for (int i = 0; i < 4; ++i) s[kQ0 + i] = qn[i];
  normalize_quat(s);
  if (s[kQ0] < 0.0f) {  // Cast2TopHalfHyperspherePSOstateVect, main.h:223-234
    s[kQ0] = -s[kQ0];
    s[kQ1] = -s[kQ1];
    s[kQ2] = -s[kQ2];
    s[kQ3] = -s[kQ3];
  }
}

// ------------------------------------------------------------------------
// Solve parameters (QPSOParams_t, main.h:182-204, plus the main.h macros
// this library makes runtime parameters).
struct SolveParams {
  float c1, c2;
  double w;
  float vdot;
  float ang_lo, ang_hi;
  float qinit[4];
  float t_lo[3], t_hi[3];
  int32_t cl_min_x, cl_max_x, cl_min_y, cl_max_y;
  uint32_t num_points;
  uint32_t num_particles;
  uint32_t iterations;
  uint64_t seed;
  uint32_t stream;
  uint32_t raster_mode;  // kRasterRef or kRasterEdge
};

// InitQPSO, main.cu:72-198 (draw group 0).
__device__ __forceinline__ void init_particle(const SolveParams& prm, uint32_t p, float s[7],
                                              float v[7]) {
  float u[12];
  draw_group(prm.seed, prm.stream, p, 0u, u);
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    s[d] = prm.t_lo[d] + (prm.t_hi[d] - prm.t_lo[d]) * u[2 * d];
    v[d] = -prm.vdot + (2.0f * prm.vdot) * u[2 * d + 1];
  }
  const float qinit[7] = {0.f, 0.f, 0.f, prm.qinit[0], prm.qinit[1], prm.qinit[2], prm.qinit[3]};
  float wpert[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  const float span = prm.ang_hi - prm.ang_lo;
  wpert[kQ1] = prm.ang_lo + span * u[6];
  wpert[kQ2] = prm.ang_lo + span * u[7];
  wpert[kQ3] = prm.ang_lo + span * u[8];
  kinematics(qinit, s, wpert);
  v[kQ0] = 0.0f;
  v[kQ1] = prm.ang_lo + span * u[9];
  v[kQ2] = prm.ang_lo + span * u[10];
  v[kQ3] = prm.ang_lo + span * u[11];
}

// UpdateParticlesEquationKernel, main.cu:858-1060, with the iteration's 12
// uniforms already drawn (draw group `iter`).
__device__ __forceinline__ void update_particle_drawn(const SolveParams& prm, float s[7], float v[7],
                                                      const float b[7], const float g[7], const float u[12]) {
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float r1 = prm.c1 * u[2 * d];
    const float r2 = prm.c2 * u[2 * d + 1];
    const float iV = (float)(prm.w * (double)v[d]);
    const float cV = r1 * (b[d] - s[d]);
    const float sV = r2 * (g[d] - s[d]);
    v[d] = iV + cV + sV;
    s[d] = s[d] + v[d];
    if (s[d] < prm.t_lo[d]) {
      s[d] = prm.t_lo[d];
      v[d] = 0.0f;
    } else if (s[d] > prm.t_hi[d]) {
      s[d] = prm.t_hi[d];
      v[d] = 0.0f;
    }
  }
  float qc[4], qs[4];
  float wc[3] = {0.f, 0.f, 0.f}, ws[3] = {0.f, 0.f, 0.f};
  quat_prod_conj(b, s, qc);
  cast_top_half(qc);
  const float nc = sqrtf(qc[1] * qc[1] + qc[2] * qc[2] + qc[3] * qc[3]);
  if (nc > kMinNorm) {
    const float rn = 1.0f / nc;
    const float a = 2.0f * facos(qc[0]) * rn;
    wc[0] = qc[1] * a;
    wc[1] = qc[2] * a;
    wc[2] = qc[3] * a;
  }
  quat_prod_conj(g, s, qs);
  cast_top_half(qs);
  const float ns = sqrtf(qs[1] * qs[1] + qs[2] * qs[2] + qs[3] * qs[3]);
  if (ns > kMinNorm) {
    const float rn = 1.0f / ns;
    const float a = 2.0f * facos(qs[0]) * rn;
    ws[0] = qs[1] * a;
    ws[1] = qs[2] * a;
    ws[2] = qs[3] * a;
  }
  v[kQ0] = 0.0f;
#pragma unroll
  for (int i = 1; i < 4; ++i) {
    const float r1 = prm.c1 * u[6 + 2 * (i - 1)];
    const float r2 = prm.c2 * u[7 + 2 * (i - 1)];
    const float iW = (float)(prm.w * (double)v[kQ0 + i]);
    const float cW = r1 * wc[i - 1];
    const float sW = r2 * ws[i - 1];
    v[kQ0 + i] = iW + cW + sW;
  }
  float from[7];
#pragma unroll
  for (int d = 0; d < 7; ++d) from[d] = s[d];
  kinematics(from, s, v);
}

__device__ __forceinline__ void update_particle(const SolveParams& prm, uint32_t p, uint32_t iter,
                                                float s[7], float v[7], const float b[7],
                                                const float g[7]) {
  float u[12];
  draw_group(prm.seed, prm.stream, p, iter, u);
  update_particle_drawn(prm, s, v, b, g, u);
}

// ------------------------------------------------------------------------
// Camera projection: projectModelPointsToPixels(const float*, const
// float4&, float4&), main.h:513-545, with the rotation
// quatVectRotationPSOstateVect, main.h:328-347.
struct Camera {
  float fx, fy, cx, cy;
  int32_t width, height;
  int32_t proj;  // kProjFp32 or kProjRefAccv
};

constexpr int32_t kProjFp32 = 0, kProjRefAccv = 1;


// Pose with the rotation's products hoisted: t = 2 q.xyz x v and
// k = q.xyz x t are evaluated term by term exactly as the reference does.
// kRefProj selects the projection at compile time: the fp32 fused
// multiply-add with the camera's intrinsics, or the reference's own
// expression with its compiled-in ACCV intrinsics (double macros,
// main.h:30-33), u = (float)(CX + FX * (double)(x/z)), as its kernels and
// host renderer evaluate it (main.h:537-539, 1849-1851).
template <bool kRefProj>
__device__ __forceinline__ void project_t(const float* s, float vx, float vy, float vz, const Camera& cam,
                                          float& u, float& v, float& z) {
  float t0 = s[kQ2] * vz - s[kQ3] * vy;
  float t1 = -(s[kQ1] * vz - s[kQ3] * vx);
  float t2 = s[kQ1] * vy - s[kQ2] * vx;
  t0 = 2.0f * t0;
  t1 = 2.0f * t1;
  t2 = 2.0f * t2;
  const float k0 = s[kQ2] * t2 - s[kQ3] * t1;
  const float k1 = -(s[kQ1] * t2 - s[kQ3] * t0);
  const float k2 = s[kQ1] * t1 - s[kQ2] * t0;
  float px = vx + s[kQ0] * t0 + k0;
  float py = vy + s[kQ0] * t1 + k1;
  float pz = vz + s[kQ0] * t2 + k2;
  px = px + s[kTX];
  py = py + s[kTY];
  pz = pz + s[kTZ];
  const float rz = 1.0f / pz;
  if (kRefProj) {
    u = (float)(325.26110 + 572.41140 * (double)(px * rz));
    v = (float)(242.04899 + 573.57043 * (double)(py * rz));
  } else {
    u = __fmaf_rn(cam.fx, px * rz, cam.cx);
    v = __fmaf_rn(cam.fy, py * rz, cam.cy);
  }
  z = 1000.0f * pz;
}

// The camera's own projection, chosen at run time (paths outside the fused
// kernels' inner loops).
__device__ __forceinline__ void project(const float* s, float vx, float vy, float vz, const Camera& cam,
                                        float& u, float& v, float& z) {
  if (cam.proj == kProjRefAccv)
    project_t<true>(s, vx, vy, vz, cam, u, v, z);
  else
    project_t<false>(s, vx, vy, vz, cam, u, v, z);
}

// ------------------------------------------------------------------------
// Wrapping int32 helpers.
__device__ __forceinline__ int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
__device__ __forceinline__ int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
__device__ __forceinline__ int32_t wmul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }
__device__ __forceinline__ int32_t wshl(int32_t a, int s) { return (int32_t)((uint32_t)a << s); }

// Triangle set-up of renderFixedPointAABB, main.h:1306-1430.  The face's
// integer bounding rectangle [minx,maxx) x [miny,maxy) feeds the render AABB
// whether or not the face is culled.
struct FaceSetup {
  int32_t minx, maxx, miny, maxy;
  int32_t c2, c3;             // edge functions 2,3 at pixel (0, 0), 2^8 scale: at pixel
                              // (x, y) they are c + y fdx - x fdy (32-bit wrapping, as
                              // the reference's row and column steps reach them)
  int32_t fdx23, fdx31;       // per-row steps
  int32_t fdy23, fdy31;       // per-column steps
  int32_t c1, fdx12, fdy12;   // edge function 1, set only for the EDGE raster mode
  float z1, z2, z3;           // z1 and the two depth gradients
  bool live;                  // front-facing with a non-empty rectangle
};

// Set-up from the snapped 28.4 vertex coordinates X = rn(16 u), Y = rn(16 v)
// (main.h:1333-1338) and the vertex depths in mm.
__device__ __forceinline__ void setup_face_fixed(int32_t X1, int32_t Y1, float w1, int32_t X2, int32_t Y2,
                                                 float w2, int32_t X3, int32_t Y3, float w3,
                                                 FaceSetup& f, bool edge = false) {
  f.minx = wadd(min(min(X1, X2), X3), 0xF) >> 4;
  f.maxx = wadd(max(max(X1, X2), X3), 0xF) >> 4;
  f.miny = wadd(min(min(Y1, Y2), Y3), 0xF) >> 4;
  f.maxy = wadd(max(max(Y1, Y2), Y3), 0xF) >> 4;
  const int32_t DX12 = wsub(X1, X2), DX23 = wsub(X2, X3), DX31 = wsub(X3, X1);
  const int32_t DY12 = wsub(Y1, Y2), DY23 = wsub(Y2, Y3), DY31 = wsub(Y3, Y1);
  const int32_t area = wsub(wmul(DX12, DY31), wmul(DX31, DY12));
  f.live = area > 0 && wsub(f.maxx, f.minx) > 0 && wsub(f.maxy, f.miny) > 0;
  if (!f.live) return;
  const float rA = 1.0f / (float)area;  // overA_ == 1, main.h:155
  f.fdx23 = wshl(DX23, 4);
  f.fdx31 = wshl(DX31, 4);
  f.fdy23 = wshl(DY23, 4);
  f.fdy31 = wshl(DY31, 4);
  int32_t C2 = wsub(wmul(DY23, X2), wmul(DX23, Y2));
  int32_t C3 = wsub(wmul(DY31, X3), wmul(DX31, Y3));
  C2 = wadd(C2, (DY23 < 0 || (DY23 == 0 && DX23 > 0)) ? 1 : 0);
  C3 = wadd(C3, (DY31 < 0 || (DY31 == 0 && DX31 > 0)) ? 1 : 0);
  f.c2 = C2;
  f.c3 = C3;
  if (edge) {
    f.fdx12 = wshl(DX12, 4);
    f.fdy12 = wshl(DY12, 4);
    int32_t C1 = wsub(wmul(DY12, X1), wmul(DX12, Y1));
    C1 = wadd(C1, (DY12 < 0 || (DY12 == 0 && DX12 > 0)) ? 1 : 0);
    f.c1 = C1;
  }
  f.z1 = w1;
  f.z2 = (w2 - w1) * rA;
  f.z3 = (w3 - w1) * rA;
}

__device__ __forceinline__ void setup_face(float u1, float v1, float w1, float u2, float v2,
                                           float w2, float u3, float v3, float w3, FaceSetup& f,
                                           bool edge = false) {
  setup_face_fixed(__float2int_rn(16.0f * u1), __float2int_rn(16.0f * v1), w1,
                   __float2int_rn(16.0f * u2), __float2int_rn(16.0f * v2), w2,
                   __float2int_rn(16.0f * u3), __float2int_rn(16.0f * v3), w3, f, edge);
}

// Raster modes.  REF (0): what the reference computes, every pixel of a
// front face's bounding rectangle (its inside mask, main.h:1440, is never
// applied because the guard of main.h:1473 tests a bit the mask never has).
// EDGE (1): that mask applied, pixels whose three biased edge functions are
// all > 0 (top-left fill convention).
constexpr uint32_t kRasterRef = 0, kRasterEdge = 1;

// Depth written at pixel (minx+rx, miny+ry) of a live face (main.h:1432-1448):
// every pixel of the rectangle is written (the inside mask of main.h:1440
// is a 0/1 value whose sign bit the guard of main.h:1473 tests).
__device__ __forceinline__ int32_t face_depth(const FaceSetup& f, int32_t x, int32_t y) {
  const int32_t CX2 = wsub(wadd(f.c2, wmul(y, f.fdx23)), wmul(x, f.fdy23));
  const int32_t CX3 = wsub(wadd(f.c3, wmul(y, f.fdx31)), wmul(x, f.fdy31));
  const int32_t cx2 = wadd(CX2, 0xF) >> 8;
  const int32_t cx3 = wadd(CX3, 0xF) >> 8;
  float depth = f.z1;
  depth = depth + (float)cx2 * f.z2;
  depth = depth + (float)cx3 * f.z3;
  return __float2int_rn(depth);
}

// Fitness from integer counts, main.cu:743-760.  The squared error is an
// exact 128-bit integer in mm^2; with no rendered pixel the fitness is +inf
// (the reference's 0*rcp(0) is NaN, which never became a best either).
__device__ __forceinline__ float fitness_from_counts(uint32_t nSNR, uint32_t nR, uint32_t nNo,
                                                     uint64_t lo, uint64_t hi,
                                                     uint32_t num_points) {
  if (nR == 0) return __int_as_float(0x7f800000);
  const double S = (hi != 0) ? (double)hi * 18446744073709551616.0 + (double)lo : (double)lo;
  const float ratio = (float)nSNR * (1.0f / (float)num_points);
  const float rR = 1.0f / (float)nR;
  const float ratioT = (float)nNo * rR;
  const float zerr = (float)(S * 1.0e-6) * rR;
  return (float)((double)(ratio + ratioT) * 0.05 + (double)zerr);
}

}  // namespace qpso
