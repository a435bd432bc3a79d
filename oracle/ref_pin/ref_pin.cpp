/*
 * ref_pin.cpp -- compiles the reference's own main.h helpers (quaternion
 * algebra, vertex rotation and projection, the fixed-point rasteriser and
 * its AABB reduction, the CPU twin rasteriser) for the host CPU so that the
 * oracle restatement can be checked against them.
 *
 * TEST INFRASTRUCTURE ONLY.  Built by oracle/ref_pin/build_ref_pin.sh into
 * oracle/_ref/ from the reference sources where they lie; nothing of the
 * reference is copied into this repository.  The reference header is parsed
 * by g++ with:
 *   - declaration-only stand-ins for the assimp and OpenCV names it mentions
 *     (oracle/ref_pin/stubs; the loaders that use them are never called);
 *   - host definitions of the CUDA intrinsics it calls, below, with the same
 *     IEEE meaning (rcp_rn is 1/x, float2int_rn rounds half to even and
 *     saturates) and one emulated thread for __syncthreads/atomicMin;
 *   - -DdeviceOverlap=asyncEngineCount, because CUDA 13 removed the
 *     cudaDeviceProp field that main.h:1178 reads in an unused function.
 * It is compiled with -ffp-contract=off: every float expression is rounded
 * per operation in source order, the arithmetic contract the oracle and the
 * CUDA kernels follow.
 */
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include <cuda_runtime.h>
#include <vector_types.h>

/* ---- emulated CUDA device environment (one thread, one block) ---- */
static uint3 threadIdx = {0, 0, 0};
static uint3 blockIdx = {0, 0, 0};
static dim3 blockDim(1, 1, 1);
static dim3 gridDim(1, 1, 1);

static inline void __syncthreads() {}
static inline float __frcp_rn(float x) { return 1.0f / x; }
static inline float __int2float_rn(int x) { return (float)x; }
static inline float __uint2float_rn(unsigned int x) { return (float)x; }
static inline double __uint2double_rn(unsigned int x) { return (double)x; }
static inline unsigned int __double2uint_rz(double x) { return (unsigned int)x; }
static inline float __fdividef(float a, float b) { return a / b; }
static inline float __fmaf_rn(float a, float b, float c) { return std::fma(a, b, c); }
static inline float __int_as_float(int x) { float f; std::memcpy(&f, &x, 4); return f; }
static inline unsigned int __umulhi(unsigned int a, unsigned int b)
{
    return (unsigned int)(((unsigned long long)a * b) >> 32);
}
static inline int __float2int_rn(float f)
{
    if (f != f) return 0;
    if (f >= 2147483648.0f) return INT32_MAX;
    if (f <= -2147483648.0f) return INT32_MIN;
    return (int)std::nearbyint(f);
}
static inline int atomicMin(int *addr, int v)
{
    int old = *addr;
    if (v < old) *addr = v;
    return old;
}

#include "handle_error.h"
#include "main.h"

extern "C" {

void pin_quat_prod(const float *p, const float *q, float *o) { QuatProd_pqPSOstateVect(p, q, o); }
void pin_quat_prod_conj(const float *p, const float *q, float *o) { QuatProd_pq_1PSOstateVect(p, q, o); }
void pin_normalize(float *s) { NormalizeQuaternionPSOstateVect(s); }
void pin_cast_top(float *q) { Cast2TopHalfHypersphere(q); }
void pin_kinematics(float *s, const float *w) { QuatKinematicsPSOStateVect(s, w); }
void pin_kinematics_init(float *qinit, float *s, const float *w)
{
    QuatKinematicsPSOStateVectWithInit(qinit, s, w);
}
void pin_rotate(const float *s, const float *v, float *o) { quatVectRotationPSOstateVect(s, v, o); }

/* projection used by the render kernel (main.h:513-545) with the
 * reference's compiled-in ACCV intrinsics */
void pin_project(const float *s, const float *v, float *o)
{
    float4 p = make_float4(v[0], v[1], v[2], 0.f), r;
    projectModelPointsToPixels(s, p, r);
    o[0] = r.x; o[1] = r.y; o[2] = r.z;
}
void pin_intrinsics(double *k)
{
    k[0] = FX; k[1] = FY; k[2] = CX; k[3] = CY;
}

/* One face through renderFixedPointAABB (main.h:1306-1491) on a 640x480 int
 * buffer; box receives the face's bounding rectangle from the AABB
 * reduction slots {minX, maxX, minY, maxY}.  The caller keeps the
 * rectangle inside the image (the reference does not clip). */
void pin_raster_face(const float *v1, const float *v2, const float *v3, int *buf, int *box)
{
    static int32_t sMinX[fxptThsPerBlock], sMaxX[fxptThsPerBlock];
    static int32_t sMinY[fxptThsPerBlock], sMaxY[fxptThsPerBlock];
    for (int i = 0; i < fxptThsPerBlock; ++i) {
        sMinX[i] = max_AABB_; sMaxX[i] = min_AABB_;
        sMinY[i] = max_AABB_; sMaxY[i] = min_AABB_;
    }
    static int32_t d_AABB[_8warpSize_];
    for (int i = 0; i < _8warpSize_; ++i) d_AABB[i] = 0;
    threadIdx.x = 0;
    blockIdx.x = 0;
    float4 a = make_float4(v1[0], v1[1], v1[2], 0.f);
    float4 b = make_float4(v2[0], v2[1], v2[2], 0.f);
    float4 c = make_float4(v3[0], v3[1], v3[2], 0.f);
    const uint32_t off = 0, tIdx = 0, pIdx = 0;
    renderFixedPointAABB(a, b, c, buf, off, tIdx, pIdx, sMinX, sMaxX, sMinY, sMaxY, d_AABB);
    box[0] = d_AABB[0];
    box[1] = d_AABB[64];
    box[2] = d_AABB[128];
    box[3] = d_AABB[192];
}

/* The CPU twin (main.h:1857-1991): iround and a float buffer. */
void pin_cpu_raster_face(const float *v1, const float *v2, const float *v3, float *buf)
{
    float4 a = make_float4(v1[0], v1[1], v1[2], 0.f);
    float4 b = make_float4(v2[0], v2[1], v2[2], 0.f);
    float4 c = make_float4(v3[0], v3[1], v3[2], 0.f);
    CPUfixedPointRender(buf, a, b, c);
}

/* projection of the host render (main.h:1823-1855) */
void pin_project_cpu(const float *s, const float *v, float *o)
{
    float4 p = make_float4(v[0], v[1], v[2], 0.f), r;
    projectModelPointsToPixelsCPU(s, p, r);
    o[0] = r.x; o[1] = r.y; o[2] = r.z;
}

int pin_rows(void) { return rows_; }
int pin_cols(void) { return cols_; }

} /* extern "C" */
