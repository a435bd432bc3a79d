/*
 * qpso_seg_front.c -- scalar CPU restatement of GraphCannySeg's stages
 * around the graph segmentation: the colour conversions, the depth
 * smoothing, the depth inpainting, the Canny saliency and the cluster
 * filter (GraphCannySeg<hsv>::run, GraphCannySeg.cpp:1438-1459, and
 * PostSegmFilter, GraphCannySeg.h:1639-1873).
 *
 * TEST INFRASTRUCTURE ONLY: the oracle for the GPU kernels of
 * q-pso_gb300/csrc/qpso_seg_front.cu.  The product never loads it.
 *
 * Parity status: unpinned against the reference.  The reference computes
 * these stages with OpenCV 2.4 (cvtColor, GaussianBlur, Scharr,
 * distanceTransform, integral, resize, inpaint, calcHist, PCA), which is
 * neither in the reference tree nor installed, so its outputs cannot be
 * produced here.  Each function below restates the published algorithm
 * that the reference calls, with an exact arithmetic definition (integers
 * where the data are integers, a fixed order of float operations
 * elsewhere) that the GPU kernels follow bit for bit.  Where OpenCV's own
 * rounding is an implementation detail, the definition here is stated
 * and marked DEVIATION (unpinned).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "qpso_oracle.h"

static int imin(int a, int b) { return a < b ? a : b; }
static int imax(int a, int b) { return a > b ? a : b; }

/* ---- colour conversions ------------------------------------------------
 * The HSV image of segment_image comes from cvtColor(BGR2HSV)
 * (convertMat2Image, GraphCannySeg.h:708-721), the grey image of the Canny
 * stage from cvtColor(BGR2GRAY) (constructor, GraphCannySeg.cpp:404).
 * Published definitions (OpenCV's colour-conversion documentation):
 * V = max(R,G,B); S = (V - min) / V; H = 60 (G - B) / d if V = R,
 * 120 + 60 (B - R) / d if V = G, 240 + 60 (R - G) / d otherwise, plus 360
 * when negative; for 8-bit images S and V scale by 255 and H halves.  Here
 * each 8-bit value is the exact rational rounded half up (DEVIATION: OpenCV
 * rounds through 12-bit reciprocal tables).  Grey is
 * 0.299 R + 0.587 G + 0.114 B with 14-bit fixed-point weights
 * 4899/9617/1868 and rounding. */
void qo_bgr_to_hsv_gray(const uint8_t *bgr, int32_t n, uint8_t *h, uint8_t *s, uint8_t *v,
                        uint8_t *gray)
{
    for (int32_t i = 0; i < n; ++i) {
        const int b = bgr[3 * i], g = bgr[3 * i + 1], r = bgr[3 * i + 2];
        const int mx = imax(r, imax(g, b)), mn = imin(r, imin(g, b)), d = mx - mn;
        v[i] = (uint8_t)mx;
        s[i] = mx == 0 ? 0 : (uint8_t)((510 * d + mx) / (2 * mx));
        if (d == 0) {
            h[i] = 0;
        } else {
            int num, off;
            if (mx == r) {
                num = g - b;
                off = 0;
            } else if (mx == g) {
                num = b - r;
                off = 60;
            } else {
                num = r - g;
                off = 120;
            }
            int hd = 30 * num + off * d; /* H * d, H in units of 2 degrees */
            if (hd < 0) hd += 180 * d;
            h[i] = (uint8_t)((2 * hd + d) / (2 * d));
        }
        gray[i] = (uint8_t)((4899 * r + 9617 * g + 1868 * b + 8192) >> 14);
    }
}

/* ---- dynamicDepthSmoothing (GraphCannySeg.cpp:426-634) ------------------
 * Fdc = z^2 * 2.8e-9 (float), B = beta Fdc.  Depth-change map C: for every
 * pixel not on the image border, |z(x+1) - z(x)| >= gamma Fdc marks it and
 * its left and right neighbours, |z(y+1) - z(y)| >= gamma Fdc marks it and
 * the pixels above and below; marked pixels are zeroed in a copy of the
 * depth (ModDepth).  T = the exact Euclidean distance to the nearest marked
 * pixel (distanceTransform L2 PRECISE), times sqrt(1/2) in float; R =
 * min(B, T); radius = (int)(R + 0.5).  Inside a 15-pixel border, a pixel
 * with radius > 0 becomes the mean of ModDepth's non-zero values in the
 * (2 radius + 1)^2 window, from float summed-area tables of ModDepth and of
 * its zero count: (1 / (count - zeros)) * (((D + A) - C) - B) + 0.5,
 * truncated to uint16.  A radius of 0, or a window of zeros only, keeps
 * the input depth; pixels within 15 of the border become 0 (the
 * reference's output starts zeroed).
 *
 * The float summed-area table is accumulated in the order of the published
 * definition: a running float sum along each row added to the entry above
 * (sum(y+1, x+1) = sum(y, x+1) + rowsum(y, x)).
 * DEVIATION: a window that reaches outside the image is clipped to it and
 * its pixel count taken from the clipped window; the reference indexes
 * outside its tables there (radius above 15).  With no marked pixel at all,
 * T is +infinity. */
static const float kSqrtHalf = 0.70710677f;

float qo_smooth_alfa(void) { return 0.0028f / 1e6f; }

int32_t qo_depth_smooth(const uint16_t *d, int32_t W, int32_t H, float beta, float gamma,
                        uint16_t *out, uint8_t *c_out, float *r_out)
{
    if (W <= 0 || H <= 0) return -1;
    const size_t n = (size_t)W * H;
    const float alfa = qo_smooth_alfa();
    float *fdc = (float *)malloc(n * sizeof(float));
    uint8_t *C = (uint8_t *)calloc(n, 1);
    uint16_t *mod = (uint16_t *)malloc(n * sizeof(uint16_t));
    int32_t *g = (int32_t *)malloc(n * sizeof(int32_t));
    float *R = (float *)malloc(n * sizeof(float));
    float *I = (float *)calloc((size_t)(W + 1) * (H + 1), sizeof(float));
    int32_t *N = (int32_t *)calloc((size_t)(W + 1) * (H + 1), sizeof(int32_t));
    if (!fdc || !C || !mod || !g || !R || !I || !N) {
        free(fdc); free(C); free(mod); free(g); free(R); free(I); free(N);
        return -1;
    }
    for (size_t i = 0; i < n; ++i) fdc[i] = (float)((int64_t)d[i] * d[i]) * alfa;
    for (int32_t r = 1; r < H - 1; ++r)
        for (int32_t c = 1; c < W - 1; ++c) {
            const size_t p = (size_t)r * W + c;
            const float tdc = gamma * fdc[p];
            const int ddx = (int)d[p + 1] - (int)d[p];
            const int ddy = (int)d[p + W] - (int)d[p];
            if ((float)abs(ddx) >= tdc) C[p] = C[p + 1] = C[p - 1] = 1;
            if ((float)abs(ddy) >= tdc) C[p] = C[p + W] = C[p - W] = 1;
        }
    int any = 0;
    for (size_t i = 0; i < n; ++i) {
        mod[i] = C[i] ? 0 : d[i];
        any |= C[i];
    }
    /* exact squared Euclidean distance: horizontal distance per row, then
     * the minimum over rows of dy^2 + g^2, searched outwards from the row */
    const int32_t INF = 0x3fffffff;
    for (int32_t r = 0; r < H; ++r) {
        int32_t last = -INF;
        for (int32_t c = 0; c < W; ++c) {
            if (C[(size_t)r * W + c]) last = c;
            g[(size_t)r * W + c] = last == -INF ? INF : c - last;
        }
        last = INF;
        for (int32_t c = W - 1; c >= 0; --c) {
            if (C[(size_t)r * W + c]) last = c;
            if (last != INF && last - c < g[(size_t)r * W + c]) g[(size_t)r * W + c] = last - c;
        }
    }
    for (int32_t r = 0; r < H; ++r)
        for (int32_t c = 0; c < W; ++c) {
            const size_t p = (size_t)r * W + c;
            float T;
            if (!any) {
                T = INFINITY;
            } else {
                int64_t best = g[p] == INF ? INT64_MAX : (int64_t)g[p] * g[p];
                for (int32_t dy = 1; (int64_t)dy * dy < best; ++dy) {
                    if (r - dy < 0 && r + dy >= H) break;
                    for (int sgn = -1; sgn <= 1; sgn += 2) {
                        const int32_t rr = r + sgn * dy;
                        if (rr < 0 || rr >= H) continue;
                        const int32_t gg = g[(size_t)rr * W + c];
                        if (gg == INF) continue;
                        const int64_t d2 = (int64_t)dy * dy + (int64_t)gg * gg;
                        if (d2 < best) best = d2;
                    }
                }
                T = sqrtf((float)best) * kSqrtHalf;
            }
            const float B = beta * fdc[p];
            R[p] = B < T ? B : T; /* std::min(B, T) */
        }
    for (int32_t y = 0; y < H; ++y) {
        float s = 0.0f;
        int32_t z = 0;
        for (int32_t x = 0; x < W; ++x) {
            s += (float)mod[(size_t)y * W + x];
            z += mod[(size_t)y * W + x] == 0;
            I[(size_t)(y + 1) * (W + 1) + x + 1] = I[(size_t)y * (W + 1) + x + 1] + s;
            N[(size_t)(y + 1) * (W + 1) + x + 1] = N[(size_t)y * (W + 1) + x + 1] + z;
        }
    }
    for (size_t i = 0; i < n; ++i) out[i] = 0;
    for (int32_t r = 15; r < H - 15; ++r)
        for (int32_t c = 15; c < W - 15; ++c) {
            const size_t p = (size_t)r * W + c;
            const int radi = (int)(R[p] + 0.5f);
            if (radi == 0) {
                out[p] = d[p];
                continue;
            }
            const int32_t x0 = imax(c - radi, 0), x1 = imin(c + radi + 1, W);
            const int32_t y0 = imax(r - radi, 0), y1 = imin(r + radi + 1, H);
            const int32_t den = (x1 - x0) * (y1 - y0);
            const size_t s1 = (size_t)(W + 1);
            const int32_t nz = N[y1 * s1 + x1] + N[y0 * s1 + x0] - N[y1 * s1 + x0] - N[y0 * s1 + x1];
            if (den == nz) {
                out[p] = d[p];
                continue;
            }
            const float sum = ((I[y1 * s1 + x1] + I[y0 * s1 + x0]) - I[y1 * s1 + x0]) - I[y0 * s1 + x1];
            const float v = (1.0f / (float)(den - nz)) * sum + 0.5f;
            out[p] = v <= 0.0f ? 0 : v >= 65535.0f ? 65535 : (uint16_t)v;
        }
    if (c_out) memcpy(c_out, C, n);
    if (r_out) memcpy(r_out, R, n * sizeof(float));
    free(fdc); free(C); free(mod); free(g); free(R); free(I); free(N);
    return 0;
}

/* ---- inpaintDepth (GraphCannySeg.h:1164-1230) ---------------------------
 * The smoothed depth is mapped to 8 bits by its minimum and maximum
 * (convertTo with alpha = 255 / (max - min), beta = -min alpha: float
 * product then float sum, rounded half to even and saturated), shrunk by
 * 0.2 (bilinear with half-pixel centres: at a scale of exactly 5 every
 * output pixel samples the input at (5x + 2, 5y + 2)), its zero pixels
 * inpainted (Telea's fast-marching method, radius 20), grown back to full
 * size (bilinear, qo_resize_bilinear_u8) and copied into the 8-bit map
 * where it is zero; depth pixels that were zero become
 * gray * (uint16)((max - min) / 255) + min.  When max == min nothing is
 * filled (DEVIATION: the reference divides by zero). */

/* Bilinear resize of an 8-bit image with half-pixel centres: source
 * coordinate f = (float)((x + 0.5) * (sw / dw) - 0.5) (double, then float),
 * s = floor(f), weight (1 - (f - s)) * 2048 rounded half to even, the
 * coordinate clamped to the image with weight 0 beyond it; the two passes
 * in exact integers and the result (v + 2^21) >> 22.  DEVIATION
 * (unpinned): this is the published fixed-point INTER_LINEAR definition;
 * OpenCV's vectorised paths round the vertical pass differently. */
static void lin_coef(int32_t dx, int32_t sw, int32_t dw, int32_t *s0, int32_t *s1, int32_t *a0)
{
    float f = (float)((dx + 0.5) * ((double)sw / (double)dw) - 0.5);
    int32_t s = (int32_t)floorf(f);
    f -= (float)s;
    if (s < 0) {
        f = 0.0f;
        s = 0;
    }
    if (s >= sw - 1) {
        f = 0.0f;
        s = sw - 1;
    }
    *s0 = s;
    *s1 = s + 1 < sw ? s + 1 : sw - 1;
    *a0 = (int32_t)rintf((1.0f - f) * 2048.0f);
}

void qo_resize_bilinear_u8(const uint8_t *src, int32_t sw, int32_t sh, uint8_t *dst, int32_t dw, int32_t dh)
{
    for (int32_t y = 0; y < dh; ++y) {
        int32_t sy0, sy1, b0;
        lin_coef(y, sh, dh, &sy0, &sy1, &b0);
        for (int32_t x = 0; x < dw; ++x) {
            int32_t sx0, sx1, a0;
            lin_coef(x, sw, dw, &sx0, &sx1, &a0);
            const int64_t r0 = (int64_t)a0 * src[(size_t)sy0 * sw + sx0] + (int64_t)(2048 - a0) * src[(size_t)sy0 * sw + sx1];
            const int64_t r1 = (int64_t)a0 * src[(size_t)sy1 * sw + sx0] + (int64_t)(2048 - a0) * src[(size_t)sy1 * sw + sx1];
            const int64_t v = ((int64_t)b0 * r0 + (int64_t)(2048 - b0) * r1 + (1 << 21)) >> 22;
            dst[(size_t)y * dw + x] = (uint8_t)(v < 0 ? 0 : v > 255 ? 255 : v);
        }
    }
}

/* Telea's inpainting (A. Telea, "An Image Inpainting Technique Based on the
 * Fast Marching Method", J. Graphics Tools 9(1), 2004), as the reference
 * calls it through cv::inpaint(INPAINT_TELEA) on the 8-bit map, restated in
 * an order that lets pixels at the same distance from the known region be
 * filled together (DEVIATION, unpinned against OpenCV's implementation):
 *   - arrival times T: 0 on known pixels, and on masked pixels the fixed
 *     point of the first-order upwind update of |grad T| = 1 over the
 *     4-neighbourhood (Jacobi iterations from +infinity: a = the smaller of
 *     the left/right times, b = of the up/down times; |a - b| >= 1: the
 *     smaller + 1, else (a + b + sqrt(2 - (a - b)^2)) / 2); the march's
 *     own discretisation, without the march's order;
 *   - masked pixels are filled in increasing T; a pixel at time L is
 *     computed from the pixels with T < L only (the known ones and those
 *     filled before), so all pixels at time L are independent;
 *   - the value of pixel n: over every such pixel k != n with
 *     |n - k| <= radius (r = n - k): dir = |r . grad T(n)| / |r|,
 *     dst = 1 / |r|^2, lev = 1 / (1 + |T(k) - T(n)|), w = (dir dst) lev,
 *     value I(k) + grad I(k) . r; grad T by central differences over the
 *     finite neighbours, grad I over the neighbours with T < L (one-sided
 *     where one is missing, 0 where both are); the sums of w and w * value
 *     in 32.32 fixed point (exact, order-free); I(n) = round-half-even(sum /
 *     weights), saturated to 8 bits; with all weights 0, dir is taken as 1;
 *     with no usable pixel, 0;
 *   - a masked pixel that no known pixel reaches (T infinite) stays 0. */
float qo_eikonal2(float a, float b)
{
    if (a == INFINITY && b == INFINITY) return INFINITY;
    const float d = a - b;
    if (fabsf(d) >= 1.0f) return (a < b ? a : b) + 1.0f;
    return (a + b + sqrtf(2.0f - d * d)) * 0.5f;
}

/* gradient of a field along one axis at a pixel, from its two neighbours
 * (am = the one before, ap = the one after; valid flags km, kp) */
static float grad1(int km, float am, int kp, float ap, float a0)
{
    if (km && kp) return (ap - am) * 0.5f;
    if (kp) return ap - a0;
    if (km) return a0 - am;
    return 0.0f;
}

static const double kFix = 4294967296.0; /* 2^32 */

/* the value of pixel (x, y) at arrival time L = T[p] */
static uint8_t telea_value(const uint8_t *img, const float *T, int32_t w, int32_t h, int32_t x, int32_t y,
                           int32_t rad)
{
    const size_t p = (size_t)y * w + x;
    const float L = T[p];
    const int fxm = x > 0 && T[p - 1] != INFINITY, fxp = x + 1 < w && T[p + 1] != INFINITY;
    const int fym = y > 0 && T[p - w] != INFINITY, fyp = y + 1 < h && T[p + w] != INFINITY;
    const float gtx = grad1(fxm, fxm ? T[p - 1] : 0.0f, fxp, fxp ? T[p + 1] : 0.0f, L);
    const float gty = grad1(fym, fym ? T[p - w] : 0.0f, fyp, fyp ? T[p + w] : 0.0f, L);
    for (int pass = 0; pass < 2; ++pass) {
        int64_t num = 0, den = 0;
        for (int32_t dy = -rad; dy <= rad; ++dy)
            for (int32_t dx = -rad; dx <= rad; ++dx) {
                if (dx == 0 && dy == 0) continue;
                if (dx * dx + dy * dy > rad * rad) continue;
                const int32_t kx = x + dx, ky = y + dy;
                if (kx < 0 || kx >= w || ky < 0 || ky >= h) continue;
                const size_t k = (size_t)ky * w + kx;
                if (!(T[k] < L)) continue;
                const int32_t rx = -dx, ry = -dy;
                const float len2 = (float)(rx * rx + ry * ry);
                const float len = sqrtf(len2);
                const float dir = pass == 0 ? fabsf((float)rx * gtx + (float)ry * gty) / len : 1.0f;
                const float dst = 1.0f / len2;
                const float lev = 1.0f / (1.0f + fabsf(T[k] - L));
                const float wt = (dir * dst) * lev;
                const int ixm = kx > 0 && T[k - 1] < L, ixp = kx + 1 < w && T[k + 1] < L;
                const int iym = ky > 0 && T[k - w] < L, iyp = ky + 1 < h && T[k + w] < L;
                const float a0 = (float)img[k];
                const float gix = grad1(ixm, ixm ? (float)img[k - 1] : 0.0f, ixp, ixp ? (float)img[k + 1] : 0.0f, a0);
                const float giy = grad1(iym, iym ? (float)img[k - w] : 0.0f, iyp, iyp ? (float)img[k + w] : 0.0f, a0);
                const float val = a0 + (gix * (float)rx + giy * (float)ry);
                den += llrint((double)wt * kFix);
                num += llrint((double)(wt * val) * kFix);
            }
        if (den > 0) {
            double q = rint((double)num / (double)den);
            return (uint8_t)(q < 0.0 ? 0.0 : q > 255.0 ? 255.0 : q);
        }
    }
    return 0;
}

/* arrival times of the masked pixels (T, w * h); returns the Jacobi
 * iterations used, or -1 without convergence within 4 (w + h) + 8 */
int32_t qo_telea_times(const uint8_t *mask, int32_t w, int32_t h, float *T)
{
    const size_t n = (size_t)w * h;
    float *U = (float *)malloc(n * sizeof(float));
    if (!U) return -1;
    for (size_t i = 0; i < n; ++i) T[i] = mask[i] ? INFINITY : 0.0f;
    const int32_t cap = 4 * (w + h) + 8;
    int32_t it = 0;
    for (;;) {
        int changed = 0;
        for (int32_t y = 0; y < h; ++y)
            for (int32_t x = 0; x < w; ++x) {
                const size_t p = (size_t)y * w + x;
                if (!mask[p]) {
                    U[p] = 0.0f;
                    continue;
                }
                const float l = x > 0 ? T[p - 1] : INFINITY, r = x + 1 < w ? T[p + 1] : INFINITY;
                const float u = y > 0 ? T[p - w] : INFINITY, d = y + 1 < h ? T[p + w] : INFINITY;
                const float a = l < r ? l : r, b = u < d ? u : d;
                U[p] = qo_eikonal2(a, b);
                changed |= U[p] != T[p];
            }
        memcpy(T, U, n * sizeof(float));
        ++it;
        if (!changed) break;
        if (it > cap) {
            free(U);
            return -1;
        }
    }
    free(U);
    return it;
}

int32_t qo_telea(uint8_t *img, const uint8_t *mask, int32_t w, int32_t h, int32_t radius)
{
    if (w <= 0 || h <= 0 || radius < 1) return -1;
    const size_t n = (size_t)w * h;
    float *T = (float *)malloc(n * sizeof(float));
    if (!T) return -1;
    if (qo_telea_times(mask, w, h, T) < 0) {
        free(T);
        return -1;
    }
    for (size_t i = 0; i < n; ++i)
        if (mask[i]) img[i] = 0;
    int32_t filled = 0;
    float last = 0.0f;
    for (;;) {
        /* the next arrival time */
        float L = INFINITY;
        for (size_t i = 0; i < n; ++i)
            if (mask[i] && T[i] > last && T[i] < L) L = T[i];
        if (L == INFINITY) break;
        /* its pixels read only pixels of smaller time: fill them in place */
        for (int32_t y = 0; y < h; ++y)
            for (int32_t x = 0; x < w; ++x) {
                const size_t p = (size_t)y * w + x;
                if (mask[p] && T[p] == L) {
                    img[p] = telea_value(img, T, w, h, x, y, radius);
                    ++filled;
                }
            }
        last = L;
    }
    free(T);
    return filled;
}

int32_t qo_inpaint_depth(const uint16_t *sm, int32_t W, int32_t H, int32_t radius, uint16_t *out,
                         uint8_t *small_out, int32_t *small_w, int32_t *small_h)
{
    if (W <= 0 || H <= 0) return -1;
    const size_t n = (size_t)W * H;
    uint16_t mn = sm[0], mx = sm[0];
    for (size_t i = 1; i < n; ++i) {
        if (sm[i] < mn) mn = sm[i];
        if (sm[i] > mx) mx = sm[i];
    }
    const int32_t w = (int32_t)rint(W * 0.2), h = (int32_t)rint(H * 0.2);
    if (small_w) *small_w = w;
    if (small_h) *small_h = h;
    memcpy(out, sm, n * sizeof(uint16_t));
    if (mx == mn || w < 1 || h < 1) return 0;
    const double alpha = 255.0 / (double)(mx - mn), beta = -(double)mn * 255.0 / (double)(mx - mn);
    const float af = (float)alpha, bf = (float)beta;
    uint8_t *j1 = (uint8_t *)malloc(n);
    uint8_t *small = (uint8_t *)malloc((size_t)w * h);
    uint8_t *mask = (uint8_t *)malloc((size_t)w * h);
    uint8_t *up = (uint8_t *)malloc(n);
    if (!j1 || !small || !mask || !up) {
        free(j1); free(small); free(mask); free(up);
        return -1;
    }
    for (size_t i = 0; i < n; ++i) {
        const float f = (float)sm[i] * af + bf;
        const float q = rintf(f);
        j1[i] = (uint8_t)(q < 0.0f ? 0.0f : q > 255.0f ? 255.0f : q);
    }
    for (int32_t y = 0; y < h; ++y)
        for (int32_t x = 0; x < w; ++x) {
            const int32_t sy = imin(5 * y + 2, H - 1), sx = imin(5 * x + 2, W - 1);
            small[(size_t)y * w + x] = j1[(size_t)sy * W + sx];
            mask[(size_t)y * w + x] = small[(size_t)y * w + x] == 0;
        }
    qo_telea(small, mask, w, h, radius);
    if (small_out) memcpy(small_out, small, (size_t)w * h);
    qo_resize_bilinear_u8(small, w, h, up, W, H);
    const uint16_t dgs = (uint16_t)((double)(mx - mn) / 255.0);
    for (size_t i = 0; i < n; ++i) {
        if (sm[i] != 0) continue;
        const int gv = j1[i] == 0 ? up[i] : j1[i];
        out[i] = (uint16_t)(gv * dgs + mn);
    }
    free(j1); free(small); free(mask); free(up);
    return 0;
}

/* ---- myCannyWithOri2 (GraphCannySeg.cpp:638-1050) -----------------------
 * GaussianBlur 5x5 of the grey image, Scharr dx and -dy (scale -1) with
 * border reflect-101, magnitude sqrt(gx^2 + gy^2) in float, orientation
 * binned to 0/45/90/135, non-maximum suppression over the interior, the
 * thresholds low * max and high * max, one 8-neighbour hysteresis pass,
 * the removal of texture edges by the inpainted depth (an edge pixel is
 * dropped when the depth changes by less than DTH at plusD pixels on both
 * sides across it and the 3D angle at point3D pixels passes the angle
 * test), a zeroed border of max(plusD, point3D) + 1 pixels, GaussianBlur
 * 7x7 and a min-max map to [0, 1] floats.
 *
 * Exact definitions (DEVIATION, unpinned against OpenCV): the Gaussian
 * blurs use the kernel of the published formula (sigma = 0.3 ((k - 1) / 2
 * - 1) + 0.8 for a k-tap kernel) quantised to integers summing to 256
 * (qo_gauss_taps), two integer passes and (v + 2^15) >> 16; the
 * orientation bin comes from exact integer geometry (tan 22.5 = sqrt2 - 1)
 * where the reference bins atan2f in degrees: the two differ only for
 * gradients within float rounding of a bin edge; the hysteresis reads
 * outside the image as 0 (the reference reads outside its buffer in the
 * first and last rows, which the border rule zeroes anyway); the angle
 * test computes the 3D points as K^-1 (u z, v z, z) with
 * K^-1 = [1/fx 0 -cx/fx; 0 1/fy -cy/fy; 0 0 1] in float and double
 * accumulation, and theta = atan2 in double rounded to float; with a
 * saliency map that is constant (no edge left) the saliency is 0 (the
 * reference divides by zero). */
int32_t qo_gauss_taps(int32_t ksize, int32_t *taps)
{
    if (ksize < 1 || (ksize & 1) == 0 || ksize > 31) return -1;
    const double sigma = 0.3 * ((ksize - 1) * 0.5 - 1.0) + 0.8;
    const int32_t c = ksize / 2;
    double g[31], sum = 0.0;
    for (int32_t i = 0; i < ksize; ++i) {
        const double x = (double)(i - c);
        g[i] = exp(-(x * x) / (2.0 * sigma * sigma));
        sum += g[i];
    }
    int32_t tot = 0;
    for (int32_t i = 0; i < ksize; ++i) {
        taps[i] = (int32_t)floor(g[i] / sum * 256.0 + 0.5);
        tot += taps[i];
    }
    taps[c] += 256 - tot;
    return ksize;
}

static int32_t reflect101(int32_t i, int32_t n)
{
    if (n == 1) return 0;
    while (i < 0 || i >= n) {
        if (i < 0) i = -i;
        if (i >= n) i = 2 * (n - 1) - i;
    }
    return i;
}

void qo_blur_u8(const uint8_t *src, int32_t W, int32_t H, int32_t ksize, uint8_t *dst)
{
    int32_t taps[31];
    qo_gauss_taps(ksize, taps);
    const int32_t c = ksize / 2;
    int32_t *tmp = (int32_t *)malloc((size_t)W * H * sizeof(int32_t));
    for (int32_t y = 0; y < H; ++y)
        for (int32_t x = 0; x < W; ++x) {
            int32_t s = 0;
            for (int32_t i = 0; i < ksize; ++i) s += taps[i] * src[(size_t)y * W + reflect101(x + i - c, W)];
            tmp[(size_t)y * W + x] = s;
        }
    for (int32_t y = 0; y < H; ++y)
        for (int32_t x = 0; x < W; ++x) {
            int64_t s = 0;
            for (int32_t i = 0; i < ksize; ++i) s += (int64_t)taps[i] * tmp[(size_t)reflect101(y + i - c, H) * W + x];
            dst[(size_t)y * W + x] = (uint8_t)((s + 32768) >> 16);
        }
    free(tmp);
}

/* orientation bin of the gradient (x, y): 0, 45, 90 or 135 (degrees),
 * the direction of (x, y) modulo 180 against the edges 22.5, 67.5, 112.5
 * and 157.5 degrees */
int32_t qo_orient_bin(int32_t x, int32_t y)
{
    if (y < 0 || (y == 0 && x < 0)) {
        x = -x;
        y = -y;
    }
    if (x == 0 && y == 0) return 0;
    const int64_t a = x < 0 ? -(int64_t)x : x, b = y;
    /* b < (sqrt2 - 1) a  <=>  (a + b)^2 < 2 a^2 ;  b > (sqrt2 + 1) a  <=>  b > a and (b - a)^2 > 2 a^2 */
    const int low = (a + b) * (a + b) < 2 * a * a;
    const int high = b > a && (b - a) * (b - a) > 2 * a * a;
    if (low) return 0;
    if (high) return 90;
    return x >= 0 ? 45 : 135;
}

static void back_project(const float kinv[4], int32_t u, int32_t v, uint16_t z, float out[3])
{
    /* K^-1 (u z, v z, z): kinv = {1/fx, -cx/fx, 1/fy, -cy/fy} */
    const float p0 = (float)(u * (int32_t)z), p1 = (float)(v * (int32_t)z), p2 = (float)z;
    out[0] = (float)((double)kinv[0] * p0 + (double)kinv[1] * p2);
    out[1] = (float)((double)kinv[2] * p1 + (double)kinv[3] * p2);
    out[2] = p2;
}

float qo_angle3(const float p1[3], const float p0[3], const float p2[3])
{
    float a[3], b[3], c[3];
    for (int k = 0; k < 3; ++k) {
        a[k] = p1[k] - p0[k];
        b[k] = p2[k] - p0[k];
    }
    const float la = (float)sqrt((double)a[0] * a[0] + (double)a[1] * a[1] + (double)a[2] * a[2]);
    const float lb = (float)sqrt((double)b[0] * b[0] + (double)b[1] * b[1] + (double)b[2] * b[2]);
    const float dot = (float)((double)a[0] * b[0] + (double)a[1] * b[1] + (double)a[2] * b[2]);
    const float cs = dot / (la * lb);
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
    const float lc = (float)sqrt((double)c[0] * c[0] + (double)c[1] * c[1] + (double)c[2] * c[2]);
    const float sn = lc / (la * lb);
    float th = (float)atan2((double)sn, (double)cs);
    if (c[0] < 0.0f) th = -th;
    return th;
}

void qo_seg_front_default_params(qo_seg_front_params *fp)
{
    fp->beta = 2000.0f;
    fp->gamma = 18000.0f;
    fp->inpaint_radius = 20;
    fp->canny_low = (float)50 / 1000.f;
    fp->canny_high = (float)75 / 1000.f;
    fp->dth = 30;
    fp->plus_d = 7;
    fp->point_3d = 5;
    /* ((float)angle) * deg2rad, deg2rad = M_PI / 180.0f (GraphCannySeg.h:39), in double */
    fp->g_angle = (float)((double)148.0f * 3.14159265358979323846 / 180.0);
    fp->l_angle = (float)((double)151.0f * 3.14159265358979323846 / 180.0);
    fp->fx = 572.41140f;
    fp->fy = 573.57043f;
    fp->cx = 325.26110f;
    fp->cy = 242.04899f;
    fp->far_obj_z = 1500.0f;
    fp->max_ecc = 0.978f;
    fp->max_l1 = 13800.0f;
    fp->max_l2 = 1950.0f;
}

int32_t qo_canny_saliency(const uint8_t *gray, const uint16_t *inp, int32_t W, int32_t H,
                          const qo_seg_front_params *fp, float *sal, uint8_t *edges_out)
{
    if (W < 3 || H < 3) return -1;
    const size_t n = (size_t)W * H;
    uint8_t *bl = (uint8_t *)malloc(n);
    int32_t *gx = (int32_t *)malloc(n * sizeof(int32_t));
    int32_t *gy = (int32_t *)malloc(n * sizeof(int32_t));
    float *G = (float *)malloc(n * sizeof(float));
    float *BW = (float *)calloc(n, sizeof(float));
    uint8_t *bin = (uint8_t *)malloc(n);
    uint8_t *mag = (uint8_t *)calloc(n, 1);
    uint8_t *mb = (uint8_t *)malloc(n);
    if (!bl || !gx || !gy || !G || !BW || !bin || !mag || !mb) {
        free(bl); free(gx); free(gy); free(G); free(BW); free(bin); free(mag); free(mb);
        return -1;
    }
    qo_blur_u8(gray, W, H, 5, bl);
    for (int32_t y = 0; y < H; ++y)
        for (int32_t x = 0; x < W; ++x) {
            const int32_t xm = reflect101(x - 1, W), xp = reflect101(x + 1, W);
            const int32_t ym = reflect101(y - 1, H), yp = reflect101(y + 1, H);
#define B_(yy, xx) ((int32_t)bl[(size_t)(yy) * W + (xx)])
            const int32_t dx = 3 * (B_(ym, xp) - B_(ym, xm)) + 10 * (B_(y, xp) - B_(y, xm)) + 3 * (B_(yp, xp) - B_(yp, xm));
            const int32_t dy = 3 * (B_(yp, xm) - B_(ym, xm)) + 10 * (B_(yp, x) - B_(ym, x)) + 3 * (B_(yp, xp) - B_(ym, xp));
#undef B_
            const size_t p = (size_t)y * W + x;
            gx[p] = dx;
            gy[p] = -dy;
            G[p] = sqrtf((float)(dx * dx) + (float)(dy * dy));
            bin[p] = (uint8_t)qo_orient_bin(gx[p], gy[p]);
        }
    float mx = 0.0f;
    for (int32_t i = 1; i < H - 1; ++i)
        for (int32_t j = 1; j < W - 1; ++j) {
            const size_t p = (size_t)i * W + j;
            float a, b;
            switch (bin[p]) {
            case 0: a = G[p + 1]; b = G[p - 1]; break;
            case 45: a = G[p + W - 1]; b = G[p - W + 1]; break;
            case 90: a = G[p + W]; b = G[p - W]; break;
            default: a = G[p + W + 1]; b = G[p - W - 1]; break;
            }
            const float m3 = G[p] >= a ? (G[p] >= b ? G[p] : b) : (a >= b ? a : b);
            if (G[p] == m3) BW[p] = G[p];
        }
    for (size_t p = 0; p < n; ++p)
        if (BW[p] > mx) mx = BW[p];
    const float tl = (float)((double)fp->canny_low * (double)mx);
    const float th = (float)((double)fp->canny_high * (double)mx);
    for (int32_t i = 0; i < H; ++i)
        for (int32_t j = 0; j < W; ++j) {
            const size_t p = (size_t)i * W + j;
            if (BW[p] < tl) continue;
            if (BW[p] > th) {
                mag[p] = 255;
                continue;
            }
            int strong = 0;
            for (int dy = -1; dy <= 1 && !strong; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    if (!dx && !dy) continue;
                    const int32_t y = i + dy, x = j + dx;
                    if (y < 0 || y >= H || x < 0 || x >= W) continue;
                    if (BW[(size_t)y * W + x] > th) {
                        strong = 1;
                        break;
                    }
                }
            if (strong) mag[p] = 255;
        }
    const float kinv[4] = {1.0f / fp->fx, -fp->cx / fp->fx, 1.0f / fp->fy, -fp->cy / fp->fy};
    const int32_t pd = fp->plus_d, p3 = fp->point_3d;
    const int32_t sp = (pd > p3 ? pd : p3) + 1;
    for (int32_t i = 0; i < H; ++i)
        for (int32_t j = 0; j < W; ++j) {
            const size_t c = (size_t)i * W + j;
            if (i < sp || i > H - sp || j < sp || j > W - sp) {
                mag[c] = 0;
                continue;
            }
            if (mag[c] == 0) continue;
            int32_t ex, ey; /* the +plusD / +point3D direction across the edge */
            switch (bin[c]) {
            case 0: ex = 1; ey = 0; break;
            case 45: ex = 1; ey = -1; break;
            case 90: ex = 0; ey = -1; break;
            default: ex = -1; ey = -1; break;
            }
#define Z_(xx, yy) inp[(size_t)(yy) * W + (xx)]
            const int z0 = Z_(j, i);
            const uint16_t dp2 = (uint16_t)abs(z0 - (int)Z_(j + ex * pd, i + ey * pd));
            const uint16_t dm2 = (uint16_t)abs(z0 - (int)Z_(j - ex * pd, i - ey * pd));
            float q0[3], q1[3], q2[3];
            back_project(kinv, j, i, Z_(j, i), q0);
            back_project(kinv, j + ex * p3, i + ey * p3, Z_(j + ex * p3, i + ey * p3), q1);
            back_project(kinv, j - ex * p3, i - ey * p3, Z_(j - ex * p3, i - ey * p3), q2);
#undef Z_
            const float theta = qo_angle3(q1, q0, q2);
            if (dp2 < fp->dth && dm2 < fp->dth && (theta > fp->g_angle || theta < fp->l_angle)) mag[c] = 0;
        }
    if (edges_out) memcpy(edges_out, mag, n);
    qo_blur_u8(mag, W, H, 7, mb);
    int32_t vmn = 255, vmx = 0;
    for (size_t p = 0; p < n; ++p) {
        if (mb[p] < vmn) vmn = mb[p];
        if (mb[p] > vmx) vmx = mb[p];
    }
    if (vmx == vmn) {
        for (size_t p = 0; p < n; ++p) sal[p] = 0.0f;
    } else {
        const float a = (float)(1.0 / (double)(vmx - vmn));
        const float b = (float)(-(double)vmn * 1.0 / (double)(vmx - vmn));
        for (size_t p = 0; p < n; ++p) sal[p] = (float)mb[p] * a + b;
    }
    free(bl); free(gx); free(gy); free(G); free(BW); free(bin); free(mag); free(mb);
    return 0;
}

/* ---- PostSegmFilter (GraphCannySeg.h:1639-1873) -------------------------
 * For every set, in the order collectSets lists them (by smallest pixel):
 * the 3D centroid of its pixels with inpainted depth (compute3DCentroid,
 * GraphCannySeg.h:2569-2597: X = (u - cx) z / fx, Y = (v - cy) z / fy,
 * Z = z, mm) and its norm; the PCA of its pixel coordinates (computePCA,
 * GraphCannySeg.cpp:1376-1435: the eigenvalues of the covariance
 * normalised by the point count, eccentricity sqrt(1 - l2 / l1)); the share
 * of pixels without depth; the share of pixels whose HSV value falls in
 * the first three of 32 bins (calcHist over [0, 256), computeValueHist,
 * GraphCannySeg.h:2644-2700).  A set is dropped when its centroid is
 * farther than far_obj_z, its eccentricity is above max_ecc or an
 * eigenvalue is above max_l1 / max_l2, at least 30% of its pixels have no
 * depth, or at least 30% fall in the three darkest value bins.
 *
 * The reference's list for a set of n pixels holds n + 1 entries (one
 * pixel twice, collectSets); the shares divide by n + 1 as it does, and
 * num_points is n + 1.  DEVIATION: the centroid and the PCA here are over
 * the set's n distinct pixels, from exact integer moments (the reference
 * counts the repeated pixel twice and accumulates in float/double). */
int32_t qo_seg_clusters(const int32_t *labels, int32_t n_sets, const uint16_t *inp, const uint8_t *v8,
                        int32_t W, int32_t H, const qo_seg_front_params *fp, qo_seg_cluster *out,
                        int32_t keep_all)
{
    if (n_sets <= 0) return 0;
    typedef struct {
        int64_t n, sx, sy, sxx, syy, sxy, nz, sz, suz, svz, nzero, vb[3];
        int32_t minx, maxx, miny, maxy;
    } acc_t;
    acc_t *a = (acc_t *)calloc((size_t)n_sets, sizeof(acc_t));
    if (!a) return -1;
    for (int32_t k = 0; k < n_sets; ++k) {
        a[k].minx = a[k].miny = 0x7fffffff;
        a[k].maxx = a[k].maxy = -1;
    }
    for (int32_t y = 0; y < H; ++y)
        for (int32_t x = 0; x < W; ++x) {
            const size_t p = (size_t)y * W + x;
            const int32_t k = labels[p];
            if (k < 0 || k >= n_sets) continue;
            acc_t *c = &a[k];
            c->n++;
            c->sx += x;
            c->sy += y;
            c->sxx += (int64_t)x * x;
            c->syy += (int64_t)y * y;
            c->sxy += (int64_t)x * y;
            const int64_t z = inp[p];
            if (z) {
                c->nz++;
                c->sz += z;
                c->suz += (int64_t)x * z;
                c->svz += (int64_t)y * z;
            } else {
                c->nzero++;
            }
            if (v8[p] < 24) c->vb[v8[p] >> 3]++;
            if (x < c->minx) c->minx = x;
            if (x > c->maxx) c->maxx = x;
            if (y < c->miny) c->miny = y;
            if (y > c->maxy) c->maxy = y;
        }
    int32_t kept = 0;
    for (int32_t k = 0; k < n_sets; ++k) {
        const acc_t *c = &a[k];
        if (c->n == 0) continue;
        qo_seg_cluster r;
        memset(&r, 0, sizeof(r));
        r.label = k;
        r.num_points = (uint32_t)(c->n + 1);
        r.pixels = (uint32_t)c->n;
        r.min_x = c->minx;
        r.max_x = c->maxx + 1;
        r.min_y = c->miny;
        r.max_y = c->maxy + 1;
        qo_seg_cluster_stats(c->n, c->sx, c->sy, c->sxx, c->syy, c->sxy, c->nz, c->sz, c->suz, c->svz,
                             c->nzero, c->vb, fp, &r);
        if (keep_all || r.kept) out[kept++] = r;
    }
    free(a);
    return kept;
}

/* The record of one set from its exact moments; shared by the oracle's
 * filter above and checked against the product's host filter. */
void qo_seg_cluster_stats(int64_t n, int64_t sx, int64_t sy, int64_t sxx, int64_t syy, int64_t sxy,
                          int64_t nz, int64_t sz, int64_t suz, int64_t svz, int64_t nzero, const int64_t vb[3],
                          const qo_seg_front_params *fp, qo_seg_cluster *r)
{
    const double cx = fp->cx, cy = fp->cy, fx = fp->fx, fy = fp->fy;
    if (nz > 0) {
        r->centroid_mm[0] = (float)(((double)suz - cx * (double)sz) / (fx * (double)nz));
        r->centroid_mm[1] = (float)(((double)svz - cy * (double)sz) / (fy * (double)nz));
        r->centroid_mm[2] = (float)((double)sz / (double)nz);
    }
    const float cxm = r->centroid_mm[0], cym = r->centroid_mm[1], czm = r->centroid_mm[2];
    const float l2c = sqrtf(czm * czm + cym * cym + cxm * cxm);
    const double dn = (double)n;
    const double mx = (double)sx / dn, my = (double)sy / dn;
    const double vxx = ((double)sxx - (double)sx * mx) / dn;
    const double vyy = ((double)syy - (double)sy * my) / dn;
    const double vxy = ((double)sxy - (double)sx * my) / dn;
    const double hm = 0.5 * (vxx + vyy);
    const double hd = 0.5 * (vxx - vyy);
    const double rt = sqrt(hd * hd + vxy * vxy);
    r->eig[0] = hm + rt;
    r->eig[1] = hm - rt;
    r->eccentricity = r->eig[0] > 0.0 ? sqrt(1.0 - r->eig[1] / r->eig[0]) : 0.0;
    const float area = (float)(n + 1);
    r->nan_ratio = (float)nzero / area;
    r->dark_ratio = ((float)vb[0] / area + (float)vb[1] / area) + (float)vb[2] / area;
    r->far = l2c > fp->far_obj_z;
    r->kept = !r->far && !(r->eccentricity > fp->max_ecc || r->eig[0] > fp->max_l1 || r->eig[1] > fp->max_l2) &&
              !(r->nan_ratio >= 0.3f) && !(r->dark_ratio >= 0.3f);
}
