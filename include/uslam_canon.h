/*
 * uslam_canon.h — canonical f32 transcendentals shared by the CUDA kernels
 * and the CPU oracle.
 *
 * The reference computes the keypoint orientation with WGSL `atan2` and the
 * BRIEF rotation with WGSL `cos`/`sin` (resources/generate_features.wgsl:98,
 * :102-103).  WGSL leaves the accuracy of these functions implementation
 * defined (atan2 may be off by up to 4096 ULP), so no implementation can be
 * bit-exact against "the" reference.  This header fixes ONE definition that
 * both sides evaluate with identical IEEE-754 binary32 operations
 * (+ - * / only, round-to-nearest-even, no contraction), so the GPU and the
 * oracle agree bit for bit.  Build flags that keep it so: host
 * `-ffp-contract=off` (no -ffast-math), device `--fmad=false`.
 *
 * Methods (written for this project from the mathematics):
 *  - atan2: octant reduction to t = min/max in [0,1]; t > tan(pi/8) is mapped
 *    through atan(t) = pi/4 + atan((t-1)/(t+1)); atan on |t| <= tan(pi/8) is
 *    the Gregory (Taylor) series to t^19, evaluated by Horner's rule.
 *  - sin/cos: Cody & Waite additive argument reduction by pi/2 split into
 *    three parts (C1, C2 exact to 12 bits, C3 the remainder), quadrant
 *    selection, then Taylor series on |r| <= pi/4 (sin to r^11, cos to r^12).
 * Coefficients are 1/n! and 1/(2k+1) rounded to nearest binary32.
 * Accuracy versus a correctly rounded result: a few ULP (tested).
 */
#ifndef USLAM_CANON_H
#define USLAM_CANON_H

#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define USLAM_HD __host__ __device__ __forceinline__
#else
#define USLAM_HD static inline
#endif

/* pi and its fractions, rounded to nearest binary32 */
#define USLAM_PI_F 0x1.921fb6p+1f
#define USLAM_PI_2_F 0x1.921fb6p+0f
#define USLAM_PI_4_F 0x1.921fb6p-1f
#define USLAM_2_PI_F 0x1.45f306p-1f
#define USLAM_TAN_PI_8_F 0x1.a8279ap-2f

/* Cody-Waite split of pi/2: C1 + C2 + C3 */
#define USLAM_PIO2_C1 0x1.922p+0f
#define USLAM_PIO2_C2 (-0x1.2aep-18f)
#define USLAM_PIO2_C3 (-0x1.de973ep-31f)

USLAM_HD float uslam_atan_reduced(float t) {
    /* Gregory series: t - t^3/3 + t^5/5 - ... - t^19/19, |t| <= tan(pi/8) */
    const float z = t * t;
    float p = -0x1.af286cp-5f;          /* -1/19 */
    p = p * z + 0x1.e1e1e2p-5f;         /*  1/17 */
    p = p * z + -0x1.111112p-4f;        /* -1/15 */
    p = p * z + 0x1.3b13b2p-4f;         /*  1/13 */
    p = p * z + -0x1.745d18p-4f;        /* -1/11 */
    p = p * z + 0x1.c71c72p-4f;         /*  1/9  */
    p = p * z + -0x1.24924ap-3f;        /* -1/7  */
    p = p * z + 0x1.99999ap-3f;         /*  1/5  */
    p = p * z + -0x1.555556p-2f;        /* -1/3  */
    return t + (t * z) * p;
}

/* atan2(y, x) for finite y, x.  Signed zeros follow C99 Annex F. */
USLAM_HD float uslam_atan2f(float y, float x) {
    const float ax = fabsf(x);
    const float ay = fabsf(y);
    const int x_neg = signbit(x) != 0;
    const int y_neg = signbit(y) != 0;
    float r;
    if (ax == 0.0f && ay == 0.0f) {
        r = x_neg ? USLAM_PI_F : 0.0f;
    } else {
        const int swap = ay > ax;
        const float num = swap ? ax : ay;
        const float den = swap ? ay : ax;
        float t = num / den;
        float off = 0.0f;
        if (t > USLAM_TAN_PI_8_F) {
            t = (t - 1.0f) / (t + 1.0f);
            off = USLAM_PI_4_F;
        }
        r = off + uslam_atan_reduced(t);
        if (swap) r = USLAM_PI_2_F - r;
        if (x_neg) r = USLAM_PI_F - r;
    }
    return y_neg ? -r : r;
}

/* sin and cos of a binary32 angle with |a| <= ~8 (the callers pass atan2
 * results in [-pi, pi]). */
USLAM_HD void uslam_sincosf(float a, float* s_out, float* c_out) {
    const float kf = rintf(a * USLAM_2_PI_F);
    float r = a - kf * USLAM_PIO2_C1;
    r = r - kf * USLAM_PIO2_C2;
    r = r - kf * USLAM_PIO2_C3;
    const float z = r * r;
    float ps = -0x1.ae6456p-26f;        /* -1/11! */
    ps = ps * z + 0x1.71de3ap-19f;      /*  1/9!  */
    ps = ps * z + -0x1.a01a02p-13f;     /* -1/7!  */
    ps = ps * z + 0x1.111112p-7f;       /*  1/5!  */
    ps = ps * z + -0x1.555556p-3f;      /* -1/3!  */
    const float sr = r + (r * z) * ps;
    float pc = 0x1.1eed8ep-29f;         /*  1/12! */
    pc = pc * z + -0x1.27e4fcp-22f;     /* -1/10! */
    pc = pc * z + 0x1.a01a02p-16f;      /*  1/8!  */
    pc = pc * z + -0x1.6c16c2p-10f;     /* -1/6!  */
    pc = pc * z + 0x1.555556p-5f;       /*  1/4!  */
    pc = pc * z + -0x1p-1f;             /* -1/2!  */
    const float cr = 1.0f + z * pc;
    const int q = ((int)kf) & 3;
    float s, c;
    switch (q) {
        case 0: s = sr; c = cr; break;
        case 1: s = cr; c = -sr; break;
        case 2: s = -sr; c = -cr; break;
        default: s = -cr; c = sr; break;
    }
    *s_out = s;
    *c_out = c;
}

#endif /* USLAM_CANON_H */
