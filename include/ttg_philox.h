/*
 * ttg_philox.h — seeded, portable input generator shared by the device code
 * and the CPU oracle.
 *
 * The workloads are defined on seeded random matrices (G iid N(0,1),
 * A/B iid U[-1,1], right-hand sides iid N(0,1)).  std::normal_distribution
 * is implementation defined, so the generator is spelled out here:
 *
 *   - Philox-4x32-10, the counter-based generator of Salmon, Moraes, Dror and
 *     Shaw, "Parallel random numbers: as easy as 1, 2, 3" (SC'11).  Key =
 *     (seed, stream), counter = (index lo, index hi, 0, 0).
 *   - 53-bit uniforms in the open interval (0,1) from two 32-bit words.
 *   - Box–Muller (1958) for normals, with a natural logarithm and a sine /
 *     cosine written below from their Taylor/atanh series.  Only IEEE
 *     add/sub/mul/div/sqrt are used, each correctly rounded, so the host and
 *     the device produce the same bits provided no multiply-add contraction
 *     happens: device code uses the explicit round-to-nearest intrinsics and
 *     host code must be compiled with -ffp-contract=off.
 *
 * Element e of a matrix uses counter e/2 and takes the first or second of the
 * two values one Philox call yields, so any element can be generated alone.
 *
 * Quantised Gaussian (for A = G·Gᵀ/N + αI): g = rint(16 z) clamped to
 * [-127,127].  Integer g lets G·Gᵀ be formed exactly (int32 accumulation) on
 * both sides, so A is bit-identical between device and oracle; the variance of
 * g/16 differs from 1 by about 3e-4.
 */
#ifndef TTG_PHILOX_H
#define TTG_PHILOX_H

#include <stdint.h>

#if defined(__CUDACC__)
#define TTG_HD __host__ __device__ __forceinline__
#else
#define TTG_HD static inline
#endif

#if defined(__CUDA_ARCH__)
#define TTG_ADD(a, b) __dadd_rn((a), (b))
#define TTG_SUB(a, b) __dsub_rn((a), (b))
#define TTG_MUL(a, b) __dmul_rn((a), (b))
#define TTG_DIV(a, b) __ddiv_rn((a), (b))
#define TTG_SQRT(a) __dsqrt_rn((a))
#else
#include <math.h>
#define TTG_ADD(a, b) ((a) + (b))
#define TTG_SUB(a, b) ((a) - (b))
#define TTG_MUL(a, b) ((a) * (b))
#define TTG_DIV(a, b) ((a) / (b))
#define TTG_SQRT(a) sqrt((a))
#endif

/* Stream ids used by the workloads (the second key word). */
enum {
    TTG_STREAM_G = 0,      /* G of A = G·Gᵀ/N + αI                        */
    TTG_STREAM_RHS = 1,    /* right-hand sides                              */
    TTG_STREAM_GEMM_A = 2, /* A of the block GEMM                           */
    TTG_STREAM_GEMM_B = 3  /* B of the block GEMM                           */
};

typedef struct { uint32_t v[4]; } ttg_u32x4;

TTG_HD void ttg_mulhilo32(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo) {
    uint64_t p = (uint64_t)a * (uint64_t)b;
    *hi = (uint32_t)(p >> 32);
    *lo = (uint32_t)p;
}

/* Philox-4x32 with 10 rounds (multipliers and Weyl key increments as
 * published by Salmon et al.). */
TTG_HD ttg_u32x4 ttg_philox4x32_10(ttg_u32x4 ctr, uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        ttg_mulhilo32(0xD2511F53u, ctr.v[0], &hi0, &lo0);
        ttg_mulhilo32(0xCD9E8D57u, ctr.v[2], &hi1, &lo1);
        ttg_u32x4 n;
        n.v[0] = hi1 ^ ctr.v[1] ^ k0;
        n.v[1] = lo1;
        n.v[2] = hi0 ^ ctr.v[3] ^ k1;
        n.v[3] = lo0;
        ctr = n;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return ctr;
}

/* 53-bit uniform in (0,1): (k + 1/2) * 2^-53. */
TTG_HD double ttg_u01(uint32_t hi, uint32_t lo) {
    uint64_t k = (((uint64_t)hi << 32) | (uint64_t)lo) >> 11;
    return TTG_MUL(TTG_ADD((double)k, 0.5), 1.1102230246251565404e-16);
}

/* Natural log for x in (0, +inf) from x = m 2^e, m in [1/sqrt2, sqrt2),
 * ln m = 2 atanh((m-1)/(m+1)) by its odd power series. */
TTG_HD double ttg_ln(double x) {
    union { double d; uint64_t u; } b;
    b.d = x;
    int e = (int)((b.u >> 52) & 0x7ff) - 1022; /* x = f 2^e, f in [0.5,1) */
    b.u = (b.u & 0x000fffffffffffffULL) | 0x3fe0000000000000ULL;
    double m = b.d;
    if (m < 0.70710678118654752440) { m = TTG_MUL(m, 2.0); e -= 1; }
    double s = TTG_DIV(TTG_SUB(m, 1.0), TTG_ADD(m, 1.0));
    double s2 = TTG_MUL(s, s);
    double term = s, sum = 0.0;
    for (int n = 0; n < 14; ++n) {
        sum = TTG_ADD(sum, TTG_DIV(term, (double)(2 * n + 1)));
        term = TTG_MUL(term, s2);
    }
    return TTG_ADD(TTG_MUL((double)e, 0.69314718055994530942), TTG_MUL(2.0, sum));
}

/* sin and cos of 2*pi*f for f in [0, 1/8]: Taylor series to x^23. */
TTG_HD void ttg_sincos_small(double f, double* s, double* c) {
    double x = TTG_MUL(f, 6.28318530717958647692);
    double x2 = TTG_MUL(x, x);
    double ts = x, tc = 1.0, ss = 0.0, cc = 0.0;
    for (int n = 0; n < 12; ++n) {
        ss = TTG_ADD(ss, ts);
        cc = TTG_ADD(cc, tc);
        double a = (double)((2 * n + 2) * (2 * n + 3));
        double bb = (double)((2 * n + 1) * (2 * n + 2));
        ts = TTG_DIV(TTG_MUL(-ts, x2), a);
        tc = TTG_DIV(TTG_MUL(-tc, x2), bb);
    }
    *s = ss;
    *c = cc;
}

/* sin and cos of 2*pi*u for u in [0,1): exact quadrant / octant reduction. */
TTG_HD void ttg_sincos2pi(double u, double* s, double* c) {
    int q = (int)(u * 4.0);
    if (q > 3) q = 3;
    double f = TTG_SUB(u, TTG_MUL((double)q, 0.25)); /* exact, in [0, 1/4) */
    double s0, c0;
    if (f <= 0.125) {
        ttg_sincos_small(f, &s0, &c0);
    } else {
        double cs, cc;
        ttg_sincos_small(TTG_SUB(0.25, f), &cs, &cc);
        s0 = cc;
        c0 = cs;
    }
    switch (q) {
        case 0: *s = s0; *c = c0; break;
        case 1: *s = c0; *c = -s0; break;
        case 2: *s = -s0; *c = -c0; break;
        default: *s = -c0; *c = s0; break;
    }
}

/* Two independent N(0,1) values from counter `ctr` under key (seed, stream). */
TTG_HD void ttg_normal2(uint64_t ctr, uint32_t seed, uint32_t stream, double* z0, double* z1) {
    ttg_u32x4 c;
    c.v[0] = (uint32_t)ctr;
    c.v[1] = (uint32_t)(ctr >> 32);
    c.v[2] = 0u;
    c.v[3] = 0u;
    ttg_u32x4 r = ttg_philox4x32_10(c, seed, stream);
    double u1 = ttg_u01(r.v[0], r.v[1]);
    double u2 = ttg_u01(r.v[2], r.v[3]);
    double rad = TTG_SQRT(TTG_MUL(-2.0, ttg_ln(u1)));
    double sn, cs;
    ttg_sincos2pi(u2, &sn, &cs);
    *z0 = TTG_MUL(rad, cs);
    *z1 = TTG_MUL(rad, sn);
}

/* Element e of an iid N(0,1) sequence. */
TTG_HD double ttg_normal_at(uint64_t e, uint32_t seed, uint32_t stream) {
    double z0, z1;
    ttg_normal2(e >> 1, seed, stream, &z0, &z1);
    return (e & 1) ? z1 : z0;
}

/* Element e of an iid U[-1,1] sequence. */
TTG_HD double ttg_uniform_pm1_at(uint64_t e, uint32_t seed, uint32_t stream) {
    ttg_u32x4 c;
    uint64_t ctr = e >> 1;
    c.v[0] = (uint32_t)ctr;
    c.v[1] = (uint32_t)(ctr >> 32);
    c.v[2] = 0u;
    c.v[3] = 0u;
    ttg_u32x4 r = ttg_philox4x32_10(c, seed, stream);
    double u = (e & 1) ? ttg_u01(r.v[2], r.v[3]) : ttg_u01(r.v[0], r.v[1]);
    return TTG_SUB(TTG_MUL(2.0, u), 1.0);
}

/* Element e of the quantised Gaussian: rint(16 z) clamped to [-127, 127]. */
TTG_HD int ttg_qnormal_at(uint64_t e, uint32_t seed, uint32_t stream) {
    double z = ttg_normal_at(e, seed, stream);
    double t = TTG_MUL(z, 16.0);
    if (t > 127.0) t = 127.0;
    if (t < -127.0) t = -127.0;
    return (int)rint(t);
}

#endif /* TTG_PHILOX_H */
