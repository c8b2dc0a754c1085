/*
 * orc_math.h -- portable FP64 elementary functions for the CPU oracle.
 *
 * TEST INFRASTRUCTURE: this file belongs to the CPU oracle.  Only the test
 * suite, the smoke check and the CPU-baseline leg of bench.py use it.
 *
 * Why: FP64 replay must give bit-identical results on the host (x86-64 or
 * aarch64 gcc, -ffp-contract=off) and on the GPU (nvcc -fmad=false).  libm and
 * CUDA's libdevice give different last bits, so the transport restatement uses
 * these functions, built only from IEEE +,-,*,/ and sqrt (all correctly
 * rounded everywhere) and exact bit manipulation.
 *
 * Methods (all textbook, coefficients are exact Taylor coefficients rounded
 * to double, written as hex literals so every compiler reads the same bits):
 *   log : x = m*2^k, m in (sqrt(1/2), sqrt(2)];  log m = 2 atanh(s),
 *         s = (m-1)/(m+1), series sum_{j>=0} s^(2j+1)/(2j+1) to j = 11;
 *         k*ln2 added with a two-part (Cody-Waite) split of ln2.
 *   exp : k = round(x/ln2), r = x - k*ln2 (two-part split), Taylor to r^13,
 *         scaled by 2^k through the exponent bits.
 *   sin/cos : n = round(x*2/pi), r = x - n*(pi/2) with a three-part split of
 *         pi/2 (each part 33 significant bits), Taylor series on |r| <= pi/4
 *         (sin to r^17, cos to r^18), quadrant chosen by n mod 4.
 * Accuracy is a few ulp, checked against libm in the tests; determinism is
 * the point.
 */
#ifndef ORC_MATH_H
#define ORC_MATH_H

#include <stdint.h>
#include <string.h>

static inline uint64_t orc_bits(double x) { uint64_t b; memcpy(&b, &x, 8); return b; }
static inline double orc_from_bits(uint64_t b) { double x; memcpy(&x, &b, 8); return x; }

#define ORC_LN2_HI   0x1.62e42fefa2000p-1   /* ln2 truncated to 40 bits */
#define ORC_LN2_LO   0x1.9ef35793c7673p-41  /* ln2 - ORC_LN2_HI */
#define ORC_INV_LN2  0x1.71547652b82fep+0
#define ORC_SQRT2    0x1.6a09e667f3bcdp+0
#define ORC_PIO2_1   0x1.921fb54400000p+0   /* pi/2, first 33 bits */
#define ORC_PIO2_2   0x1.0b4611a600000p-34  /* next 33 bits */
#define ORC_PIO2_3   0x1.3198a2e037073p-69  /* remainder */
#define ORC_2_OVER_PI 0x1.45f306dc9c883p-1

static inline double orc_log(double x)
{
    /* x > 0 and finite (the transport only takes logs of (0,1) draws and
     * positive products of them). */
    int k = 0;
    uint64_t b = orc_bits(x);
    if (b < 0x0010000000000000ULL) {          /* subnormal: rescale */
        x = x * 0x1p54;
        b = orc_bits(x);
        k = -54;
    }
    k += (int)(b >> 52) - 1023;
    double m = orc_from_bits((b & 0x000FFFFFFFFFFFFFULL) | 0x3FF0000000000000ULL);
    if (m > ORC_SQRT2) { m = m * 0.5; k += 1; }
    double f = m - 1.0;
    double s = f / (2.0 + f);
    double z = s * s;
    double p = 0x1.642c8590b2164p-5;          /* 1/23 */
    p = 0x1.8618618618618p-5 + z * p;         /* 1/21 */
    p = 0x1.af286bca1af28p-5 + z * p;         /* 1/19 */
    p = 0x1.e1e1e1e1e1e1ep-5 + z * p;         /* 1/17 */
    p = 0x1.1111111111111p-4 + z * p;         /* 1/15 */
    p = 0x1.3b13b13b13b14p-4 + z * p;         /* 1/13 */
    p = 0x1.745d1745d1746p-4 + z * p;         /* 1/11 */
    p = 0x1.c71c71c71c71cp-4 + z * p;         /* 1/9  */
    p = 0x1.2492492492492p-3 + z * p;         /* 1/7  */
    p = 0x1.999999999999ap-3 + z * p;         /* 1/5  */
    p = 0x1.5555555555555p-2 + z * p;         /* 1/3  */
    double two_s = 2.0 * s;
    double r = two_s + two_s * (z * p);
    double kd = (double)k;
    return kd * ORC_LN2_HI + (r + kd * ORC_LN2_LO);
}

static inline double orc_exp(double x)
{
    /* |x| < 700 (only used to build energy-filter grids at set-up). */
    double kd = x * ORC_INV_LN2;
    kd = (kd >= 0.0) ? (double)(int64_t)(kd + 0.5) : -(double)(int64_t)(-kd + 0.5);
    int k = (int)kd;
    double r = (x - kd * ORC_LN2_HI) - kd * ORC_LN2_LO;
    double p = 0x1.6124613a86d09p-33;         /* 1/13! */
    p = 0x1.1eed8eff8d898p-29 + r * p;        /* 1/12! */
    p = 0x1.ae64567f544e4p-26 + r * p;        /* 1/11! */
    p = 0x1.27e4fb7789f5cp-22 + r * p;        /* 1/10! */
    p = 0x1.71de3a556c734p-19 + r * p;        /* 1/9!  */
    p = 0x1.a01a01a01a01ap-16 + r * p;        /* 1/8!  */
    p = 0x1.a01a01a01a01ap-13 + r * p;        /* 1/7!  */
    p = 0x1.6c16c16c16c17p-10 + r * p;        /* 1/6!  */
    p = 0x1.1111111111111p-7 + r * p;         /* 1/5!  */
    p = 0x1.5555555555555p-5 + r * p;         /* 1/4!  */
    p = 0x1.5555555555555p-3 + r * p;         /* 1/3!  */
    p = 0x1.0000000000000p-1 + r * p;         /* 1/2!  */
    p = 1.0 + r * p;
    p = 1.0 + r * p;
    /* scale by 2^k in two steps so that k down to -1074 stays exact enough */
    int k1 = k / 2, k2 = k - k / 2;
    double s1 = orc_from_bits((uint64_t)(k1 + 1023) << 52);
    double s2 = orc_from_bits((uint64_t)(k2 + 1023) << 52);
    return (p * s1) * s2;
}

static inline double orc_sin_poly(double r)
{
    double z = r * r;
    double p = 0x1.952c77030ad4ap-49;         /* +1/17! */
    p = -0x1.ae7f3e733b81fp-41 + z * p;       /* -1/15! */
    p = 0x1.6124613a86d09p-33 + z * p;        /* +1/13! */
    p = -0x1.ae64567f544e4p-26 + z * p;       /* -1/11! */
    p = 0x1.71de3a556c734p-19 + z * p;        /* +1/9!  */
    p = -0x1.a01a01a01a01ap-13 + z * p;       /* -1/7!  */
    p = 0x1.1111111111111p-7 + z * p;         /* +1/5!  */
    p = -0x1.5555555555555p-3 + z * p;        /* -1/3!  */
    return r + r * (z * p);
}

static inline double orc_cos_poly(double r)
{
    double z = r * r;
    double p = -0x1.6827863b97d97p-53;        /* -1/18! */
    p = 0x1.ae7f3e733b81fp-45 + z * p;        /* +1/16! */
    p = -0x1.93974a8c07c9dp-37 + z * p;       /* -1/14! */
    p = 0x1.1eed8eff8d898p-29 + z * p;        /* +1/12! */
    p = -0x1.27e4fb7789f5cp-22 + z * p;       /* -1/10! */
    p = 0x1.a01a01a01a01ap-16 + z * p;        /* +1/8!  */
    p = -0x1.6c16c16c16c17p-10 + z * p;       /* -1/6!  */
    p = 0x1.5555555555555p-5 + z * p;         /* +1/4!  */
    /* 1 - z/2 + z^2 * p */
    return 1.0 - (0.5 * z - (z * z) * p);
}

/* Reduce x to r in [-pi/4, pi/4] and the quadrant n mod 4 (|x| < 2^20). */
static inline double orc_reduce(double x, int *quad)
{
    double t = x * ORC_2_OVER_PI;
    double n = (t >= 0.0) ? (double)(int64_t)(t + 0.5) : -(double)(int64_t)(-t + 0.5);
    *quad = (int)((int64_t)n & 3);
    return ((x - n * ORC_PIO2_1) - n * ORC_PIO2_2) - n * ORC_PIO2_3;
}

static inline double orc_sin(double x)
{
    int q; double r = orc_reduce(x, &q);
    switch (q) {
    case 0: return orc_sin_poly(r);
    case 1: return orc_cos_poly(r);
    case 2: return -orc_sin_poly(r);
    default: return -orc_cos_poly(r);
    }
}

static inline double orc_cos(double x)
{
    int q; double r = orc_reduce(x, &q);
    switch (q) {
    case 0: return orc_cos_poly(r);
    case 1: return -orc_sin_poly(r);
    case 2: return -orc_cos_poly(r);
    default: return orc_sin_poly(r);
    }
}

#endif /* ORC_MATH_H */
