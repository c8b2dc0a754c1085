// mc_math.cuh -- deterministic FP64 elementary functions and the Philox
// stream, callable from host and device code.
//
// FP64 replay mode must give the same bits on the GPU as the CPU oracle gives
// on the host, so it cannot use libm or CUDA's math library (their last bits
// differ).  These functions use only IEEE +,-,*,/ and sqrt (correctly rounded
// on both sides; device code is built with -fmad=false so nothing is fused)
// and exact bit manipulation:
//   log      x = m 2^k, m in (sqrt(1/2), sqrt(2)]; log m = 2 atanh(s),
//            s = (m-1)/(m+1), series to s^23; k ln2 via a two-part split.
//   exp      k = round(x/ln2), r = x - k ln2 (two-part), Taylor to r^13.
//   sin/cos  Cody-Waite reduction by pi/2 in three 33-bit parts, Taylor
//            series on [-pi/4, pi/4] (sin to r^17, cos to r^18).
// Coefficients are the exact Taylor coefficients rounded to double, written
// as hex literals.
//
// Philox4x32-10 follows Salmon, Moraes, Dror, Shaw, SC'11.  Stream layout:
//   key = (seed_lo, seed_hi ^ history_hi), counter = (draw>>1, event, id,
//   history_lo); even draws use words (0,1), odd draws (2,3); a 64-bit word
//   v maps to ((v >> 12) + 0.5) * 2^-52 in (0, 1).
#pragma once

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define MC_HD __host__ __device__ __forceinline__
#else
#define MC_HD inline
#endif

namespace mc {

MC_HD uint64_t dbits(double x)
{
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    memcpy(&b, &x, 8);
    return b;
#endif
}

MC_HD double dfrom(uint64_t b)
{
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double x;
    memcpy(&x, &b, 8);
    return x;
#endif
}

MC_HD double dsqrt(double x)
{
#ifdef __CUDA_ARCH__
    return __dsqrt_rn(x);
#else
    return __builtin_sqrt(x);
#endif
}

MC_HD double dround_half_up(double t)
{
    return (t >= 0.0) ? (double)(int64_t)(t + 0.5) : -(double)(int64_t)(-t + 0.5);
}

constexpr double kLn2Hi = 0x1.62e42fefa2000p-1;
constexpr double kLn2Lo = 0x1.9ef35793c7673p-41;
constexpr double kInvLn2 = 0x1.71547652b82fep+0;
constexpr double kSqrt2 = 0x1.6a09e667f3bcdp+0;
constexpr double kPio2_1 = 0x1.921fb54400000p+0;
constexpr double kPio2_2 = 0x1.0b4611a600000p-34;
constexpr double kPio2_3 = 0x1.3198a2e037073p-69;
constexpr double kTwoOverPi = 0x1.45f306dc9c883p-1;

MC_HD double plog(double x)
{
    int k = 0;
    uint64_t b = dbits(x);
    if (b < 0x0010000000000000ULL) {
        x = x * 0x1p54;
        b = dbits(x);
        k = -54;
    }
    k += (int)(b >> 52) - 1023;
    double m = dfrom((b & 0x000FFFFFFFFFFFFFULL) | 0x3FF0000000000000ULL);
    if (m > kSqrt2) { m = m * 0.5; k += 1; }
    const double f = m - 1.0;
    const double s = f / (2.0 + f);
    const double z = s * s;
    double p = 0x1.642c8590b2164p-5;
    p = 0x1.8618618618618p-5 + z * p;
    p = 0x1.af286bca1af28p-5 + z * p;
    p = 0x1.e1e1e1e1e1e1ep-5 + z * p;
    p = 0x1.1111111111111p-4 + z * p;
    p = 0x1.3b13b13b13b14p-4 + z * p;
    p = 0x1.745d1745d1746p-4 + z * p;
    p = 0x1.c71c71c71c71cp-4 + z * p;
    p = 0x1.2492492492492p-3 + z * p;
    p = 0x1.999999999999ap-3 + z * p;
    p = 0x1.5555555555555p-2 + z * p;
    const double two_s = 2.0 * s;
    const double r = two_s + two_s * (z * p);
    const double kd = (double)k;
    return kd * kLn2Hi + (r + kd * kLn2Lo);
}

MC_HD double pexp(double x)
{
    const double kd = dround_half_up(x * kInvLn2);
    const int k = (int)kd;
    const double r = (x - kd * kLn2Hi) - kd * kLn2Lo;
    double p = 0x1.6124613a86d09p-33;
    p = 0x1.1eed8eff8d898p-29 + r * p;
    p = 0x1.ae64567f544e4p-26 + r * p;
    p = 0x1.27e4fb7789f5cp-22 + r * p;
    p = 0x1.71de3a556c734p-19 + r * p;
    p = 0x1.a01a01a01a01ap-16 + r * p;
    p = 0x1.a01a01a01a01ap-13 + r * p;
    p = 0x1.6c16c16c16c17p-10 + r * p;
    p = 0x1.1111111111111p-7 + r * p;
    p = 0x1.5555555555555p-5 + r * p;
    p = 0x1.5555555555555p-3 + r * p;
    p = 0x1.0000000000000p-1 + r * p;
    p = 1.0 + r * p;
    p = 1.0 + r * p;
    const int k1 = k / 2, k2 = k - k / 2;
    const double s1 = dfrom((uint64_t)(k1 + 1023) << 52);
    const double s2 = dfrom((uint64_t)(k2 + 1023) << 52);
    return (p * s1) * s2;
}

MC_HD double psin_poly(double r)
{
    const double z = r * r;
    double p = 0x1.952c77030ad4ap-49;
    p = -0x1.ae7f3e733b81fp-41 + z * p;
    p = 0x1.6124613a86d09p-33 + z * p;
    p = -0x1.ae64567f544e4p-26 + z * p;
    p = 0x1.71de3a556c734p-19 + z * p;
    p = -0x1.a01a01a01a01ap-13 + z * p;
    p = 0x1.1111111111111p-7 + z * p;
    p = -0x1.5555555555555p-3 + z * p;
    return r + r * (z * p);
}

MC_HD double pcos_poly(double r)
{
    const double z = r * r;
    double p = -0x1.6827863b97d97p-53;
    p = 0x1.ae7f3e733b81fp-45 + z * p;
    p = -0x1.93974a8c07c9dp-37 + z * p;
    p = 0x1.1eed8eff8d898p-29 + z * p;
    p = -0x1.27e4fb7789f5cp-22 + z * p;
    p = 0x1.a01a01a01a01ap-16 + z * p;
    p = -0x1.6c16c16c16c17p-10 + z * p;
    p = 0x1.5555555555555p-5 + z * p;
    return 1.0 - (0.5 * z - (z * z) * p);
}

MC_HD double preduce(double x, int &quad)
{
    const double n = dround_half_up(x * kTwoOverPi);
    quad = (int)((int64_t)n & 3);
    return ((x - n * kPio2_1) - n * kPio2_2) - n * kPio2_3;
}

MC_HD double psin(double x)
{
    int q;
    const double r = preduce(x, q);
    switch (q) {
    case 0: return psin_poly(r);
    case 1: return pcos_poly(r);
    case 2: return -psin_poly(r);
    default: return -pcos_poly(r);
    }
}

MC_HD double pcos(double x)
{
    int q;
    const double r = preduce(x, q);
    switch (q) {
    case 0: return pcos_poly(r);
    case 1: return -psin_poly(r);
    case 2: return -pcos_poly(r);
    default: return psin_poly(r);
    }
}

// ----------------------------------------------------------------------------
// Philox4x32-10
// ----------------------------------------------------------------------------
struct U4 { uint32_t x, y, z, w; };

MC_HD void mulhilo32(uint32_t a, uint32_t b, uint32_t &hi, uint32_t &lo)
{
#ifdef __CUDA_ARCH__
    lo = a * b;
    hi = __umulhi(a, b);
#else
    const uint64_t p = (uint64_t)a * b;
    hi = (uint32_t)(p >> 32);
    lo = (uint32_t)p;
#endif
}

MC_HD U4 philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(0xD2511F53u, c0, hi0, lo0);
        mulhilo32(0xCD9E8D57u, c2, hi1, lo1);
        const uint32_t n0 = hi1 ^ c1 ^ k0;
        const uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    }
    return U4{c0, c1, c2, c3};
}

MC_HD uint32_t fmix32(uint32_t h)
{
    h ^= h >> 16; h *= 0x85EBCA6Bu;
    h ^= h >> 13; h *= 0xC2B2AE35u;
    h ^= h >> 16;
    return h;
}

// id of the k-th copy (k >= 1) made by a split during event `event`
MC_HD uint32_t child_id(uint32_t parent, uint32_t event, uint32_t k)
{
    return fmix32(parent * 0x9E3779B1u + fmix32(event * 0x85EBCA77u + k));
}

MC_HD double u01(uint32_t lo, uint32_t hi)
{
    const uint64_t v = ((uint64_t)hi << 32) | lo;
    return ((double)(v >> 12) + 0.5) * 0x1p-52;
}

// float draw in (0,1) from one 32-bit word (24 significant bits)
MC_HD float u01f(uint32_t x) { return ((float)(x >> 9) + 0.5f) * 0x1p-23f; }

// Sequential draws of one particle within one event.  Caches the current
// Philox block so the two draws of a block cost one evaluation.
struct Stream {
    uint32_t k0, k1;      // key
    uint32_t hist_lo;
    uint32_t id;
    uint32_t event;
    uint32_t draw;
    uint32_t cached;      // block index + 1 held in blk (0 = none)
    U4 blk;

    MC_HD void init(uint64_t seed, uint64_t history)
    {
        k0 = (uint32_t)seed;
        k1 = (uint32_t)(seed >> 32) ^ (uint32_t)(history >> 32);
        hist_lo = (uint32_t)history;
        id = 0; event = 0; draw = 0; cached = 0;
    }
    MC_HD void start_event(uint32_t ev) { event = ev; draw = 0; cached = 0; }
    MC_HD double next()
    {
        const uint32_t b = draw >> 1;
        if (cached != b + 1) {
            blk = philox(b, event, id, hist_lo, k0, k1);
            cached = b + 1;
        }
        const double u = (draw & 1u) ? u01(blk.z, blk.w) : u01(blk.x, blk.y);
        ++draw;
        return u;
    }
};

}  // namespace mc
