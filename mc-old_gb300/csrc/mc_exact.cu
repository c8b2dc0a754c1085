// mc_exact.cu -- exact per-bin tally sums of the FP64 modes, for merging
// disjoint history ranges (several GPUs, several processes) bit for bit.
//
// The reference folds each history's tally into a running FP64 sum
// (Estimator.cpp:339-346): sum += h, squared += h * h.  FP64 replay keeps that
// order, so one run over [0, n) equals the reference bit for bit; but the
// sum of two runs over [0, a) and [a, n) rounds differently from the single
// run, because FP64 addition is not associative.  So beside the running sums
// the FP64 modes accumulate every bin's sum of history totals and sum of
// their (FP64-rounded) squares exactly, as an integer multiple of 2^-1074
// (every double is one).  Integer addition is associative: exact sums of
// disjoint ranges added in any order, then rounded once to the nearest
// double, give what one run over the union gives, bit for bit.
//
// Representation of one exact value: kExactLimbs signed 64-bit limbs,
// value = sum_j limb[j] * 2^(32 j - 1074).  A double's 53-bit significand
// at its binary position lands in three consecutive limbs as 32-bit digits
// (carry-save: a limb absorbs 2^31 such adds before it could overflow), and
// normalising propagates the carries so that limbs 0..kExactLimbs-2 hold
// digits in [0, 2^32) and the last limb holds the signed rest -- one
// representation per value, which is what mc_exact_sums_read returns.
#include <cmath>
#include <cstring>

#include "mc_device.h"
#include "mc_engine.h"

namespace mc {

namespace {

constexpr uint32_t kExactSlice = 4096;   // histories one thread folds into its own accumulator

// v (finite) into acc as three signed 32-bit digits
__device__ __forceinline__ void exact_add(long long *acc, double v)
{
    const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
    const int e = (int)((bits >> 52) & 0x7FF);
    unsigned long long m = bits & ((1ull << 52) - 1);
    int p = 0;                       // v = m * 2^(p - 1074)
    if (e != 0) {
        m |= 1ull << 52;
        p = e - 1;
    }
    const int j = p >> 5, sh = p & 31;
    const unsigned __int128 t = (unsigned __int128)m << sh;   // < 2^85
    const long long d0 = (long long)(unsigned long long)(t & 0xFFFFFFFFull);
    const long long d1 = (long long)(unsigned long long)((t >> 32) & 0xFFFFFFFFull);
    const long long d2 = (long long)(unsigned long long)(t >> 64);
    if (bits >> 63) {
        acc[j] -= d0; acc[j + 1] -= d1; acc[j + 2] -= d2;
    } else {
        acc[j] += d0; acc[j + 1] += d1; acc[j + 2] += d2;
    }
}

__device__ __forceinline__ void exact_normalize(long long *acc)
{
    for (int j = 0; j < kExactLimbs - 1; ++j) {
        const long long carry = acc[j] >> 32;     // arithmetic: floor division by 2^32
        acc[j] -= carry * 4294967296ll;
        acc[j + 1] += carry;
    }
}

// Thread (bin b, slice of histories, which = sum / squares): accumulates the
// slice's nonzero history totals (or their FP64 squares) exactly in a local
// accumulator, normalises it and adds its limbs to the bin's exact value with
// 64-bit integer atomics (exact, in any order).
__global__ void k_fold_exact(const double *__restrict__ hist, uint32_t n, long long nb, long long *ex)
{
    const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const int which = blockIdx.z;
    const uint32_t h0 = blockIdx.y * kExactSlice;
    const uint32_t h1 = min(n, h0 + kExactSlice);
    long long acc[kExactLimbs];
    for (int j = 0; j < kExactLimbs; ++j) acc[j] = 0;
    bool any = false;
    for (uint32_t h = h0; h < h1; ++h) {
        const double v = hist[(size_t)h * nb + b];
        if (v == 0.0) continue;
        const double x = which ? v * v : v;
        // a square below the smallest subnormal adds nothing; a non-finite
        // value (an overflowed square) has no exact value and is left out
        if (x == 0.0 || !(fabs(x) <= 1.7976931348623157e308)) continue;
        exact_add(acc, x);
        any = true;
    }
    if (!any) return;
    exact_normalize(acc);
    unsigned long long *dst = reinterpret_cast<unsigned long long *>(ex + ((size_t)b * 2 + which) * kExactLimbs);
    for (int j = 0; j < kExactLimbs; ++j)
        if (acc[j] != 0) atomicAdd(dst + j, (unsigned long long)acc[j]);   // two's complement: signed add
}

__global__ void k_exact_normalize(long long *ex, long long count)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    long long a[kExactLimbs];
    long long *p = ex + (size_t)i * kExactLimbs;
    for (int j = 0; j < kExactLimbs; ++j) a[j] = p[j];
    exact_normalize(a);
    for (int j = 0; j < kExactLimbs; ++j) p[j] = a[j];
}

}  // namespace

cudaError_t launch_fold_exact(const double *hist, uint32_t n, long long nb, long long *ex, cudaStream_t st)
{
    if (nb <= 0 || n == 0) return cudaSuccess;
    const int block = 128;
    dim3 grid((unsigned)((nb + block - 1) / block), (n + kExactSlice - 1) / kExactSlice, 2);
    k_fold_exact<<<grid, block, 0, st>>>(hist, n, nb, ex);
    return cudaGetLastError();
}

cudaError_t launch_exact_normalize(long long *ex, long long nb, cudaStream_t st)
{
    if (nb <= 0) return cudaSuccess;
    const long long count = 2 * nb;
    k_exact_normalize<<<(unsigned)((count + 127) / 128), 128, 0, st>>>(ex, count);
    return cudaGetLastError();
}

// Nearest double (ties to even) of one exact value: the limbs are
// normalised on a copy, the sign taken from the top, the magnitude's top 64
// bits rounded to 53 with the lower bits as a sticky bit.  Every value is a
// multiple of 2^-1074, so a magnitude below 2^-1022 is exactly a subnormal.
double exact_round(const int64_t *limbs)
{
    long long a[kExactLimbs];
    std::memcpy(a, limbs, sizeof(a));
    for (int j = 0; j < kExactLimbs - 1; ++j) {
        const long long carry = a[j] >> 32;
        a[j] -= carry * 4294967296ll;
        a[j + 1] += carry;
    }
    const bool neg = a[kExactLimbs - 1] < 0;
    if (neg) {   // magnitude: negate the whole number, then normalise again
        for (int j = 0; j < kExactLimbs; ++j) a[j] = -a[j];
        for (int j = 0; j < kExactLimbs - 1; ++j) {
            const long long carry = a[j] >> 32;
            a[j] -= carry * 4294967296ll;
            a[j + 1] += carry;
        }
    }
    // digits d[0..K-1] in [0, 2^32) except possibly the top one (>= 0)
    int top = kExactLimbs - 1;
    while (top >= 0 && a[top] == 0) --top;
    if (top < 0) return 0.0;
    // the top limb may exceed 32 bits only for magnitudes far above DBL_MAX
    if (top == kExactLimbs - 1 && (unsigned long long)a[top] >= (1ull << 32)) return neg ? -HUGE_VAL : HUGE_VAL;
    const int lz = __builtin_clzll((unsigned long long)a[top]);
    const int msb = 32 * top + (63 - lz);          // bit index of the leading one
    if (msb < 53) {                                 // below 2^-1021: exact (a multiple of 2^-1074, < 2^53 units)
        unsigned long long v = 0;
        for (int j = top; j >= 0; --j) v = (v << 32) | (unsigned long long)a[j];
        const double r = std::ldexp((double)v, -1074);
        return neg ? -r : r;
    }
    // the 64 bits below and including the leading one, and whether anything
    // below them is nonzero
    unsigned long long hi = 0;
    bool sticky = false;
    for (int bit = msb, k = 0; k < 64; ++k, --bit) {
        unsigned long long b = 0;
        if (bit >= 0) b = ((unsigned long long)a[bit >> 5] >> (bit & 31)) & 1ull;
        hi = (hi << 1) | b;
    }
    for (int bit = msb - 64; bit >= 0 && !sticky; --bit)
        if (((unsigned long long)a[bit >> 5] >> (bit & 31)) & 1ull) sticky = true;
    unsigned long long mant = hi >> 11;             // 53 bits
    const unsigned long long rest = hi & 0x7FFull;  // 11 bits below
    const bool up = rest > 0x400ull || (rest == 0x400ull && (sticky || (mant & 1ull)));
    int e = msb - 52 - 1074;                        // value = mant * 2^e
    if (up) {
        ++mant;
        if (mant == (1ull << 53)) { mant >>= 1; ++e; }
    }
    if (e > 1023 - 52) return neg ? -HUGE_VAL : HUGE_VAL;
    const double r = std::ldexp((double)mant, e);
    return neg ? -r : r;
}

}  // namespace mc
