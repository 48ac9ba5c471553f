// rt_fixed.cuh — exact conversions in integer arithmetic.
//
// GB300 executes FP64 (and 64-bit float<->int conversions) at a small fraction of its FP32
// rate, so the three places that need double semantics do them with integer instructions and
// give the very bits the FP64 expressions give:
//   * ray generation: (float)((double)X * dp) for an integer X (RayTracer.cpp:14-18 computes the
//     pixel offset times dp in double and stores it as float);
//   * frame resolve: (float)((double)acc * scale), acc a 64-bit fixed-point colour sum;
//   * accumulation: llrint(v * 2^32), the fixed-point value of a float colour.
// Round-to-nearest-even at every step, as IEEE-754 does.
#pragma once
#include <cstdint>

namespace rtg {

__device__ __forceinline__ int bitlen64(unsigned long long v) { return v ? 64 - __clzll((long long)v) : 0; }

// Round the 128-bit value (hi:lo) to `bits` (<= 63) significant bits, nearest-even. Returns the
// significand k and sets `shift` so that the rounded value is k * 2^shift.
__device__ __forceinline__ unsigned long long round_sig(unsigned long long hi, unsigned long long lo, int bits, int &shift)
{
    const int L = hi ? 128 - __clzll((long long)hi) : bitlen64(lo);
    if (L <= bits) {   // exact (hi is 0 here because bits < 64)
        shift = 0;
        return lo;
    }
    const int s = L - bits;   // 1 .. 127 bits dropped
    unsigned long long k, rb, st;
    if (s >= 64) {
        k = hi >> (s - 64);
        const int r = s - 1;   // index of the round bit, >= 63
        if (r >= 64) {
            rb = (hi >> (r - 64)) & 1ull;
            st = lo | (r > 64 ? (hi & ((1ull << (r - 64)) - 1ull)) : 0ull);
        } else {
            rb = lo >> 63;
            st = lo & ((1ull << 63) - 1ull);
        }
    } else {
        k = (hi << (64 - s)) | (lo >> s);
        rb = (lo >> (s - 1)) & 1ull;
        st = s > 1 ? (lo & ((1ull << (s - 1)) - 1ull)) : 0ull;
    }
    shift = s;
    if (rb && (st || (k & 1ull))) {
        ++k;
        if (k >> bits) {   // carried into a new leading bit
            k >>= 1;
            ++shift;
        }
    }
    return k;
}

// k * 2^E as float for k < 2^24 (exact while the result is a normal float)
__device__ __forceinline__ float scale_pow2(unsigned k, int E)
{
    float f = __uint2float_rn(k);
    while (E > 127) {
        f *= 1.7014118346046923e38f;   // 2^127
        E -= 127;
    }
    while (E < -126) {
        f *= 1.1754943508222875e-38f;   // 2^-126
        E += 126;
    }
    return f * __int_as_float((E + 127) << 23);
}

// the significand and exponent of a positive normal double: d = m * 2^e, 2^52 <= m < 2^53
struct DSplit {
    unsigned long long m;
    int e;
};
__host__ __device__ __forceinline__ DSplit split_double_bits(unsigned long long bits)
{
    return DSplit{(bits & ((1ull << 52) - 1ull)) | (1ull << 52), (int)((bits >> 52) & 0x7ff) - 1075};
}

// (float)((double)x * d) for a 64-bit integer x and a positive normal double d = m * 2^e:
// x rounded to double, the product rounded to double, then to float.
__device__ __forceinline__ float dmul_to_float(long long x, DSplit d)
{
    if (x == 0) return 0.0f;
    const bool neg = x < 0;
    const unsigned long long ax = neg ? 0ull - (unsigned long long)x : (unsigned long long)x;
    // d a power of two (the resolve scale 2^-32 / spp for a power-of-two spp) and |x| < 2^53:
    // (double)x and the product are exact, so the value is x rounded once to float (the
    // hardware's round-to-nearest-even conversion) times d, exact while it stays a normal float
    if (d.m == (1ull << 52) && ax < (1ull << 53) && d.e >= -178 && d.e <= 22) {
        const float f = __ull2float_rn(ax) * __int_as_float((d.e + 52 + 127) << 23);
        return neg ? -f : f;
    }
    int s0, s1, s2;
    const unsigned long long xr = round_sig(0ull, ax, 53, s0);   // (double)x
    const unsigned long long hi = __umul64hi(xr, d.m), lo = xr * d.m;
    const unsigned long long k53 = round_sig(hi, lo, 53, s1);     // the double product
    const unsigned long long k24 = round_sig(0ull, k53, 24, s2);  // to float
    const float f = scale_pow2((unsigned)k24, s0 + s1 + s2 + d.e);
    return neg ? -f : f;
}

// llrint(v * 2^32) for a finite float v with |v| < 2^31 (the fixed-point colour unit)
__device__ __forceinline__ long long float_to_fix32(float v)
{
    const unsigned b = __float_as_uint(v);
    const int ex = (int)((b >> 23) & 0xffu);
    if (ex == 0) return 0;   // zero or subnormal: |v * 2^32| < 2^-94
    const unsigned long long m = (b & 0x7fffffu) | 0x800000u;
    const int sh = ex - 127 - 23 + 32;   // v * 2^32 = m * 2^sh
    unsigned long long r;
    if (sh >= 0)
        r = m << sh;
    else if (sh < -25)
        r = 0;   // below 1/2
    else {
        r = m >> (-sh);
        const unsigned long long rb = (m >> (-sh - 1)) & 1ull, st = m & ((1ull << (-sh - 1)) - 1ull);
        if (rb && (st || (r & 1ull))) ++r;
    }
    return (b >> 31) ? -(long long)r : (long long)r;
}

} // namespace rtg
