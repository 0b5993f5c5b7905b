// lg_ozdigits.cuh -- split-precision digit arithmetic shared by the
// tensor-core kernels (lg_ozaki.cu, lg_ozgemm.cu).  See lg_ozaki.cu for the
// scheme.  Everything here is integer work on IEEE bit patterns.
#pragma once

#include <stdint.h>

namespace lg {
namespace oz {

constexpr int NS = 8;  // digits per value
constexpr uint32_t LBO = 128;   // K-adjacent core matrices (8 rows x 16 B) are contiguous

__device__ __forceinline__ int bexp(unsigned long long b) { return (int)((b >> 52) & 0x7FF); }

// round(x * 2^(56-e)) with 2^e = 2^(emax-1022) > |x|; 0 for zero / subnormal.
__device__ __forceinline__ long long fixed56(unsigned long long b, int emax)
{
    int ex = bexp(b);
    if (ex == 0 || emax == 0) return 0;
    long long mant = (long long)((b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull);
    int sh = ex - emax + 3;
    long long X;
    if (sh >= 0)
        X = mant << sh;
    else if (sh > -60)
        X = (mant + (1LL << (-sh - 1))) >> (-sh);
    else
        X = 0;
    return (b >> 63) ? -X : X;
}

// Balanced base-128 digits of X (|X| < 2^56), most significant first, as FP32
// bit patterns whose upper halves are the BF16 encodings of the digits:
// X = sum_s d_s 2^(7(7-s)), d_0 in [-128, 128], d_1..d_7 in [-64, 63].
// The low seven digits come from biasing X by 64 in every low digit position
// (B = 64 (2^49 - 1) / 127) and taking plain 7-bit chunks c of X + B, so each
// is c - 64; small integers become floats through a magic-number add, so the
// whole split is integer ALU work plus one FADD per digit.
__device__ __forceinline__ void digit_floats(long long X, uint32_t (&f)[NS])
{
    const long long B = 64LL * (((1LL << 49) - 1) / 127);
    const long long T = X + B;
    const uint32_t lo = (uint32_t)T, hi = (uint32_t)((unsigned long long)T >> 32);
    const int top = ((int)hi) >> 17;  // floor(T / 2^49)
    f[0] = __float_as_uint(__int_as_float(0x4B400000 + top) - 12582912.0f);
    const float bias = 8388672.0f;  // 2^23 + 64
    f[1] = __float_as_uint(__int_as_float(0x4B000000 | ((hi >> 10) & 127u)) - bias);
    f[2] = __float_as_uint(__int_as_float(0x4B000000 | ((hi >> 3) & 127u)) - bias);
    f[3] = __float_as_uint(__int_as_float(0x4B000000 | (__funnelshift_r(lo, hi, 28) & 127u)) - bias);
    f[4] = __float_as_uint(__int_as_float(0x4B000000 | ((lo >> 21) & 127u)) - bias);
    f[5] = __float_as_uint(__int_as_float(0x4B000000 | ((lo >> 14) & 127u)) - bias);
    f[6] = __float_as_uint(__int_as_float(0x4B000000 | ((lo >> 7) & 127u)) - bias);
    f[7] = __float_as_uint(__int_as_float(0x4B000000 | (lo & 127u)) - bias);
}

// Two BF16 digits (upper halves of two FP32 patterns) packed into one word.
__device__ __forceinline__ uint32_t pack_hi(uint32_t a, uint32_t b) { return __byte_perm(a, b, 0x7632); }

// Exact integer value of an FP32 accumulator holding an integer |v| < 2^22.
__device__ __forceinline__ int acc_int(uint32_t vbits)
{
    return __float_as_int(__uint_as_float(vbits) + 12582912.0f) - 0x4B400000;
}

// Double of (hi * 2^28 + lo) * 2^sc from integer work only (|hi|, |lo| < 2^43):
// J = hi * 2^19 + floor(lo / 2^9) fits in 63 bits and keeps every bit down to
// 2^-54 of the group scale (the digit truncation itself is 2^-56); J is then
// rounded to 53 bits to nearest.
__device__ __forceinline__ double assemble_fast(long long hi, long long lo, int sc)
{
    const long long J = hi * (1LL << 19) + (lo >> 9);
    if (J == 0) return 0.0;
    unsigned long long sign = 0;
    unsigned long long a = (unsigned long long)J;
    if (J < 0) {
        sign = 1ull << 63;
        a = (unsigned long long)(-J);
    }
    int msb = 63 - __clzll((long long)a);
    unsigned long long mant;
    if (msb <= 52) {
        mant = a << (52 - msb);
    } else {
        const int sh = msb - 52;
        mant = (a + (1ull << (sh - 1))) >> sh;
        if (mant >> 53) {
            mant >>= 1;
            msb++;
        }
    }
    const int be = msb + sc + 9 + 1023;
    if (be <= 0) return sign ? -0.0 : 0.0;
    if (be >= 2047) return __longlong_as_double((long long)(sign | 0x7FF0000000000000ull));
    return __longlong_as_double((long long)(sign | ((unsigned long long)be << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}

// (hi * 2^28 + lo) * 2^sc rounded to nearest even double; integer-only.
__device__ __forceinline__ double assemble(long long hi, long long lo, int sc)
{
    __int128 I = ((__int128)hi << 28) + (__int128)lo;
    if (I == 0) return 0.0;
    unsigned long long sign = 0;
    unsigned __int128 a;
    if (I < 0) {
        sign = 1ull << 63;
        a = (unsigned __int128)(-I);
    } else {
        a = (unsigned __int128)I;
    }
    unsigned long long ah = (unsigned long long)(a >> 64), al = (unsigned long long)a;
    int msb = ah ? 127 - __clzll((long long)ah) : 63 - __clzll((long long)al);
    unsigned long long mant;
    if (msb <= 52) {
        mant = al << (52 - msb);
    } else {
        int sh = msb - 52;
        unsigned __int128 q = a >> sh;
        unsigned __int128 rem = a - (q << sh);
        unsigned __int128 half = (unsigned __int128)1 << (sh - 1);
        mant = (unsigned long long)q;
        if (rem > half || (rem == half && (mant & 1ull))) {
            mant++;
            if (mant == (1ull << 53)) {
                mant >>= 1;
                msb++;
            }
        }
    }
    int be = msb + sc + 1023;
    if (be <= 0) return sign ? -0.0 : 0.0;
    if (be >= 2047) return __longlong_as_double((long long)(sign | 0x7FF0000000000000ull));
    unsigned long long bits = sign | ((unsigned long long)be << 52) | (mant & 0xFFFFFFFFFFFFFull);
    return __longlong_as_double((long long)bits);
}

}  // namespace oz
}  // namespace lg
