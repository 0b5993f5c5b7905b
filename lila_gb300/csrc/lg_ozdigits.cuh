// lg_ozdigits.cuh -- split-precision digit arithmetic shared by the
// tensor-core kernels (lg_ozaki.cu, lg_ozgemm.cu).  See lg_ozaki.cu for the
// scheme.  Integer work on IEEE bit patterns, plus one FP32 or BF16x2
// subtraction per digit word.
#pragma once

#include <stdint.h>

#include <cuda_bf16.h>

namespace lg {
namespace oz {

constexpr int NS = 8;  // digits per value
constexpr uint32_t LBO = 128;   // K-adjacent core matrices (8 rows x 16 B) are contiguous

__device__ __forceinline__ int bexp(unsigned long long b) { return (int)((b >> 52) & 0x7FF); }

// round(x * 2^(56-e)) with 2^e = 2^(emax-1022) > |x|; 0 for zero / subnormal.
// The scaling is an add to the exponent field (the scaled exponent stays in
// [1, 1078], so the sign bit is untouched and |x 2^(56-e)| < 2^56), the
// rounding (to nearest even) the double -> int64 conversion.
__device__ __forceinline__ long long fixed56(unsigned long long b, int emax)
{
    const int ex = bexp(b);
    if (ex == 0 || emax == 0 || ex + 1078 - emax <= 0) return 0;
    return __double2ll_rn(__longlong_as_double((long long)(b + ((unsigned long long)(long long)(1078 - emax) << 52))));
}

// Balanced base-128 digits of X (|X| < 2^56), most significant first:
// X = sum_s d_s 2^(7(7-s)), d_0 in [-128, 128], d_1..d_7 in [-64, 63], each
// exact in BF16.  The low seven digits come from biasing X by 64 in every low
// digit position (B = 64 (2^49 - 1) / 127) and taking plain 7-bit chunks c
// of T = X + B, so each is c - 64; d_0 = floor(T / 2^49).
//
// digit_pair gives the digit words of two values: w[s] holds d_s of X0 in
// the low half and d_s of X1 in the high half (BF16 bits), the pairs the
// K-major shared-memory layout stores.  The low seven digits are built two
// at a time: both values' chunks are brought to bits 0..6 and 16..22 of one
// word (byte permutes and one shift), put into the mantissas of BF16 128.0
// (0x4300 | c = 128 + c, exact), and one BF16x2 subtraction of 192 gives
// c - 64 in both halves exactly; d_0 goes through an FP32 magic-number add.
__device__ __forceinline__ uint32_t chunk_pair_to_bf16(uint32_t p)
{
    const uint32_t v = (p & 0x007F007Fu) | 0x43004300u;
    __nv_bfloat162 x = *reinterpret_cast<const __nv_bfloat162 *>(&v);
    const uint32_t k192 = 0x43404340u;  // (192, 192)
    x = __hsub2(x, *reinterpret_cast<const __nv_bfloat162 *>(&k192));
    return *reinterpret_cast<const uint32_t *>(&x);
}

__device__ __forceinline__ void digit_pair(long long X0, long long X1, uint32_t (&w)[NS])
{
    const long long B = 64LL * (((1LL << 49) - 1) / 127);
    const long long T0 = X0 + B, T1 = X1 + B;
    const uint32_t lo0 = (uint32_t)T0, hi0 = (uint32_t)((unsigned long long)T0 >> 32);
    const uint32_t lo1 = (uint32_t)T1, hi1 = (uint32_t)((unsigned long long)T1 >> 32);
    // digit 0 in [-128, 128] through the FP32 path
    const float f0 = __int_as_float(0x4B400000 + (((int)hi0) >> 17)) - 12582912.0f;
    const float f1 = __int_as_float(0x4B400000 + (((int)hi1) >> 17)) - 12582912.0f;
    w[0] = __byte_perm(__float_as_uint(f0), __float_as_uint(f1), 0x7632);
    const uint32_t hl = __byte_perm(hi0, hi1, 0x5410);  // T bits 32..47 of each
    const uint32_t hm = __byte_perm(hi0, hi1, 0x6521);  // T bits 40..55
    w[1] = chunk_pair_to_bf16(hm >> 2);                 // T bits 42..48
    w[2] = chunk_pair_to_bf16(hl >> 3);                 // T bits 35..41
    w[3] = chunk_pair_to_bf16(__byte_perm(__funnelshift_r(lo0, hi0, 28), __funnelshift_r(lo1, hi1, 28), 0x5410));
    const uint32_t lh = __byte_perm(lo0, lo1, 0x7632);  // T bits 16..31
    const uint32_t lm = __byte_perm(lo0, lo1, 0x6521);  // T bits 8..23
    const uint32_t ll = __byte_perm(lo0, lo1, 0x5410);  // T bits 0..15
    w[4] = chunk_pair_to_bf16(lh >> 5);                 // T bits 21..27
    w[5] = chunk_pair_to_bf16(lm >> 6);                 // T bits 14..20
    w[6] = chunk_pair_to_bf16(ll >> 7);                 // T bits 7..13
    w[7] = chunk_pair_to_bf16(ll);                      // T bits 0..6
}

// P0 2^21 + P1 2^14 + P2 2^7 + P3 for four FP32 accumulator words holding
// exact integers |P_d| < 2^22.  P_d is the bit pattern of
// v + 1.5 * 2^23 minus that of 1.5 * 2^23 (0x4B400000); pairs are combined
// in 32 bits, P0 2^7 + P1 = f0 2^7 + f1 - 129 * 0x4B400000 (mod 2^32, exact
// since |P0 2^7 + P1| < 2^30), and only the final combination is 64-bit.
__device__ __forceinline__ long long combine4(uint32_t v0, uint32_t v1, uint32_t v2, uint32_t v3)
{
    const uint32_t f0 = __float_as_uint(__uint_as_float(v0) + 12582912.0f);
    const uint32_t f1 = __float_as_uint(__uint_as_float(v1) + 12582912.0f);
    const uint32_t f2 = __float_as_uint(__uint_as_float(v2) + 12582912.0f);
    const uint32_t f3 = __float_as_uint(__uint_as_float(v3) + 12582912.0f);
    const uint32_t off = 129u * 0x4B400000u;
    const int p01 = (int)(f0 * 128u + f1 - off);
    const int p23 = (int)(f2 * 128u + f3 - off);
    return (long long)p01 * 16384 + p23;
}

// Double of (hi * 2^28 + lo) * 2^sc (|hi|, |lo| < 2^43): J = hi * 2^19 +
// floor(lo / 2^9) fits in 63 bits and keeps every bit down to 2^-54 of the
// group scale (the digit truncation itself is 2^-56); J is rounded to 53
// bits to nearest by the int64 conversion, no FP64 arithmetic.
__device__ __forceinline__ double assemble_fast(long long hi, long long lo, int sc)
{
    const long long J = hi * (1LL << 19) + (lo >> 9);
    if (J == 0) return 0.0;
    // the int64 -> double conversion rounds J to 53 bits (nearest even); the
    // scale 2^(sc + 9) is then an exponent-field add
    const long long b = __double_as_longlong(__ll2double_rn(J));
    const int be = (int)((b >> 52) & 0x7FF) + sc + 9;
    const long long sign = b & (long long)0x8000000000000000ull;
    if (be <= 0) return __longlong_as_double(sign);
    if (be >= 2047) return __longlong_as_double(sign | 0x7FF0000000000000ll);
    return __longlong_as_double(b + ((long long)(sc + 9) << 52));
}

// The same value as assemble_fast, bit for bit, with the int64 -> double
// rounding done by integer instructions (no FP64-pipe conversion): |J| is
// normalised by its leading-zero count, rounded to 53 bits (nearest, ties to
// even) and placed in the exponent and fraction fields; a carry out of the
// rounding moves into the exponent field by itself.
__device__ __forceinline__ double assemble_int(long long hi, long long lo, int sc)
{
    const long long J = hi * (1LL << 19) + (lo >> 9);
    if (J == 0) return 0.0;
    const unsigned long long sign = (unsigned long long)J & 0x8000000000000000ull;
    unsigned long long a = J < 0 ? 0ull - (unsigned long long)J : (unsigned long long)J;
    const int lz = __clzll((long long)a);  // a < 2^63, so lz >= 1
    a <<= lz;
    unsigned long long mant = a >> 11;  // bit 52 set
    const unsigned rb = (unsigned)a & 0x7FFu;
    mant += (rb > 0x400u || (rb == 0x400u && (mant & 1ull))) ? 1ull : 0ull;
    // value = mant 2^(11 - lz) 2^(sc + 9); biased exponent of mant 2^-52 scaled
    const int be = 1023 + 72 - lz + sc;
    const int bec = be + (int)(mant >> 53);  // with the rounding carry
    if (bec <= 0) return __longlong_as_double((long long)sign);
    if (bec >= 2047) return __longlong_as_double((long long)(sign | 0x7FF0000000000000ull));
    // (be - 1) << 52 plus mant (whose bit 52 is the implicit one) is the
    // exponent and fraction field; a carry (mant = 2^53) lands in the exponent
    return __longlong_as_double((long long)(sign | ((((unsigned long long)(long long)(be - 1)) << 52) + mant)));
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
