// Fixed-point cosine and sine in 64-bit integer arithmetic (sm_103a): GB300's FP64 pipe is its slow
// one, so the walks evaluate cos of a phase (the internal-field echo energy) and of k.dR (the PFGSE
// phase sums along a general direction) on the integer pipes.
//
//   1. An angle is held as a fraction of a turn, theta in units of 2^-64 turns plus two more bits g
//      (2^-65, 2^-66). From an FP64 angle x (turns_of): the 53-bit mantissa times 2^128 / (2 pi)
//      (two words) and the exponent's 66-bit window of that product -- the idea of Payne and Hanek's
//      reduction with a fixed window of the constant, enough for |x| < 2^40 -- error below 2^-66
//      turns. Angles that are integer combinations of known angles can be formed in turns directly
//      (the sum wraps modulo one turn), with no reduction at all.
//   2. k = theta rounded to 1/4096 turn, r = 2 pi (theta - k / 4096) with |r| <= pi / 4096.
//   3. cos / sin (k pi / 2048 + r) from the quadrant k / 1024, the table cos / sin (j pi / 2048),
//      j = k mod 1024 (shared memory, 16 KB), and cos r = 1 - r^2/2 + r^4/24,
//      sin r = r - r^3/6 + r^5/120 (the next terms are below 2^-71): r and r^2 in 64-bit fixed
//      point, the higher terms in 32-bit multiplies. Results are value * 2^62 as signed integers,
//      within 2.1 units of the exact values (cos_table.py's 256-bit arithmetic).
// The constants and the table are generated by cos_table.py in exact integer arithmetic.
#pragma once
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

namespace rwnmr
{
namespace fxcos
{
#include "cos_table.inc"

// Copies the quadrant table into shared memory (every thread of the block calls it; the caller
// synchronises before the first use).
__device__ __forceinline__ void load_quadrant_table(ulonglong2 *quad)
{
    for (int k = threadIdx.x; k < kQuadrant; k += blockDim.x)
        quad[k] = make_ulonglong2(kQuadrantCosSin[k][0], kQuadrantCosSin[k][1]);
}

// |x| / (2 pi) mod 1 as theta (2^-64 turns) and g (the next two bits); false for |x| >= 2^40, inf, nan.
__device__ __forceinline__ bool turns_of(double x, uint64_t &theta, uint32_t &g)
{
    const uint64_t bits = (uint64_t)__double_as_longlong(x);
    const int ex = (int)((bits >> 52) & 0x7ff);
    theta = 0;
    g = 0;
    if (ex >= 1063) return false;
    const int sh = 1139 - ex; // theta = (mantissa * 2^128 / (2 pi)) >> sh, modulo 2^64
    if (ex != 0 && sh < 178)
    {
        const uint64_t m = (bits & ((1ull << 52) - 1)) | (1ull << 52);
        const uint64_t lo2 = m * INV_2PI_HI;
        const uint64_t q1 = __umul64hi(m, INV_2PI_LO) + lo2;
        const uint64_t q2 = __umul64hi(m, INV_2PI_HI) + (q1 < lo2 ? 1 : 0);
        theta = sh < 128 ? (q1 >> (sh - 64)) | (q2 << (128 - sh)) : q2 >> (sh - 128);
        g = (uint32_t)(sh < 130 ? q1 >> (sh - 66) : q2 >> (sh - 130)) & 3u;
    }
    return true;
}

// The shared part of cos and sin of the angle (theta, g): the table entry pair, the quadrant, and
// cos r, sin r in fixed point.
struct TurnParts
{
    uint64_t C, S;    // cos, sin (j pi / 2048) * 2^63
    uint64_t dev;     // (1 - cos r) * 2^63
    uint64_t sr;      // |sin r| * 2^73
    int quadrant;     // 0..3
    bool neg_r;
};

__device__ __forceinline__ TurnParts turn_parts(uint64_t theta, uint32_t g, const ulonglong2 *__restrict__ quad)
{
    TurnParts t;
    const uint64_t tr = theta + (1ull << 51);
    const int k = (int)(tr >> 52);
    const long long d = (long long)(theta - (tr & ~((1ull << 52) - 1))) * 4 + g; // [-2^53, 2^53) 2^-66 turns
    t.neg_r = d < 0;
    const uint64_t a = (uint64_t)(t.neg_r ? -d : d);
    const uint64_t R = __umul64hi(a << 10, TWO_PI_Q61); // |r| 2^73
    const uint64_t u = __umul64hi(R, R);                // r^2 2^82
    const uint32_t u32 = (uint32_t)(u >> 31);           // r^2 2^51
    const uint32_t r32 = (uint32_t)(R >> 31);           // |r| 2^42
    const uint32_t hi3 = __umulhi(r32, u32);            // |r|^3 2^61
    // 1 - cos r = r^2/2 - r^4/24 (times 2^63), used as A cos r = A/2 - A (1 - cos r): two-term
    // differences only (the fused form 2^63 - x + t came out wrong on sm_103a when x = t = 0)
    t.dev = (u >> 20) - __umulhi(__umulhi(u32, u32), C_INV3072);
    t.sr = R - (((uint64_t)hi3 * C_INV6) >> 20) + __umulhi(__umulhi(hi3, u32), C_INV15360);
    const ulonglong2 cs = quad[k & (kQuadrant - 1)];
    t.C = cs.x;
    t.S = cs.y;
    t.quadrant = (k >> 10) & 3;
    return t;
}

// A cos r and A |sin r| at 2^62 for a table value A (2^63)
__device__ __forceinline__ long long mul_cos_r(uint64_t A, const TurnParts &t)
{
    return (long long)((A >> 1) - __umul64hi(A, t.dev));
}
__device__ __forceinline__ long long mul_sin_r(uint64_t A, const TurnParts &t)
{
    return (long long)((__umul64hi(A, t.sr) + 512) >> 10);
}

// cos(angle) * 2^62 for the angle (theta, g) in turns
__device__ __forceinline__ long long cos_turns_q62(uint64_t theta, uint32_t g, const ulonglong2 *__restrict__ quad)
{
    const TurnParts t = turn_parts(theta, g, quad);
    const bool odd = t.quadrant & 1;
    // quadrants 0..3: cos(phi), -sin(phi), -cos(phi), sin(phi) with phi = j pi / 2048 + r
    const long long p1 = mul_cos_r(odd ? t.S : t.C, t);
    const long long p2 = mul_sin_r(odd ? t.C : t.S, t);
    const long long v = odd == t.neg_r ? p1 - p2 : p1 + p2;
    return ((t.quadrant + 1) & 2) ? -v : v;
}

// cos and sin (angle) * 2^62 for the angle (theta, g) in turns
__device__ __forceinline__ void sincos_turns_q62(uint64_t theta, uint32_t g, const ulonglong2 *__restrict__ quad,
                                                 long long &c, long long &s)
{
    const TurnParts t = turn_parts(theta, g, quad);
    // cos(phi) = C cos r - S sin r, sin(phi) = S cos r + C sin r, sin r signed by neg_r
    const long long cc = mul_cos_r(t.C, t), sc = mul_cos_r(t.S, t);
    const long long cs = mul_sin_r(t.C, t), ss = mul_sin_r(t.S, t);
    const long long cphi = t.neg_r ? cc + ss : cc - ss;
    const long long sphi = t.neg_r ? sc - cs : sc + cs;
    // quadrant q: cos = cos(phi), -sin(phi), -cos(phi), sin(phi); sin = sin(phi), cos(phi), -sin(phi), -cos(phi)
    const bool odd = t.quadrant & 1, high = t.quadrant & 2;
    const long long c0 = odd ? sphi : cphi, s0 = odd ? cphi : sphi;
    c = (odd != high) ? -c0 : c0;
    s = high ? -s0 : s0;
}

// cos(x) * 2^62 for an FP64 angle; false (out untouched) for |x| >= 2^40 and non-finite x
__device__ __forceinline__ bool cos_q62(double x, const ulonglong2 *__restrict__ quad, long long &out)
{
    uint64_t theta;
    uint32_t g;
    if (!turns_of(x, theta, g)) return false;
    out = cos_turns_q62(theta, g, quad);
    return true;
}

// round(p * 2^63), half to even (the survival tables' rounding), for an FP64 probability p in
// [0, 1], from its bits.
__device__ __forceinline__ uint64_t prob_q63(double p)
{
    const uint64_t bits = (uint64_t)__double_as_longlong(p);
    const int ex = (int)((bits >> 52) & 0x7ff);
    if (ex < 959) return 0; // below 2^-64
    const uint64_t m = (bits & ((1ull << 52) - 1)) | (1ull << 52);
    const int sh = ex - 1012; // p 2^63 = m 2^(ex - 1075 + 63), sh <= 11
    if (sh >= 0) return m << sh;
    const int r = -sh; // 1 .. 53
    const uint64_t q = m >> r, rem = m & ((1ull << r) - 1), half = 1ull << (r - 1);
    return q + ((rem > half || (rem == half && (q & 1))) ? 1 : 0);
}

// Host: x / (2 pi) mod 1 in units of 2^-64 turns, rounded to nearest (x of either sign, |x| < 2^40;
// 0 for larger x), by the same product of the mantissa with 2^128 / (2 pi) as turns_of.
inline uint64_t turns_q64_host(double x)
{
    typedef unsigned __int128 u128;
    const double ax = x < 0 ? -x : x;
    uint64_t bits;
    std::memcpy(&bits, &ax, 8);
    const int ex = (int)(bits >> 52);
    if (ex == 0 || ex >= 1063) return 0; // zero and subnormals are below 2^-64 turns
    const int s = 1139 - ex - 66;        // the 66-bit window starts at bit s of (m K) >> 64; s >= 11
    if (s >= 128) return 0;
    const uint64_t m = (bits & ((1ull << 52) - 1)) | (1ull << 52);
    const u128 A = (u128)m * INV_2PI_LO, B = (u128)m * INV_2PI_HI;
    const u128 W = (A >> 64) + B; // (m K) >> 64, K = 2^128 / (2 pi)
    const u128 t66 = (W >> s) & (((u128)1 << 66) - 1);
    const uint64_t theta = (uint64_t)((t66 + 2) >> 2);
    return x < 0 ? 0 - theta : theta;
}
} // namespace fxcos
} // namespace rwnmr
