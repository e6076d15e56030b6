// Device-side building blocks shared by the sweep, trial and rebuild kernels.
//
// Number formats (why they are what they are):
//  * Positions are 64-bit fixed point per axis, X = x/L * 2^64 (two's
//    complement). Periodic wrapping (Cuboid::boundary, geometry.h:539-547) is
//    integer overflow, the minimum image (Cuboid::vdist, geometry.h:519-537)
//    is a 32-bit integer difference of the high words, and k.r phases for
//    k = 2*pi*n/L are exact integers (n.X mod 2^32 turns).
//  * Per-pair and per-k terms are FP32. The per-move sums, Q(k), the running
//    energy and the Metropolis threshold use "df" numbers: an unevaluated sum
//    hi + lo of two floats updated with error-free transformations (Knuth's
//    TwoSum, Dekker's FastTwoSum), giving ~48 significant bits. GB300 issues
//    FP64 at a small fraction of its FP32 rate, so the per-move loop carries no
//    FP64 instruction at all; FP64 appears only when values are exported.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace fg {

// 2*pi / 2^32: radians per unit of a 32-bit turn fraction
__device__ __constant__ static const float kRadPerTurnUnit = 1.46291807926715968e-09f;

struct df {
    float hi, lo;
};

// Knuth TwoSum: s + e == a + b exactly.
__device__ __forceinline__ df two_sum(float a, float b) {
    float s = __fadd_rn(a, b);
    float bp = __fsub_rn(s, a);
    float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
    return {s, e};
}
// Dekker FastTwoSum (|a| >= |b|).
__device__ __forceinline__ df fast_two_sum(float a, float b) {
    float s = __fadd_rn(a, b);
    float e = __fsub_rn(b, __fsub_rn(s, a));
    return {s, e};
}
__device__ __forceinline__ df df_add(df a, df b) {
    df s = two_sum(a.hi, b.hi);
    df t = two_sum(a.lo, b.lo);
    s.lo = __fadd_rn(s.lo, t.hi);
    s = fast_two_sum(s.hi, s.lo);
    s.lo = __fadd_rn(s.lo, t.lo);
    return fast_two_sum(s.hi, s.lo);
}
// a + b with one TwoSum on the high parts (the low parts added plainly):
// fewer dependent steps than df_add, relative error ~2^-44 when a and b do
// not nearly cancel.
__device__ __forceinline__ df df_add_quick(df a, df b) {
    df s = two_sum(a.hi, b.hi);
    s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_add_f(df a, float b) {
    df s = two_sum(a.hi, b);
    s.lo = __fadd_rn(s.lo, a.lo);
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_neg(df a) { return {-a.hi, -a.lo}; }
// a > b for df numbers (both finite or hi infinite)
__device__ __forceinline__ bool df_gt(df a, df b) {
    if (a.hi != b.hi) return a.hi > b.hi;
    return a.lo > b.lo;
}

// Warp-wide df sum (all lanes get the result).
__device__ __forceinline__ df warp_sum_df(df v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        df w;
        w.hi = __shfl_xor_sync(0xffffffffu, v.hi, o);
        w.lo = __shfl_xor_sync(0xffffffffu, v.lo, o);
        v = df_add(v, w);
    }
    return v;
}

// int64 -> float through two 32-bit conversions (the 64-bit conversion runs
// on the FP64 pipe): hi * 2^32 + lo, one FMA rounding.
__device__ __forceinline__ float i64_to_float(long long v) {
    return fmaf((float)(int)(v >> 32), 4294967296.0f, (float)(unsigned)v);
}

// Fixed point helpers ------------------------------------------------------
// High 32 bits of a 64-bit coordinate, rounded to nearest.
__device__ __forceinline__ int32_t hi32(int64_t X) {
    return (int32_t)((uint64_t)(X + 0x80000000LL) >> 32);
}

// cos/sin of 2*pi*ph/2^32 for an exact 32-bit turn fraction `ph`.
// Table of cos/sin at multiples of 2*pi/256 (in shared memory) times a short
// Taylor polynomial of the remainder angle |d| <= pi/256 (truncation < 1e-11).
__device__ __forceinline__ float2 sincos_turns(uint32_t ph, const float2 *__restrict__ tab) {
    const uint32_t i = (ph + (1u << 23)) >> 24;
    // rem = ph - i 2^24 in [-2^23, 2^23) is the sign-extended low 24 bits of
    // ph; h = floor(rem / 2) enters the mantissa of 1.5 2^23 (|h| <= 2^22),
    // so the angle is one FMA with no conversion. Folding the magic constant
    // into the FMA shifts every angle by the same < 2e-9 rad: a global phase
    // of all e^{ik.r}, which no energy (|Q|^2, Re conj(Q) D) can see.
    const int32_t h = (int32_t)(ph << 8) >> 9;
    const float d = fmaf(__int_as_float(0x4B400000 + h), 2.0f * kRadPerTurnUnit,
                         -12582912.0f * (2.0f * kRadPerTurnUnit));
    float d2 = d * d;
    float s = fmaf(d2 * (-1.0f / 6.0f), d, d);
    float c = fmaf(d2, fmaf(d2, 1.0f / 24.0f, -0.5f), 1.0f);
    float2 t = tab[i & 255u];
    return make_float2(t.x * c - t.y * s, t.x * s + t.y * c);
}

// e^{i phi} - 1 = (cos phi - 1, sin phi) with error relative to |phi|, from
// the Taylor series of sin and of 1 - cos in Horner form on the coefficients
// +-1/n! (one FMA per term); valid for |phi| <= 1.6 rad (next terms < 1e-9).
__device__ __forceinline__ float2 expm1_i_horner(float phi) {
    const float p2 = phi * phi;
    float s = fmaf(p2, 1.6059043836821613e-10f, -2.5052108385441720e-08f);
    s = fmaf(p2, s, 2.7557319223985893e-06f);
    s = fmaf(p2, s, -1.9841269841269841e-04f);
    s = fmaf(p2, s, 8.3333333333333333e-03f);
    s = fmaf(p2, s, -1.6666666666666667e-01f);
    s = fmaf(p2 * phi, s, phi);                         // sin(phi)
    float c = fmaf(p2, 1.1470745597729725e-11f, -2.0876756987868099e-09f);
    c = fmaf(p2, c, 2.7557319223985891e-07f);
    c = fmaf(p2, c, -2.4801587301587302e-05f);
    c = fmaf(p2, c, 1.3888888888888889e-03f);
    c = fmaf(p2, c, -4.1666666666666667e-02f);
    c = fmaf(p2, c, 0.5f);
    return make_float2(-(p2 * c), s);                   // (cos - 1, sin)
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Small integers to float without the conversion pipe (|n| < 2^22).
__device__ __forceinline__ float small_int_to_float(int n) {
    return __int_as_float(0x4B400000 + n) - 12582912.0f;
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw: "Parallel random numbers: as
// easy as 1, 2, 3", SC'11), the published round function and key schedule.
struct u4 {
    uint32_t x, y, z, w;
};
__host__ __device__ __forceinline__ u4 philox4x32_10(u4 c, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; r++) {
        uint64_t p0 = (uint64_t)M0 * c.x;
        uint64_t p1 = (uint64_t)M1 * c.z;
        u4 n;
        n.x = (uint32_t)(p1 >> 32) ^ c.y ^ k0;
        n.y = (uint32_t)p1;
        n.z = (uint32_t)(p0 >> 32) ^ c.w ^ k1;
        n.w = (uint32_t)p0;
        c = n;
        k0 += W0;
        k1 += W1;
    }
    return c;
}

}  // namespace fg
