// Paired double-float arithmetic: two independent double-float numbers per
// thread, one in each lane of a float2, computed with the paired FP32
// instructions of sm_100 and later (__fadd2_rn, __fmul2_rn, __ffma2_rn: one
// issued instruction performs the operation on both lanes).  The error-free
// transformations are those of tm_df64.cuh (Knuth's TwoSum, Dekker's
// Fast2Sum, the FMA form of TwoProduct); every step is an explicit
// round-to-nearest paired intrinsic, which the compiler does not contract.
//
// The P1 assembly kernels carry two elements per thread through these
// operations (lane x: one element, lane y: the other) and accumulate a
// target's stiffness and mass sums in the two lanes of one pair, so that the
// double-float work, which bounds those kernels, issues half the
// instructions.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace tmk {

__device__ __forceinline__ float2 p_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 p_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 p_sub(float2 a, float2 b) { return __fadd2_rn(a, p_neg(b)); }
__device__ __forceinline__ float2 p_mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 p_fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 p_set(float v) { return make_float2(v, v); }

// two double-float numbers: (hi.x + lo.x, hi.y + lo.y)
struct pf2 {
    float2 hi, lo;
};

// s + e == a + b exactly, lane by lane (Knuth)
__device__ __forceinline__ pf2 p_two_sum(float2 a, float2 b) {
    const float2 s = p_add(a, b);
    const float2 bb = p_sub(s, a);
    const float2 e = p_add(p_sub(a, p_sub(s, bb)), p_sub(b, bb));
    return {s, e};
}

// s + e == a + b exactly when |a| >= |b| in each lane (Dekker)
__device__ __forceinline__ pf2 p_fast_two_sum(float2 a, float2 b) {
    const float2 s = p_add(a, b);
    const float2 e = p_sub(b, p_sub(s, a));
    return {s, e};
}

__device__ __forceinline__ pf2 p_neg(pf2 a) { return {p_neg(a.hi), p_neg(a.lo)}; }

__device__ __forceinline__ pf2 p_add(pf2 a, pf2 b) {
    const pf2 s = p_two_sum(a.hi, b.hi);
    const float2 e = p_add(s.lo, p_add(a.lo, b.lo));
    return p_fast_two_sum(s.hi, e);
}

__device__ __forceinline__ pf2 p_mul(pf2 a, pf2 b) {
    const float2 p = p_mul(a.hi, b.hi);
    float2 e = p_fma(a.hi, b.hi, p_neg(p));
    e = p_fma(a.hi, b.lo, e);
    e = p_fma(a.lo, b.hi, e);
    return p_fast_two_sum(p, e);
}

// a * b - c * d with one normalisation
__device__ __forceinline__ pf2 p_diff_of_products(pf2 a, pf2 b, pf2 c, pf2 d) {
    const float2 p = p_mul(a.hi, b.hi);
    const float2 pe = p_fma(a.hi, b.hi, p_neg(p));
    const float2 q = p_mul(c.hi, d.hi);
    const float2 qe = p_fma(c.hi, d.hi, p_neg(q));
    const pf2 s = p_two_sum(p, p_neg(q));
    float2 e = p_add(s.lo, p_sub(pe, qe));
    e = p_fma(a.hi, b.lo, e);
    e = p_fma(a.lo, b.hi, e);
    e = p_fma(p_neg(c.hi), d.lo, e);
    e = p_fma(p_neg(c.lo), d.hi, e);
    return p_fast_two_sum(s.hi, e);
}

// a0 b0 + a1 b1 + a2 b2 with one normalisation
__device__ __forceinline__ pf2 p_dot3(const pf2* a, const pf2* b) {
    const float2 p0 = p_mul(a[0].hi, b[0].hi), p1 = p_mul(a[1].hi, b[1].hi), p2 = p_mul(a[2].hi, b[2].hi);
    const float2 e0 = p_fma(a[0].hi, b[0].hi, p_neg(p0));
    const float2 e1 = p_fma(a[1].hi, b[1].hi, p_neg(p1));
    const float2 e2 = p_fma(a[2].hi, b[2].hi, p_neg(p2));
    const pf2 s01 = p_two_sum(p0, p1);
    const pf2 s = p_two_sum(s01.hi, p2);
    float2 e = p_add(p_add(s01.lo, s.lo), p_add(p_add(e0, e1), e2));
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        e = p_fma(a[k].hi, b[k].lo, e);
        e = p_fma(a[k].lo, b[k].hi, e);
    }
    return p_fast_two_sum(s.hi, e);
}

// a0 b0 + a1 b1 with one normalisation
__device__ __forceinline__ pf2 p_dot2(const pf2* a, const pf2* b) {
    const float2 p0 = p_mul(a[0].hi, b[0].hi), p1 = p_mul(a[1].hi, b[1].hi);
    const float2 e0 = p_fma(a[0].hi, b[0].hi, p_neg(p0));
    const float2 e1 = p_fma(a[1].hi, b[1].hi, p_neg(p1));
    const pf2 s = p_two_sum(p0, p1);
    float2 e = p_add(s.lo, p_add(e0, e1));
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        e = p_fma(a[k].hi, b[k].lo, e);
        e = p_fma(a[k].lo, b[k].hi, e);
    }
    return p_fast_two_sum(s.hi, e);
}

// 1 / a for a.hi > 0 normal: the hardware approximation of 1 / a.hi
// (rcp.approx, relative error below 2^-22), one Newton step in float that
// brings it to about 2^-24, and one in double-float, r + r (1 - a r): the
// relative error of the result is about 2^-47
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ pf2 p_recip(pf2 a) {
    float2 r = make_float2(rcp_approx(a.hi.x), rcp_approx(a.hi.y));
    float2 e = p_fma(p_neg(a.hi), r, p_set(1.0f));
    r = p_fma(r, e, r);
    e = p_fma(p_neg(a.hi), r, p_set(1.0f));       // 1 - a.hi r: exact up to the FMA's rounding of a tiny value
    e = p_fma(p_neg(a.lo), r, e);
    return p_fast_two_sum(r, p_mul(r, e));
}

__device__ __forceinline__ pf2 p_abs(pf2 a) {
    const bool nx = a.hi.x < 0.0f, ny = a.hi.y < 0.0f;
    return {make_float2(nx ? -a.hi.x : a.hi.x, ny ? -a.hi.y : a.hi.y),
            make_float2(nx ? -a.lo.x : a.lo.x, ny ? -a.lo.y : a.lo.y)};
}

// ------------------------------------------------------------ conversions
// double -> hi + lo on the integer pipe, without branches.  hi is x
// truncated to 24 significant bits, lo the remaining 29 bits rounded to 24
// (|x - hi - lo| <= 2^-47 |x|; hi and lo have the sign of x).  Valid for
// 2^-75 <= |x| < 2^128; smaller values give (0, 0), an absolute error below
// 2^-75 (callers check that their data's scale lies far above it and below
// the upper limit).
__device__ __forceinline__ void split_to_pair(double x, float& hi, float& lo) {
    const uint32_t H = (uint32_t)__double2hiint(x), L = (uint32_t)__double2loint(x);
    const uint32_t t = H - (896u << 20);                               // float exponent bias
    const uint32_t hb = __funnelshift_l(L, t, 3) | (H & 0x80000000u);  // sign, exponent, 23 bits
    const uint32_t pw = (hb & 0xFF800000u) - (52u << 23);              // +-2^(e - 52): lo's unit
    const float l = __uint2float_rn(L & 0x1FFFFFFFu) * __uint_as_float(pw);
    const bool tiny = (H & 0x7FFFFFFFu) < (949u << 20);               // |x| < 2^-74
    hi = tiny ? 0.0f : __uint_as_float(hb);
    lo = tiny ? 0.0f : l;
}

// float -> double, exact, on the integer pipe (normal floats and zero)
__device__ __forceinline__ double widen(float f) {
    const uint32_t b = __float_as_uint(f);
    const uint32_t hw = (((b >> 3) & 0x0FFFFFFFu) + (896u << 20)) | (b & 0x80000000u);
    const bool zero = (b & 0x7FFFFFFFu) == 0;
    return __hiloint2double((int)(zero ? (b & 0x80000000u) : hw), (int)(zero ? 0u : (b << 29)));
}

// the nearest double to hi + lo (one FP64 add)
__device__ __forceinline__ double pair_to_double(float hi, float lo) { return widen(hi) + widen(lo); }

}  // namespace tmk
