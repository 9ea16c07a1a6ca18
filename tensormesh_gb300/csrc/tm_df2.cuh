// Double-float arithmetic on one or two lanes: a value is an unevaluated sum
// hi + lo of two floats (about 48 significant bits), and a "lane" type L is
// either float (one number) or float2 (two independent numbers, one per
// lane, computed with the paired FP32 instructions of sm_100 and later:
// __fadd2_rn, __fmul2_rn, __ffma2_rn perform the operation on both lanes in
// one issued instruction).  The error-free transformations are the
// classical ones (Knuth's TwoSum, Dekker's Fast2Sum, the FMA form of
// TwoProduct; Dekker 1971, Knuth TAOCP vol. 2 4.2.2, the double-float
// formulation of Hida, Li & Bailey's QD library); every step is an explicit
// round-to-nearest intrinsic, which the compiler does not contract.
//
// The P1 assembly kernels use float2 lanes to carry two elements per
// thread, or float lanes for one element per thread, and float2 lanes to
// accumulate a target's stiffness and mass sums side by side.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace tmk {

// ------------------------------------------------------------ lane primitives
__device__ __forceinline__ float l_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float l_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float l_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float l_neg(float a) { return -a; }
__device__ __forceinline__ float2 l_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 l_mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 l_fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// negation and subtraction on pairs as single paired instructions
// (multiplication by -1 is exact; fma(b, -1, a) rounds a - b once)
__device__ __forceinline__ float2 l_neg(float2 a) { return __fmul2_rn(a, make_float2(-1.0f, -1.0f)); }
__device__ __forceinline__ float l_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float2 l_sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a); }

template <class L> __device__ __forceinline__ L l_set(float v);
template <> __device__ __forceinline__ float l_set<float>(float v) { return v; }
template <> __device__ __forceinline__ float2 l_set<float2>(float v) { return make_float2(v, v); }

// lane access (k a compile-time constant after unrolling)
__device__ __forceinline__ float l_get(float v, int) { return v; }
__device__ __forceinline__ float l_get(float2 v, int k) { return k ? v.y : v.x; }
__device__ __forceinline__ void l_put(float& v, int, float x) { v = x; }
__device__ __forceinline__ void l_put(float2& v, int k, float x) {
    if (k)
        v.y = x;
    else
        v.x = x;
}

// hardware approximation of 1 / x (rcp.approx, relative error below 2^-22)
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float l_rcp(float x) { return rcp_approx(x); }
__device__ __forceinline__ float2 l_rcp(float2 x) { return make_float2(rcp_approx(x.x), rcp_approx(x.y)); }

// v with the sign flipped where s is negative
__device__ __forceinline__ float l_abs_sel(float v, float s) { return s < 0.0f ? -v : v; }
__device__ __forceinline__ float2 l_abs_sel(float2 v, float2 s) {
    return make_float2(s.x < 0.0f ? -v.x : v.x, s.y < 0.0f ? -v.y : v.y);
}

// ------------------------------------------------------------ double-float
template <class L>
struct ddv {
    L hi, lo;
};
using pf2 = ddv<float2>;

// s + e == a + b exactly, lane by lane (Knuth)
template <class L>
__device__ __forceinline__ ddv<L> p_two_sum(L a, L b) {
    const L s = l_add(a, b);
    const L bb = l_sub(s, a);
    const L e = l_add(l_sub(a, l_sub(s, bb)), l_sub(b, bb));
    return {s, e};
}

// s + e == a + b exactly when |a| >= |b| in each lane (Dekker)
template <class L>
__device__ __forceinline__ ddv<L> p_fast_two_sum(L a, L b) {
    const L s = l_add(a, b);
    const L e = l_sub(b, l_sub(s, a));
    return {s, e};
}

template <class L>
__device__ __forceinline__ ddv<L> p_neg(ddv<L> a) { return {l_neg(a.hi), l_neg(a.lo)}; }

template <class L>
__device__ __forceinline__ ddv<L> p_const(float hi, float lo) { return {l_set<L>(hi), l_set<L>(lo)}; }

template <class L>
__device__ __forceinline__ ddv<L> p_add(ddv<L> a, ddv<L> b) {
    const ddv<L> s = p_two_sum(a.hi, b.hi);
    const L e = l_add(s.lo, l_add(a.lo, b.lo));
    return p_fast_two_sum(s.hi, e);
}

template <class L>
__device__ __forceinline__ ddv<L> p_mul(ddv<L> a, ddv<L> b) {
    const L p = l_mul(a.hi, b.hi);
    L e = l_fma(a.hi, b.hi, l_neg(p));
    e = l_fma(a.hi, b.lo, e);
    e = l_fma(a.lo, b.hi, e);
    return p_fast_two_sum(p, e);
}

// a * b - c * d with one normalisation
template <class L>
__device__ __forceinline__ ddv<L> p_diff_of_products(ddv<L> a, ddv<L> b, ddv<L> c, ddv<L> d) {
    const L p = l_mul(a.hi, b.hi);
    const L pe = l_fma(a.hi, b.hi, l_neg(p));
    const L q = l_mul(c.hi, d.hi);
    const L qe = l_fma(c.hi, d.hi, l_neg(q));
    const ddv<L> s = p_two_sum(p, l_neg(q));
    L e = l_add(s.lo, l_sub(pe, qe));
    e = l_fma(a.hi, b.lo, e);
    e = l_fma(a.lo, b.hi, e);
    e = l_fma(l_neg(c.hi), d.lo, e);
    e = l_fma(l_neg(c.lo), d.hi, e);
    return p_fast_two_sum(s.hi, e);
}

// a0 b0 + a1 b1 + a2 b2 with one normalisation
template <class L>
__device__ __forceinline__ ddv<L> p_dot3(const ddv<L>* a, const ddv<L>* b) {
    const L p0 = l_mul(a[0].hi, b[0].hi), p1 = l_mul(a[1].hi, b[1].hi), p2 = l_mul(a[2].hi, b[2].hi);
    const L e0 = l_fma(a[0].hi, b[0].hi, l_neg(p0));
    const L e1 = l_fma(a[1].hi, b[1].hi, l_neg(p1));
    const L e2 = l_fma(a[2].hi, b[2].hi, l_neg(p2));
    const ddv<L> s01 = p_two_sum(p0, p1);
    const ddv<L> s = p_two_sum(s01.hi, p2);
    L e = l_add(l_add(s01.lo, s.lo), l_add(l_add(e0, e1), e2));
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        e = l_fma(a[k].hi, b[k].lo, e);
        e = l_fma(a[k].lo, b[k].hi, e);
    }
    return p_fast_two_sum(s.hi, e);
}

// a0 b0 + a1 b1 with one normalisation
template <class L>
__device__ __forceinline__ ddv<L> p_dot2(const ddv<L>* a, const ddv<L>* b) {
    const L p0 = l_mul(a[0].hi, b[0].hi), p1 = l_mul(a[1].hi, b[1].hi);
    const L e0 = l_fma(a[0].hi, b[0].hi, l_neg(p0));
    const L e1 = l_fma(a[1].hi, b[1].hi, l_neg(p1));
    const ddv<L> s = p_two_sum(p0, p1);
    L e = l_add(s.lo, l_add(e0, e1));
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        e = l_fma(a[k].hi, b[k].lo, e);
        e = l_fma(a[k].lo, b[k].hi, e);
    }
    return p_fast_two_sum(s.hi, e);
}

// 1 / a for a.hi > 0 normal: the hardware approximation, one Newton step in
// float (relative error about 2^-24), one in double-float, r + r (1 - a r):
// relative error of the result about 2^-47
template <class L>
__device__ __forceinline__ ddv<L> p_recip(ddv<L> a) {
    L r = l_rcp(a.hi);
    L e = l_fma(l_neg(a.hi), r, l_set<L>(1.0f));
    r = l_fma(r, e, r);
    e = l_fma(l_neg(a.hi), r, l_set<L>(1.0f));
    e = l_fma(l_neg(a.lo), r, e);
    return p_fast_two_sum(r, l_mul(r, e));
}

template <class L>
__device__ __forceinline__ ddv<L> p_abs(ddv<L> a) {
    return {l_abs_sel(a.hi, a.hi), l_abs_sel(a.lo, a.hi)};
}

// an unnormalised double-float accumulator per lane: s + e, every term's
// rounding error collected in e (TwoSum on the leading parts); the same
// steps, lane by lane, as the single-lane acc2 of the double-float header
template <class L>
struct dacc {
    L s, e;
};

// acc += a * b (a.lo * b.lo dropped: below 2^-96 of the product)
template <class L>
__device__ __forceinline__ void d_fma(dacc<L>& acc, ddv<L> a, ddv<L> b) {
    const L p = l_mul(a.hi, b.hi);
    const L pe = l_fma(a.hi, b.hi, l_neg(p));
    const ddv<L> t = p_two_sum(acc.s, p);
    L e = l_add(acc.e, l_add(t.lo, pe));
    e = l_fma(a.hi, b.lo, e);
    e = l_fma(a.lo, b.hi, e);
    acc.s = t.hi;
    acc.e = e;
}

// acc += a
template <class L>
__device__ __forceinline__ void d_add(dacc<L>& acc, ddv<L> a) {
    const ddv<L> t = p_two_sum(acc.s, a.hi);
    acc.s = t.hi;
    acc.e = l_add(acc.e, l_add(t.lo, a.lo));
}

template <class L>
__device__ __forceinline__ ddv<L> d_value(dacc<L> acc) { return p_fast_two_sum(acc.s, acc.e); }

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
