// Double-float ("df64") arithmetic on the FP32 pipes.
//
// GB300 executes FP64 at 1/62 of its FP32 rate (1.25 vs 77.7 TFLOP/s FMA,
// measured), so the P1 assembly kernels carry their arithmetic as unevaluated
// sums hi + lo of two floats (about 48 significant bits) built from the
// classical error-free transformations: Knuth's TwoSum, Dekker's Fast2Sum and
// the FMA form of TwoProduct (Dekker 1971; Knuth, TAOCP vol. 2, 4.2.2; the
// double-float formulation of Hida, Li & Bailey's QD library and of Thall,
// "Extended-precision floating-point numbers for GPU computation", 2006).
// Every step uses the _rn intrinsics so that the compiler cannot fuse a
// product and a sum into an FMA, which would break the error terms.
//
// Conversions between double and df64 are done on the integer pipe by
// moving exponent and mantissa bits, so that no FP64 instruction is issued
// for them.  They are valid for normal numbers in the float exponent range;
// callers check the range (exponent_in_band) and fall back to FP64 code
// outside it.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace tmk {

struct f2 {
    float hi, lo;
};

__device__ __forceinline__ f2 f2_make(float h, float l) { return {h, l}; }

// s + e == a + b exactly (Knuth)
__device__ __forceinline__ f2 two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

// s + e == a + b exactly when |a| >= |b| (Dekker)
__device__ __forceinline__ f2 fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float e = __fsub_rn(b, __fsub_rn(s, a));
    return {s, e};
}

// p + e == a * b exactly (FMA)
__device__ __forceinline__ f2 two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    const float e = __fmaf_rn(a, b, -p);
    return {p, e};
}

__device__ __forceinline__ f2 f2_neg(f2 a) { return {-a.hi, -a.lo}; }

__device__ __forceinline__ f2 f2_add(f2 a, f2 b) {
    const f2 s = two_sum(a.hi, b.hi);
    const float e = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
    return fast_two_sum(s.hi, e);
}

__device__ __forceinline__ f2 f2_sub(f2 a, f2 b) { return f2_add(a, f2_neg(b)); }

__device__ __forceinline__ f2 f2_mul(f2 a, f2 b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return fast_two_sum(p, e);
}

// a * b - c * d with one normalisation
__device__ __forceinline__ f2 f2_diff_of_products(f2 a, f2 b, f2 c, f2 d) {
    const f2 p = two_prod(a.hi, b.hi);
    const f2 q = two_prod(c.hi, d.hi);
    const f2 s = two_sum(p.hi, -q.hi);
    float e = __fadd_rn(s.lo, __fsub_rn(p.lo, q.lo));
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    e = __fmaf_rn(-c.hi, d.lo, e);
    e = __fmaf_rn(-c.lo, d.hi, e);
    return fast_two_sum(s.hi, e);
}

// a0*b0 + a1*b1 + a2*b2 with one normalisation
__device__ __forceinline__ f2 f2_dot3(const f2* a, const f2* b) {
    const f2 p0 = two_prod(a[0].hi, b[0].hi);
    const f2 p1 = two_prod(a[1].hi, b[1].hi);
    const f2 p2 = two_prod(a[2].hi, b[2].hi);
    const f2 s01 = two_sum(p0.hi, p1.hi);
    const f2 s = two_sum(s01.hi, p2.hi);
    float e = __fadd_rn(__fadd_rn(s01.lo, s.lo), __fadd_rn(__fadd_rn(p0.lo, p1.lo), p2.lo));
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        e = __fmaf_rn(a[k].hi, b[k].lo, e);
        e = __fmaf_rn(a[k].lo, b[k].hi, e);
    }
    return fast_two_sum(s.hi, e);
}

__device__ __forceinline__ f2 f2_dot2(const f2* a, const f2* b) {
    const f2 p0 = two_prod(a[0].hi, b[0].hi);
    const f2 p1 = two_prod(a[1].hi, b[1].hi);
    const f2 s = two_sum(p0.hi, p1.hi);
    float e = __fadd_rn(s.lo, __fadd_rn(p0.lo, p1.lo));
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        e = __fmaf_rn(a[k].hi, b[k].lo, e);
        e = __fmaf_rn(a[k].lo, b[k].hi, e);
    }
    return fast_two_sum(s.hi, e);
}

// 1 / a: correctly rounded float reciprocal of a.hi refined by one Newton
// step r1 = r0 + r0 (1 - a r0) evaluated in double-float
__device__ __forceinline__ f2 f2_recip(f2 a) {
    const float r0 = __frcp_rn(a.hi);
    const f2 p = two_prod(a.hi, r0);                  // a.hi * r0 = 1 - small
    float e = __fsub_rn(1.0f, p.hi);                  // exact (Sterbenz)
    e = __fsub_rn(e, p.lo);
    e = __fmaf_rn(-a.lo, r0, e);
    return fast_two_sum(r0, __fmul_rn(r0, e));
}

__device__ __forceinline__ f2 f2_abs(f2 a) { return a.hi < 0.0f ? f2_neg(a) : a; }

__device__ __forceinline__ bool f2_finite(f2 a) { return isfinite(a.hi) && isfinite(a.lo); }

// |a.hi| in [2^lo_exp, 2^hi_exp) or a == 0: the range in which every
// error term of the kernels' products stays a normal float
__device__ __forceinline__ bool f2_in_band(f2 a, int lo_exp, int hi_exp) {
    const uint32_t b = __float_as_uint(a.hi) & 0x7FFFFFFFu;
    if (b == 0) return true;
    const int e = (int)(b >> 23) - 127;
    return e >= lo_exp && e < hi_exp;
}

// biased double exponent of x (0 for zero and subnormals)
__device__ __forceinline__ int biased_exponent(double x) {
    return (int)(((uint64_t)__double_as_longlong(x) >> 52) & 0x7FF);
}

// |x| in [2^-band, 2^band] or x == +-0
__device__ __forceinline__ bool exponent_in_band(double x, int band) {
    const uint64_t u = (uint64_t)__double_as_longlong(x);
    if ((u << 1) == 0) return true;
    const int e = (int)((u >> 52) & 0x7FF) - 1023;
    return e >= -band && e < band;
}

// double -> hi + lo (both truncated toward zero, |x - hi - lo| < 2^-47 |x|
// + 2^-126), on the integer pipe.  Values below 2^-126 become 0 and bits of
// lo below 2^-126 are dropped; |x| must be below 2^128 (callers check the
// scale of their data with exponent_in_band / biased_exponent).
__device__ __forceinline__ f2 split_double(double x) {
    const uint64_t u = (uint64_t)__double_as_longlong(x);
    const int e = (int)((u >> 52) & 0x7FF);
    if (e < 1023 - 126) return {0.0f, 0.0f};          // |x| < 2^-126: below float range, kept as 0
    const uint32_t sign = (uint32_t)(u >> 32) & 0x80000000u;
    const uint64_t m = u & 0xFFFFFFFFFFFFFull;
    const uint32_t hib = sign | ((uint32_t)(e - 1023 + 127) << 23) | (uint32_t)(m >> 29);
    const uint32_t rem = (uint32_t)(m & 0x1FFFFFFFu);
    float lo = 0.0f;
    if (rem != 0) {
        const int lz = __clz(rem);                    // >= 3
        const int p = 31 - lz;                        // leading one of rem
        const int le = p + e - 1075 + 127;            // float exponent of lo
        if (le > 0) {
            const uint32_t mant = (uint32_t)(rem << (lz + 1)) >> 9;
            lo = __uint_as_float(sign | ((uint32_t)le << 23) | mant);
        }
    }
    return {__uint_as_float(hib), lo};
}

// x * 2^-s as hi + lo (split_double of the scaled value); the exponent is
// moved on the integer pipe, so that the scaling is exact, and a scaled
// value below the double range becomes 0.  The caller picks s so that
// |x| 2^-s < 1.
__device__ __forceinline__ f2 split_scaled(double x, int s) {
    const uint64_t u = (uint64_t)__double_as_longlong(x);
    const int e = (int)((u >> 52) & 0x7FF);
    const int ne = e - s;
    if (e == 0 || ne <= 0) return {0.0f, 0.0f};
    const uint64_t v = (u & ~(0x7FFull << 52)) | ((uint64_t)ne << 52);
    return split_double(__longlong_as_double((long long)v));
}

// 2^k as a float, k in [-126, 127]
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((k + 127) << 23); }

// an unnormalised double-float accumulator: s + e, where every term's
// rounding error is collected in e (TwoSum on the leading parts)
struct acc2 {
    float s, e;
};

// acc += a * b for double-float a, b (a.lo * b.lo dropped: below 2^-96)
__device__ __forceinline__ void acc_fma(acc2& acc, f2 a, f2 b) {
    const f2 p = two_prod(a.hi, b.hi);
    const f2 t = two_sum(acc.s, p.hi);
    float e = __fadd_rn(acc.e, __fadd_rn(t.lo, p.lo));
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    acc.s = t.hi;
    acc.e = e;
}

// acc += a for double-float a
__device__ __forceinline__ void acc_add(acc2& acc, f2 a) {
    const f2 t = two_sum(acc.s, a.hi);
    acc.s = t.hi;
    acc.e = __fadd_rn(acc.e, __fadd_rn(t.lo, a.lo));
}

__device__ __forceinline__ f2 acc_value(acc2 acc) { return fast_two_sum(acc.s, acc.e); }

// float -> double, exact, on the integer pipe (normal floats and zero)
__device__ __forceinline__ double float_to_double(float f) {
    const uint32_t b = __float_as_uint(f);
    const uint32_t e = (b >> 23) & 0xFF;
    if (e == 0) return __longlong_as_double((long long)((uint64_t)(b & 0x80000000u) << 32));
    if (e == 255) return (double)f;                   // inf / nan (not produced on the checked path)
    const uint32_t hiw = (b & 0x80000000u) | ((e - 127 + 1023) << 20) | ((b & 0x7FFFFFu) >> 3);
    const uint64_t u = ((uint64_t)hiw << 32) | ((uint64_t)(b & 7u) << 29);
    return __longlong_as_double((long long)u);
}

// nearest double to hi + lo (one FP64 add)
__device__ __forceinline__ double f2_to_double(f2 a) {
    return float_to_double(a.hi) + float_to_double(a.lo);
}

}  // namespace tmk
