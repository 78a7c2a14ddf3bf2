// Float-float arithmetic: a value is the unevaluated sum h + l of two floats
// with |l| <= ulp(h) / 2, about 48 significant bits, evaluated on the FP32
// pipes (on GB300 FP64 issues at 2 operations per clock per SM against 128 for
// FP32).  The building blocks are the published error-free transformations:
// Knuth's TwoSum, Dekker's Fast2Sum (quick_two_sum) and the FMA-based exact
// product; the compound operations follow the usual "sloppy" double-word
// forms (Dekker 1971; Hida, Li and Bailey's QD library paper, 2001), whose
// relative error is a few 2^-48 except under cancellation, where it is a few
// 2^-48 of the operands' magnitude.
#pragma once

#include <cuda_runtime.h>

namespace nlgpu {

struct ff {
    float h, l;
};

__device__ __forceinline__ ff ff_make(float h, float l = 0.0f) { return ff{h, l}; }

// nearest float-float of a double (exact for doubles with <= 48 significant bits)
__device__ __forceinline__ ff ff_from(double x) {
    const float h = __double2float_rn(x);
    return ff{h, __double2float_rn(x - double(h))};
}

__device__ __forceinline__ double ff_to(ff a) { return double(a.h) + double(a.l); }

// s + e = a + b exactly (any a, b)
__device__ __forceinline__ ff two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return ff{s, e};
}

// s + e = a + b exactly when |a| >= |b|
__device__ __forceinline__ ff quick_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return ff{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ ff ff_add(ff a, ff b) {
    const ff s = two_sum(a.h, b.h);
    return quick_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}

__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.h, -a.l}; }

__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }

__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return quick_two_sum(p, e);
}

// a * b for a float b
__device__ __forceinline__ ff ff_mul_f(ff a, float b) {
    const float p = __fmul_rn(a.h, b);
    const float e = __fmaf_rn(a.l, b, __fmaf_rn(a.h, b, -p));
    return quick_two_sum(p, e);
}

// acc + a * b
__device__ __forceinline__ ff ff_fma(ff acc, ff a, ff b) { return ff_add(acc, ff_mul(a, b)); }

__device__ __forceinline__ bool ff_lt(ff a, float b) { return a.h < b || (a.h == b && a.l < 0.0f); }
__device__ __forceinline__ ff ff_abs(ff a) { return a.h < 0.0f ? ff_neg(a) : a; }

// x^n, n >= 0, by repeated squaring
__device__ __forceinline__ ff ff_ipow(ff x, int n) {
    ff r = ff_make(1.0f);
    while (n > 0) {
        if (n & 1) { r = ff_mul(r, x); --n; } else { x = ff_mul(x, x); n >>= 1; }
    }
    return r;
}

// Compensated dot product of float-float operands (the Dot2 scheme of Ogita,
// Rump and Oishi, 2005, with float-float inputs): each product's high part
// goes into a running float sum through TwoSum, and every rounding error --
// the product's (FMA-exact, with the two cross terms of the low parts) and the
// sum's -- into one float compensation, folded in once at the end.  12
// FP32 operations per term instead of the 17 of a renormalised float-float
// multiply-add; the result is as accurate as float-float arithmetic (errors
// of order n^2 2^-48 of the terms' magnitudes).
struct ffdot {
    float s = 0.0f, c = 0.0f;
};

__device__ __forceinline__ void ffdot_add(ffdot& acc, ff a, ff b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    const ff t = two_sum(acc.s, p);
    acc.s = t.h;
    acc.c = __fadd_rn(acc.c, __fadd_rn(t.l, e));
}

__device__ __forceinline__ ff ffdot_value(const ffdot& acc) { return quick_two_sum(acc.s, acc.c); }

// exp(k / 64) for k = -FF_EXP_K .. FF_EXP_K as float-float pairs, filled on the
// host (exp of a double, split hi = float(x), lo = float(x - hi))
constexpr int FF_EXP_K = 23;
struct FFExpTable {
    float2 v[2 * FF_EXP_K + 1];
};

// exp(t) for t <= 0 from the mathematics of the exponential: t = m ln2 + f with
// |f| <= ln2 / 2, f = k / 64 + g with |g| <= 1/128, exp(f) = exp(k / 64) exp(g)
// with exp(k / 64) from the table and exp(g) by its Taylor series through g^6
// (remainder below 4e-19), every step in float-float.  Results below 1e-37
// are flushed to zero.  ln2 and 1/k! are split into two floats each.
__device__ __forceinline__ ff ff_exp_nonpositive(ff t, const ff* table) {
    if (t.h < -85.0f) return ff_make(0.0f);
    const ff ln2{0.6931471824645996f, -1.9046542121259336e-09f};
    const float m = rintf(t.h * 1.4426950216293335f);
    const ff f = ff_sub(t, ff_mul_f(ln2, m));
    const float k = rintf(f.h * 64.0f);
    const ff g = ff_sub(f, ff_make(k * 0.015625f));
    const ff inv_fact[7] = {{1.0f, 0.0f},
                            {1.0f, 0.0f},
                            {0.5f, 0.0f},
                            {0.1666666716337204f, -4.967053879312289e-09f},
                            {0.0416666679084301f, -1.2417634698280722e-09f},
                            {0.008333333767950535f, -4.34617203337595e-10f},
                            {0.0013888889225199819f, -3.3631094437103215e-11f}};
    ff p = inv_fact[6];
#pragma unroll
    for (int j = 5; j >= 0; --j) p = ff_add(ff_mul(p, g), inv_fact[j]);
    const int ki = min(FF_EXP_K, max(-FF_EXP_K, int(k)));
    p = ff_mul(p, table[ki + FF_EXP_K]);
    const int e = int(m);
    return ff{ldexpf(p.h, e), ldexpf(p.l, e)};
}

}  // namespace nlgpu
