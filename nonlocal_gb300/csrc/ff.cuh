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

// 8-byte aligned, so that a float-float moves as one 64-bit access wherever it
// lives (a 4-byte aligned array of them, after a 4-byte shared variable, gave
// misaligned 64-bit shared-memory loads)
struct __align__(8) ff {
    float h, l;
};

__device__ __forceinline__ ff ff_make(float h, float l = 0.0f) { return ff{h, l}; }

// nearest float-float of a double (exact for doubles with <= 48 significant bits)
__device__ __forceinline__ ff ff_from(double x) {
    const float h = __double2float_rn(x);
    return ff{h, __double2float_rn(x - double(h))};
}

__device__ __forceinline__ double ff_to(ff a) { return double(a.h) + double(a.l); }

// float-float of a double by integer operations only (no FP64 instruction):
// h = the double truncated to 24 significant bits, l = the remaining 29 bits
// rounded to a float, so h + l carries about 48 bits; |x| outside
// [2^-100, 2^127] gives (0, 0) (or h = +-inf for a too large or non-finite x)
__device__ __forceinline__ ff ff_split(double x) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
    const unsigned sign = unsigned(b >> 32) & 0x80000000u;
    const int e = int((b >> 52) & 0x7ff) - 1023;
    if (e < -100) return ff{0.0f, 0.0f};
    if (e > 127) return ff{__uint_as_float(sign | 0x7f800000u), 0.0f};
    const unsigned long long mant = b & 0xfffffffffffffull;
    const float h = __uint_as_float(sign | (unsigned(e + 127) << 23) | unsigned(mant >> 29));
    const unsigned rest = unsigned(mant & 0x1fffffffull);   // 29 bits below h's last
    // rest * 2^(e - 52), e - 52 in [-152, 75]: below 2^-126 the power of two is
    // built as 2^(e - 52 + 64) * 2^-64
    const int s = e - 52;
    const float r = __uint2float_rn(rest);
    const float l = s >= -126 ? __fmul_rn(r, __uint_as_float(unsigned(s + 127) << 23))
                              : __fmul_rn(__fmul_rn(r, __uint_as_float(unsigned(s + 64 + 127) << 23)), 5.421010862427522e-20f);
    return ff{h, sign ? -l : l};
}

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

// exp(k / 256) for k = -FF_EXP_K .. FF_EXP_K as float-float pairs, filled on
// the host (exp of a double, split hi = float(x), lo = float(x - hi))
constexpr int FF_EXP_K = 89;
constexpr float FF_EXP_STEPS = 256.0f;
struct FFExpTable {
    float2 v[2 * FF_EXP_K + 1];
};

// exp(t) for t <= 0 from the mathematics of the exponential:
//   t = m ln2 + f, |f| <= ln2 / 2 (ln2 split into two floats);
//   f = k / 256 + g, |g| <= 1/512 (f.h - k/256 is exact by Sterbenz's lemma);
//   exp(f) = exp(k / 256) exp(g), exp(k / 256) from the table and
//   exp(g) = 1 + g + g^2/2 + g^3 (1/6 + g/24 + g^2/120) + O(g^6),
// the first three terms in float-float (g^2 by the FMA exact product), the
// bracket in FP32: its term is below 2^-27 and needs only 2^-21 relative
// accuracy for a result good to about 2^-48, and the omitted g^6 / 720 is
// below 2^-63.  The scaling by 2^m builds the power of two from its exponent
// bits (m >= -123 here).  Results below 1e-37 are flushed to zero.
__device__ __forceinline__ ff ff_exp_nonpositive(ff t, const ff* table) {
    if (t.h < -85.0f) return ff_make(0.0f);
    const ff ln2{0.6931471824645996f, -1.9046542121259336e-09f};
    const float m = rintf(t.h * 1.4426950216293335f);
    const ff f = ff_sub(t, ff_mul_f(ln2, m));
    const float k = rintf(f.h * FF_EXP_STEPS);
    const ff g = quick_two_sum(__fsub_rn(f.h, k * (1.0f / FF_EXP_STEPS)), f.l);
    const float p2 = __fmul_rn(g.h, g.h);
    const float e2 = __fmaf_rn(2.0f * g.h, g.l, __fmaf_rn(g.h, g.h, -p2));   // g^2 = p2 + e2
    const float q = __fmul_rn(__fmul_rn(p2, g.h),
                              __fmaf_rn(g.h, __fmaf_rn(g.h, 0.008333333767950535f, 0.0416666679084301f),
                                        0.1666666716337204f));
    const float low = __fadd_rn(__fadd_rn(g.l, 0.5f * e2), q);
    const ff u = quick_two_sum(g.h, 0.5f * p2);       // |g| >= g^2 / 2
    const ff v = quick_two_sum(1.0f, u.h);
    ff p = quick_two_sum(v.h, __fadd_rn(v.l, __fadd_rn(u.l, low)));
    const int ki = min(FF_EXP_K, max(-FF_EXP_K, int(k)));
    p = ff_mul(p, table[ki + FF_EXP_K]);
    const float scale = __int_as_float((127 + int(m)) << 23);
    return ff{__fmul_rn(p.h, scale), __fmul_rn(p.l, scale)};
}

}  // namespace nlgpu
