// Float-float evaluation of the double-precision sub-expressions of the cut
// arithmetic, with a rounding test and a double-precision fallback.
//
// The reference computes many float results through double intermediates
// (unqualified sqrt/atan2/sin on promoted floats, double constants); the
// device reproduces them exactly.  GB300 runs FP64 at a small fraction of its
// FP32 rate, so each such result is first evaluated here in float-float
// arithmetic (pairs hi + lo of floats, about 44 significant bits) together
// with a bound on its distance to the value the double evaluation produces.
// If no float rounding boundary lies within that bound, the float the double
// evaluation rounds to is known: it is returned.  Otherwise (a fraction of
// about 2^-15 of the inputs) the caller evaluates the expression in double as
// before.  The results are therefore identical to the double evaluation's.
//
// sincos_ff is out of line: one copy shared by the sine and the cosine keeps
// the mini-doublet kernel's code within the instruction caches.
//
// Published methods used: Dekker's and Knuth's error-free transformations
// (TwoSum, FastTwoSum, TwoProd via fused multiply-add), Dekker's double-length
// division and square root, argument reduction of atan by a 33-entry table of
// atan(k/32) and its Taylor series on |u| <= 1/64, and Ziv's rounding test.
// Table and constants were computed with mpmath at 200 bits.
#pragma once

namespace sdlg {
namespace ffm {

struct ff {
    float hi, lo;
};

__device__ __forceinline__ ff two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}
// |a| >= |b| or a == 0
__device__ __forceinline__ ff fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ ff two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ ff neg(ff a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ ff fabs_ff(ff a) { return a.hi < 0.f ? neg(a) : a; }
__device__ __forceinline__ ff add(ff a, ff b) {
    ff s = two_sum(a.hi, b.hi);
    const ff t = two_sum(a.lo, b.lo);
    s.lo = __fadd_rn(s.lo, t.hi);
    s = fast_two_sum(s.hi, s.lo);
    s.lo = __fadd_rn(s.lo, t.lo);
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ ff add(ff a, float b) {
    ff s = two_sum(a.hi, b);
    s.lo = __fadd_rn(s.lo, a.lo);
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ ff sub(ff a, ff b) { return add(a, neg(b)); }
__device__ __forceinline__ ff mul(ff a, ff b) {
    ff p = two_prod(a.hi, b.hi);
    p.lo = __fadd_rn(p.lo, __fadd_rn(__fmul_rn(a.hi, b.lo), __fmul_rn(a.lo, b.hi)));
    return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ ff mul(ff a, float b) {
    ff p = two_prod(a.hi, b);
    p.lo = __fadd_rn(p.lo, __fmul_rn(a.lo, b));
    return fast_two_sum(p.hi, p.lo);
}
// a / b (b.hi != 0): relative error below 2^-44
__device__ __forceinline__ ff div(ff a, ff b) {
    const float q1 = __fdiv_rn(a.hi, b.hi);
    const ff r = sub(a, mul(b, q1));
    const float q2 = __fdiv_rn(r.hi, b.hi);
    return fast_two_sum(q1, q2);
}
// sqrt(a) (a.hi > 0, normal): relative error below 2^-45
__device__ __forceinline__ ff sqrt_ff(ff a) {
    const float s0 = __fsqrt_rn(a.hi);
    const ff p = two_prod(s0, s0);
    const float r = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p.hi), p.lo), a.lo);
    return fast_two_sum(s0, __fdiv_rn(r, __fmul_rn(2.f, s0)));
}

// Ziv's rounding test.  If every real number within err of v rounds to the
// same float, store it in out and return true.  Zero, subnormal, very small,
// very large and non-finite values return false.
__device__ __forceinline__ bool round_unique(ff v, float err, float& out) {
    const float r = __fadd_rn(v.hi, v.lo);
    const uint32_t ur = __float_as_uint(r) & 0x7fffffffu;
    const uint32_t e = ur >> 23;
    if (e < 40u || e > 215u) return false;
    float h = __uint_as_float((e - 24u) << 23);  // half an ulp of r
    if ((ur & 0x7fffffu) == 0u) h = __fmul_rn(h, 0.5f);  // below a power of two the gap halves
    // v - r (hi - r is exact; the sum and the test below round by at most
    // 2^-24 relative, which the factor on h covers)
    const float d = __fadd_rn(__fsub_rn(v.hi, r), v.lo);
    if (!(__fadd_rn(fabsf(d), err) < __fmul_rn(0.99999f, h))) return false;
    out = r;
    return true;
}
// the same with err = |v| * 2^-40 (results with relative error below 2^-42)
__device__ __forceinline__ bool round_unique_rel(ff v, float& out) {
    return round_unique(v, __fmul_rn(fabsf(v.hi), 0x1p-40f), out);
}

// atan(k/32), k = 0..32, as hi + lo
__device__ constexpr float kAtanTabHi[33] = {
    0x0.0p+0f, 0x1.ffd55cp-6f, 0x1.ff55bcp-5f, 0x1.7ee182p-4f, 0x1.fd5baap-4f, 0x1.3d6eeep-3f, 0x1.7b97b4p-3f,
    0x1.b90d76p-3f, 0x1.f5b760p-3f, 0x1.18bf5ap-2f, 0x1.362774p-2f, 0x1.530adap-2f, 0x1.6f6194p-2f, 0x1.8b24d4p-2f,
    0x1.a64eecp-2f, 0x1.c0db4cp-2f, 0x1.dac670p-2f, 0x1.f40dd0p-2f, 0x1.0657eap-1f, 0x1.1255dap-1f, 0x1.1e00bap-1f,
    0x1.2958e6p-1f, 0x1.345f02p-1f, 0x1.3f13fcp-1f, 0x1.4978fap-1f, 0x1.538f58p-1f, 0x1.5d5898p-1f, 0x1.66d664p-1f,
    0x1.700a7cp-1f, 0x1.78f6bcp-1f, 0x1.819d0cp-1f, 0x1.89ff60p-1f, 0x1.921fb6p-1f};
__device__ constexpr float kAtanTabLo[33] = {
    0x0.0p+0f, -0x1.15a276p-32f, -0x1.1a6042p-30f, 0x1.80bc44p-30f, -0x1.54f424p-30f, 0x1.18cc4ep-28f,
    0x1.79cb60p-28f, -0x1.adb3ecp-28f, -0x1.b4dfc8p-29f, 0x1.85f8bcp-29f, -0x1.1f0286p-27f, -0x1.ab8caep-28f,
    0x1.e4def0p-30f, -0x1.ad7936p-28f, 0x1.e611fep-29f, 0x1.29d93ep-27f, 0x1.586ed4p-28f, 0x1.6a8282p-27f,
    -0x1.6499e6p-26f, -0x1.010b56p-27f, 0x1.7bdfd6p-26f, -0x1.b3dc74p-27f, -0x1.98e422p-28f, -0x1.d85a42p-27f,
    0x1.934f70p-28f, -0x1.1dbe78p-27f, 0x1.c5a6c6p-27f, -0x1.b707dep-27f, 0x1.5e118cp-27f, -0x1.516750p-28f,
    -0x1.1d4eb6p-26f, -0x1.501c10p-30f, -0x1.777a5cp-26f};
__device__ constexpr ff kPiFF = {0x1.921fb6p+1f, -0x1.777a5cp-24f};
__device__ constexpr ff kPi2FF = {0x1.921fb6p+0f, -0x1.777a5cp-25f};
__device__ constexpr ff kThirdFF = {0x1.555556p-2f, -0x1.555556p-27f};

// atan(u) for |u| <= 1/64 + 2^-20: u + u P(u^2), P = -u^2/3 + u^4/5 - u^6/7 + u^8/9;
// the truncation error is below |u| u^10/11 < |u| 2^-63, the rounding error
// below |u| 2^-44
__device__ __forceinline__ ff atan_small(ff u) {
    const ff u2 = add(two_prod(u.hi, u.hi), __fmul_rn(__fmul_rn(2.f, u.hi), u.lo));
    const float z = u2.hi;
    const float tail = __fmul_rn(__fmul_rn(z, z), __fsub_rn(0.2f, __fmul_rn(z, __fsub_rn(0x1.24924ap-3f, __fmul_rn(z, 0x1.c71c72p-4f)))));
    const ff p = add(neg(mul(u2, kThirdFF)), tail);
    return add(u, mul(u, p));
}

// atan(t) for t >= 0 (t.hi normal, below 2^60): relative error below 2^-42
__device__ __forceinline__ ff atan_ff(ff t) {
    const bool inv = t.hi > 1.f;
    if (inv) t = div(ff{1.f, 0.f}, t);
    const int k = __float2int_rn(__fmul_rn(t.hi, 32.f));  // 0..32
    const float c = __fmul_rn((float)k, 0.03125f);
    const ff num = add(t, -c);
    const ff den = add(mul(t, c), 1.f);
    const ff a = add(ff{kAtanTabHi[k], kAtanTabLo[k]}, atan_small(div(num, den)));
    return inv ? sub(kPi2FF, a) : a;
}

// atan2(y, x) for nonzero, normal x and y with |y/x| and |x/y| above 2^-60:
// relative error below 2^-42.  Returns false when the arguments are outside
// that range.
__device__ __forceinline__ bool atan2_ff(ff y, ff x, ff& out) {
    const float ax = fabsf(x.hi), ay = fabsf(y.hi);
    if (!(ax > 0x1p-60f && ax < 0x1p60f && ay > 0x1p-60f && ay < 0x1p60f)) return false;
    const bool swap = ay > ax;
    const ff t = swap ? div(fabs_ff(x), fabs_ff(y)) : div(fabs_ff(y), fabs_ff(x));
    if (!(t.hi > 0x1p-60f)) return false;
    ff a = atan_ff(t);
    if (swap) a = sub(kPi2FF, a);
    if (x.hi < 0.f) a = sub(kPiFF, a);
    if (y.hi < 0.f) a = neg(a);
    out = a;
    return true;
}

// asin(x) for 0 < |x| <= 0.95 as atan(x / sqrt(1 - x^2)): relative error below 2^-42
__device__ __forceinline__ ff asin_ff(float x) {
    const ff w = add(neg(two_prod(x, x)), 1.f);
    const ff t = div(ff{fabsf(x), 0.f}, sqrt_ff(w));
    const ff a = atan_ff(t);
    return x < 0.f ? neg(a) : a;
}

// sin(x) for |x| <= 0.8: x + x P(x^2) with the Taylor series to x^13 (the
// truncation error is below |x| 2^-45); the x^2..x^6 terms in float-float,
// the rest in float.  Relative error below 2^-42.
__device__ __forceinline__ ff sin_small_ff(float x) {
    const ff x2 = two_prod(x, x);
    const float z = x2.hi;
    const float t = __fadd_rn(0x1.71de3ap-19f, __fmul_rn(z, __fsub_rn(__fmul_rn(z, 0x1.612462p-33f), 0x1.ae6456p-26f)));
    ff h = add(ff{-0x1.a01a02p-13f, 0x1.7f97fap-39f}, __fmul_rn(z, t));
    h = add(ff{0x1.111112p-7f, -0x1.dddddep-32f}, mul(x2, h));
    h = add(ff{-0x1.555556p-3f, 0x1.555556p-28f}, mul(x2, h));
    return add(mul(mul(x2, h), x), x);
}

// cos(x) for |x| <= 0.8: Taylor series to x^14 (truncation below 2^-49),
// the x^2..x^8 terms in float-float.  Relative error below 2^-43.
__device__ __forceinline__ ff cos_small_ff(float x) {
    const ff x2 = two_prod(x, x);
    const float z = x2.hi;
    const float t = __fsub_rn(__fmul_rn(z, __fsub_rn(0x1.1eed8ep-29f, __fmul_rn(z, 0x1.93974ap-37f))), 0x1.27e4fcp-22f);
    ff h = add(ff{0x1.a01a02p-16f, -0x1.7f97fap-42f}, __fmul_rn(z, t));
    h = add(ff{-0x1.6c16c2p-10f, 0x1.27d27ep-35f}, mul(x2, h));
    h = add(ff{0x1.555556p-5f, -0x1.555556p-30f}, mul(x2, h));
    h = add(ff{-0.5f, 0.f}, mul(x2, h));
    return add(mul(x2, h), 1.f);
}

// sin(x) (cosine: shift = 1) for |x| <= 8: x = r + k pi/2 with pi/2 split in
// three parts (the first two with at most 20 significant bits, so k times
// them is exact; the split is 2e-21 off), then the series on |r| <= pi/4.
// Relative error below 2^-42; false when |r| < 2^-16 after a reduction
// (a result near a zero of the function).
static __device__ __noinline__ bool sincos_ff(float x, int shift, ff& out) {
    if (!(fabsf(x) <= 8.f)) return false;
    const int k = __float2int_rn(__fmul_rn(x, 0x1.45f306p-1f));
    ff s, c;
    if (k == 0) {
        if (shift == 0) {
            out = sin_small_ff(x);
            return true;
        }
        s = sin_small_ff(x);
        c = cos_small_ff(x);
    } else {
        const float fk = (float)k;
        const float r1 = __fsub_rn(x, __fmul_rn(fk, 0x1.921fc0p+0f));
        ff r = two_sum(r1, -__fmul_rn(fk, -0x1.5777a0p-21f));
        r = add(r, -__fmul_rn(fk, -0x1.73dcb4p-43f));
        if (!(fabsf(r.hi) > 0x1p-16f)) return false;
        const ff s0 = sin_small_ff(r.hi), c0 = cos_small_ff(r.hi);
        s = add(s0, __fmul_rn(c0.hi, r.lo));  // sin(hi + lo) = sin hi + lo cos hi + O(lo^2)
        c = add(c0, -__fmul_rn(s0.hi, r.lo));
    }
    switch ((k + shift) & 3) {
        case 0: out = s; break;
        case 1: out = c; break;
        case 2: out = neg(s); break;
        default: out = neg(c);
    }
    return true;
}

}  // namespace ffm
}  // namespace sdlg
