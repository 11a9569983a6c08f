// Device-side arithmetic of the segment-linking cuts for sm_103a.
//
// Every function keeps the reference's precision and operation order so that
// the object sets match the reference CPU chain exactly:
//  * the reference's unqualified sqrt/sin/tan/cos/atan2/pow/fabs/copysign are
//    the double overloads (evaluated here in double);
//  * its std::asin/atan/sin/cos/tan on floats are float functions; here they
//    are evaluated in double and rounded once to float, i.e. correctly
//    rounded, which is what the host library returns for all but a small
//    fraction of inputs;
//  * pow(x, 2) of a float is exact in double and is written x*x;
//  * the integer abs of a truncated float (MiniDoublet.cc:273,787,
//    Segment.cc:743-744) uses x86-64 truncation semantics (out of range and
//    NaN give INT_MIN);
//  * the library is compiled with -fmad=false so nothing is contracted.
#pragma once
#include <cstdint>

#include "sdl_ffmath.cuh"

namespace sdlg {

constexpr double kPi = 3.14159265358979323846;
constexpr float kSdlInf = 123456789.0f;  // MiniDoublet.cc:3 compared as float (123456792)

enum : uint8_t { kEndcap = 4, kBarrel = 5 };
enum : uint8_t { kNegZ = 1, kPosZ = 2, kCenter = 3 };
enum : uint8_t { kPS = 0, kTwoS = 1 };
enum : uint8_t { kPixel = 0, kStrip = 1 };

// Decoded module plus the geometry-table values the cuts read, one entry per
// sensor module (Module.cc:159-358, TiltedGeometry.cc:43-51,
// EndcapGeometry.cc:63-101, MiniDoublet.cc:1260-1332).
struct ModDev {
    uint32_t detid;
    int32_t partner;     // module index of the partner sensor, -1 if unknown
    uint8_t subdet, side, layer, ring;
    uint8_t rod, module, lower, inverted;
    uint8_t type, ltype, layer_slot, pad;  // layer_slot: 0..5 barrel, 6..10 endcap
    float gap;           // moduleGapSize of this module
    float drdz_s;        // tilted drdz of the strip sensor of the pair
    float slope_s;       // strip-direction slope of the strip sensor of the pair
    float edge_x, edge_y;  // (float)(2.5*cos(phi_c)), (float)(2.5*sin(phi_c)) of this sensor
    float tilt;          // (float)((double)(0.5f*pitchPS*drdz_s) / sqrt((double)(1.f + drdz_s*drdz_s)) / (double)gap)
    // the module-only terms of the strip shift (MiniDoublet.cc:1260-1332),
    // from the host's float functions when the module table is built: angleB
    // ((float)(pi / 2) for endcap modules, else atanf(drdz_s)) and the sine
    // and cosine of angleM for the four quadrants of the anchoring hit (x > 0
    // and y > 0; x > 0 and y < 0; x < 0 and y < 0; any other)
    float sh_angle_b;
    float sh_sin[4], sh_cos[4];
};

// ------------------------------------------------------------------ math
// The double-precision math routines are kept out of line: one copy of each
// in the binary instead of one per call site keeps the cut kernels small
// enough for the instruction caches.
static __device__ __noinline__ float f_asin_d(float x) { return (float)asin((double)x); }
static __device__ __noinline__ float f_atan_d(float x) { return (float)atan((double)x); }
static __device__ __noinline__ float f_sin_d(float x) { return (float)sin((double)x); }
static __device__ __noinline__ float f_cos_d(float x) { return (float)cos((double)x); }
static __device__ __noinline__ float f_tan(float x) { return (float)tan((double)x); }
static __device__ __noinline__ double d_sin(double x) { return sin(x); }
__device__ __forceinline__ float fmin_ref(float a, float b) { return (b < a) ? b : a; }  // std::min
__device__ __forceinline__ float fmax_ref(float a, float b) { return (a < b) ? b : a; }  // std::max
__device__ __forceinline__ int trunc_i32(float f) {
    if (!(f > -2147483649.0f && f < 2147483648.0f)) return (int)0x80000000;
    return __float2int_rz(f);
}
__device__ __forceinline__ int iabs(int v) { return v < 0 ? (int)(0u - (unsigned)v) : v; }
__device__ __forceinline__ float f_copysign(float a, float b) { return copysignf(a, b); }

// Each function below returns the float the double evaluation gives: the
// float-float evaluation of sdl_ffmath.cuh when its rounding is certain, the
// double evaluation otherwise.

// (float)asin((double)x) (std::asin of a float)
__device__ __forceinline__ bool f_asin_fast(float x, float& r) {
    if (x == 0.f) {
        r = x;
        return true;
    }
    return fabsf(x) <= 0.95f && ffm::round_unique_rel(ffm::asin_ff(x), r);
}
static __device__ __noinline__ float f_asin(float x) {
    float r;
    return f_asin_fast(x, r) ? r : f_asin_d(x);
}

// (float)atan((double)x), (float)sin((double)x), (float)cos((double)x)
__device__ __forceinline__ bool f_atan_fast(float x, float& r) {
    if (x == 0.f) {
        r = x;
        return true;
    }
    const float ax = fabsf(x);
    if (!(ax > 0x1p-60f && ax < 0x1p60f)) return false;
    const ffm::ff a = ffm::atan_ff(ffm::ff{ax, 0.f});
    return ffm::round_unique_rel(x < 0.f ? ffm::neg(a) : a, r);
}
static __device__ __noinline__ float f_atan(float x) {
    float r;
    return f_atan_fast(x, r) ? r : f_atan_d(x);
}
__device__ __forceinline__ bool f_sincos_fast(float x, int shift, float& r) {
    if (shift == 0 && x == 0.f) {
        r = x;
        return true;
    }
    if (!(fabsf(x) > 0x1p-60f)) return false;
    ffm::ff v;
    return ffm::sincos_ff(x, shift, v) && ffm::round_unique_rel(v, r);
}
// (float)tan((double)x) and (float)(tan((double)x) / (double)x), the hits'
// tan of their asin angle (0 < x <= asin(0.95)): sine over cosine in
// float-float (relative error below 2^-41), answered when the rounding is
// unique; the double evaluation otherwise
static __device__ __noinline__ float f_tan_over_d(float x) { return (float)(tan((double)x) / (double)x); }
__device__ __forceinline__ bool f_tan_fast(float x, bool over_x, float& r) {
    if (!(x > 0x1p-30f && x < 1.5f)) return false;
    ffm::ff s, c;
    if (!ffm::sincos_ff(x, 0, s) || !ffm::sincos_ff(x, 1, c)) return false;
    ffm::ff t = ffm::div(s, c);
    if (over_x) t = ffm::div(t, ffm::ff{x, 0.f});
    return ffm::round_unique_rel(t, r);
}
static __device__ __noinline__ float f_tan_ff(float x) {
    float r;
    return f_tan_fast(x, false, r) ? r : f_tan(x);
}
static __device__ __noinline__ float f_tan_over(float x) {
    float r;
    return f_tan_fast(x, true, r) ? r : f_tan_over_d(x);
}
static __device__ __noinline__ float f_sin(float x) {
    float r;
    return f_sincos_fast(x, 0, r) ? r : f_sin_d(x);
}
static __device__ __noinline__ float f_cos(float x) {
    float r;
    return f_sincos_fast(x, 1, r) ? r : f_cos_d(x);
}

// ------------------------------------------------------------------ host libm
// The reference's std::asin/atan/sin/cos/tan on floats are the host libm's
// float functions (glibc's asinf, atanf, sinf, cosf, tanf), which are not
// correctly rounded: on glibc 2.39 they differ from the correctly rounded
// value on 0.4-3 % of the floats, always by one float step, and the cut
// decisions see it.  The host library tabulates, for every |x| bit pattern
// in [lo, lo + n), whether its float function returns the correctly rounded
// value of |x| (code 0), the next float up (1), the next float down (2) or a
// value kept in a sorted exception list (3); outside [lo, lo + n) it returns
// the correctly rounded value (checked on every float of each function's
// domain by the library's self-check).  The functions are odd (asin, atan,
// sin, tan) or even (cos) in the host libm as well, so |x| indexes the table.
struct LibmTab {
    const uint32_t* code;   // 2 bits per float, 16 per word
    const uint32_t* exc_x;  // exceptions: |x| bit patterns (sorted) and their values
    const float* exc_v;
    uint32_t lo, n, n_exc, pad;
};
enum { kLmAsin = 0, kLmAtan, kLmSin, kLmCos, kLmTan, kLmCount };
static __constant__ LibmTab c_libm[kLmCount];

// The table word of |x| (ax) is loaded first and the correctly rounded value
// computed while the load is in flight (the float-float paths are inlined;
// only their rare double fallbacks are calls); libm_pick then moves the value.
struct LibmWord {
    uint32_t w, k;
    bool in;
};
__device__ __forceinline__ LibmWord libm_word(int fn, float ax) {
    const LibmTab& t = c_libm[fn];
    LibmWord r;
    r.k = __float_as_uint(ax) - t.lo;
    r.in = r.k < t.n;
    r.w = r.in ? __ldg(t.code + (r.k >> 4)) : 0u;
    return r;
}
// the host libm's value for |x| (ax), given the correctly rounded value r of ax
static __device__ __noinline__ float libm_exception(int fn, float ax, float r) {
    const LibmTab& t = c_libm[fn];
    const uint32_t u = __float_as_uint(ax);
    uint32_t a = 0, b = t.n_exc;
    while (a < b) {
        const uint32_t m = (a + b) >> 1;
        if (__ldg(t.exc_x + m) < u) a = m + 1;
        else b = m;
    }
    return (a < t.n_exc && __ldg(t.exc_x + a) == u) ? __ldg(t.exc_v + a) : r;
}
__device__ __forceinline__ float libm_pick(int fn, LibmWord lw, float ax, float r) {
    if (!lw.in) return r;
    const uint32_t c = (lw.w >> ((lw.k & 15u) * 2u)) & 3u;
    if (c == 1u) return nextafterf(r, INFINITY);
    if (c == 2u) return nextafterf(r, -INFINITY);
    if (c == 3u) return libm_exception(fn, ax, r);
    return r;
}
// std::asin, std::atan, std::sin, std::tan (odd) and std::cos (even) of a
// float, as the host libm computes them
static __device__ __noinline__ float g_asin(float x) {
    const float ax = fabsf(x);
    const LibmWord lw = libm_word(kLmAsin, ax);
    float r;
    if (!f_asin_fast(ax, r)) r = f_asin_d(ax);
    r = libm_pick(kLmAsin, lw, ax, r);
    return x < 0.f ? -r : r;
}
static __device__ __noinline__ float g_atan(float x) {
    const float ax = fabsf(x);
    const LibmWord lw = libm_word(kLmAtan, ax);
    float r;
    if (!f_atan_fast(ax, r)) r = f_atan_d(ax);
    r = libm_pick(kLmAtan, lw, ax, r);
    return x < 0.f ? -r : r;
}
static __device__ __noinline__ float g_sin(float x) {
    const float ax = fabsf(x);
    const LibmWord lw = libm_word(kLmSin, ax);
    float r;
    if (!f_sincos_fast(ax, 0, r)) r = f_sin_d(ax);
    r = libm_pick(kLmSin, lw, ax, r);
    return x < 0.f ? -r : r;
}
static __device__ __noinline__ float g_cos(float x) {
    const float ax = fabsf(x);
    const LibmWord lw = libm_word(kLmCos, ax);
    float r;
    if (!f_sincos_fast(ax, 1, r)) r = f_cos_d(ax);
    return libm_pick(kLmCos, lw, ax, r);
}
static __device__ __noinline__ float g_tan(float x) {
    const float ax = fabsf(x);
    const LibmWord lw = libm_word(kLmTan, ax);
    float r;
    if (!f_tan_fast(ax, false, r)) r = f_tan(ax);
    r = libm_pick(kLmTan, lw, ax, r);
    return x < 0.f ? -r : r;
}


// (float)sqrt((double)a*a + (double)b*b)
static __device__ __noinline__ float hypot_d(float a, float b) {
    const double da = a, db = b;
    return (float)sqrt(da * da + db * db);
}
__device__ __forceinline__ bool hypot_fast(float a, float b, float& r) {
    const float m = fmaxf(fabsf(a), fabsf(b));
    if (!(m > 0x1p-50f && m < 0x1p50f)) return false;
    return ffm::round_unique_rel(ffm::sqrt_ff(ffm::add(ffm::two_prod(a, a), ffm::two_prod(b, b))), r);
}
static __device__ __noinline__ float hypot_ref(float a, float b) {
    float r;
    return hypot_fast(a, b, r) ? r : hypot_d(a, b);
}
// (float)((double)a * 15.0 / (double)b): the product is exact in double
static __device__ __noinline__ float times15_over_d(float a, float b) { return (float)((double)a * 15.0 / (double)b); }
__device__ __forceinline__ bool times15_over_fast(float a, float b, float& r) {
    if (!(fabsf(a) > 0x1p-60f && fabsf(a) < 0x1p60f && fabsf(b) > 0x1p-60f && fabsf(b) < 0x1p60f)) return false;
    return ffm::round_unique_rel(ffm::div(ffm::two_prod(a, 15.f), ffm::ff{b, 0.f}), r);
}
static __device__ __noinline__ float times15_over(float a, float b) {
    float r;
    return times15_over_fast(a, b, r) ? r : times15_over_d(a, b);
}

// (float)((double)num / sin((double)beta)), the tracklets' pT from a turning angle
static __device__ __noinline__ float pt_from_d(float num, float beta) { return (float)((double)num / d_sin((double)beta)); }
__device__ __forceinline__ bool pt_from_fast(float num, float beta, float& r) {
    const float ab = fabsf(beta);
    if (!(ab > 0x1p-30f && ab <= 0.8f && fabsf(num) > 0x1p-60f && fabsf(num) < 0x1p60f)) return false;
    return ffm::round_unique_rel(ffm::div(ffm::ff{num, 0.f}, ffm::sin_small_ff(beta)), r);
}
static __device__ __noinline__ float pt_from(float num, float beta) {
    float r;
    return pt_from_fast(num, beta, r) ? r : pt_from_d(num, beta);
}

// Tracklet.cc multiple-scattering factor
// (float)((double)0.015f * sqrt((double)0.1f + 0.2 * (double)d / (double)50.f) [* sqrt((double)q)])
static __device__ __noinline__ float muls_d(float d, float q, bool two) {
    const double m = (double)0.015f * sqrt((double)0.1f + 0.2 * (double)d / (double)50.f);
    return two ? (float)(m * sqrt((double)q)) : (float)m;
}
__device__ __forceinline__ bool muls_fast(float d, float q, bool two, float& r) {
    if (!(d >= 0.f && d < 1e4f)) return false;  // no cancellation in 0.1 + 0.004 d
    if (two && !(q > 0x1p-60f && q < 0x1p60f)) return false;
    // the double 0.2 as hi + lo is 5.6e-17 off
    const ffm::ff t = ffm::div(ffm::mul(ffm::ff{0x1.99999ap-3f, -0x1.99999ap-29f}, d), ffm::ff{50.f, 0.f});
    ffm::ff m = ffm::mul(ffm::sqrt_ff(ffm::add(t, 0.1f)), 0.015f);
    if (two) m = ffm::mul(m, ffm::sqrt_ff(ffm::ff{q, 0.f}));
    return ffm::round_unique_rel(m, r);
}
static __device__ __noinline__ float muls(float d, float q, bool two) {
    float r;
    return muls_fast(d, q, two, r) ? r : muls_d(d, q, two);
}
// muls(d, S.lr3z / rtIn, true) with sqrt(S.lr3z / rtIn) precomputed for the
// inner segment S (sg_pack_record: the same sqrt_ff, NaN outside muls_fast's
// range of the quotient); the same arithmetic as muls_fast
__device__ __forceinline__ bool muls_fast_sq(float d, float sqh, float sql, float& r) {
    if (!(d >= 0.f && d < 1e4f)) return false;
    if (!(sqh > 0.f)) return false;  // NaN: the quotient is outside the fast path's range
    const ffm::ff t = ffm::div(ffm::mul(ffm::ff{0x1.99999ap-3f, -0x1.99999ap-29f}, d), ffm::ff{50.f, 0.f});
    ffm::ff m = ffm::mul(ffm::sqrt_ff(ffm::add(t, 0.1f)), 0.015f);
    m = ffm::mul(m, ffm::ff{sqh, sql});
    return ffm::round_unique_rel(m, r);
}
static __device__ __noinline__ float muls_sq(float d, float sqh, float sql, float lr3z, float rtIn) {
    float r;
    return muls_fast_sq(d, sqh, sql, r) ? r : muls_d(d, lr3z / rtIn, true);
}

// (float)((double)head + 0.25 * ((double)t * (double)t)): the square is exact in double
static __device__ __noinline__ float add_quarter_sq_d(float head, float t) {
    const double dt = t;
    return (float)((double)head + 0.25 * (dt * dt));
}
__device__ __forceinline__ bool add_quarter_sq_fast(float head, float t, float& r) {
    if (!(fabsf(t) < 0x1p50f && fabsf(head) < 0x1p100f)) return false;
    const ffm::ff q = ffm::two_prod(t, t);
    const ffm::ff v = ffm::add(ffm::ff{__fmul_rn(q.hi, 0.25f), __fmul_rn(q.lo, 0.25f)}, head);
    return ffm::round_unique(v, __fmul_rn(__fadd_rn(fabsf(head), __fmul_rn(q.hi, 0.25f)), 0x1p-44f), r);
}
static __device__ __noinline__ float add_quarter_sq(float head, float t) {
    float r;
    return add_quarter_sq_fast(head, t, r) ? r : add_quarter_sq_d(head, t);
}

// (float)((double)x + sqrt((double)y)), the reference's float + double sqrt of a float
static __device__ __noinline__ float add_dsqrt_d(float x, float y) { return (float)((double)x + sqrt((double)y)); }
__device__ __forceinline__ bool add_dsqrt_fast(float x, float y, float& r) {
    if (!(y > 0x1p-100f && y < 0x1p100f)) return false;
    const ffm::ff s = ffm::sqrt_ff(ffm::ff{y, 0.f});
    return ffm::round_unique(ffm::add(s, x), __fmul_rn(__fadd_rn(fabsf(x), s.hi), 0x1p-40f), r);
}
static __device__ __noinline__ float add_dsqrt(float x, float y) {
    float r;
    return add_dsqrt_fast(x, y, r) ? r : add_dsqrt_d(x, y);
}
// (float)(s + sqrt(a*a + b*b + c*c)) with a, b, c floats promoted to double
static __device__ __noinline__ float add_dsqrt3_d(float s, float a, float b, float c) {
    const double da = a, db = b, dc = c;
    return (float)((double)s + sqrt(da * da + db * db + dc * dc));
}
__device__ __forceinline__ bool add_dsqrt3_fast(float s, float a, float b, float c, float& r) {
    const float m = fmaxf(fabsf(a), fmaxf(fabsf(b), fabsf(c)));
    if (!(m > 0x1p-50f && m < 0x1p50f)) return false;
    const ffm::ff q = ffm::add(ffm::add(ffm::two_prod(a, a), ffm::two_prod(b, b)), ffm::two_prod(c, c));
    const ffm::ff r0 = ffm::sqrt_ff(q);
    return ffm::round_unique(ffm::add(r0, s), __fmul_rn(__fadd_rn(fabsf(s), r0.hi), 0x1p-40f), r);
}
static __device__ __noinline__ float add_dsqrt3(float s, float a, float b, float c) {
    float r;
    return add_dsqrt3_fast(s, a, b, c, r) ? r : add_dsqrt3_d(s, a, b, c);
}

// MathUtil.cc:3-19; the loop is bounded (|x| stays within a few pi here).
// 0x1.921fb6p+1f is the float just above pi: |x| below it is in [-pi, pi).
static __device__ __noinline__ float phi_mpi_pi_d(float x) {
    if (isnan(x)) return x;
#pragma unroll 1
    for (int it = 0; it < 64 && (double)x >= kPi; ++it) x = (float)((double)x - 2. * kPi);
#pragma unroll 1
    for (int it = 0; it < 64 && (double)x < -kPi; ++it) x = (float)((double)x + 2. * kPi);
    return x;
}
// one step of the loop, (float)((double)x -+ 2 M_PI), when it is enough
// (2 M_PI as hi + lo is 7.1e-15 off; the sum's error is below 1e-13)
__device__ __forceinline__ bool phi_mpi_pi_fast(float x, float& r) {
    const float ax = fabsf(x);
    if (ax < 0x1.921fb6p+1f) {
        r = x;
        return true;
    }
    if (!(ax < 9.f)) return false;
    const ffm::ff tp = x > 0.f ? ffm::ff{-0x1.921fb6p+2f, 0x1.777a5cp-23f} : ffm::ff{0x1.921fb6p+2f, -0x1.777a5cp-23f};
    return ffm::round_unique(ffm::add(tp, x), 2e-13f, r) && fabsf(r) < 0x1.921fb6p+1f;
}
static __device__ __noinline__ float phi_mpi_pi_slow(float x) {
    float r;
    return phi_mpi_pi_fast(x, r) ? r : phi_mpi_pi_d(x);
}
__device__ __forceinline__ float phi_mpi_pi(float x) {
    if (fabsf(x) < 0x1.921fb6p+1f) return x;
    return phi_mpi_pi_slow(x);
}
// MathUtil.cc:21-27
static __device__ __noinline__ float atan2_d(float y, float x) { return (float)atan2((double)y, (double)x); }
__device__ __forceinline__ bool atan2_fast(float y, float x, float& r) {
    ffm::ff a;
    return y != 0.f && x != 0.f && ffm::atan2_ff(ffm::ff{y, 0.f}, ffm::ff{x, 0.f}, a) && ffm::round_unique_rel(a, r);
}
__device__ __forceinline__ float atan2_ref(float y, float x) {
    if (x != 0) {
        float r;
        return atan2_fast(y, x, r) ? r : atan2_d(y, x);
    }
    if (y == 0) return 0.f;
    if (y > 0) return (float)(kPi / 2);
    return (float)(-kPi / 2);
}
// phi of a point (Hit.cc:68-83 via MathUtil.cc): Phi_mpi_pi(M_PI + ATan2(-y, -x))
static __device__ __noinline__ float phi_of_d(float x, float y) {
    const float a = x != 0 ? atan2_d(-y, -x) : atan2_ref(-y, -x);
    return phi_mpi_pi_d((float)(kPi + (double)a));
}
// (float)(M_PI + (double)a): M_PI as hi + lo is 3.6e-15 off; error below 1e-13
__device__ __forceinline__ bool add_pi_fast(float a, float& p) {
    return ffm::round_unique(ffm::add(ffm::ff{0x1.921fb6p+1f, -0x1.777a5cp-24f}, a), 1e-13f, p);
}
static __device__ __noinline__ float phi_of(float x, float y) {
    const float a = atan2_ref(-y, -x);
    float p;
    if (!add_pi_fast(a, p)) p = (float)(kPi + (double)a);
    return phi_mpi_pi(p);
}

// A point with the derived quantities (Hit.cc:68-83).
struct P3 {
    float x, y, z, rt, phi, r3;
};
__device__ __forceinline__ P3 mk(float x, float y, float z) {
    P3 p;
    p.x = x; p.y = y; p.z = z;
    // float sqrt == double sqrt rounded to float for float arguments
    p.rt = __fsqrt_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)));
    p.r3 = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z)));
    p.phi = phi_of(x, y);
    return p;
}
// rt and phi only (r3 unused)
__device__ __forceinline__ P3 mk2(float x, float y, float z) {
    P3 p;
    p.x = x; p.y = y; p.z = z;
    p.rt = __fsqrt_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)));
    p.r3 = 0.f;
    p.phi = phi_of(x, y);
    return p;
}
__device__ __forceinline__ P3 sub(const P3& a, const P3& b) { return mk2(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float dphi(const P3& a, const P3& b) { return phi_mpi_pi(b.phi - a.phi); }
__device__ __forceinline__ float dphichange(const P3& a, const P3& b) { return dphi(a, sub(b, a)); }
__device__ __forceinline__ float rt_of_diff(const P3& a, const P3& b) {
    const float x = a.x - b.x, y = a.y - b.y;
    return __fsqrt_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)));
}
__device__ __forceinline__ P3 midpoint(const P3& a, const P3& b) {
    float x = 0.f, y = 0.f, z = 0.f;
    x += a.x; y += a.y; z += a.z;
    x += b.x; y += b.y; z += b.z;
    x /= 2.f; y /= 2.f; z /= 2.f;
    return mk2(x, y, z);
}
// GeometryUtil.cc:3-23 (edge offsets precomputed per module)
__device__ __forceinline__ P3 strip_edge(const P3& h, const ModDev& m, bool up) {
    float ex = up ? m.edge_x : -m.edge_x;
    float ey = up ? m.edge_y : -m.edge_y;
    float ez = 0.f;
    ex += h.x; ey += h.y; ez += h.z;
    return mk2(ex, ey, ez);
}

// constants as the reference spells them
__device__ constexpr float kRinv1GeVf = (float)(2.99792458e-3 * 3.8);
__device__ constexpr float k2Rinv1GeVf = (float)((double)(float)(2.99792458e-3 * 3.8) / 2.);
__device__ constexpr float kSinAlphaMax = 0.95f;
__device__ constexpr float kPtCut = 1.0f;
__device__ constexpr float kPixelPSZpitch = 0.15f;
__device__ constexpr float kStrip2SZpitch = 5.0f;
__device__ constexpr float kDeltaZLum = 15.f;

// ------------------------------------------------------------------ mini-doublets
// MiniDoublet.cc:741-810
__device__ __forceinline__ float dphi_threshold(float rt, float asin_rt1, const ModDev& m, float dPhi, float dz) {
    const float mulsB[6] = {0.0052f, 0.0038f, 0.0034f, 0.0034f, 0.0032f, 0.0034f};
    const unsigned iL = m.layer - 1;
    const float miniSlope = asin_rt1;  // asin(min(rt * k2Rinv1GeVf / 1, 0.95))
    (void)rt;
    const bool barrel = m.subdet == kBarrel;
    // (float)(0.1 / (double)rLay) for the layer radii 21.8 ... 106.8 (barrel) and
    // 131.4 ... 261.5 (endcap) of MiniDoublet.cc:763-767: constant per layer
    constexpr float pvB[6] = {(float)(0.1 / (double)21.8f), (float)(0.1 / (double)34.6f), (float)(0.1 / (double)49.6f),
                              (float)(0.1 / (double)67.4f), (float)(0.1 / (double)87.6f), (float)(0.1 / (double)106.8f)};
    constexpr float pvE[5] = {(float)(0.1 / (double)131.4f), (float)(0.1 / (double)156.2f), (float)(0.1 / (double)185.6f),
                              (float)(0.1 / (double)220.3f), (float)(0.1 / (double)261.5f)};
    const float miniPVoff = barrel ? pvB[iL] : pvE[iL];
    const float miniMuls = barrel ? mulsB[iL] * 3.f / kPtCut : 0.006f * 3.f / kPtCut;
    if (barrel && m.side == kCenter) return add_dsqrt3(miniSlope, miniMuls, miniPVoff, 0.f);
    if (barrel) return add_dsqrt3(miniSlope, miniMuls, miniPVoff, m.tilt * miniSlope);
    const float miniLum = (float)iabs(trunc_i32(dPhi * kDeltaZLum / dz));
    return add_dsqrt3(miniSlope, miniMuls, miniPVoff, miniLum);
}

// MiniDoublet.cc:989-1209 (shiftStripHits), split in two.  Everything up to
// the shifted anchor point (xa, ya) and the new z depends only on the
// anchoring hit `pix` and the lower module lm of its pair, so shift_anchor
// runs once per hit (k_hit_scatter); shift_finish projects onto the strip
// through the other hit `str` per mini-doublet candidate.  The arithmetic and
// its order are the reference's.
__device__ __forceinline__ void shift_anchor(const P3& pix, const ModDev& lm, float& xa, float& ya, float& zn) {
    const bool ps = lm.type == kPS;
    const bool pixLower = lm.ltype == kPixel;
    const float angleA = fabsf(g_atan(pix.rt / pix.z));
    const float angleB = lm.sh_angle_b;  // (float)(pi / 2) for endcap modules
    float sep = lm.gap;
    if (ps && !pixLower) sep *= -1;
    const float sAB = g_sin(angleA + angleB);
    const float drprime = (sep / sAB) * g_sin(angleA);
    // angleM: |atan(slope)| (pi / 2 for the "infinite" slope), pi - it, pi +
    // it, 2 pi - it by quadrant; its sine and cosine come with the module
    const float xp = pix.x, yp = pix.y;
    const int q = (xp > 0 && yp > 0) ? 0 : (xp > 0 && yp < 0) ? 1 : (xp < 0 && yp < 0) ? 2 : 3;
    const float dx = drprime * lm.sh_sin[q];
    const float dy = drprime * lm.sh_cos[q];
    xa = xp + dx;
    ya = yp + dy;
    const float absdzprime = fabsf(sep / sAB * g_cos(angleA));
    float abszn;
    // one double operation on two floats rounded to float: the float operation
    if (pixLower) abszn = fabsf(pix.z) + absdzprime;
    else abszn = fabsf(pix.z) - absdzprime;
    zn = abszn * ((pix.z > 0) ? 1 : -1);
}
__device__ __forceinline__ void shift_finish(float xa, float ya, const P3& str, const ModDev& lm, float& xn, float& yn) {
    const float slope = lm.slope_s;
    const float xo = str.x, yo = str.y;
    if (slope == kSdlInf) { xn = xa; yn = yo; }
    else if (slope == 0) { xn = xo; yn = ya; }
    else {
        xn = (slope * xa + (1.f / slope) * xo - ya + yo) / (slope + (1.f / slope));
        yn = (xn - xa) * slope + ya;
    }
}
// whether the mini-doublets of the pair with lower module lm shift a strip
// hit, and whether the upper hit anchors (MiniDoublet.cc:60-81)
__device__ __forceinline__ bool md_shifts(const ModDev& lm) { return lm.subdet == kEndcap || lm.side != kCenter; }
__device__ __forceinline__ bool md_upper_anchors(const ModDev& lm) { return lm.type == kPS && lm.ltype != kPixel; }

struct MDVals {
    float dz, shiftedDz, dphi, dphichange;
};

// ---- single-precision directions with error bounds, for decisions that only
// reject (or accept) by more than the bound and leave the rest to the exact
// code: a direction difference with one direction from atan2f is within
// kB2qDir of the exact float (3 ulp of pi for atan2f, the exact value's own
// rounding, the subtraction and the wrap at +-pi), and the decisions take
// kB2qSafety times their bounds.
constexpr float kPiF = 3.14159265f;
constexpr float kB2qSafety = 4.f;
constexpr float kB2qDir = 2e-6f;  // a direction difference from atan2f: 3 ulp of pi, the exact value's rounding, the wrap
constexpr float kB2qSin = 4e-7f;  // __sinf on [-pi, pi]: absolute error below 2^-21.41 (CUDA)
__device__ __forceinline__ float ulp_of(float x) { return fabsf(x) * 0x1p-23f + 0x1p-126f; }
// the exact code's dphi(a, b) = phi_mpi_pi(b - a) of two directions in
// [-pi, pi] (one of them approximate); false near the wrap at +-pi
__device__ __forceinline__ bool dphi_q(float a, float b, float& d) {
    float v = b - a;
    if (v >= kPiF) v -= 2.f * kPiF;
    else if (v < -kPiF) v += 2.f * kPiF;
    d = v;
    return fabsf(fabsf(v) - kPiF) > 1e-4f;
}

// MiniDoublet.cc:243-447.  pixAsin is asin(min(rt*k, .95)) of the hit that
// dPhiThreshold reads (the pixel-side hit); sh is shift_anchor's (xa, ya, zn)
// of the anchoring hit.
__device__ __forceinline__ bool md_barrel(const P3& lo, const P3& up, float pixAsin, const ModDev& lm, const float* sh,
                                          MDVals& v) {
    v.dz = lo.z - up.z;
    const float dz = v.dz;
    const float dzCut = lm.type == kPS ? 2.f : 10.f;
    const float sign = (float)(((dz > 0) - (dz < 0)) * ((lo.z > 0) - (lo.z < 0)));
    const float inverted = (float)(iabs(trunc_i32(dz)) > 2) * sign;
    if (!(fabsf(dz) < dzCut && inverted <= 0)) return false;
    const float miniCut = dphi_threshold(0.f, pixAsin, lm, 0.f, 1.f);
    P3 shifted;
    if (lm.side != kCenter) {
        float xn, yn;
        shift_finish(sh[0], sh[1], md_upper_anchors(lm) ? lo : up, lm, xn, yn);
        if (lm.ltype == kPixel) { shifted = mk2(xn, yn, up.z); v.dphi = dphi(lo, shifted); }
        else { shifted = mk2(xn, yn, lo.z); v.dphi = dphi(shifted, up); }
    } else {
        v.dphi = dphi(lo, up);
    }
    if (!(fabsf(v.dphi) < miniCut)) return false;
    // the two points of the direction change (dphichange(a, b): the direction of
    // b - a against a's), as the reference picks them
    const P3* a = &lo;
    const P3* b = &up;
    if (lm.side != kCenter) {
        if (lm.ltype == kPixel) { a = lo.rt < shifted.rt ? &lo : &shifted; b = lo.rt < shifted.rt ? &shifted : &lo; }
        else { a = shifted.rt < up.rt ? &shifted : &up; b = shifted.rt < up.rt ? &up : &shifted; }
    }
    // most candidates fail this cut: the direction of b - a from atan2f (a's
    // direction is exact) rejects those clearly outside it before the exact one
    float q;
    if (dphi_q(a->phi, atan2f(b->y - a->y, b->x - a->x), q) && fabsf(q) >= miniCut + kB2qSafety * kB2qDir) return false;
    v.dphichange = dphichange(*a, *b);
    return fabsf(v.dphichange) < miniCut;
}

// MiniDoublet.cc:449-684
__device__ __forceinline__ bool md_endcap(const P3& lo, const P3& up, float pixAsin, const ModDev& lm, const float* sh,
                                          MDVals& v) {
    v.dz = lo.z - up.z;
    float dz = v.dz;
    if (!(fabsf(dz) < 10.f)) return false;  // side() is never SubDet::Endcap (MiniDoublet.cc:470)
    const float drtCut = lm.type == kPS ? 2.f : 10.f;
    if (!(fabsf(lo.rt - up.rt) < drtCut)) return false;
    float xn, yn;
    const float zn = sh[2];
    shift_finish(sh[0], sh[1], md_upper_anchors(lm) ? lo : up, lm, xn, yn);
    P3 shifted;
    if (lm.type == kPS && lm.ltype != kPixel) { shifted = mk2(xn, yn, lo.z); v.dphi = dphi(shifted, up); }
    else { shifted = mk2(xn, yn, up.z); v.dphi = dphi(lo, shifted); }
    if (lm.type == kPS) {
        v.shiftedDz = lm.ltype == kPixel ? lo.z - zn : up.z - zn;
        dz = v.shiftedDz;
    }
    const float miniCut = dphi_threshold(0.f, pixAsin, lm, v.dphi, dz);
    if (!(fabsf(v.dphi) < miniCut)) return false;
    const float dzFrac = fabsf(dz) / fabsf(lo.z);  // a double division of two floats rounded to float
    v.dphichange = v.dphi / dzFrac * (1.f + dzFrac);
    return fabsf(v.dphichange) < miniCut;
}

// ------------------------------------------------------------------ segments
struct MDView {
    P3 a;          // anchor hit
    float dphi, dphichange, dz, shiftedDz;
    const ModDev* m;  // lower module
};
constexpr int kMdPack = 16;  // floats per packed mini-doublet record

// Segment.cc:886-994 (the three thresholds)
// host: the host libm's asin (the reference's), else the correctly rounded one
__device__ __forceinline__ void dalpha_threshold(const MDView& im, const MDView& om, float th[3], bool host) {
    const float mulsB[6] = {0.0052f, 0.0038f, 0.0034f, 0.0034f, 0.0032f, 0.0034f};
    const ModDev& I = *im.m;
    const ModDev& O = *om.m;
    const float sdMuls = I.subdet == kBarrel ? mulsB[I.layer - 1] * 3.f / kPtCut : 0.006f * 3.f / kPtCut;
    const float segmentDr = hypot_ref(om.a.y - im.a.y, om.a.x - im.a.x);
    const float a = fmin_ref(segmentDr * k2Rinv1GeVf / kPtCut, kSinAlphaMax);
    const float dAlpha_Bfield = host ? g_asin(a) : f_asin(a);
    const bool inTilt = I.subdet == kBarrel && I.side != kCenter;
    const bool outTilt = O.subdet == kBarrel && O.side != kCenter;
    const float iTilt = inTilt ? I.tilt : 0.f;
    const float oTilt = outTilt ? O.tilt : 0.f;
    const float miniDelta = I.gap;
    float lumIn, lumOut;
    if (I.subdet == kBarrel) lumIn = iTilt * dAlpha_Bfield;
    else if (I.type == kPS) lumIn = times15_over(im.dphi, im.shiftedDz);
    else lumIn = times15_over(im.dphi, im.dz);
    if (O.subdet == kBarrel) lumOut = oTilt * dAlpha_Bfield;
    else if (O.type == kPS) lumOut = times15_over(om.dphi, om.shiftedDz);
    else lumOut = times15_over(om.dphi, om.dz);
    const float resIn = 0.02f / miniDelta * (I.subdet == kBarrel ? 1.0f : fabsf(im.a.z / im.a.rt));
    const float resOut = 0.02f / miniDelta * (O.subdet == kBarrel ? 1.0f : fabsf(om.a.z / om.a.rt));
    const float res = resIn + resOut;
    th[0] = add_dsqrt3(dAlpha_Bfield, res, sdMuls, (I.subdet == kBarrel && I.side == kCenter) ? 0.f : lumIn);
    th[1] = add_dsqrt3(dAlpha_Bfield, res, sdMuls, (O.subdet == kBarrel && O.side == kCenter) ? 0.f : lumOut);
    th[2] = add_dsqrt3(dAlpha_Bfield, res, sdMuls, 0.f);
}

// |v - t| small enough that replacing the correctly rounded value of one
// float libm call behind t by the host libm's (one float step away) could
// move t across v
__device__ __forceinline__ bool near_cut(float v, float t, float rel) { return fabsf(v - t) <= fabsf(t) * rel; }

// the three dAlpha cuts with the host libm's asin (the reference's)
static __device__ __noinline__ bool dalpha_cuts_host(const MDView& im, const MDView& om, float sg_alpha) {
    float th[3];
    dalpha_threshold(im, om, th, true);
    if (!(fabsf(im.dphichange - sg_alpha) < th[0])) return false;
    if (!(fabsf(om.dphichange - sg_alpha) < th[1])) return false;
    return fabsf(om.dphichange - im.dphichange) < th[2];
}
// The three dAlpha cuts are decided with the correctly rounded asin first.
// The host libm's asin is within one float step of it (dAlpha_Bfield >= 0);
// each threshold, dAlpha_Bfield + a square root (with dAlpha_Bfield inside it
// for tilted modules, times a tilt factor below 1) rounded to float, moves
// by at most three float steps, 2^-21 |t|; a comparison at least 2^-19 |t|
// from its threshold is therefore the host's decision too, and the rare
// closer ones are decided again with the host libm's asin.
__device__ __forceinline__ bool dalpha_cuts(const MDView& im, const MDView& om, float sg_alpha) {
    constexpr float rel = 0x1p-19f;
    float th[3];
    dalpha_threshold(im, om, th, false);
    const float v0 = fabsf(im.dphichange - sg_alpha);
    if (near_cut(v0, th[0], rel)) return dalpha_cuts_host(im, om, sg_alpha);
    if (!(v0 < th[0])) return false;
    const float v1 = fabsf(om.dphichange - sg_alpha);
    if (near_cut(v1, th[1], rel)) return dalpha_cuts_host(im, om, sg_alpha);
    if (!(v1 < th[1])) return false;
    const float v2 = fabsf(om.dphichange - im.dphichange);
    if (near_cut(v2, th[2], rel)) return dalpha_cuts_host(im, om, sg_alpha);
    return v2 < th[2];
}

struct SGVals {
    float dphi, dphimin, dphimax, dphichange, dphiminchange, dphimaxchange;
};

// Segment.cc:364-599: sdCut of an outer barrel anchor (rtOut, asin term)
// for inner barrel layer lIn
__device__ __forceinline__ float sg_barrel_cut(int lIn, float rtOut, float outAsin) {
    const float mulsB[6] = {0.0052f, 0.0038f, 0.0034f, 0.0034f, 0.0032f, 0.0034f};
    const float sdMuls = mulsB[lIn - 1] * 3.f / kPtCut;
    const float sdPVoff = 0.1f / rtOut;
    return add_dsqrt(outAsin, sdMuls * sdMuls + sdPVoff * sdPVoff);
}

// Segment.cc:364-599.  outAsin / outTanf: asin(min(rtOut*k,.95)) of the
// outer anchor and its float tan; cutPrev: sg_barrel_cut for the barrel
// layer below the outer one (k_md_pack).
// kPre: only the first cuts (the z window and the phi cut), for the segment
// stage's first pass; a candidate they reject fails the whole algorithm
template <bool kPre = false>
__device__ __forceinline__ bool sg_barrel(const MDView& im, const MDView& om, float outAsin, float outTanf, float cutPrev,
                                          SGVals& v) {
    const float rtIn = im.a.rt, rtOut = om.a.rt, zIn = im.a.z, zOut = om.a.z;
    const float sdSlope = outAsin;
    const float dzDrtScale = outTanf / sdSlope;
    const float zGeom = im.m->layer <= 2 ? 2.f * kPixelPSZpitch : 2.f * kStrip2SZpitch;
    const float zLo = zIn + (zIn - kDeltaZLum) * (rtOut / rtIn - 1.f) * (zIn > 0.f ? 1.f : dzDrtScale) - zGeom;
    const float zHi = zIn + (zIn + kDeltaZLum) * (rtOut / rtIn - 1.f) * (zIn < 0.f ? 1.f : dzDrtScale) + zGeom;
    if (!(zOut >= zLo && zOut <= zHi)) return false;
    const bool prev = im.m->subdet == kBarrel && im.m->layer + 1 == om.m->layer;
    const float sdCut = prev ? cutPrev : sg_barrel_cut(im.m->layer, rtOut, outAsin);
    const float deltaPhi = dphi(im.a, om.a);
    if (!(fabsf(deltaPhi) <= sdCut)) return false;
    if (kPre) return true;
    v.dphichange = dphichange(im.a, om.a);
    if (!(fabsf(v.dphichange) <= sdCut)) return false;
    return dalpha_cuts(im, om, v.dphichange);
}

// Segment.cc:601-859.  connected: outer module is in the inner module's
// connection list (cut #0); phiHi / phiLo: the phi of the outer anchor's
// strip-edge points (the anchor itself for PS modules; k_md_pack).
// kPre: only the first cuts (connection, rt window and phi cut), as sg_barrel
template <bool kPre = false>
__device__ __forceinline__ bool sg_endcap(const MDView& im, const MDView& om, float outAsin, float outTanf,
                                          bool connected, float phiHi, float phiLo, SGVals& v) {
    const ModDev& I = *im.m;
    const bool l2r123 = (I.ring == 1 || I.ring == 2 || I.ring == 3) && I.layer == 2;
    if (!(connected || l2r123)) return false;
    const float rtIn = im.a.rt, rtOut = om.a.rt, zIn = im.a.z, zOut = om.a.z;
    const float sdSlope = outAsin;
    const float disks2SMinRadius = 60.f;
    const float rtGeom = (rtIn < disks2SMinRadius && rtOut < disks2SMinRadius) ? (2.f * kPixelPSZpitch)
                       : ((rtIn < disks2SMinRadius || rtOut < disks2SMinRadius) ? (kPixelPSZpitch + kStrip2SZpitch)
                       : (2.f * kStrip2SZpitch));
    if (zIn * zOut < 0) return false;
    const float dz = zOut - zIn;
    const float dLum = f_copysign(kDeltaZLum, zIn);
    const float drtDzScale = sdSlope / outTanf;
    const float rtLo = fmax_ref(rtIn * (1.f + dz / (zIn + dLum) * drtDzScale) - rtGeom, rtIn - 0.5f * rtGeom);
    const float rtHi = rtIn * (zOut - dLum) / (zIn - dLum) + rtGeom;
    if (!(rtOut >= rtLo && rtOut <= rtHi)) return false;
    const float dPhiPos = dphi(im.a, om.a);
    const float sdCut = sdSlope;
    if (!(fabsf(dPhiPos) <= sdCut)) return false;
    if (kPre) return true;
    const float hiP = phi_mpi_pi(phiHi - im.a.phi);  // dphi(im.a, oHi)
    const float loP = phi_mpi_pi(phiLo - im.a.phi);
    const bool hiBigger = iabs(trunc_i32(hiP)) > iabs(trunc_i32(loP));
    v.dphi = dPhiPos;
    v.dphimax = hiBigger ? hiP : loP;
    v.dphimin = hiBigger ? loP : hiP;
    const float dzFrac = dz / zIn;
    v.dphichange = dPhiPos / dzFrac * (1.f + dzFrac);
    if (!(fabsf(v.dphichange) <= sdCut)) return false;
    v.dphiminchange = v.dphimin / dzFrac * (1.f + dzFrac);
    v.dphimaxchange = v.dphimax / dzFrac * (1.f + dzFrac);
    return dalpha_cuts(im, om, v.dphichange);
}

// ------------------------------------------------------------------ tracklets
// The tracklet stage reads each segment through a packed 128-byte record
// built once per segment (k_sg_pack): both anchor hits with their derived
// quantities, the segment's angles and the per-segment sub-expressions of
// the tracklet algorithms (all evaluated exactly as in the per-candidate
// formulas, so the results do not change).
enum SGPackField : int {
    PK_LX, PK_LY, PK_LZ, PK_LRT,            // inner-MD anchor
    PK_LPHI, PK_LR3, PK_LA1, PK_LTD,        //   phi, r3, asin(min(rt*k,.95)), (float)(tan(a1)/a1)
    PK_LA3, PK_LR3Z, PK_UX, PK_UY,          //   asin(min(rt*k/3,.95)), sqrt(z*z+rt*rt); outer-MD anchor x, y
    PK_UZ, PK_URT, PK_UPHI, PK_UR3,         //   outer-MD anchor
    PK_DPC, PK_DPMIN, PK_DPMAX, PK_DPMINC,  // segment dPhiChange, dPhiMin, dPhiMax, dPhiMinChange
    PK_DPMAXC, PK_RTSEG, PK_ALPHAUP, PK_DPHILU,  // dPhiMaxChange, rt of (up - lo), dphi(up, up - lo), dphi(lo, up)
    PK_EX, PK_EY, PK_FLAGS, PK_G2,          // outer anchor module's strip-edge offset; flags; module of the outer MD
    PK_S0, PK_S1, PK_S2, PK_S3,             // dz/drt and dr3/drt of the segment; sqrt(lr3z/lrt) in float-float
    PK_N
};
enum : uint32_t {
    F_LO_B = 1u, F_LO_E = 2u, F_LO_PS = 4u,
    F_UP_B = 8u, F_UP_E = 16u, F_UP_PS = 32u, F_UP_2S = 64u,
};

struct SGV {
    float lx, ly, lz, lrt, lphi, lr3, la1, ltd, la3, lr3z;
    float ux, uy, uz, urt, uphi, ur3;
    float dpc, dpmin, dpmax, dpminc, dpmaxc, rtseg, alphaup, dphilu, ex, ey;
    uint32_t flags;
    // the inner role's per-segment terms (sg_pack_record): (uz - lz) / (urt -
    // lrt), (ur3 - lr3) / (urt - lrt), and sqrt(lr3z / lrt) in float-float
    // (NaN outside the multiple-scattering factor's fast-path range)
    float dzdr, cosh, sqq_hi, sqq_lo;
    __device__ P3 lo() const { P3 p; p.x = lx; p.y = ly; p.z = lz; p.rt = lrt; p.phi = lphi; p.r3 = lr3; return p; }
    __device__ P3 up() const { P3 p; p.x = ux; p.y = uy; p.z = uz; p.rt = urt; p.phi = uphi; p.r3 = ur3; return p; }
};

__device__ __forceinline__ SGV load_sgv(const float* __restrict__ pack, int64_t s) {
    const float4* q = reinterpret_cast<const float4*>(pack + s * PK_N);
    const float4 a = __ldg(q + 0), c = __ldg(q + 1), d = __ldg(q + 2), e = __ldg(q + 3);
    const float4 f = __ldg(q + 4), g = __ldg(q + 5), h = __ldg(q + 6), i = __ldg(q + 7);
    SGV v;
    v.lx = a.x; v.ly = a.y; v.lz = a.z; v.lrt = a.w;
    v.lphi = c.x; v.lr3 = c.y; v.la1 = c.z; v.ltd = c.w;
    v.la3 = d.x; v.lr3z = d.y; v.ux = d.z; v.uy = d.w;
    v.uz = e.x; v.urt = e.y; v.uphi = e.z; v.ur3 = e.w;
    v.dpc = f.x; v.dpmin = f.y; v.dpmax = f.z; v.dpminc = f.w;
    v.dpmaxc = g.x; v.rtseg = g.y; v.alphaup = g.z; v.dphilu = g.w;
    v.ex = h.x; v.ey = h.y; v.flags = __float_as_uint(h.z);
    v.dzdr = i.x; v.cosh = i.y; v.sqq_hi = i.z; v.sqq_lo = i.w;
    return v;
}

// the same from a record held in registers or local memory
__device__ __forceinline__ SGV sgv_from(const float* p) {
    SGV v;
    v.lx = p[PK_LX]; v.ly = p[PK_LY]; v.lz = p[PK_LZ]; v.lrt = p[PK_LRT];
    v.lphi = p[PK_LPHI]; v.lr3 = p[PK_LR3]; v.la1 = p[PK_LA1]; v.ltd = p[PK_LTD];
    v.la3 = p[PK_LA3]; v.lr3z = p[PK_LR3Z]; v.ux = p[PK_UX]; v.uy = p[PK_UY];
    v.uz = p[PK_UZ]; v.urt = p[PK_URT]; v.uphi = p[PK_UPHI]; v.ur3 = p[PK_UR3];
    v.dpc = p[PK_DPC]; v.dpmin = p[PK_DPMIN]; v.dpmax = p[PK_DPMAX]; v.dpminc = p[PK_DPMINC];
    v.dpmaxc = p[PK_DPMAXC]; v.rtseg = p[PK_RTSEG]; v.alphaup = p[PK_ALPHAUP]; v.dphilu = p[PK_DPHILU];
    v.ex = p[PK_EX]; v.ey = p[PK_EY]; v.flags = __float_as_uint(p[PK_FLAGS]);
    v.dzdr = p[PK_S0]; v.cosh = p[PK_S1]; v.sqq_hi = p[PK_S2]; v.sqq_lo = p[PK_S3];
    return v;
}

// Features of a tracklet candidate for the learned pre-filter (float
// arithmetic only, no counterpart in the reference): anchor radii and z of
// the innermost and outermost mini-doublets, the azimuthal opening between
// them, the two segments' direction angles, float estimates of the betaIn /
// betaOut angles the exact cuts test (Tracklet.cc:1205-1260), the rz
// pointing residual of the outer anchor against the inner segment, a signed
// 1/pT estimate from the mean beta, and a code of the anchor module types.
// Every feature is scaled to O(1) and clamped to [-16, 16].  They read one
// 32-byte record of each segment (k_sg_pack): the inner segment's in its
// inner role, the outer segment's in its outer role.
__device__ __forceinline__ float wrap_pi_f(float x) { return x - 6.28318531f * rintf(x * 0.159154943f); }
constexpr int kFeatN = 16;  // floats per segment: inner-role record, outer-role record
struct FeatS {               // a segment as the inner one
    float lx, ly, lz, lrt, lphi, dpc, slope, code;  // lower anchor; dPhiChange; rz slope; module code
};
struct FeatT {               // a segment as the outer one
    float ux, uy, uz, urt, uphi, alphaup, code, pad;  // upper anchor; direction angle; module code
};
__device__ __forceinline__ FeatS feat_s(const float* __restrict__ f, int64_t s) {
    const float4* q = reinterpret_cast<const float4*>(f + s * kFeatN);
    const float4 a = __ldg(q), b = __ldg(q + 1);
    return FeatS{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
}
__device__ __forceinline__ FeatT feat_t(const float* __restrict__ f, int64_t t) {
    const float4* q = reinterpret_cast<const float4*>(f + t * kFeatN + 8);
    const float4 a = __ldg(q), b = __ldg(q + 1);
    return FeatT{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
}
__device__ __forceinline__ void tl_features(const FeatS& S, const FeatT& T, float* f) {
    const float ax = T.ux - S.lx, ay = T.uy - S.ly;
    const float dr = sqrtf(ax * ax + ay * ay);
    const float phiAxis = atan2f(ay, ax);
    const float betaIn = S.dpc - wrap_pi_f(phiAxis - S.lphi);
    const float betaOut = -T.alphaup + wrap_pi_f(phiAxis - T.uphi);
    const float zRes = T.uz - (S.lz + S.slope * (T.urt - S.lrt));
    const float invPt = __fdividef(__sinf(0.5f * (betaIn + betaOut)), fmaxf(dr, 1e-3f) * k2Rinv1GeVf);
    float v[12];
    v[0] = S.lrt * 0.01f;
    v[1] = S.lz * 0.01f;
    v[2] = T.urt * 0.01f;
    v[3] = T.uz * 0.01f;
    v[4] = wrap_pi_f(T.uphi - S.lphi) * 10.f;
    v[5] = S.dpc * 10.f;
    v[6] = T.alphaup * 10.f;
    v[7] = betaIn * 10.f;
    v[8] = betaOut * 10.f;
    v[9] = zRes * 0.1f;
    v[10] = invPt;
    v[11] = S.code + T.code;
#pragma unroll
    for (int k = 0; k < 12; ++k) f[k] = fmaxf(fminf(v[k], 16.f), -16.f);
}

// strip-edge point of a 2S endcap hit (GeometryUtil.cc:3-23) from the edge offset
__device__ __forceinline__ P3 edge_point(float x, float y, float z, float ex, float ey, bool up) {
    float px = up ? ex : -ex, py = up ? ey : -ey, pz = 0.f;
    px += x; py += y; pz += z;
    return mk2(px, py, pz);
}
__device__ __forceinline__ float edge_rt(float x, float y, float ex, float ey, bool up) {
    float px = up ? ex : -ex, py = up ? ey : -ey;
    px += x; py += y;
    return __fsqrt_rn(__fadd_rn(__fmul_rn(px, px), __fmul_rn(py, py)));
}

// Tracklet.cc:3181-3324.  The reference adds the double copysign term to a
// float and rounds to float; a double sum of two floats rounded to float
// equals the float sum (53 >= 2*24+2), so the additions are done in float.
__device__ __forceinline__ void delta_beta_iterations(float& betaIn, float& betaOut, float& betaAv, float& pt_beta, float sdIn_dr,
                                                      float sdOut_dr, float dr, int lIn, float pt_betaMax) {
    const float sinAlphaMax = 0.95f;
    if (betaIn * betaOut > 0.f &&
        (fabsf(pt_beta) < 4.f * pt_betaMax || (lIn >= 11 && fabsf(pt_beta) < 8.f * pt_betaMax))) {
        const float betaInUpd = betaIn + copysignf(g_asin(fmin_ref(sdIn_dr * k2Rinv1GeVf / fabsf(pt_beta), sinAlphaMax)), betaIn);
        const float betaOutUpd = betaOut + copysignf(g_asin(fmin_ref(sdOut_dr * k2Rinv1GeVf / fabsf(pt_beta), sinAlphaMax)), betaOut);
        betaAv = 0.5f * (betaInUpd + betaOutUpd);
        pt_beta = pt_from(dr * k2Rinv1GeVf, betaAv);
        betaIn = betaIn + copysignf(g_asin(fmin_ref(sdIn_dr * k2Rinv1GeVf / fabsf(pt_beta), sinAlphaMax)), betaIn);
        betaOut = betaOut + copysignf(g_asin(fmin_ref(sdOut_dr * k2Rinv1GeVf / fabsf(pt_beta), sinAlphaMax)), betaOut);
        betaAv = 0.5f * (betaIn + betaOut);
        pt_beta = pt_from(dr * k2Rinv1GeVf, betaAv);
    } else if (lIn < 11 && (double)fabsf(betaOut) < 0.2 * (double)fabsf(betaIn) && fabsf(pt_beta) < 12.f * pt_betaMax) {
        const float pt_betaIn = pt_from(dr * k2Rinv1GeVf, betaIn);
        const float betaInUpd = betaIn + copysignf(g_asin(fmin_ref(sdIn_dr * k2Rinv1GeVf / fabsf(pt_betaIn), sinAlphaMax)), betaIn);
        const float betaOutUpd = betaOut + copysignf(g_asin(fmin_ref(sdOut_dr * k2Rinv1GeVf / fabsf(pt_betaIn), sinAlphaMax)), betaIn);
        betaAv = (fabsf(betaOut) > 0.2f * fabsf(betaIn)) ? (0.5f * (betaInUpd + betaOutUpd)) : betaInUpd;
        pt_beta = pt_from(dr * k2Rinv1GeVf, betaAv);
        betaIn = betaIn + copysignf(g_asin(fmin_ref(sdIn_dr * k2Rinv1GeVf / fabsf(pt_beta), sinAlphaMax)), betaIn);
        betaOut = betaOut + copysignf(g_asin(fmin_ref(sdOut_dr * k2Rinv1GeVf / fabsf(pt_beta), sinAlphaMax)), betaIn);
        betaAv = 0.5f * (betaIn + betaOut);
        pt_beta = pt_from(dr * k2Rinv1GeVf, betaAv);
    }
}

__device__ __forceinline__ float dbeta_cut2(float dBetaRes, float dBetaMuls, float dBetaLum2, float dBetaROut2, float inMin,
                                            float inMax, float outMin, float outMax) {
    const float dBetaRIn2 = 0;
    const float head = dBetaRes * dBetaRes * 2.0f + dBetaMuls * dBetaMuls + dBetaLum2 + dBetaRIn2 + dBetaROut2;
    return add_quarter_sq(head, fabsf(inMin - inMax) + fabsf(outMin - outMax));
}


// What phase A reads of the outer segment, from arrays of one float per
// segment (consecutive outer segments of a warp's candidates are then read
// with coalesced loads); the same values as the packed record's fields.
struct SGOuter {
    float lrt, lz, ltd, la1, uphi;
    uint32_t flags;
    float pvoff;  // 0.1f / lrt
};
__device__ __forceinline__ SGOuter load_sgo(const float* __restrict__ a, int64_t cap, int64_t t) {
    SGOuter o;
    o.lrt = __ldg(a + t);
    o.lz = __ldg(a + cap + t);
    o.ltd = __ldg(a + 2 * cap + t);
    o.la1 = __ldg(a + 3 * cap + t);
    o.uphi = __ldg(a + 4 * cap + t);
    o.flags = __float_as_uint(__ldg(a + 5 * cap + t));
    o.pvoff = __ldg(a + 6 * cap + t);
    return o;
}
// the outer segment's anchor points as phase B1 reads them: (lx, ly, ux, uy),
// arrays 7 to 10 of the same layout
__device__ __forceinline__ float4 load_sgo_xy(const float* __restrict__ a, int64_t cap, int64_t t) {
    return make_float4(__ldg(a + 7 * cap + t), __ldg(a + 8 * cap + t), __ldg(a + 9 * cap + t), __ldg(a + 10 * cap + t));
}
// the PV-offset term 0.1f / rtOut of the tracklet cuts (Tracklet.cc:1056 and
// the like), precomputed for an SGOuter
__device__ __forceinline__ float pv_off(const SGOuter& T) { return T.pvoff; }
__device__ __forceinline__ float pv_off(const SGV& T) { return 0.1f / T.lrt; }

// Tracklet algorithm ids carried between the two phases
enum : int { kAlgoNone = 0, kAlgoBBBB = 1, kAlgoBBEE = 2, kAlgoEEEE = 3 };

// ---- phase A: dispatch (Tracklet.cc:144-296) and the cuts that need only
// float arithmetic and square roots.  Returns the algorithm or kAlgoNone,
// and the two quantities phase B reuses.
// (T: an SGV or an SGOuter, the outer segment)
template <class TSeg>
__device__ __forceinline__ int tl_phaseA(const SGV& S, const TSeg& T, float& sdlCut, float& mulsF) {
    const uint32_t fs = S.flags, ft = T.flags;
    const bool b1 = fs & F_LO_B, b2 = fs & F_UP_B, b3 = ft & F_LO_B, b4 = ft & F_UP_B;
    const bool e1 = fs & F_LO_E, e2 = fs & F_UP_E, e3 = ft & F_LO_E, e4 = ft & F_UP_E;
    const float rtIn = S.lrt, rtOut = T.lrt, zIn = S.lz, zOut = T.lz;
    if (b1 && b2 && b3 && (b4 || e4)) {
        // Tracklet.cc:902-1132 (cuts 1, 3 and 2)
        const float zpitch_InLo = (fs & F_LO_PS) ? kPixelPSZpitch : kStrip2SZpitch;
        const float zpitch_OutLo = (ft & F_LO_PS) ? kPixelPSZpitch : kStrip2SZpitch;
        const float rtRatio = rtOut / rtIn;
        const float dzDrtScale = T.ltd;
        const float zHi = zIn + (zIn + kDeltaZLum) * (rtRatio - 1.f) * (zIn < 0.f ? 1.f : dzDrtScale) + (zpitch_InLo + zpitch_OutLo);
        const float zLo = zIn + (zIn - kDeltaZLum) * (rtRatio - 1.f) * (zIn > 0.f ? 1.f : dzDrtScale) - (zpitch_InLo + zpitch_OutLo);
        if (!(zOut >= zLo && zOut <= zHi)) return kAlgoNone;
        mulsF = muls_sq(rtOut - rtIn, S.sqq_hi, S.sqq_lo, S.lr3z, rtIn);
        const float sdlMuls = mulsF * 3.f / kPtCut * 4.f;
        const float sdlPVoff = pv_off(T);
        sdlCut = add_dsqrt(T.la1, sdlMuls * sdlMuls + sdlPVoff * sdlPVoff);
        if (!(fabsf(phi_mpi_pi(T.uphi - S.uphi)) <= sdlCut)) return kAlgoNone;
        const float drt_OutLo_InLo = rtOut - rtIn;
        const float drt_InSeg = S.urt - S.lrt;
        const float coshEta = S.cosh;  // (S.ur3 - S.lr3) / drt_InSeg
        float dzErr = (zpitch_InLo + zpitch_OutLo) * (zpitch_InLo + zpitch_OutLo) * 2.f;
        dzErr += sdlMuls * sdlMuls * drt_OutLo_InLo * drt_OutLo_InLo / 3.f * coshEta * coshEta;
        dzErr = __fsqrt_rn(dzErr);
        const float dzMean = S.dzdr * drt_OutLo_InLo;  // dz_InSeg / drt_InSeg * drt_OutLo_InLo
        const float zWindow = dzErr / drt_InSeg * drt_OutLo_InLo + (zpitch_InLo + zpitch_OutLo);
        const float zLoPointed = zIn + dzMean * (zIn > 0.f ? 1.f : dzDrtScale) - zWindow;
        const float zHiPointed = zIn + dzMean * (zIn < 0.f ? 1.f : dzDrtScale) + zWindow;
        if (!(zOut >= zLoPointed && zOut <= zHiPointed)) return kAlgoNone;
        return kAlgoBBBB;
    }
    if (b1 && e3 && e4 && (b2 || e2)) {
        // Tracklet.cc:1540-1720
        const float zGeom = ((fs & F_LO_PS) ? kPixelPSZpitch : kStrip2SZpitch) + ((ft & F_LO_PS) ? kPixelPSZpitch : kStrip2SZpitch);
        const float dzDrtScale = T.ltd;
        if (!(zIn * zOut > 0)) return kAlgoNone;
        const float dLum = f_copysign(kDeltaZLum, zIn);
        const float rtGeom1 = (ft & F_LO_PS) ? kPixelPSZpitch : kStrip2SZpitch;
        const float zGeom1 = f_copysign(zGeom, zIn);
        const float rtLo = rtIn * (1.f + (zOut - zIn - zGeom1) / (zIn + zGeom1 + dLum) / dzDrtScale) - rtGeom1;
        if (!(rtOut >= rtLo)) return kAlgoNone;
        float zInForHi = zIn - zGeom1 - dLum;
        if (zInForHi * zIn < 0) zInForHi = f_copysign(0.1f, zIn);
        const float rtHi = rtIn * (1.f + (zOut - zIn + zGeom1) / zInForHi) + rtGeom1;
        if (!(rtOut >= rtLo && rtOut <= rtHi)) return kAlgoNone;
        const float kZ = (zOut - zIn) / (S.uz - S.lz);
        if (!(kZ >= 0)) return kAlgoNone;
        mulsF = muls_sq(rtOut - rtIn, S.sqq_hi, S.sqq_lo, S.lr3z, rtIn);
        const float sdlMuls = mulsF * 3.f / kPtCut * 4.f;
        const float sdlPVoff = pv_off(T);
        sdlCut = add_dsqrt(T.la1, sdlMuls * sdlMuls + sdlPVoff * sdlPVoff);
        if (!(fabsf(phi_mpi_pi(T.uphi - S.uphi)) <= sdlCut)) return kAlgoNone;
        return kAlgoBBEE;
    }
    if (e1 && e2 && e3 && e4) {
        // Tracklet.cc:2018-2218
        const float dzDrtScale = T.ltd;
        if (!(zIn * zOut > 0)) return kAlgoNone;
        const float dLum = f_copysign(kDeltaZLum, zIn);
        const bool inPS = fs & F_LO_PS, outPS = ft & F_LO_PS;
        const float rtGeom = (inPS && outPS) ? 2.f * kPixelPSZpitch : (inPS || outPS) ? (kPixelPSZpitch + kStrip2SZpitch) : 2.f * kStrip2SZpitch;
        const float dz = zOut - zIn;
        const float rtLo = rtIn * (1.f + dz / (zIn + dLum) / dzDrtScale) - rtGeom;
        if (!(rtOut >= rtLo)) return kAlgoNone;
        const float rtHi = rtIn * (1.f + dz / (zIn - dLum)) + rtGeom;
        if (!(rtOut >= rtLo && rtOut <= rtHi)) return kAlgoNone;
        mulsF = muls(rtOut - rtIn, 0.f, false);
        const float sdlMuls = mulsF * 3.f / kPtCut * 4.f;
        const float sdlPVoff = pv_off(T);
        sdlCut = add_dsqrt(T.la1, sdlMuls * sdlMuls + sdlPVoff * sdlPVoff);
        if (!(fabsf(phi_mpi_pi(T.uphi - S.uphi)) <= sdlCut)) return kAlgoNone;
        if (inPS && (fs & F_UP_PS)) {
            const float drtSDIn = S.urt - S.lrt;
            const float dzSDIn = S.uz - S.lz;
            const float coshEta = S.cosh;  // (S.ur3 - S.lr3) / drtSDIn
            const float dzOutInAbs = fabsf(zOut - zIn);
            const float multDzDr = dzOutInAbs * coshEta / (coshEta * coshEta - 1.f);
            const float kZ = (zOut - zIn) / dzSDIn;
            float drtErr = kPixelPSZpitch * kPixelPSZpitch * 2.f / dzSDIn / dzSDIn * dzOutInAbs * dzOutInAbs;
            drtErr += sdlMuls * sdlMuls * multDzDr * multDzDr / 3.f * coshEta * coshEta;
            drtErr = __fsqrt_rn(drtErr);
            const float drtMean = drtSDIn * dzOutInAbs / fabsf(dzSDIn);
            const float rtWindow = drtErr + rtGeom;
            const float rtLo_point = rtIn + drtMean / dzDrtScale - rtWindow;
            const float rtHi_point = rtIn + drtMean + rtWindow;
            if (!(kZ >= 0 && rtOut >= rtLo_point && rtOut <= rtHi_point)) return kAlgoNone;
        }
        return kAlgoEEEE;
    }
    return kAlgoNone;
}

// The two quantities phase A hands to phase B for a candidate it accepts
// with algorithm algo: the multiple-scattering factor and the width of the
// phi cut (Tracklet.cc:1049-1057, 1669-1677, 2127-2135), exactly as
// tl_phaseA computes them.
template <class TSeg>
__device__ __forceinline__ void tl_cut_values(int algo, const SGV& S, const TSeg& T, float& sdlCut, float& mulsF) {
    const float rtIn = S.lrt, rtOut = T.lrt;
    mulsF = algo == kAlgoEEEE ? muls(rtOut - rtIn, 0.f, false) : muls_sq(rtOut - rtIn, S.sqq_hi, S.sqq_lo, S.lr3z, rtIn);
    const float sdlMuls = mulsF * 3.f / kPtCut * 4.f;
    const float sdlPVoff = pv_off(T);
    sdlCut = add_dsqrt(T.la1, sdlMuls * sdlMuls + sdlPVoff * sdlPVoff);
}

// ---- phase A's decision alone, from single-precision approximations of the
// multiple-scattering factor and of the quantities built on it (the phi-cut
// width, the pointed z window of BBBB, the pointed rt window of EEEE with PS
// inner modules).  Everything else is the exact float arithmetic of
// tl_phaseA.  The approximation of the factor, 0.015 sqrt(0.1 + 0.004 d) [x
// sqrt(q)] with sqrt(u) = u * rsqrtf(u) (rsqrtf: at most 2 ulp), is within
// 11 * 2^-24 of the exact float, and every quantity compared is then within
// 2^-24 * 53 * (the sum of the magnitudes of its terms) of its exact value
// (3 of the 53 from the pointed windows' square roots as u * rsqrtf(u)).
// A comparison is decided here only when it holds by kQuickMargin times that
// sum (2^-16: over 4.8 times the bound); otherwise, and for NaNs or the
// exact functions' fallback ranges, the result is kAlgoUnsure and the caller
// runs tl_phaseA.  Returns the algorithm, kAlgoNone or kAlgoUnsure.
constexpr int kAlgoUnsure = -1;
constexpr float kQuickMargin = 0x1p-16f;

// sdlMuls = mulsF * 3 / ptCut * 4 from the approximate factor (NaN when d is
// outside the exact function's fast range or sq is NaN)
__device__ __forceinline__ float sdl_muls_quick(float d, float sq) {
    if (!(d >= 0.f && d < 1e4f)) return __int_as_float(0x7fc00000);
    const float u = __fadd_rn(0.1f, __fmul_rn(d, 0.004f));
    const float m = __fmul_rn(__fmul_rn(0.015f, __fmul_rn(u, rsqrtf(u))), sq);
    return m * 3.f / kPtCut * 4.f;
}
// |dphi| <= la1 + sqrt(sdlMuls^2 + pvoff^2): 1 holds, 0 fails, -1 not
// decided.  cut: the approximate width (within 25 * 2^-24 * (|la1| + r) of
// the exact one, below 3e-6 where it is set), NaN where |la1| + r >= 2.
__device__ __forceinline__ int phi_cut_quick(float adphi, float la1, float sdlMuls, float pvoff, float& cut) {
    cut = __int_as_float(0x7fc00000);
    const float y = sdlMuls * sdlMuls + pvoff * pvoff;
    if (!(y > 0x1p-100f && y < 0x1p100f)) return -1;
    const float r = __fmul_rn(y, rsqrtf(y));
    const float c = la1 + r;
    const float m = kQuickMargin * (fabsf(la1) + r);
    if (fabsf(la1) + r < 2.f) cut = c;
    if (adphi > c + m) return 0;
    if (adphi < c - m) return 1;
    return -1;
}
// lo <= v <= hi with both bounds within m of their exact values
__device__ __forceinline__ int window_quick(float v, float lo, float hi, float m) {
    if (v < lo - m || v > hi + m) return 0;
    if (v >= lo + m && v <= hi - m) return 1;
    return -1;
}

template <class TSeg>
__device__ __forceinline__ int tl_phaseA_quick(const SGV& S, const TSeg& T, float& cut) {
    cut = __int_as_float(0x7fc00000);
    const uint32_t fs = S.flags, ft = T.flags;
    const bool b1 = fs & F_LO_B, b2 = fs & F_UP_B, b3 = ft & F_LO_B, b4 = ft & F_UP_B;
    const bool e1 = fs & F_LO_E, e2 = fs & F_UP_E, e3 = ft & F_LO_E, e4 = ft & F_UP_E;
    const float rtIn = S.lrt, rtOut = T.lrt, zIn = S.lz, zOut = T.lz;
    if (b1 && b2 && b3 && (b4 || e4)) {
        const float zpitch_InLo = (fs & F_LO_PS) ? kPixelPSZpitch : kStrip2SZpitch;
        const float zpitch_OutLo = (ft & F_LO_PS) ? kPixelPSZpitch : kStrip2SZpitch;
        const float rtRatio = rtOut / rtIn;
        const float dzDrtScale = T.ltd;
        const float zHi = zIn + (zIn + kDeltaZLum) * (rtRatio - 1.f) * (zIn < 0.f ? 1.f : dzDrtScale) + (zpitch_InLo + zpitch_OutLo);
        const float zLo = zIn + (zIn - kDeltaZLum) * (rtRatio - 1.f) * (zIn > 0.f ? 1.f : dzDrtScale) - (zpitch_InLo + zpitch_OutLo);
        if (!(zOut >= zLo && zOut <= zHi)) return kAlgoNone;
        const float sdlMuls = sdl_muls_quick(rtOut - rtIn, S.sqq_hi);
        const int c3 = phi_cut_quick(fabsf(phi_mpi_pi(T.uphi - S.uphi)), T.la1, sdlMuls, pv_off(T), cut);
        if (c3 <= 0) return c3 == 0 ? kAlgoNone : kAlgoUnsure;
        const float drt_OutLo_InLo = rtOut - rtIn;
        const float drt_InSeg = S.urt - S.lrt;
        const float coshEta = S.cosh;
        const float zp = zpitch_InLo + zpitch_OutLo;
        // (the two quotients by __fdividef: 2 ulp instead of 0.5, inside the bound)
        float dzErr = zp * zp * 2.f;
        dzErr += __fdividef(sdlMuls * sdlMuls * drt_OutLo_InLo * drt_OutLo_InLo, 3.f) * coshEta * coshEta;
        dzErr = dzErr * rsqrtf(dzErr);  // (>= 2 zp^2 > 0; 3 ulp, inside the margin)
        const float dzMean = S.dzdr * drt_OutLo_InLo;
        const float pw = __fdividef(dzErr, drt_InSeg) * drt_OutLo_InLo;
        const float zWindow = pw + zp;
        const float mLo = dzMean * (zIn > 0.f ? 1.f : dzDrtScale), mHi = dzMean * (zIn < 0.f ? 1.f : dzDrtScale);
        const float zLoPointed = zIn + mLo - zWindow;
        const float zHiPointed = zIn + mHi + zWindow;
        const float m = kQuickMargin * (fabsf(zIn) + fabsf(mLo) + fabsf(mHi) + 2.f * (fabsf(pw) + zp));
        const int c2 = window_quick(zOut, zLoPointed, zHiPointed, m);
        return c2 > 0 ? kAlgoBBBB : (c2 == 0 ? kAlgoNone : kAlgoUnsure);
    }
    if (b1 && e3 && e4 && (b2 || e2)) {
        const float zGeom = ((fs & F_LO_PS) ? kPixelPSZpitch : kStrip2SZpitch) + ((ft & F_LO_PS) ? kPixelPSZpitch : kStrip2SZpitch);
        const float dzDrtScale = T.ltd;
        if (!(zIn * zOut > 0)) return kAlgoNone;
        const float dLum = f_copysign(kDeltaZLum, zIn);
        const float rtGeom1 = (ft & F_LO_PS) ? kPixelPSZpitch : kStrip2SZpitch;
        const float zGeom1 = f_copysign(zGeom, zIn);
        const float rtLo = rtIn * (1.f + (zOut - zIn - zGeom1) / (zIn + zGeom1 + dLum) / dzDrtScale) - rtGeom1;
        if (!(rtOut >= rtLo)) return kAlgoNone;
        float zInForHi = zIn - zGeom1 - dLum;
        if (zInForHi * zIn < 0) zInForHi = f_copysign(0.1f, zIn);
        const float rtHi = rtIn * (1.f + (zOut - zIn + zGeom1) / zInForHi) + rtGeom1;
        if (!(rtOut >= rtLo && rtOut <= rtHi)) return kAlgoNone;
        const float kZ = (zOut - zIn) / (S.uz - S.lz);
        if (!(kZ >= 0)) return kAlgoNone;
        const float sdlMuls = sdl_muls_quick(rtOut - rtIn, S.sqq_hi);
        const int c3 = phi_cut_quick(fabsf(phi_mpi_pi(T.uphi - S.uphi)), T.la1, sdlMuls, pv_off(T), cut);
        return c3 > 0 ? kAlgoBBEE : (c3 == 0 ? kAlgoNone : kAlgoUnsure);
    }
    if (e1 && e2 && e3 && e4) {
        const float dzDrtScale = T.ltd;
        if (!(zIn * zOut > 0)) return kAlgoNone;
        const float dLum = f_copysign(kDeltaZLum, zIn);
        const bool inPS = fs & F_LO_PS, outPS = ft & F_LO_PS;
        const float rtGeom = (inPS && outPS) ? 2.f * kPixelPSZpitch : (inPS || outPS) ? (kPixelPSZpitch + kStrip2SZpitch) : 2.f * kStrip2SZpitch;
        const float dz = zOut - zIn;
        const float rtLo = rtIn * (1.f + dz / (zIn + dLum) / dzDrtScale) - rtGeom;
        if (!(rtOut >= rtLo)) return kAlgoNone;
        const float rtHi = rtIn * (1.f + dz / (zIn - dLum)) + rtGeom;
        if (!(rtOut >= rtLo && rtOut <= rtHi)) return kAlgoNone;
        const float sdlMuls = sdl_muls_quick(rtOut - rtIn, 1.f);
        const int c3 = phi_cut_quick(fabsf(phi_mpi_pi(T.uphi - S.uphi)), T.la1, sdlMuls, pv_off(T), cut);
        if (c3 <= 0) return c3 == 0 ? kAlgoNone : kAlgoUnsure;
        if (inPS && (fs & F_UP_PS)) {
            const float drtSDIn = S.urt - S.lrt;
            const float dzSDIn = S.uz - S.lz;
            const float coshEta = S.cosh;
            const float dzOutInAbs = fabsf(zOut - zIn);
            const float multDzDr = dzOutInAbs * coshEta / (coshEta * coshEta - 1.f);
            const float kZ = (zOut - zIn) / dzSDIn;
            if (!(kZ >= 0)) return kAlgoNone;
            float drtErr = kPixelPSZpitch * kPixelPSZpitch * 2.f / dzSDIn / dzSDIn * dzOutInAbs * dzOutInAbs;
            drtErr += sdlMuls * sdlMuls * multDzDr * multDzDr / 3.f * coshEta * coshEta;
            drtErr = drtErr * rsqrtf(drtErr);  // (3 ulp, inside the margin; NaN for 0: undecided)
            const float drtMean = drtSDIn * dzOutInAbs / fabsf(dzSDIn);
            const float rtWindow = drtErr + rtGeom;
            const float mLo = drtMean / dzDrtScale;
            const float rtLo_point = rtIn + mLo - rtWindow;
            const float rtHi_point = rtIn + drtMean + rtWindow;
            const float m = kQuickMargin * (fabsf(rtIn) + fabsf(mLo) + fabsf(drtMean) + 2.f * fabsf(rtWindow));
            const int c2 = window_quick(rtOut, rtLo_point, rtHi_point, m);
            return c2 > 0 ? kAlgoEEEE : (c2 == 0 ? kAlgoNone : kAlgoUnsure);
        }
        return kAlgoEEEE;
    }
    return kAlgoNone;
}

// Phase B1 decides most candidates from single-precision approximations of
// its two angles: atan2f for the directions and asinf for the betaIn cut's
// asin, whose errors CUDA documents as at most 3 and 2 ulp.  The exact values
// are the floats nearest the reference's double evaluations; for angles
// below pi the two differ by about 1e-6 at most, and the compared quantities
// (a difference of two directions wrapped into [-pi, pi], minus a float;
// an asin plus a float) by a few 1e-6.  A comparison is decided from the
// approximations only when it holds by kB1Margin (about 400 ulp of pi), and
// only away from the wrap at +-pi; otherwise the exact evaluation decides.
// The self-check (functions 16 and 17 of k_math_check) bounds both
// approximation errors by 2e-6 on the GPU itself.
constexpr float kB1Margin = 1e-4f;

// approximate direction of (x, y) (Hit.cc:68-83's phi), or false when the
// point is at the origin, tiny, huge or not finite
__device__ __forceinline__ bool phi_approx(float x, float y, float& p) {
    const float m = fabsf(x) + fabsf(y);
    if (!(m > 0x1p-60f && m < 0x1p60f)) return false;
    p = atan2f(y, x);
    return true;
}
// atan(q) for q in [0, 1] as q * P(q^2) with P of degree 5, fitted to atan
// near-minimax (least squares at Chebyshev nodes, reweighted by the error)
// and rounded to float: evaluated in float as below, within 1.76e-6 of
// atan(q) for every float q in [0, 1] (tests/test_atan_approx.py runs them
// all with these coefficients)
__device__ constexpr float kAtanP[6] = {0.999977231f, -0.332622826f, 0.193540379f, -0.116426416f, 0.052647233f,
                                       -0.0117190806f};
__device__ __forceinline__ float atan01_approx(float q) {
    const float s = __fmul_rn(q, q);
    float p = kAtanP[5];
#pragma unroll
    for (int k = 4; k >= 0; --k) p = __fadd_rn(__fmul_rn(p, s), kAtanP[k]);
    return __fmul_rn(q, p);
}
// direction of (x, y) from atan01_approx: q = min / max by __fdividef (2 ulp,
// below 1.2e-7 in q), then pi/2 - r and pi - r in float (constants and
// roundings below 4.2e-7): within 2.5e-6 of atan2(y, x); false where
// phi_approx is false
__device__ __forceinline__ bool phi_fast(float x, float y, float& p) {
    const float ax = fabsf(x), ay = fabsf(y);
    const float m = ax + ay;
    if (!(m > 0x1p-60f && m < 0x1p60f)) return false;
    float r = atan01_approx(__fdividef(fminf(ax, ay), fmaxf(ax, ay)));
    if (ay > ax) r = 1.57079637f - r;
    if (x < 0.f) r = 3.14159274f - r;
    p = copysignf(r, y);
    return true;
}

// a difference of two directions in [-pi, pi], into [-pi, pi]
__device__ __forceinline__ float wrap_approx(float d) {
    return d > kPiF ? d - 2.f * kPiF : (d < -kPiF ? d + 2.f * kPiF : d);
}
// 1 when |v| < cut (or <= cut) holds by the margin, 0 when it fails by the
// margin, -1 when the approximations cannot tell (v or cut not usable)
__device__ __forceinline__ int clear_within(float v, float cut) {
    const float a = fabsf(v);
    if (!(a < 3.f && fabsf(cut) < 3.f)) return -1;
    if (a > cut + kB1Margin) return 0;
    if (a < cut - kB1Margin) return 1;
    return -1;
}

// ---- phase B1: the mid-point direction cut and the betaIn cut
// (Tracklet.cc:1139-1222 BBBB, 1765-1819 BBEE, 2258-2292 EEEE; EEEE has no
// betaIn cut).  Its code is the same for the three algorithms.
__device__ __forceinline__ bool tl_phaseB1_sgv(int algo, const SGV& S, const SGV& T, float sdlCut) {
    // cut #5: dphi(midpoint(InLo, OutLo), OutLo - InLo) (the same float
    // operations as midpoint() and sub())
    float mx = 0.f, my = 0.f;
    mx += S.lx; my += S.ly;
    mx += T.lx; my += T.ly;
    mx /= 2.f; my /= 2.f;
    const float dx = T.lx - S.lx, dy = T.ly - S.ly;
    int c5 = -1;
    float pm, pd;
    if (phi_approx(mx, my, pm) && phi_approx(dx, dy, pd)) c5 = clear_within(wrap_approx(pd - pm), sdlCut);
    if (c5 < 0) {
        const P3 InLo = S.lo(), OutLo = T.lo();
        const float dPhi = dphi(midpoint(InLo, OutLo), sub(OutLo, InLo));
        c5 = fabsf(dPhi) <= sdlCut ? 1 : 0;
    }
    if (!c5) return false;
    if (algo == kAlgoEEEE) return true;
    // betaIn = alphaIn - dphi(InLo, axis), axis = OutUp - InLo (tl_axis / dr3);
    // betaIn_cut = asin(min((-sdIn_dr + dr) k / ptCut, sinAlphaMax)) + 0.02 / sdIn_d
    const float ax = T.ux - S.lx, ay = T.uy - S.ly;
    const float dr = __fsqrt_rn(__fadd_rn(__fmul_rn(ax, ax), __fmul_rn(ay, ay)));  // as mk2()
    const float sdIn_d = S.urt - S.lrt;
    const float arg = fmin_ref((-S.rtseg * 1.f + dr) * k2Rinv1GeVf / kPtCut, kSinAlphaMax);
    int cb = -1;
    float pa;
    if (phi_approx(ax, ay, pa) && fabsf(arg) <= kSinAlphaMax) {
        const float w = wrap_approx(pa - S.lphi);
        if (fabsf(w) < 3.f) cb = clear_within(S.dpc - w, asinf(arg) + (0.02f / sdIn_d));
    }
    if (cb < 0) {
        const P3 InLo = S.lo();
        const float betaIn = S.dpc - dphi(InLo, sub(T.up(), InLo));
        cb = fabsf(betaIn) < g_asin(arg) + (0.02f / sdIn_d) ? 1 : 0;  // betaInRHmin == betaIn here
    }
    return cb != 0;
}
static __device__ __noinline__ bool tl_phaseB1(int algo, const float* __restrict__ pack, int s, int t, float sdlCut) {
    return tl_phaseB1_sgv(algo, load_sgv(pack, s), load_sgv(pack, t), sdlCut);
}
// Phase B1 from the approximations alone, with an approximate phi-cut width
// (tl_phaseA_quick's, within 3e-6 of the exact one, or the exact one): the
// directions (phi_fast) are within 2.5e-6 of the exact angles and asinf
// within 2e-6 (functions 20 and 17 of the math self-check), so with the
// width's error every comparison clear_within decides holds by over 9e-5 in
// exact arithmetic as well, and the result is tl_phaseB1_sgv's.  txy: the outer segment's (lx, ly, ux, uy).
// 1: passes, 0: fails, -1: left to tl_phaseB1_sgv (NaN width included).
__device__ __forceinline__ int tl_phaseB1_quick(int algo, const SGV& S, float4 txy, float cut) {
    float mx = 0.f, my = 0.f;
    mx += S.lx; my += S.ly;
    mx += txy.x; my += txy.y;
    mx /= 2.f; my /= 2.f;
    const float dx = txy.x - S.lx, dy = txy.y - S.ly;
    // the angle from the mid-point direction M to D = OutLo - InLo as one
    // atan2 of (M x D, M . D): the rounding of the cross and dot products
    // (below 2^-23 |M| |D| each) moves it by under 2^-22 whatever the lengths,
    // so it is within 4e-6 of the reference's difference of the two
    // directions wrapped into [-pi, pi] away from the wrap
    if (!(fabsf(mx) + fabsf(my) > 0x1p-40f && fabsf(mx) + fabsf(my) < 0x1p40f && fabsf(dx) + fabsf(dy) > 0x1p-40f &&
          fabsf(dx) + fabsf(dy) < 0x1p40f))
        return -1;
    float v;
    if (!phi_fast(mx * dx + my * dy, mx * dy - my * dx, v)) return -1;
    const int c5 = clear_within(v, cut);
    if (c5 <= 0 || algo == kAlgoEEEE) return c5;
    const float ax = txy.z - S.lx, ay = txy.w - S.ly;
    const float dr2 = __fadd_rn(__fmul_rn(ax, ax), __fmul_rn(ay, ay));
    const float dr = dr2 * rsqrtf(dr2);  // (3 ulp: a few 1e-7 on the angle, far inside kB1Margin; NaN for 0: undecided)
    const float sdIn_d = S.urt - S.lrt;
    const float arg = fmin_ref((-S.rtseg * 1.f + dr) * k2Rinv1GeVf / kPtCut, kSinAlphaMax);
    float pa;
    if (!(phi_fast(ax, ay, pa) && fabsf(arg) <= kSinAlphaMax)) return -1;
    const float w = wrap_approx(pa - S.lphi);
    if (!(fabsf(w) < 3.f) || !(fabsf(sdIn_d) > 1e-3f)) return -1;
    return clear_within(S.dpc - w, asinf(arg) + __fdividef(0.02f, sdIn_d));  // 2 ulp of at most 20
}

// the multiple-scattering factor of a candidate whose phase B1 passed already
static __device__ __noinline__ float tl_muls_entry(int algo, const float* __restrict__ pack, int s, int t) {
    const float rtIn = __ldg(pack + (int64_t)s * PK_N + PK_LRT), rtOut = __ldg(pack + (int64_t)t * PK_N + PK_LRT);
    if (algo == kAlgoEEEE) return muls(rtOut - rtIn, 0.f, false);
    return muls_sq(rtOut - rtIn, __ldg(pack + (int64_t)s * PK_N + PK_S2), __ldg(pack + (int64_t)s * PK_N + PK_S3),
                   __ldg(pack + (int64_t)s * PK_N + PK_LR3Z), rtIn);
}

// phase B1 of a candidate through phase A (tl_phaseA_quick's survivors carry
// no cut values): the exact phi-cut width and multiple-scattering factor
// (tl_cut_values), then the cuts; the factor goes on to phase B2
struct B1Result {
    bool pass;
    float muls;
};
static __device__ __noinline__ B1Result tl_phaseB1_entry(int algo, const float* __restrict__ pack, int s, int t) {
    const SGV S = load_sgv(pack, s), T = load_sgv(pack, t);
    float cut, muls;
    tl_cut_values(algo, S, T, cut, muls);
    return B1Result{tl_phaseB1_sgv(algo, S, T, cut), muls};
}

// ---- phase B2: betaIn, betaOut, the deltaBeta iterations, the betaOut cut
// and the deltaBeta cut, on the candidates through phase B1 (exact values
// throughout).  kSet restricts the algorithms compiled in (kB2All, kB2BBBB:
// BBBB only, kB2Others: BBEE and EEEE), so that a kernel running one group
// keeps only that code resident.
enum : int { kB2All = 0, kB2BBBB = 1, kB2Others = 2 };
// The tracklet's final cut variables as the reference records them
// (Tracklet.cc:1440-1495 and the same block of the other algorithms), in the
// order of the kTLVar* names
enum : int {
    kTLVarBetaIn, kTLVarBetaInRHmin, kTLVarBetaInRHmax, kTLVarBetaOut, kTLVarBetaOutRHmin, kTLVarBetaOutRHmax,
    kTLVarBetaAv, kTLVarPtBeta, kTLVarDBeta, kTLVarDBetaCut2, kTLVarDBetaLum2, kTLVarDBetaMuls, kTLVarDBetaRes,
    kTLVarDBetaRIn2, kTLVarDBetaROut2, kTLVarN
};

// rec (optional, kTLVarN floats): the final cut variables of a candidate
// that reaches the deltaBeta cut
template <int kSet>
__device__ __forceinline__ bool tl_phaseB2_sgv(int algo, const SGV& S, const SGV& T, float mulsF, bool nm1,
                                               float* rec = nullptr) {
    if (kSet == kB2BBBB) algo = kAlgoBBBB;
    if (kSet == kB2Others && algo == kAlgoBBBB) return false;
    const float pt_betaMax = 7.0f;
    const P3 InLo = S.lo(), InUp = S.up(), OutLo = T.lo(), OutUp = T.up();
    const P3 axis = sub(OutUp, InLo);
    float betaIn = S.dpc - dphi(InLo, axis);
    const float dr = axis.rt;
    const float sdIn_dr = S.rtseg;
    const float sdIn_d = InUp.rt - InLo.rt;
    const float sdOut_dr = T.rtseg;
    const float sdOut_d = OutUp.rt - OutLo.rt;
    const float alphaIn = S.dpc;
    float betaOut, betaInRHmin, betaInRHmax, betaOutRHmin, betaOutRHmax;
    float alphaOutReg;
    int lIn, lOut;
    float dBetaROut2 = 0.f;
    if (kSet != kB2Others && algo == kAlgoBBBB) {
        // Tracklet.cc:1205-1538
        betaInRHmin = betaIn; betaInRHmax = betaIn;
        betaOut = -T.alphaup + dphi(OutUp, axis);
        const bool ec2s = (T.flags & F_UP_E) && (T.flags & F_UP_2S);
        if (ec2s) {
            const P3 hiE = edge_point(OutUp.x, OutUp.y, OutUp.z, T.ex, T.ey, true);
            const P3 loE = edge_point(OutUp.x, OutUp.y, OutUp.z, T.ex, T.ey, false);
            betaOutRHmin = -dphi(hiE, sub(hiE, OutLo)) + dphi(hiE, sub(hiE, InLo));
            betaOutRHmax = -dphi(loE, sub(loE, OutLo)) + dphi(loE, sub(loE, InLo));
            const float sinDPhi = g_sin(dphi(midpoint(InLo, OutLo), sub(OutLo, InLo)));
            const float rr = (hiE.rt - loE.rt) * sinDPhi / dr;
            dBetaROut2 = rr * rr;  // the double square of a float is exact: one rounding to float
        } else {
            // (rt - rt) * sin(dPhi) / dr squared: sin(dPhi) is finite here
            // (|dPhi| <= sdlCut), so the product is a signed zero and only
            // its square matters
            betaOutRHmin = betaOut; betaOutRHmax = betaOut;
            const float rr = (OutUp.rt - OutUp.rt) * 0.f / dr;
            dBetaROut2 = rr * rr;
        }
        alphaOutReg = T.dpc;
        lIn = 5;
        lOut = ec2s ? 11 : 5;
    } else if (kSet != kB2BBBB && algo == kAlgoBBEE) {
        // Tracklet.cc:1765-2016
        const float sdOut_alphaOut = T.alphaup;
        const float sdOut_alphaOut_min = phi_mpi_pi(T.dpminc - T.dpmin);
        const float sdOut_alphaOut_max = phi_mpi_pi(T.dpmaxc - T.dpmax);
        betaOut = -sdOut_alphaOut + dphi(OutUp, axis);
        betaInRHmin = betaIn; betaInRHmax = betaIn;  // isEC_secondLayer is always false (Tracklet.cc:1798)
        betaOutRHmin = betaOut - sdOut_alphaOut_min + sdOut_alphaOut;
        betaOutRHmax = betaOut - sdOut_alphaOut_max + sdOut_alphaOut;
        if (fabsf(betaOutRHmin) > fabsf(betaOutRHmax)) { const float t = betaOutRHmin; betaOutRHmin = betaOutRHmax; betaOutRHmax = t; }
        if (T.flags & F_UP_2S) {
            const float sinDPhi = g_sin(dphi(midpoint(InLo, OutLo), sub(OutLo, InLo)));
            const float hrt = edge_rt(OutUp.x, OutUp.y, T.ex, T.ey, true);
            const float lrt = edge_rt(OutUp.x, OutUp.y, T.ex, T.ey, false);
            const float rr = (hrt - lrt) * sinDPhi / dr;
            dBetaROut2 = rr * rr;
        } else {
            const float rr = (OutUp.rt - OutUp.rt) * 0.f / dr;  // see the BBBB branch
            dBetaROut2 = rr * rr;
        }
        alphaOutReg = S.dpc;  // sdOut_alpha is the inner segment's (Tracklet.cc:1790)
        lIn = 5;
        lOut = 11;
    } else {
        // Tracklet.cc:2220-2665
        const float sdOut_dPhiPos = T.dphilu;
        const float sdOut_alphaOutRHmin = phi_mpi_pi(T.dpminc - sdOut_dPhiPos);
        const float sdOut_alphaOutRHmax = phi_mpi_pi(T.dpmaxc - sdOut_dPhiPos);
        const float sdOut_alphaOut = phi_mpi_pi(T.dpc - sdOut_dPhiPos);
        betaOut = -sdOut_alphaOut + dphi(OutUp, axis);
        betaInRHmin = betaIn + S.dpminc - alphaIn;
        betaInRHmax = betaIn + S.dpmaxc - alphaIn;
        if (fabsf(betaInRHmin) > fabsf(betaInRHmax)) { const float t = betaInRHmin; betaInRHmin = betaInRHmax; betaInRHmax = t; }
        betaOutRHmin = betaOut - sdOut_alphaOutRHmin + sdOut_alphaOut;
        betaOutRHmax = betaOut - sdOut_alphaOutRHmax + sdOut_alphaOut;
        if (fabsf(betaOutRHmin) > fabsf(betaOutRHmax)) { const float t = betaOutRHmin; betaOutRHmin = betaOutRHmax; betaOutRHmax = t; }
        // cut #6 never rejects here (Tracklet.cc:2327-2336)
        alphaOutReg = S.dpc;  // (sic)
        lIn = 11;
        lOut = 13;
    }
    float betaAv = 0.5f * (betaIn + betaOut);
    float pt_beta = pt_from(dr * k2Rinv1GeVf, betaAv);
    delta_beta_iterations(betaIn, betaOut, betaAv, pt_beta, sdIn_dr, sdOut_dr, dr, lIn, pt_betaMax);
    const float betaInMMSF = (fabsf(betaInRHmin + betaInRHmax) > 0) ? (2.f * betaIn / fabsf(betaInRHmin + betaInRHmax)) : 0.f;
    const float betaOutMMSF = (fabsf(betaOutRHmin + betaOutRHmax) > 0) ? (2.f * betaOut / fabsf(betaOutRHmin + betaOutRHmax)) : 0.f;
    betaInRHmin *= betaInMMSF; betaInRHmax *= betaInMMSF;
    betaOutRHmin *= betaOutMMSF; betaOutRHmax *= betaOutMMSF;
    const float dBetaMuls = mulsF * 4.f / fmin_ref(fabsf(pt_beta), pt_betaMax);
    const float alphaInAbsReg = fmax_ref(fabsf(alphaIn), S.la3);
    const float alphaOutAbsReg = fmax_ref(fabsf(alphaOutReg), T.la3);
    const float dBetaInLum = lIn < 11 ? 0.0f : fabsf(alphaInAbsReg * kDeltaZLum / InLo.z);
    const float dBetaOutLum = lOut < 11 ? 0.0f : fabsf(alphaOutAbsReg * kDeltaZLum / OutLo.z);
    const float dBetaLum2 = (dBetaInLum + dBetaOutLum) * (dBetaInLum + dBetaOutLum);
    const float betaOut_cut = add_dsqrt(g_asin(fmin_ref(dr * k2Rinv1GeVf / kPtCut, kSinAlphaMax)) + (0.02f / sdOut_d),
                                        dBetaLum2 + dBetaMuls * dBetaMuls);
    if (!(fabsf(betaOut) < betaOut_cut)) return false;
    const float dBetaRes = 0.02f / fmin_ref(sdOut_d, sdIn_d);
    const float dBetaCut2 = dbeta_cut2(dBetaRes, dBetaMuls, dBetaLum2, dBetaROut2, betaInRHmin, betaInRHmax, betaOutRHmin, betaOutRHmax);
    const float dBeta = betaIn - betaOut;
    if (rec) {
        rec[kTLVarBetaIn] = betaIn; rec[kTLVarBetaInRHmin] = betaInRHmin; rec[kTLVarBetaInRHmax] = betaInRHmax;
        rec[kTLVarBetaOut] = betaOut; rec[kTLVarBetaOutRHmin] = betaOutRHmin; rec[kTLVarBetaOutRHmax] = betaOutRHmax;
        rec[kTLVarBetaAv] = betaAv; rec[kTLVarPtBeta] = pt_beta; rec[kTLVarDBeta] = dBeta;
        rec[kTLVarDBetaCut2] = dBetaCut2; rec[kTLVarDBetaLum2] = dBetaLum2; rec[kTLVarDBetaMuls] = dBetaMuls;
        rec[kTLVarDBetaRes] = dBetaRes; rec[kTLVarDBetaRIn2] = 0.f; rec[kTLVarDBetaROut2] = dBetaROut2;
    }
    return (dBeta * dBeta <= dBetaCut2) || nm1;
}
template <int kSet>
static __device__ __noinline__ bool tl_phaseB2(int algo, const float* __restrict__ pack, int s, int t, float mulsF,
                                                bool nm1) {
    return tl_phaseB2_sgv<kSet>(algo, load_sgv(pack, s), load_sgv(pack, t), mulsF, nm1);
}

// ---- Phase B2's decision from single-precision approximations: a filter
// ahead of the exact phases B1 and B2 (no counterpart in the reference).  The
// directions come from atan2f and the deltaBeta iterations' functions from
// asinf and __sinf (CUDA: at most 3 and 2 ulp, and 2^-21.41 absolute on
// [-pi, pi]) instead of the host libm and the double sub-expressions; every
// other input is the exact code's own float (the packed segment fields, dr,
// sdOut_d, the luminous-region terms, dBetaRes, the alpha terms of the BBEE
// and EEEE algorithms).  Each compared quantity carries a bound on its
// distance to the exact value, propagated through the iterations with the
// derivatives of asin and 1/sin, and every bound is taken kB2qSafety times at
// the decisions: a candidate is rejected only when a cut fails by more than
// that, and a branch condition within its bound, a non-finite value or an
// angle too close to the wrap at +-pi leaves it to the exact phases.  So the
// tracklets do not change; the filter only spares the exact phases the
// candidates that certainly fail.  Returns 0 (phase B2 rejects the candidate),
// 3 (phase B2 accepts it: both cuts hold by more than their bounds, so the
// exact phase need not run), or 1 (not decided here); with kDefer, 2 for the
// entries whose evaluation
// takes the long branches (BBEE and EEEE, and BBBB with a 2S endcap outer
// anchor, about one entry in six), which a second pass evaluates on full
// warps instead of holding a warp of the common case for one lane.
// (the bounds' own arithmetic uses __fdividef and rsqrtf, within 2 and 2 ulp,
// and widens its results by a relative 1e-6; the few quantities the exact
// code computes with the same float operations keep IEEE division)


// pt = D / sin(b) (approximate) and bounds [lo, hi] of |D / sin(b')| over
// every b' within e of b
__device__ __forceinline__ float pt_range(float D, float b, float e, float& lo, float& hi) {
    const float sb = __sinf(b), s = fabsf(sb);  // |b| <= pi here
    const float es = e + kB2qSin + 2.f * ulp_of(s) + 1e-30f;
    lo = __fdividef(D, s + es) * (1.f - 1e-6f);
    hi = s > es ? __fdividef(D, s - es) * (1.f + 1e-6f) : __int_as_float(0x7f800000);
    return __fdividef(D, sb);
}
// 1: |pt| < c for every pt in [lo, hi]; 0: for none; -1: not decided
__device__ __forceinline__ int pt_below(float lo, float hi, float c) { return hi < c ? 1 : (lo >= c ? 0 : -1); }

// one update of the deltaBeta iterations, asin(min(a / |pt|, 0.95)) with a =
// sd_dr * k, for |pt| = p (approximate) within [lo, hi]: value and bound
__device__ __forceinline__ float b2q_update(float a, float p, float lo, float hi, float& e) {
    const float arg = fmin_ref(__fdividef(a, fabsf(p)), kSinAlphaMax);
    const float alo = fmin_ref(__fdividef(a, hi) * (1.f - 1e-6f), kSinAlphaMax);
    const float ahi = fmin_ref(__fdividef(a, lo) * (1.f + 1e-6f), kSinAlphaMax);
    const float earg = fmaxf(ahi - arg, arg - alo) + 2.f * ulp_of(arg);
    const float v = asinf(arg);
    // asin' <= 1 / sqrt(1 - 0.95^2) = 3.2026 on [0, 0.95]
    const float slope = rsqrtf(fmaxf(1.f - ahi * ahi, 0.0975f)) * (1.f + 1e-6f);
    e = earg * slope + 3.f * ulp_of(v);
    return v;
}

// the filter's values and bounds (for the self-check)
struct B2Quick {
    float dbeta, e_dbeta, cut2, e_cut2, bout, e_bout, bout_cut, e_bout_cut;
    bool complete;  // the function reached the cuts
};

template <bool kDefer = false>
__device__ __forceinline__ int tl_b2_quick(int algo, const SGV& S, const SGV& T, B2Quick* q = nullptr) {
    constexpr float K = kB2qSafety;
    const float pt_betaMax = 7.0f;
    if (q) q->complete = false;
    if (kDefer && (algo != kAlgoBBBB || ((T.flags & F_UP_E) && (T.flags & F_UP_2S)))) return 2;
    // axis = OutUp - InLo: the float differences and IEEE square root of sub()
    const float ax = T.ux - S.lx, ay = T.uy - S.ly;
    const float dr = __fsqrt_rn(__fadd_rn(__fmul_rn(ax, ax), __fmul_rn(ay, ay)));
    if (!(dr > 1e-3f && dr < 1e5f)) return 1;
    const float axphi = atan2f(ay, ax);
    float d;
    if (!dphi_q(S.lphi, axphi, d)) return 1;
    const float betaIn0 = S.dpc - d;
    const float eIn = kB2qDir + ulp_of(betaIn0);
    const float sdIn_dr = S.rtseg, sdOut_dr = T.rtseg;
    const float sdIn_d = S.urt - S.lrt, sdOut_d = T.urt - T.lrt;
    const float alphaIn = S.dpc;
    if (!dphi_q(T.uphi, axphi, d)) return 1;
    float betaOut0, eOut, inMin, inMax, outMin, outMax, eInRH, eOutRH, alphaOutReg;
    float dBetaROut2 = 0.f, eROut2 = 0.f;
    int lIn, lOut;
    // (rt - rt') * sin(dPhi(midpoint(InLo, OutLo), OutLo - InLo)) / dr with an
    // approximate sine: value of the square and its bound
    auto rout2 = [&](float drt, float& e2) -> bool {
        const float mx = (0.f + S.lx + T.lx) / 2.f, my = (0.f + S.ly + T.ly) / 2.f;
        float dm;
        if (!dphi_q(atan2f(my, mx), atan2f(T.ly - S.ly, T.lx - S.lx), dm)) return false;
        const float sd = __sinf(dm);
        const float rr = __fdividef(drt * sd, dr);
        // (both directions approximate)
        const float err = __fdividef(fabsf(drt), dr) * (2.f * kB2qDir + kB2qSin + 2.f * ulp_of(sd)) * (1.f + 1e-6f) +
                          4.f * ulp_of(rr);
        dBetaROut2 = rr * rr;
        e2 = 2.f * fabsf(rr) * err + err * err + ulp_of(dBetaROut2);
        return true;
    };
    if (algo == kAlgoBBBB) {
        // Tracklet.cc:1205-1538
        betaOut0 = -T.alphaup + d;
        eOut = kB2qDir + ulp_of(betaOut0);
        inMin = inMax = betaIn0;
        eInRH = eIn;
        const bool ec2s = (T.flags & F_UP_E) && (T.flags & F_UP_2S);
        if (ec2s) {
            // the strip-edge points of the outer anchor (edge_point's float sums)
            const float hx = T.ux + T.ex, hy = T.uy + T.ey, lx = T.ux + -T.ex, ly = T.uy + -T.ey;
            const float hphi = atan2f(hy, hx), lphi = atan2f(ly, lx);
            float d1, d2, d3, d4;
            if (!dphi_q(hphi, atan2f(hy - T.ly, hx - T.lx), d1) || !dphi_q(hphi, atan2f(hy - S.ly, hx - S.lx), d2) ||
                !dphi_q(lphi, atan2f(ly - T.ly, lx - T.lx), d3) || !dphi_q(lphi, atan2f(ly - S.ly, lx - S.lx), d4))
                return 1;
            outMin = -d1 + d2;
            outMax = -d3 + d4;
            eOutRH = 4.f * kB2qDir + ulp_of(outMin) + ulp_of(outMax);
            const float hrt = __fsqrt_rn(__fadd_rn(__fmul_rn(hx, hx), __fmul_rn(hy, hy)));
            const float lrt = __fsqrt_rn(__fadd_rn(__fmul_rn(lx, lx), __fmul_rn(ly, ly)));
            if (!rout2(hrt - lrt, eROut2)) return 1;
        } else {
            outMin = outMax = betaOut0;
            eOutRH = eOut;
        }
        alphaOutReg = T.dpc;
        lIn = 5;
        lOut = ec2s ? 11 : 5;
    } else if (algo == kAlgoBBEE) {
        // Tracklet.cc:1765-2016 (the alpha terms are the exact code's floats)
        const float aOut = T.alphaup;
        const float aMin = phi_mpi_pi(T.dpminc - T.dpmin), aMax = phi_mpi_pi(T.dpmaxc - T.dpmax);
        betaOut0 = -aOut + d;
        eOut = kB2qDir + ulp_of(betaOut0);
        inMin = inMax = betaIn0;
        eInRH = eIn;
        outMin = betaOut0 - aMin + aOut;
        outMax = betaOut0 - aMax + aOut;
        eOutRH = eOut + 2.f * ulp_of(fabsf(outMin) + fabsf(outMax) + fabsf(aOut));
        if (T.flags & F_UP_2S) {
            const float hrt = edge_rt(T.ux, T.uy, T.ex, T.ey, true), lrt = edge_rt(T.ux, T.uy, T.ex, T.ey, false);
            if (!rout2(hrt - lrt, eROut2)) return 1;
        }
        alphaOutReg = S.dpc;
        lIn = 5;
        lOut = 11;
    } else if (algo == kAlgoEEEE) {
        // Tracklet.cc:2220-2665
        const float dPhiPos = T.dphilu;
        const float aOutMin = phi_mpi_pi(T.dpminc - dPhiPos), aOutMax = phi_mpi_pi(T.dpmaxc - dPhiPos);
        const float aOut = phi_mpi_pi(T.dpc - dPhiPos);
        betaOut0 = -aOut + d;
        eOut = kB2qDir + ulp_of(betaOut0);
        inMin = betaIn0 + S.dpminc - alphaIn;
        inMax = betaIn0 + S.dpmaxc - alphaIn;
        eInRH = eIn + 2.f * ulp_of(fabsf(inMin) + fabsf(inMax) + fabsf(alphaIn));
        outMin = betaOut0 - aOutMin + aOut;
        outMax = betaOut0 - aOutMax + aOut;
        eOutRH = eOut + 2.f * ulp_of(fabsf(outMin) + fabsf(outMax) + fabsf(aOut));
        alphaOutReg = S.dpc;
        lIn = 11;
        lOut = 13;
    } else {
        return 1;
    }
    // ---- the deltaBeta iterations (Tracklet.cc:3181-3324) with bounds
    const float D = dr * k2Rinv1GeVf;
    const float aIn = sdIn_dr * k2Rinv1GeVf, aOut = sdOut_dr * k2Rinv1GeVf;
    float betaIn = betaIn0, betaOut = betaOut0, eBi = eIn, eBo = eOut;
    if (!(fabsf(betaIn) < 1.5f && fabsf(betaOut) < 1.5f)) return 1;  // keeps every pt_range argument within pi
    float betaAv = 0.5f * (betaIn + betaOut);
    float eAv = 0.5f * (eBi + eBo) + ulp_of(betaAv);
    float lo, hi;
    float pt = pt_range(D, betaAv, K * eAv, lo, hi);
    const int ptc = pt_below(lo, hi, (lIn >= 11 ? 8.f : 4.f) * pt_betaMax);
    const int same = (fabsf(betaIn) > K * eBi && fabsf(betaOut) > K * eBo) ? ((betaIn > 0.f) == (betaOut > 0.f)) : -1;
    int mode;  // 1, 2 or 0 (no update)
    if (same == 1 && ptc == 1) mode = 1;
    else if (same == 0 || ptc == 0) mode = 0;
    else return 1;
    if (mode == 0 && lIn < 11) {
        // (double)|betaOut| < 0.2 (double)|betaIn| && |pt| < 12 pt_betaMax
        const float slack = 1e-7f * fabsf(betaIn);
        const int small = (fabsf(betaOut) + K * eBo < 0.2f * (fabsf(betaIn) - K * eBi) - slack)
                              ? 1
                              : ((fabsf(betaOut) - K * eBo > 0.2f * (fabsf(betaIn) + K * eBi) + slack) ? 0 : -1);
        const int ptc2 = pt_below(lo, hi, 12.f * pt_betaMax);
        if (small == 1 && ptc2 == 1) mode = 2;
        else if (!(small == 0 || ptc2 == 0)) return 1;
    }
    if (mode == 1) {
        float e1, e2;
        const float uIn = b2q_update(aIn, pt, lo, hi, e1), uOut = b2q_update(aOut, pt, lo, hi, e2);
        const float bIn1 = betaIn + copysignf(uIn, betaIn), bOut1 = betaOut + copysignf(uOut, betaOut);
        const float av1 = 0.5f * (bIn1 + bOut1);
        const float eAv1 = 0.5f * (eBi + e1 + eBo + e2) + ulp_of(bIn1) + ulp_of(bOut1) + ulp_of(av1);
        float lo1, hi1;
        const float p1 = pt_range(D, av1, K * eAv1, lo1, hi1);
        const float vIn = b2q_update(aIn, p1, lo1, hi1, e1), vOut = b2q_update(aOut, p1, lo1, hi1, e2);
        betaIn = betaIn + copysignf(vIn, betaIn);
        betaOut = betaOut + copysignf(vOut, betaOut);
        eBi = eBi + e1 + ulp_of(betaIn);
        eBo = eBo + e2 + ulp_of(betaOut);
    } else if (mode == 2) {
        // the sign of betaIn is certain here (|betaIn| > 5 |betaOut| + the bounds)
        float loI, hiI;
        const float pI = pt_range(D, betaIn, K * eBi, loI, hiI);
        float e1, e2;
        const float uIn = b2q_update(aIn, pI, loI, hiI, e1);
        // |betaOut| > 0.2f |betaIn| is false here, so betaAv = betaInUpd (betaOutUpd is unused)
        const float av1 = betaIn + copysignf(uIn, betaIn);
        const float eAv1 = eBi + e1 + ulp_of(av1);
        float lo1, hi1;
        const float p1 = pt_range(D, av1, K * eAv1, lo1, hi1);
        const float vIn = b2q_update(aIn, p1, lo1, hi1, e1), vOut = b2q_update(aOut, p1, lo1, hi1, e2);
        betaIn = betaIn + copysignf(vIn, betaIn);
        betaOut = betaOut + copysignf(vOut, betaIn);
        eBi = eBi + e1 + ulp_of(betaIn);
        eBo = eBo + e2 + ulp_of(betaOut);
    }
    if (mode != 0) {
        betaAv = 0.5f * (betaIn + betaOut);
        eAv = 0.5f * (eBi + eBo) + ulp_of(betaAv);
        pt = pt_range(D, betaAv, K * eAv, lo, hi);
    }
    // ---- the cut values
    // betaRH * (2 beta / |RHmin + RHmax|): the spread |RHmin - RHmax| scaled
    auto spread = [&](float mn, float mx, float eRH, float beta, float eBeta, float& e) -> bool {
        if (mn == mx) {  // the same float in both codes: the difference is 0
            e = 0.f;
            return true;
        }
        const float sum = fabsf(mn + mx), eSum = 2.f * eRH + ulp_of(sum);
        if (!(sum > 2.f * K * eSum)) return false;
        const float m = 2.f * beta / sum;
        const float eM = __fdividef(2.f * eBeta + fabsf(m) * eSum, sum - K * eSum) * (1.f + 1e-6f) + 2.f * ulp_of(m);
        const float s = fabsf(mn * m - mx * m);
        const float eD = 2.f * eRH;
        e = fabsf(mn - mx) * eM + fabsf(m) * eD + eD * eM + 3.f * ulp_of(fabsf(mn * m) + fabsf(mx * m));
        return s == s;
    };
    float eTin, eTout;
    if (!spread(inMin, inMax, eInRH, betaIn, eBi, eTin) || !spread(outMin, outMax, eOutRH, betaOut, eBo, eTout)) return 1;
    float tIn = 0.f, tOut = 0.f;
    if (inMin != inMax) {
        const float m = 2.f * betaIn / fabsf(inMin + inMax);
        tIn = fabsf(inMin * m - inMax * m);
    }
    if (outMin != outMax) {
        const float m = 2.f * betaOut / fabsf(outMin + outMax);
        tOut = fabsf(outMin * m - outMax * m);
    }
    const float t = tIn + tOut, eT = eTin + eTout + ulp_of(t);
    // the multiple-scattering factor: phase A's approximation (relative 11 * 2^-24)
    const float dd = T.lrt - S.lrt;
    if (!(dd >= 0.f && dd < 1e4f)) return 1;
    const float u = __fadd_rn(0.1f, __fmul_rn(dd, 0.004f));
    const float mulsF = __fmul_rn(__fmul_rn(0.015f, __fmul_rn(u, rsqrtf(u))), algo == kAlgoEEEE ? 1.f : S.sqq_hi);
    const float rMuls = 2e-6f;
    const float ptm = fmin_ref(fabsf(pt), pt_betaMax);
    const float ptmLo = fminf(lo, pt_betaMax), ptmHi = fminf(hi, pt_betaMax);
    if (!(ptmLo > 0.f)) return 1;
    const float rPt = __fdividef(fmaxf(ptmHi - ptm, ptm - ptmLo) + ulp_of(ptm), ptmLo) * (1.f + 1e-6f);
    const float dBetaMuls = __fdividef(mulsF * 4.f, ptm);
    const float eMuls = dBetaMuls * (K * rMuls + rPt) * (1.f + K * rMuls + rPt) + 4.f * ulp_of(dBetaMuls);
    // the luminous-region terms and dBetaRes: the exact code's floats
    const float alphaInAbsReg = fmax_ref(fabsf(alphaIn), S.la3);
    const float alphaOutAbsReg = fmax_ref(fabsf(alphaOutReg), T.la3);
    const float dBetaInLum = lIn < 11 ? 0.0f : fabsf(alphaInAbsReg * kDeltaZLum / S.lz);
    const float dBetaOutLum = lOut < 11 ? 0.0f : fabsf(alphaOutAbsReg * kDeltaZLum / T.lz);
    const float dBetaLum2 = (dBetaInLum + dBetaOutLum) * (dBetaInLum + dBetaOutLum);
    const float ey = 2.f * dBetaMuls * eMuls + eMuls * eMuls;
    // betaOut_cut = asin(min(dr k / ptCut, 0.95)) + 0.02 / sdOut_d + sqrt(dBetaLum2 + dBetaMuls^2)
    const float x = asinf(fmin_ref(dr * k2Rinv1GeVf / kPtCut, kSinAlphaMax)) + (0.02f / sdOut_d);
    const float ex = 3.f * ulp_of(1.3f) + ulp_of(x);
    const float y = dBetaLum2 + dBetaMuls * dBetaMuls;
    const float eY = ey + 2.f * ulp_of(y);
    const float sy = y > 0.f ? y * rsqrtf(y) : 0.f;
    const float eS = (y > 2.f * K * eY ? __fdividef(K * eY, sy) : sqrtf(K * eY)) * (1.f + 1e-6f);
    const float boutCut = x + sy;
    const float eBoutCut = K * ex + eS + 2.f * ulp_of(boutCut) + 4.f * ulp_of(sy);
    const float dBetaRes = 0.02f / fmin_ref(sdOut_d, sdIn_d);
    const float head = dBetaRes * dBetaRes * 2.0f + dBetaMuls * dBetaMuls + dBetaLum2 + dBetaROut2;
    const float eHead = ey + eROut2 + 5.f * ulp_of(head);
    const float cut2 = head + 0.25f * t * t;
    const float eCut2 = eHead + 0.5f * t * eT + 0.25f * eT * eT + 3.f * ulp_of(cut2);
    const float dBeta = betaIn - betaOut;
    const float eD = eBi + eBo + ulp_of(dBeta);
    if (q) {
        q->dbeta = dBeta; q->e_dbeta = eD; q->cut2 = cut2; q->e_cut2 = eCut2;
        q->bout = betaOut; q->e_bout = eBo; q->bout_cut = boutCut; q->e_bout_cut = eBoutCut;
        q->complete = true;
    }
    if (!(dBeta == dBeta && cut2 == cut2 && boutCut == boutCut && betaOut == betaOut)) return 1;
    // betaOut cut: rejected when |betaOut| >= betaOut_cut
    if (fabsf(betaOut) - K * eBo >= boutCut + K * eBoutCut) return 0;
    // deltaBeta cut: rejected when dBeta^2 > dBetaCut2 (the square rounded to float)
    const float lowD = fabsf(dBeta) - K * eD;
    if (lowD > 0.f && lowD * lowD * (1.f - 0x1p-21f) > cut2 + K * eCut2) return 0;
    // both cuts hold: |betaOut| < betaOut_cut and dBeta^2 <= dBetaCut2 for the exact
    // values (the comparisons' own roundings are ulps, far below the bounds)
    const float hiO = fabsf(betaOut) + K * eBo, hiD = fabsf(dBeta) + K * eD;
    if (hiO + ulp_of(hiO) < boutCut - K * eBoutCut - ulp_of(boutCut) &&
        hiD * hiD * (1.f + 0x1p-21f) < cut2 - K * eCut2 - ulp_of(cut2))
        return 3;
    return 1;
}

// phase B in one call (phase B1, then phase B2 on its survivors)
__device__ __forceinline__ bool tl_phaseB(int algo, const float* __restrict__ pack, int s, int t, float sdlCut, float mulsF,
                                          bool nm1) {
    return tl_phaseB1(algo, pack, s, t, sdlCut) && tl_phaseB2<kB2All>(algo, pack, s, t, mulsF, nm1);
}

}  // namespace sdlg
