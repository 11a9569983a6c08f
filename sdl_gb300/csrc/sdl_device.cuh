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
};

// ------------------------------------------------------------------ math
__device__ __forceinline__ float f_asin(float x) { return (float)asin((double)x); }
__device__ __forceinline__ float f_atan(float x) { return (float)atan((double)x); }
__device__ __forceinline__ float f_sin(float x) { return (float)sin((double)x); }
__device__ __forceinline__ float f_cos(float x) { return (float)cos((double)x); }
__device__ __forceinline__ float f_tan(float x) { return (float)tan((double)x); }
__device__ __forceinline__ float fmin_ref(float a, float b) { return (b < a) ? b : a; }  // std::min
__device__ __forceinline__ float fmax_ref(float a, float b) { return (a < b) ? b : a; }  // std::max
__device__ __forceinline__ int trunc_i32(float f) {
    if (!(f > -2147483649.0f && f < 2147483648.0f)) return (int)0x80000000;
    return __float2int_rz(f);
}
__device__ __forceinline__ int iabs(int v) { return v < 0 ? (int)(0u - (unsigned)v) : v; }
__device__ __forceinline__ float f_copysign(float a, float b) { return copysignf(a, b); }

// MathUtil.cc:3-19; the loop is bounded (|x| stays within a few pi here)
__device__ __forceinline__ float phi_mpi_pi(float x) {
    if (isnan(x)) return x;
#pragma unroll 1
    for (int it = 0; it < 64 && (double)x >= kPi; ++it) x = (float)((double)x - 2. * kPi);
#pragma unroll 1
    for (int it = 0; it < 64 && (double)x < -kPi; ++it) x = (float)((double)x + 2. * kPi);
    return x;
}
// MathUtil.cc:21-27
__device__ __forceinline__ float atan2_ref(float y, float x) {
    if (x != 0) return (float)atan2((double)y, (double)x);
    if (y == 0) return 0.f;
    if (y > 0) return (float)(kPi / 2);
    return (float)(-kPi / 2);
}
__device__ __forceinline__ float phi_of(float x, float y) {
    return phi_mpi_pi((float)(kPi + (double)atan2_ref(-y, -x)));
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
    const float rB[6] = {21.8f, 34.6f, 49.6f, 67.4f, 87.6f, 106.8f};
    const float rE[5] = {131.4f, 156.2f, 185.6f, 220.3f, 261.5f};
    const unsigned iL = m.layer - 1;
    const float miniSlope = asin_rt1;  // asin(min(rt * k2Rinv1GeVf / 1, 0.95))
    (void)rt;
    const bool barrel = m.subdet == kBarrel;
    const float rLay = barrel ? rB[iL] : rE[iL];
    const float miniPVoff = (float)(0.1 / (double)rLay);
    const float miniMuls = barrel ? mulsB[iL] * 3.f / kPtCut : 0.006f * 3.f / kPtCut;
    if (barrel && m.side == kCenter) {
        const double a = miniMuls, b = miniPVoff;
        return (float)((double)miniSlope + sqrt(a * a + b * b));
    }
    if (barrel) {
        const float drdz = m.drdz_s;
        const float miniTilt = (float)((double)(0.5f * kPixelPSZpitch * drdz) / sqrt((double)(1.f + drdz * drdz)) / (double)m.gap);
        const double a = miniMuls, b = miniPVoff, c = miniTilt * miniSlope;
        return (float)((double)miniSlope + sqrt(a * a + b * b + c * c));
    }
    const float miniLum = (float)iabs(trunc_i32(dPhi * kDeltaZLum / dz));
    const double a = miniMuls, b = miniPVoff, c = miniLum;
    return (float)((double)miniSlope + sqrt(a * a + b * b + c * c));
}

// MiniDoublet.cc:989-1209.  pix/str are the anchoring and the shifted hit.
__device__ __forceinline__ void shift_strip(const P3& lo, const P3& up, const ModDev& lm, float& xn, float& yn, float& zn) {
    const bool ps = lm.type == kPS;
    const bool pixLower = lm.ltype == kPixel;
    const P3& pix = (ps && !pixLower) ? up : lo;
    const P3& str = (ps && !pixLower) ? lo : up;
    const bool isEndcap = lm.subdet == kEndcap;
    const float angleA = (float)fabs((double)f_atan(pix.rt / pix.z));
    const float angleB = isEndcap ? (float)(kPi / 2.) : f_atan(lm.drdz_s);
    float sep = lm.gap;
    if (ps && !pixLower) sep *= -1;
    const float sAB = f_sin(angleA + angleB);
    const float drprime = (sep / sAB) * f_sin(angleA);
    const float slope = lm.slope_s;
    const float absArctanSlope = (slope != kSdlInf) ? (float)fabs((double)f_atan(slope)) : (float)(kPi / 2);
    const float xp = pix.x, yp = pix.y;
    float angleM;
    if (xp > 0 && yp > 0) angleM = absArctanSlope;
    else if (xp > 0 && yp < 0) angleM = (float)(kPi - (double)absArctanSlope);
    else if (xp < 0 && yp < 0) angleM = (float)(kPi + (double)absArctanSlope);
    else angleM = (float)(2 * kPi - (double)absArctanSlope);
    const float dx = drprime * f_sin(angleM);
    const float dy = drprime * f_cos(angleM);
    const float xa = xp + dx, ya = yp + dy;
    const float xo = str.x, yo = str.y;
    if (slope == kSdlInf) { xn = xa; yn = yo; }
    else if (slope == 0) { xn = xo; yn = ya; }
    else {
        xn = (slope * xa + (1.f / slope) * xo - ya + yo) / (slope + (1.f / slope));
        yn = (xn - xa) * slope + ya;
    }
    const float absdzprime = fabsf(sep / sAB * f_cos(angleA));
    float abszn;
    if (pixLower) abszn = (float)(fabs((double)pix.z) + (double)absdzprime);
    else abszn = (float)(fabs((double)pix.z) - (double)absdzprime);
    zn = abszn * ((pix.z > 0) ? 1 : -1);
}

struct MDVals {
    float dz, shiftedDz, dphi, dphichange;
};

// MiniDoublet.cc:243-447.  pixAsin is asin(min(rt*k, .95)) of the hit that
// dPhiThreshold reads (the pixel-side hit).
__device__ __forceinline__ bool md_barrel(const P3& lo, const P3& up, float pixAsin, const ModDev& lm, MDVals& v) {
    v.dz = lo.z - up.z;
    const float dz = v.dz;
    const float dzCut = lm.type == kPS ? 2.f : 10.f;
    const float sign = (float)(((dz > 0) - (dz < 0)) * ((lo.z > 0) - (lo.z < 0)));
    const float inverted = (float)(iabs(trunc_i32(dz)) > 2) * sign;
    if (!(fabsf(dz) < dzCut && inverted <= 0)) return false;
    const float miniCut = dphi_threshold(0.f, pixAsin, lm, 0.f, 1.f);
    P3 shifted;
    if (lm.side != kCenter) {
        float xn, yn, zn;
        shift_strip(lo, up, lm, xn, yn, zn);
        if (lm.ltype == kPixel) { shifted = mk2(xn, yn, up.z); v.dphi = dphi(lo, shifted); }
        else { shifted = mk2(xn, yn, lo.z); v.dphi = dphi(shifted, up); }
    } else {
        v.dphi = dphi(lo, up);
    }
    if (!(fabsf(v.dphi) < miniCut)) return false;
    if (lm.side != kCenter) {
        if (lm.ltype == kPixel)
            v.dphichange = lo.rt < shifted.rt ? dphichange(lo, shifted) : dphichange(shifted, lo);
        else
            v.dphichange = shifted.rt < up.rt ? dphichange(shifted, up) : dphichange(up, shifted);
    } else {
        v.dphichange = dphichange(lo, up);
    }
    return fabsf(v.dphichange) < miniCut;
}

// MiniDoublet.cc:449-684
__device__ __forceinline__ bool md_endcap(const P3& lo, const P3& up, float pixAsin, const ModDev& lm, MDVals& v) {
    v.dz = lo.z - up.z;
    float dz = v.dz;
    if (!(fabsf(dz) < 10.f)) return false;  // side() is never SubDet::Endcap (MiniDoublet.cc:470)
    const float drtCut = lm.type == kPS ? 2.f : 10.f;
    if (!(fabsf(lo.rt - up.rt) < drtCut)) return false;
    float xn, yn, zn;
    shift_strip(lo, up, lm, xn, yn, zn);
    P3 shifted;
    if (lm.type == kPS && lm.ltype != kPixel) { shifted = mk2(xn, yn, lo.z); v.dphi = dphi(shifted, up); }
    else { shifted = mk2(xn, yn, up.z); v.dphi = dphi(lo, shifted); }
    if (lm.type == kPS) {
        v.shiftedDz = lm.ltype == kPixel ? lo.z - zn : up.z - zn;
        dz = v.shiftedDz;
    }
    const float miniCut = dphi_threshold(0.f, pixAsin, lm, v.dphi, dz);
    if (!(fabsf(v.dphi) < miniCut)) return false;
    const float dzFrac = (float)((double)fabsf(dz) / fabs((double)lo.z));
    v.dphichange = v.dphi / dzFrac * (1.f + dzFrac);
    return fabsf(v.dphichange) < miniCut;
}

// ------------------------------------------------------------------ segments
struct MDView {
    P3 a;          // anchor hit
    float dphi, dphichange, dz, shiftedDz;
    const ModDev* m;  // lower module
};

// Segment.cc:886-994 (the three thresholds)
__device__ __forceinline__ void dalpha_threshold(const MDView& im, const MDView& om, float th[3]) {
    const float mulsB[6] = {0.0052f, 0.0038f, 0.0034f, 0.0034f, 0.0032f, 0.0034f};
    const ModDev& I = *im.m;
    const ModDev& O = *om.m;
    const float sdMuls = I.subdet == kBarrel ? mulsB[I.layer - 1] * 3.f / kPtCut : 0.006f * 3.f / kPtCut;
    const double dyy = (double)(om.a.y - im.a.y), dxx = (double)(om.a.x - im.a.x);
    const float segmentDr = (float)sqrt(dyy * dyy + dxx * dxx);
    const float dAlpha_Bfield = f_asin(fmin_ref(segmentDr * k2Rinv1GeVf / kPtCut, kSinAlphaMax));
    const bool inTilt = I.subdet == kBarrel && I.side != kCenter;
    const bool outTilt = O.subdet == kBarrel && O.side != kCenter;
    const float iTilt = inTilt ? (float)((double)(0.5f * kPixelPSZpitch * I.drdz_s) / sqrt((double)(1.f + I.drdz_s * I.drdz_s)) / (double)I.gap) : 0.f;
    const float oTilt = outTilt ? (float)((double)(0.5f * kPixelPSZpitch * O.drdz_s) / sqrt((double)(1.f + O.drdz_s * O.drdz_s)) / (double)O.gap) : 0.f;
    const float miniDelta = I.gap;
    float lumIn, lumOut;
    if (I.subdet == kBarrel) lumIn = iTilt * dAlpha_Bfield;
    else if (I.type == kPS) lumIn = (float)((double)im.dphi * 15.0 / (double)im.shiftedDz);
    else lumIn = (float)((double)im.dphi * 15.0 / (double)im.dz);
    if (O.subdet == kBarrel) lumOut = oTilt * dAlpha_Bfield;
    else if (O.type == kPS) lumOut = (float)((double)om.dphi * 15.0 / (double)om.shiftedDz);
    else lumOut = (float)((double)om.dphi * 15.0 / (double)om.dz);
    const float resIn = 0.02f / miniDelta * (I.subdet == kBarrel ? 1.0f : fabsf(im.a.z / im.a.rt));
    const float resOut = 0.02f / miniDelta * (O.subdet == kBarrel ? 1.0f : fabsf(om.a.z / om.a.rt));
    const double res = (double)(resIn + resOut);
    const double mu = sdMuls;
    const double base = res * res + mu * mu;
    const double li = lumIn, lo = lumOut;
    th[0] = (I.subdet == kBarrel && I.side == kCenter) ? (float)((double)dAlpha_Bfield + sqrt(base)) : (float)((double)dAlpha_Bfield + sqrt(base + li * li));
    th[1] = (O.subdet == kBarrel && O.side == kCenter) ? (float)((double)dAlpha_Bfield + sqrt(base)) : (float)((double)dAlpha_Bfield + sqrt(base + lo * lo));
    th[2] = (float)((double)dAlpha_Bfield + sqrt(base));
}

__device__ __forceinline__ bool dalpha_cuts(const MDView& im, const MDView& om, float sg_alpha) {
    float th[3];
    dalpha_threshold(im, om, th);
    if (!(fabsf(im.dphichange - sg_alpha) < th[0])) return false;
    if (!(fabsf(om.dphichange - sg_alpha) < th[1])) return false;
    return fabsf(om.dphichange - im.dphichange) < th[2];
}

struct SGVals {
    float dphi, dphimin, dphimax, dphichange, dphiminchange, dphimaxchange;
};

// Segment.cc:364-599.  outAsin / outTanf: asin(min(rtOut*k,.95)) of the
// outer anchor and its float tan.
__device__ __forceinline__ bool sg_barrel(const MDView& im, const MDView& om, float outAsin, float outTanf, SGVals& v) {
    const float mulsB[6] = {0.0052f, 0.0038f, 0.0034f, 0.0034f, 0.0032f, 0.0034f};
    const float sdMuls = mulsB[im.m->layer - 1] * 3.f / kPtCut;
    const float rtIn = im.a.rt, rtOut = om.a.rt, zIn = im.a.z, zOut = om.a.z;
    const float sdSlope = outAsin;
    const float sdPVoff = 0.1f / rtOut;
    const float dzDrtScale = outTanf / sdSlope;
    const float zGeom = im.m->layer <= 2 ? 2.f * kPixelPSZpitch : 2.f * kStrip2SZpitch;
    const float zLo = zIn + (zIn - kDeltaZLum) * (rtOut / rtIn - 1.f) * (zIn > 0.f ? 1.f : dzDrtScale) - zGeom;
    const float zHi = zIn + (zIn + kDeltaZLum) * (rtOut / rtIn - 1.f) * (zIn < 0.f ? 1.f : dzDrtScale) + zGeom;
    if (!(zOut >= zLo && zOut <= zHi)) return false;
    const float sdCut = (float)((double)sdSlope + sqrt((double)(sdMuls * sdMuls + sdPVoff * sdPVoff)));
    const float deltaPhi = dphi(im.a, om.a);
    if (!(fabsf(deltaPhi) <= sdCut)) return false;
    v.dphichange = dphichange(im.a, om.a);
    if (!(fabsf(v.dphichange) <= sdCut)) return false;
    return dalpha_cuts(im, om, v.dphichange);
}

// Segment.cc:601-859.  connected: outer module is in the inner module's
// connection list (cut #0).
__device__ __forceinline__ bool sg_endcap(const MDView& im, const MDView& om, float outAsin, float outTanf,
                                          bool connected, const P3& oHi, const P3& oLo, SGVals& v) {
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
    const float hiP = dphi(im.a, oHi);
    const float loP = dphi(im.a, oLo);
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
struct AnchorView {
    P3 p;
    float asin1;   // asin(min(rt*k, .95))
    float tand1;   // (float)(tan((double)asin1) / asin1)
    float asin3;   // asin(min(rt*k/3, .95))
    const ModDev* m;
};
struct SGView {
    AnchorView lo, up;
    float dphi, dphimin, dphimax, dphichange, dphiminchange, dphimaxchange;
};

// Tracklet.cc:3181-3324
__device__ __forceinline__ void delta_beta_iterations(float& betaIn, float& betaOut, float& betaAv, float& pt_beta, float sdIn_dr,
                                                      float sdOut_dr, float dr, int lIn, float pt_betaMax) {
    const float sinAlphaMax = 0.95f;
    if (betaIn * betaOut > 0.f &&
        (fabsf(pt_beta) < 4.f * pt_betaMax || (lIn >= 11 && fabsf(pt_beta) < 8.f * pt_betaMax))) {
        const float betaInUpd = (float)((double)betaIn + copysign((double)f_asin(fmin_ref(sdIn_dr * k2Rinv1GeVf / fabsf(pt_beta), sinAlphaMax)), (double)betaIn));
        const float betaOutUpd = (float)((double)betaOut + copysign((double)f_asin(fmin_ref(sdOut_dr * k2Rinv1GeVf / fabsf(pt_beta), sinAlphaMax)), (double)betaOut));
        betaAv = 0.5f * (betaInUpd + betaOutUpd);
        pt_beta = (float)((double)(dr * k2Rinv1GeVf) / sin((double)betaAv));
        betaIn = (float)((double)betaIn + copysign((double)f_asin(fmin_ref(sdIn_dr * k2Rinv1GeVf / fabsf(pt_beta), sinAlphaMax)), (double)betaIn));
        betaOut = (float)((double)betaOut + copysign((double)f_asin(fmin_ref(sdOut_dr * k2Rinv1GeVf / fabsf(pt_beta), sinAlphaMax)), (double)betaOut));
        betaAv = 0.5f * (betaIn + betaOut);
        pt_beta = (float)((double)(dr * k2Rinv1GeVf) / sin((double)betaAv));
    } else if (lIn < 11 && (double)fabsf(betaOut) < 0.2 * (double)fabsf(betaIn) && fabsf(pt_beta) < 12.f * pt_betaMax) {
        const float pt_betaIn = (float)((double)(dr * k2Rinv1GeVf) / sin((double)betaIn));
        const float betaInUpd = (float)((double)betaIn + copysign((double)f_asin(fmin_ref(sdIn_dr * k2Rinv1GeVf / fabsf(pt_betaIn), sinAlphaMax)), (double)betaIn));
        const float betaOutUpd = (float)((double)betaOut + copysign((double)f_asin(fmin_ref(sdOut_dr * k2Rinv1GeVf / fabsf(pt_betaIn), sinAlphaMax)), (double)betaIn));
        betaAv = (fabsf(betaOut) > 0.2f * fabsf(betaIn)) ? (0.5f * (betaInUpd + betaOutUpd)) : betaInUpd;
        pt_beta = (float)((double)(dr * k2Rinv1GeVf) / sin((double)betaAv));
        betaIn = (float)((double)betaIn + copysign((double)f_asin(fmin_ref(sdIn_dr * k2Rinv1GeVf / fabsf(pt_beta), sinAlphaMax)), (double)betaIn));
        betaOut = (float)((double)betaOut + copysign((double)f_asin(fmin_ref(sdOut_dr * k2Rinv1GeVf / fabsf(pt_beta), sinAlphaMax)), (double)betaIn));
        betaAv = 0.5f * (betaIn + betaOut);
        pt_beta = (float)((double)(dr * k2Rinv1GeVf) / sin((double)betaAv));
    }
}

__device__ __forceinline__ float dbeta_cut2(float dBetaRes, float dBetaMuls, float dBetaLum2, float dBetaROut2, float inMin,
                                            float inMax, float outMin, float outMax) {
    const float dBetaRIn2 = 0;
    const float head = dBetaRes * dBetaRes * 2.0f + dBetaMuls * dBetaMuls + dBetaLum2 + dBetaRIn2 + dBetaROut2;
    const double t = (double)(fabsf(inMin - inMax) + fabsf(outMin - outMax));
    return (float)((double)head + 0.25 * (t * t));
}

// Tracklet.cc:902-1538
__device__ __forceinline__ bool tl_bbbb(const SGView& S, const SGView& T, bool nm1) {
    const float pt_betaMax = 7.0f;
    const AnchorView& InLo = S.lo;
    const AnchorView& InUp = S.up;
    const AnchorView& OutLo = T.lo;
    const AnchorView& OutUp = T.up;
    const float zpitch_InLo = InLo.m->type == kPS ? kPixelPSZpitch : kStrip2SZpitch;
    const float zpitch_OutLo = OutLo.m->type == kPS ? kPixelPSZpitch : kStrip2SZpitch;
    const float rt_InLo = InLo.p.rt, rt_OutLo = OutLo.p.rt, z_InLo = InLo.p.z, z_OutLo = OutLo.p.z;
    const float alpha1GeV_OutLo = OutLo.asin1;
    const float rtRatio = rt_OutLo / rt_InLo;
    const float dzDrtScale = OutLo.tand1;
    const float zHi = z_InLo + (z_InLo + kDeltaZLum) * (rtRatio - 1.f) * (z_InLo < 0.f ? 1.f : dzDrtScale) + (zpitch_InLo + zpitch_OutLo);
    const float zLo = z_InLo + (z_InLo - kDeltaZLum) * (rtRatio - 1.f) * (z_InLo > 0.f ? 1.f : dzDrtScale) - (zpitch_InLo + zpitch_OutLo);
    if (!(z_OutLo >= zLo && z_OutLo <= zHi)) return false;
    const float drt_OutLo_InLo = rt_OutLo - rt_InLo;
    const float drt_InSeg = InUp.p.rt - InLo.p.rt;
    const float dz_InSeg = InUp.p.z - InLo.p.z;
    const float dr3_InSeg = InUp.p.r3 - InLo.p.r3;
    const float coshEta = dr3_InSeg / drt_InSeg;
    const float r3_InLo = __fsqrt_rn(z_InLo * z_InLo + rt_InLo * rt_InLo);
    const float sdlThetaMulsF = (float)((double)0.015f * sqrt((double)0.1f + 0.2 * (double)(rt_OutLo - rt_InLo) / (double)50.f) * sqrt((double)(r3_InLo / rt_InLo)));
    const float sdlMuls = sdlThetaMulsF * 3.f / kPtCut * 4.f;
    const float sdlPVoff = 0.1f / rt_OutLo;
    const float sdlCut = (float)((double)alpha1GeV_OutLo + sqrt((double)(sdlMuls * sdlMuls + sdlPVoff * sdlPVoff)));
    // cut #3 (independent of cut #2; evaluated first because it is cheaper)
    if (!(fabsf(dphi(InUp.p, OutUp.p)) <= sdlCut)) return false;
    float dzErr = (zpitch_InLo + zpitch_OutLo) * (zpitch_InLo + zpitch_OutLo) * 2.f;
    dzErr += sdlMuls * sdlMuls * drt_OutLo_InLo * drt_OutLo_InLo / 3.f * coshEta * coshEta;
    dzErr = __fsqrt_rn(dzErr);
    const float dzMean = dz_InSeg / drt_InSeg * drt_OutLo_InLo;
    const float zWindow = dzErr / drt_InSeg * drt_OutLo_InLo + (zpitch_InLo + zpitch_OutLo);
    const float zLoPointed = z_InLo + dzMean * (z_InLo > 0.f ? 1.f : dzDrtScale) - zWindow;
    const float zHiPointed = z_InLo + dzMean * (z_InLo < 0.f ? 1.f : dzDrtScale) + zWindow;
    if (!(z_OutLo >= zLoPointed && z_OutLo <= zHiPointed)) return false;
    const P3 mid = midpoint(InLo.p, OutLo.p);
    const float dPhi = dphi(mid, sub(OutLo.p, InLo.p));
    if (!(fabsf(dPhi) <= sdlCut)) return false;
    const float alpha_InLo = S.dphichange;
    const bool isEC_lastLayer = OutUp.m->subdet == kEndcap && OutUp.m->type == kTwoS;
    const P3 tl_axis = sub(OutUp.p, InLo.p);
    const float drt_tl_axis = tl_axis.rt;
    const float rt_InSeg = rt_of_diff(InUp.p, InLo.p);
    float betaIn = alpha_InLo - dphi(InLo.p, tl_axis);
    const float betaIn_cut = f_asin(fmin_ref((-rt_InSeg * 1.f + drt_tl_axis) * k2Rinv1GeVf / kPtCut, kSinAlphaMax)) + (0.02f / drt_InSeg);
    float betaInRHmin = betaIn, betaInRHmax = betaIn;
    if (!(fabsf(betaInRHmin) < betaIn_cut)) return false;
    const float alpha_OutUp = dphi(OutUp.p, sub(OutUp.p, OutLo.p));
    float betaOut = -alpha_OutUp + dphi(OutUp.p, tl_axis);
    float betaOutRHmin, betaOutRHmax;
    P3 hiE = OutUp.p, loE = OutUp.p;
    if (isEC_lastLayer) {
        hiE = strip_edge(OutUp.p, *OutUp.m, true);
        loE = strip_edge(OutUp.p, *OutUp.m, false);
        const float alpha_hi = dphi(hiE, sub(hiE, OutLo.p));
        const float alpha_lo = dphi(loE, sub(loE, OutLo.p));
        betaOutRHmin = -alpha_hi + dphi(hiE, sub(hiE, InLo.p));
        betaOutRHmax = -alpha_lo + dphi(loE, sub(loE, InLo.p));
    } else {
        betaOutRHmin = betaOut;
        betaOutRHmax = betaOut;
    }
    float betaAv = 0.5f * (betaIn + betaOut);
    float pt_beta = (float)((double)(drt_tl_axis * k2Rinv1GeVf) / sin((double)betaAv));
    const int lIn = 5;
    const int lOut = isEC_lastLayer ? 11 : 5;
    const float sdOut_dr = rt_of_diff(OutUp.p, OutLo.p);
    const float sdOut_d = OutUp.p.rt - OutLo.p.rt;
    delta_beta_iterations(betaIn, betaOut, betaAv, pt_beta, rt_InSeg, sdOut_dr, drt_tl_axis, lIn, pt_betaMax);
    const float betaInMMSF = (fabsf(betaInRHmin + betaInRHmax) > 0) ? (2.f * betaIn / fabsf(betaInRHmin + betaInRHmax)) : 0.f;
    const float betaOutMMSF = (fabsf(betaOutRHmin + betaOutRHmax) > 0) ? (2.f * betaOut / fabsf(betaOutRHmin + betaOutRHmax)) : 0.f;
    betaInRHmin *= betaInMMSF; betaInRHmax *= betaInMMSF;
    betaOutRHmin *= betaOutMMSF; betaOutRHmax *= betaOutMMSF;
    const float dBetaMuls = sdlThetaMulsF * 4.f / fmin_ref(fabsf(pt_beta), pt_betaMax);
    const float alpha_OutLo = T.dphichange;
    const float alphaInAbsReg = fmax_ref(fabsf(alpha_InLo), InLo.asin3);
    const float alphaOutAbsReg = fmax_ref(fabsf(alpha_OutLo), OutLo.asin3);
    const float dBetaInLum = lIn < 11 ? 0.0f : fabsf(alphaInAbsReg * kDeltaZLum / InLo.p.z);
    const float dBetaOutLum = lOut < 11 ? 0.0f : fabsf(alphaOutAbsReg * kDeltaZLum / OutLo.p.z);
    const float dBetaLum2 = (dBetaInLum + dBetaOutLum) * (dBetaInLum + dBetaOutLum);
    const float sinDPhi = f_sin(dPhi);
    const double rr = (double)((hiE.rt - loE.rt) * sinDPhi / drt_tl_axis);
    const float dBetaROut2 = (float)(rr * rr);
    const float betaOut_cut = (float)((double)(f_asin(fmin_ref(drt_tl_axis * k2Rinv1GeVf / kPtCut, kSinAlphaMax)) + (0.02f / sdOut_d)) + sqrt((double)(dBetaLum2 + dBetaMuls * dBetaMuls)));
    if (!(fabsf(betaOut) < betaOut_cut)) return false;
    const float dBetaRes = 0.02f / fmin_ref(sdOut_d, drt_InSeg);
    const float dBetaCut2 = dbeta_cut2(dBetaRes, dBetaMuls, dBetaLum2, dBetaROut2, betaInRHmin, betaInRHmax, betaOutRHmin, betaOutRHmax);
    const float dBeta = betaIn - betaOut;
    return (dBeta * dBeta <= dBetaCut2) || nm1;
}

// Tracklet.cc:1540-2016
__device__ __forceinline__ bool tl_bbee(const SGView& S, const SGView& T, bool nm1) {
    const float pt_betaMax = 7.0f;
    const AnchorView& InLo = S.lo;
    const AnchorView& InUp = S.up;
    const AnchorView& OutLo = T.lo;
    const AnchorView& OutUp = T.up;
    const float zGeom = (InLo.m->type == kPS ? kPixelPSZpitch : kStrip2SZpitch) + (OutLo.m->type == kPS ? kPixelPSZpitch : kStrip2SZpitch);
    const float rtIn = InLo.p.rt, rtOut = OutLo.p.rt, zIn = InLo.p.z, zOut = OutLo.p.z;
    const float sdlSlope = OutLo.asin1;
    const float dzDrtScale = OutLo.tand1;
    if (!(zIn * zOut > 0)) return false;
    const float dLum = f_copysign(kDeltaZLum, zIn);
    const float rtGeom1 = OutLo.m->type == kPS ? kPixelPSZpitch : kStrip2SZpitch;
    const float zGeom1 = f_copysign(zGeom, zIn);
    const float rtLo = rtIn * (1.f + (zOut - zIn - zGeom1) / (zIn + zGeom1 + dLum) / dzDrtScale) - rtGeom1;
    if (!(rtOut >= rtLo)) return false;
    float zInForHi = zIn - zGeom1 - dLum;
    if (zInForHi * zIn < 0) zInForHi = f_copysign(0.1f, zIn);
    const float rtHi = rtIn * (1.f + (zOut - zIn + zGeom1) / zInForHi) + rtGeom1;
    if (!(rtOut >= rtLo && rtOut <= rtHi)) return false;
    const float dzSDIn = InUp.p.z - InLo.p.z;
    const float kZ = (zOut - zIn) / dzSDIn;
    if (!(kZ >= 0)) return false;
    const float rIn = __fsqrt_rn(zIn * zIn + rtIn * rtIn);
    const float sdlThetaMulsF = (float)((double)0.015f * sqrt((double)0.1f + 0.2 * (double)(rtOut - rtIn) / (double)50.f) * sqrt((double)(rIn / rtIn)));
    const float sdlMuls = sdlThetaMulsF * 3.f / kPtCut * 4.f;
    const float sdlPVoff = 0.1f / rtOut;
    const float sdlCut = (float)((double)sdlSlope + sqrt((double)(sdlMuls * sdlMuls + sdlPVoff * sdlPVoff)));
    if (!(fabsf(dphi(InUp.p, OutUp.p)) <= sdlCut)) return false;
    const P3 mid = midpoint(InLo.p, OutLo.p);
    const float dPhi = dphi(mid, sub(OutLo.p, InLo.p));
    if (!(fabsf(dPhi) <= sdlCut)) return false;
    const float sdIn_alpha = S.dphichange;
    const float sdOut_alpha = S.dphichange;  // (sic) Tracklet.cc:1790
    const float sdOut_alphaOut = dphi(OutUp.p, sub(OutUp.p, OutLo.p));
    const float sdOut_alphaOut_min = phi_mpi_pi(T.dphiminchange - T.dphimin);
    const float sdOut_alphaOut_max = phi_mpi_pi(T.dphimaxchange - T.dphimax);
    const P3 dr3 = sub(OutUp.p, InLo.p);
    float betaIn = sdIn_alpha - dphi(InLo.p, dr3);
    float betaOut = -sdOut_alphaOut + dphi(OutUp.p, dr3);
    float betaInRHmin = betaIn, betaInRHmax = betaIn;  // isEC_secondLayer is always false (Tracklet.cc:1798)
    float betaOutRHmin = betaOut - sdOut_alphaOut_min + sdOut_alphaOut;
    float betaOutRHmax = betaOut - sdOut_alphaOut_max + sdOut_alphaOut;
    if (fabsf(betaOutRHmin) > fabsf(betaOutRHmax)) { float t = betaOutRHmin; betaOutRHmin = betaOutRHmax; betaOutRHmax = t; }
    const float sdIn_dr = rt_of_diff(InUp.p, InLo.p);
    const float sdIn_d = InUp.p.rt - InLo.p.rt;
    const float dr = dr3.rt;
    const float betaIn_cut = f_asin(fmin_ref((-sdIn_dr * 1.f + dr) * k2Rinv1GeVf / kPtCut, kSinAlphaMax)) + (0.02f / sdIn_d);
    if (!(fabsf(betaInRHmin) < betaIn_cut)) return false;
    float betaAv = 0.5f * (betaIn + betaOut);
    float pt_beta = (float)((double)(dr * k2Rinv1GeVf) / sin((double)betaAv));
    const int lIn = 5, lOut = 11;
    const float sdOut_dr = rt_of_diff(OutUp.p, OutLo.p);
    const float sdOut_d = OutUp.p.rt - OutLo.p.rt;
    delta_beta_iterations(betaIn, betaOut, betaAv, pt_beta, sdIn_dr, sdOut_dr, dr, lIn, pt_betaMax);
    const float betaInMMSF = (fabsf(betaInRHmin + betaInRHmax) > 0) ? 2.f * betaIn / fabsf(betaInRHmin + betaInRHmax) : 0.f;
    const float betaOutMMSF = (fabsf(betaOutRHmin + betaOutRHmax) > 0) ? 2.f * betaOut / fabsf(betaOutRHmin + betaOutRHmax) : 0.f;
    betaInRHmin *= betaInMMSF; betaInRHmax *= betaInMMSF;
    betaOutRHmin *= betaOutMMSF; betaOutRHmax *= betaOutMMSF;
    const float dBetaMuls = sdlThetaMulsF * 4.f / fmin_ref(fabsf(pt_beta), pt_betaMax);
    const float alphaInAbsReg = fmax_ref(fabsf(sdIn_alpha), InLo.asin3);
    const float alphaOutAbsReg = fmax_ref(fabsf(sdOut_alpha), OutLo.asin3);
    const float dBetaInLum = lIn < 11 ? 0.0f : fabsf(alphaInAbsReg * kDeltaZLum / InLo.p.z);
    const float dBetaOutLum = lOut < 11 ? 0.0f : fabsf(alphaOutAbsReg * kDeltaZLum / OutLo.p.z);
    const float dBetaLum2 = (dBetaInLum + dBetaOutLum) * (dBetaInLum + dBetaOutLum);
    const float sinDPhi = f_sin(dPhi);
    float dBetaROut2 = 0.f;
    if (OutUp.m->type == kTwoS) {
        const P3 hiE = strip_edge(OutUp.p, *OutUp.m, true);
        const P3 loE = strip_edge(OutUp.p, *OutUp.m, false);
        const double rr = (double)((hiE.rt - loE.rt) * sinDPhi / dr);
        dBetaROut2 = (float)(rr * rr);
    } else {
        const double rr = (double)((OutUp.p.rt - OutUp.p.rt) * sinDPhi / dr);
        dBetaROut2 = (float)(rr * rr);
    }
    const float betaOut_cut = (float)((double)(f_asin(fmin_ref(dr * k2Rinv1GeVf / kPtCut, kSinAlphaMax)) + (0.02f / sdOut_d)) + sqrt((double)(dBetaLum2 + dBetaMuls * dBetaMuls)));
    if (!(fabsf(betaOut) < betaOut_cut)) return false;
    const float dBetaRes = 0.02f / fmin_ref(sdOut_d, sdIn_d);
    const float dBetaCut2 = dbeta_cut2(dBetaRes, dBetaMuls, dBetaLum2, dBetaROut2, betaInRHmin, betaInRHmax, betaOutRHmin, betaOutRHmax);
    const float dBeta = betaIn - betaOut;
    return (dBeta * dBeta <= dBetaCut2) || nm1;
}

// Tracklet.cc:2018-2665
__device__ __forceinline__ bool tl_eeee(const SGView& S, const SGView& T, bool nm1) {
    const float pt_betaMax = 7.0f;
    const AnchorView& InLo = S.lo;
    const AnchorView& InUp = S.up;
    const AnchorView& OutLo = T.lo;
    const AnchorView& OutUp = T.up;
    const float rtIn = InLo.p.rt, rtOut = OutLo.p.rt, zIn = InLo.p.z, zOut = OutLo.p.z;
    const float sdlSlope = OutLo.asin1;
    const float dzDrtScale = OutLo.tand1;
    if (!(zIn * zOut > 0)) return false;
    const float dLum = f_copysign(kDeltaZLum, zIn);
    const bool isOutSgInnerMDPS = OutLo.m->type == kPS;
    const bool isInSgInnerMDPS = InLo.m->type == kPS;
    const float rtGeom = (isInSgInnerMDPS && isOutSgInnerMDPS) ? 2.f * kPixelPSZpitch
                       : (isInSgInnerMDPS || isOutSgInnerMDPS) ? (kPixelPSZpitch + kStrip2SZpitch) : 2.f * kStrip2SZpitch;
    const float dz = zOut - zIn;
    const float rtLo = rtIn * (1.f + dz / (zIn + dLum) / dzDrtScale) - rtGeom;
    if (!(rtOut >= rtLo)) return false;
    const float rtHi = rtIn * (1.f + dz / (zIn - dLum)) + rtGeom;
    if (!(rtOut >= rtLo && rtOut <= rtHi)) return false;
    const float sdlThetaMulsF = (float)((double)0.015f * sqrt((double)0.1f + 0.2 * (double)(rtOut - rtIn) / (double)50.f));
    const float sdlMuls = sdlThetaMulsF * 3.f / kPtCut * 4.f;
    const float sdlPVoff = 0.1f / rtOut;
    const float sdlCut = (float)((double)sdlSlope + sqrt((double)(sdlMuls * sdlMuls + sdlPVoff * sdlPVoff)));
    if (!(fabsf(dphi(InUp.p, OutUp.p)) <= sdlCut)) return false;
    const bool isInSgOuterMDPS = InUp.m->type == kPS;
    const float drtSDIn = InUp.p.rt - InLo.p.rt;
    const float dzSDIn = InUp.p.z - InLo.p.z;
    if (isInSgInnerMDPS && isInSgOuterMDPS) {
        const float dr3SDIn = InUp.p.r3 - InLo.p.r3;
        const float coshEta = dr3SDIn / drtSDIn;
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
        if (!(kZ >= 0 && rtOut >= rtLo_point && rtOut <= rtHi_point)) return false;
    }
    const P3 mid = midpoint(InLo.p, OutLo.p);
    const float dPhi = dphi(mid, sub(OutLo.p, InLo.p));
    if (!(fabsf(dPhi) <= sdlCut)) return false;
    const float sdIn_alpha = S.dphichange;
    const float sdOut_alpha = S.dphichange;  // (sic)
    const float sdOut_dPhiPos = dphi(OutLo.p, OutUp.p);
    const float sdOut_alphaOutRHmin = phi_mpi_pi(T.dphiminchange - sdOut_dPhiPos);
    const float sdOut_alphaOutRHmax = phi_mpi_pi(T.dphimaxchange - sdOut_dPhiPos);
    const float sdOut_alphaOut = phi_mpi_pi(T.dphichange - sdOut_dPhiPos);
    const P3 dr3 = sub(OutUp.p, InLo.p);
    float betaIn = sdIn_alpha - dphi(InLo.p, dr3);
    float betaOut = -sdOut_alphaOut + dphi(OutUp.p, dr3);
    float betaInRHmin = betaIn + S.dphiminchange - sdIn_alpha;
    float betaInRHmax = betaIn + S.dphimaxchange - sdIn_alpha;
    if (fabsf(betaInRHmin) > fabsf(betaInRHmax)) { float t = betaInRHmin; betaInRHmin = betaInRHmax; betaInRHmax = t; }
    float betaOutRHmin = betaOut - sdOut_alphaOutRHmin + sdOut_alphaOut;
    float betaOutRHmax = betaOut - sdOut_alphaOutRHmax + sdOut_alphaOut;
    if (fabsf(betaOutRHmin) > fabsf(betaOutRHmax)) { float t = betaOutRHmin; betaOutRHmin = betaOutRHmax; betaOutRHmax = t; }
    const float sdIn_dr = rt_of_diff(InUp.p, InLo.p);
    const float sdIn_d = InUp.p.rt - InLo.p.rt;
    const float dr = dr3.rt;
    // cut #6 never rejects here (Tracklet.cc:2327-2336)
    float betaAv = 0.5f * (betaIn + betaOut);
    float pt_beta = (float)((double)(dr * k2Rinv1GeVf) / sin((double)betaAv));
    const int lIn = 11, lOut = 13;
    const float sdOut_dr = rt_of_diff(OutUp.p, OutLo.p);
    const float sdOut_d = OutUp.p.rt - OutLo.p.rt;
    delta_beta_iterations(betaIn, betaOut, betaAv, pt_beta, sdIn_dr, sdOut_dr, dr, lIn, pt_betaMax);
    const float betaInMMSF = (fabsf(betaInRHmin + betaInRHmax) > 0) ? (2.f * betaIn / fabsf(betaInRHmin + betaInRHmax)) : 0.f;
    const float betaOutMMSF = (fabsf(betaOutRHmin + betaOutRHmax) > 0) ? (2.f * betaOut / fabsf(betaOutRHmin + betaOutRHmax)) : 0.f;
    betaInRHmin *= betaInMMSF; betaInRHmax *= betaInMMSF;
    betaOutRHmin *= betaOutMMSF; betaOutRHmax *= betaOutMMSF;
    const float dBetaMuls = sdlThetaMulsF * 4.f / fmin_ref(fabsf(pt_beta), pt_betaMax);
    const float alphaInAbsReg = fmax_ref(fabsf(sdIn_alpha), InLo.asin3);
    const float alphaOutAbsReg = fmax_ref(fabsf(sdOut_alpha), OutLo.asin3);
    const float dBetaInLum = lIn < 11 ? 0.0f : fabsf(alphaInAbsReg * kDeltaZLum / InLo.p.z);
    const float dBetaOutLum = lOut < 11 ? 0.0f : fabsf(alphaOutAbsReg * kDeltaZLum / OutLo.p.z);
    const float dBetaLum2 = (dBetaInLum + dBetaOutLum) * (dBetaInLum + dBetaOutLum);
    const float betaOut_cut = (float)((double)(f_asin(fmin_ref(dr * k2Rinv1GeVf / kPtCut, kSinAlphaMax)) + (0.02f / sdOut_d)) + sqrt((double)(dBetaLum2 + dBetaMuls * dBetaMuls)));
    if (!(fabsf(betaOut) < betaOut_cut)) return false;
    const float dBetaRes = 0.02f / fmin_ref(sdOut_d, sdIn_d);
    const float dBetaCut2 = dbeta_cut2(dBetaRes, dBetaMuls, dBetaLum2, 0.f, betaInRHmin, betaInRHmax, betaOutRHmin, betaOutRHmax);
    const float dBeta = betaIn - betaOut;
    return (dBeta * dBeta <= dBetaCut2) || nm1;
}

// Tracklet.cc:144-296
__device__ __forceinline__ bool tl_dispatch(const SGView& S, const SGView& T, bool nm1) {
    const bool b1 = S.lo.m->subdet == kBarrel, b2 = S.up.m->subdet == kBarrel;
    const bool b3 = T.lo.m->subdet == kBarrel, b4 = T.up.m->subdet == kBarrel;
    const bool e1 = S.lo.m->subdet == kEndcap, e2 = S.up.m->subdet == kEndcap;
    const bool e3 = T.lo.m->subdet == kEndcap, e4 = T.up.m->subdet == kEndcap;
    if (b1 && b2 && b3 && (b4 || e4)) return tl_bbbb(S, T, nm1);
    if (b1 && ((b2 && e3) || (e2 && e3)) && e4) return tl_bbee(S, T, nm1);
    if (e1 && e2 && e3 && e4) return tl_eeee(S, T, nm1);
    return false;
}

}  // namespace sdlg
