// CPU restatement of the reference segment-linking chain -- TEST
// INFRASTRUCTURE ONLY (see sdl_oracle.h).  Every function names the
// reference lines it follows.  Arithmetic keeps the reference's types: the
// reference's unqualified sqrt/sin/tan/cos/atan2/pow/fabs/copysign resolve to
// the double overloads, std::asin/atan/sin/cos/tan/abs/min/max on floats stay
// float, and the unqualified abs at MiniDoublet.cc:273,787 and
// Segment.cc:743-744 is the integer abs of a truncated float.  Build with
// -ffp-contract=off so no multiply-add is fused.
#include "sdl_oracle.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <thread>
#include <unordered_map>
#include <utility>
#include <vector>

// The reference's unqualified math calls resolve to the double overloads;
// the explicit ::calls below must do the same in this translation unit.
static_assert(sizeof(::sqrt(1.0f)) == sizeof(double), "::sqrt must be the double overload");
static_assert(sizeof(::pow(1.0f, 2)) == sizeof(double), "::pow must be the double overload");
static_assert(sizeof(::sin(1.0f)) == sizeof(double), "::sin must be the double overload");
static_assert(sizeof(::tan(1.0f)) == sizeof(double), "::tan must be the double overload");
static_assert(sizeof(::atan2(1.0f, 1.0f)) == sizeof(double), "::atan2 must be the double overload");
static_assert(sizeof(::fabs(1.0f)) == sizeof(double), "::fabs must be the double overload");
static_assert(sizeof(::copysign(1.0f, 1.0f)) == sizeof(double), "::copysign must be the double overload");
static_assert(sizeof(std::asin(1.0f)) == sizeof(float), "std::asin(float) must be the float overload");

namespace {

// ---------------------------------------------------------------- float libm
// The reference's std::asin/atan/sin/cos/tan on floats are glibc's float
// functions, which are not always correctly rounded; the GPU chain uses the
// correctly rounded float (the double function rounded once).  A switch
// (sdlo_set_libm) makes the restatement use either, or the glibc values while
// counting the calls where the two differ, so that the effect of the libm
// difference on the objects can be measured.  Default: glibc, as the
// reference.
enum { kLibmGlibc = 0, kLibmRounded = 1, kLibmCount = 2 };
std::atomic<int> g_libm_mode(kLibmGlibc);
std::atomic<uint64_t> g_libm_calls(0), g_libm_diff(0);
thread_local int tl_libm = kLibmGlibc;
thread_local uint64_t tl_calls = 0, tl_diff = 0;

inline float libm_pick(float glibc, double exact) {
    const float r = (float)exact;
    if (tl_libm == kLibmRounded) return r;
    ++tl_calls;
    if (!(r == glibc) && !(std::isnan(r) && std::isnan(glibc))) ++tl_diff;
    return glibc;
}
inline float f_asin(float x) { return tl_libm == kLibmGlibc ? std::asin(x) : libm_pick(std::asin(x), ::asin((double)x)); }
inline float f_atan(float x) { return tl_libm == kLibmGlibc ? std::atan(x) : libm_pick(std::atan(x), ::atan((double)x)); }
inline float f_sin(float x) { return tl_libm == kLibmGlibc ? std::sin(x) : libm_pick(std::sin(x), ::sin((double)x)); }
inline float f_cos(float x) { return tl_libm == kLibmGlibc ? std::cos(x) : libm_pick(std::cos(x), ::cos((double)x)); }
inline float f_tan(float x) { return tl_libm == kLibmGlibc ? std::tan(x) : libm_pick(std::tan(x), ::tan((double)x)); }
// a worker thread takes the process-wide mode and hands back its counts
struct LibmScope {
    LibmScope() { tl_libm = g_libm_mode.load(); tl_calls = tl_diff = 0; }
    ~LibmScope() { g_libm_calls += tl_calls; g_libm_diff += tl_diff; }
};

// ---------------------------------------------------------------- cut trace
// Every cut of the algorithms goes through CUT(decision, value, lo, hi): the
// decision is returned unchanged; with a trace switched on (the near-cut
// audit, sdlo_audit), the compared value and its bounds are recorded so that
// a decision can be reported with its distance to the cut.
struct CutRec {
    const char* where;  // the algorithm
    const char* cut;    // the decision as written
    float value, lo, hi;
    bool pass;
};
thread_local std::vector<CutRec>* tl_trace = nullptr;
const float kNoBound = INFINITY;
inline bool cut_rec(bool pass, const char* where, const char* cut, float value, float lo, float hi) {
    if (tl_trace) tl_trace->push_back({where, cut, value, lo, hi, pass});
    return pass;
}
#define CUT(pass, value, lo, hi) cut_rec((pass), __func__, #pass, (value), (lo), (hi))

constexpr float kSdlInf = 123456789;  // MiniDoublet.cc:3, compared as float
const double kPi = M_PI;

// ---------------------------------------------------------------- helpers
// x86-64 truncating float->int conversion (cvttss2si): out-of-range and NaN
// give INT_MIN.  Written out so the result is the same on every host.
inline int trunc_i32(float f) {
    if (!(f > -2147483649.0f && f < 2147483648.0f)) return INT_MIN;
    return (int)f;
}
// C abs(int) as compiled on x86-64 (two's complement wrap for INT_MIN).
inline int iabs(int v) { return v < 0 ? (int)(0u - (unsigned)v) : v; }
inline float fmin_ref(float a, float b) { return (b < a) ? b : a; }  // std::min
inline float fmax_ref(float a, float b) { return (a < b) ? b : a; }  // std::max

// MathUtil.cc:3-19
float phi_mpi_pi(float x) {
    if (std::isnan(x)) return x;
    while (x >= kPi) x -= 2. * kPi;
    while (x < -kPi) x += 2. * kPi;
    return x;
}
// MathUtil.cc:21-27
float atan2_ref(float y, float x) {
    if (x != 0) return ::atan2((double)y, (double)x);
    if (y == 0) return 0;
    if (y > 0) return kPi / 2;
    return -kPi / 2;
}

// A point with the derived quantities the cuts read (Hit.cc:68-83).  eta is
// never read by the chain and is not kept.
struct P3 {
    float x, y, z, rt, phi, r3;
};
P3 mk(float x, float y, float z) {
    P3 p;
    p.x = x; p.y = y; p.z = z;
    p.r3 = ::sqrt((double)(x * x + y * y + z * z));
    p.rt = ::sqrt((double)(x * x + y * y));
    p.phi = phi_mpi_pi(kPi + atan2_ref(-y, -x));
    return p;
}
P3 sub(const P3& a, const P3& b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }  // Hit.cc:205-208
// Hit.cc:149-152
float dphi(const P3& a, const P3& b) { return phi_mpi_pi(b.phi - a.phi); }
// Hit.cc:154-173
float dphichange(const P3& a, const P3& b) { return dphi(a, sub(b, a)); }
// midpoint as Hit(); += a; += b; /= 2 (Tracklet.cc:1191-1194)
P3 midpoint(const P3& a, const P3& b) {
    float x = 0.f, y = 0.f, z = 0.f;
    x += a.x; y += a.y; z += a.z;
    x += b.x; y += b.y; z += b.z;
    const float two = 2;
    x /= two; y /= two; z /= two;
    return mk(x, y, z);
}

// ---------------------------------------------------------------- modules
enum { kEndcap = 4, kBarrel = 5 };
enum { kNegZ = 1, kPosZ = 2, kCenter = 3 };
enum { kPS = 0, kTwoS = 1 };
enum { kPixel = 0, kStrip = 1 };

struct ModInfo {
    uint32_t detid, partner;
    uint16_t subdet, side, layer, rod, ring, module;
    bool lower, inverted;
    uint8_t type, ltype;
};

// Module.cc:159-358
ModInfo decode(uint32_t d) {
    ModInfo m;
    m.detid = d;
    m.subdet = (d & (7u << 25)) >> 25;
    const bool ec = m.subdet == kEndcap, br = m.subdet == kBarrel;
    m.side = ec ? (d & (3u << 23)) >> 23 : br ? (d & (3u << 18)) >> 18 : 0;
    m.layer = ec ? (d & (7u << 18)) >> 18 : br ? (d & (7u << 20)) >> 20 : 0;
    m.rod = br ? (d & (127u << 10)) >> 10 : 0;
    m.ring = ec ? (d & (15u << 12)) >> 12 : 0;
    m.module = (d & (127u << 2)) >> 2;
    bool inv = false;
    if (ec) {
        if (m.side == kNegZ) inv = m.module % 2 == 1;
        else if (m.side == kPosZ) inv = m.module % 2 == 0;
    } else if (br) {
        if (m.side == kCenter) {
            if (m.layer <= 3) inv = m.module % 2 == 1;
            else inv = m.module % 2 == 0;   // layer >= 4
        } else if (m.side == kNegZ || m.side == kPosZ) {
            if (m.layer <= 2) inv = m.module % 2 == 1;
            else if (m.layer == 3) inv = m.module % 2 == 0;
        }
    }
    m.inverted = inv;
    m.lower = inv ? !(d & 1) : (d & 1);
    if (m.lower) m.partner = inv ? d - 1 : d + 1;
    else m.partner = inv ? d + 1 : d - 1;
    if (br) m.type = m.layer <= 3 ? kPS : kTwoS;
    else if (m.layer <= 2) m.type = m.ring <= 10 ? kPS : kTwoS;
    else m.type = m.ring <= 7 ? kPS : kTwoS;
    if (m.type == kTwoS) m.ltype = kStrip;
    else if (inv) m.ltype = m.lower ? kStrip : kPixel;
    else m.ltype = m.lower ? kPixel : kStrip;
    return m;
}

// ---------------------------------------------------------------- geometry
struct Geo {
    std::unordered_map<uint32_t, std::pair<float, float>> tilted;  // drdz, slope
    std::unordered_map<uint32_t, std::pair<float, float>> endcap;  // slope lower, centroid phi (col 7)
    std::unordered_map<uint32_t, std::vector<uint32_t>> conn;
    float drdz(uint32_t d) const { auto it = tilted.find(d); return it == tilted.end() ? 0.f : it->second.first; }
    float tslope(uint32_t d) const { auto it = tilted.find(d); return it == tilted.end() ? 0.f : it->second.second; }
    float eslope(uint32_t d) const { auto it = endcap.find(d); return it == endcap.end() ? 0.f : it->second.first; }
    float ephi(uint32_t d) const { auto it = endcap.find(d); return it == endcap.end() ? 0.f : it->second.second; }
    const std::vector<uint32_t>& connected(uint32_t d) const {
        static const std::vector<uint32_t> empty;
        auto it = conn.find(d);
        return it == conn.end() ? empty : it->second;
    }
};

// MiniDoublet.cc:1242-1257
bool tighter_tilted(const ModInfo& m) {
    const bool b = m.subdet == kBarrel;
    return (b && m.side != kCenter && m.layer == 3) ||
           (b && m.side == kNegZ && m.layer == 2 && m.rod > 5) ||
           (b && m.side == kPosZ && m.layer == 2 && m.rod < 8) ||
           (b && m.side == kNegZ && m.layer == 1 && m.rod > 9) ||
           (b && m.side == kPosZ && m.layer == 1 && m.rod < 4);
}

// MiniDoublet.cc:1260-1332
float gap_size(const ModInfo& m) {
    static const float tilted[3] = {0.26f, 0.26f, 0.26f};
    static const float loose[3] = {0.4f, 0.4f, 0.4f};
    static const float flat[6] = {0.26f, 0.16f, 0.16f, 0.18f, 0.18f, 0.18f};
    const unsigned iL = m.layer - 1;
    if (m.subdet == kBarrel && m.side == kCenter) return flat[iL];
    if (tighter_tilted(m)) return tilted[iL];
    if (m.subdet == kEndcap) {
        const int iR = m.ring - 1;
        const int lim = (iL <= 1) ? 10 : (iL <= 3) ? 8 : 9;
        return iR < lim ? 0.4f : 0.18f;
    }
    return loose[iL];
}

// constants as the reference spells them (double literals rounded to float)
const float kRinv1GeVf = (2.99792458e-3 * 3.8);
const float k2Rinv1GeVf = kRinv1GeVf / 2.;
const float kSinAlphaMax = 0.95;
const float kPtCut = 1.0;  // PTCUT (Constants.h:4)
const float kPixelPSZpitch = 0.15;
const float kStrip2SZpitch = 5.0;
const float kDeltaZLum = 15.f;

// ---------------------------------------------------------------- event
struct Hit {
    P3 p;
    int idx;
    int mod;
    bool edge;
    P3 hi, lo;  // 2S endcap strip edges (Event.cc:132-138)
};
struct MD {
    int lo, up, anchor, mod;
    float dz, shiftedDz, dphi, dphichange;
};
struct SG {
    int imd, omd, mod;
    float dphi, dphimin, dphimax, dphichange, dphiminchange, dphimaxchange;
};
struct Pair {
    int in, out;
};

struct Result {
    std::vector<int32_t> t[5];
    std::vector<float> vals[2];  // per mini-doublet 4 floats, per segment 6, in tuple order
    uint32_t counters[110];
    double seconds[5];
};

struct Event {
    const Geo& geo;
    std::vector<ModInfo> mods;
    std::unordered_map<uint32_t, int> modIndex;
    std::vector<int> lowerMods;
    std::vector<std::vector<int>> modHits, modMDs, modSGs, modTLs, modTPs;
    std::map<std::pair<int, int>, std::vector<int>> layerMDs, layerSGs, layerTLs;  // (subdet, layer)
    std::vector<Hit> hits;
    std::vector<MD> mds;
    std::vector<SG> sgs;
    std::vector<Pair> tls, tps, tcs;
    std::vector<Pair> tcsTP;  // track candidates built from two triplets (createTrackCandidatesFromTriplets)
    std::vector<int> tcLayer;
    uint32_t cnt[5][2][11];
    int tlMode = 0;  // 0 default, 1 DefaultNm1

    explicit Event(const Geo& g) : geo(g) { std::memset(cnt, 0, sizeof(cnt)); }

    // Event.cc:54-78 (modules are created on demand; lower ones are listed)
    int module(uint32_t d) {
        auto it = modIndex.find(d);
        if (it != modIndex.end()) return it->second;
        int i = (int)mods.size();
        mods.push_back(decode(d));
        modIndex.emplace(d, i);
        modHits.emplace_back(); modMDs.emplace_back(); modSGs.emplace_back();
        modTLs.emplace_back(); modTPs.emplace_back();
        if (mods[i].lower) lowerMods.push_back(i);
        return i;
    }
    bool has(uint32_t d) const { return modIndex.count(d) != 0; }
    void count(int stage, int obj, const ModInfo& m) {
        if (m.subdet == kBarrel) cnt[stage][obj][m.layer - 1]++;
        else cnt[stage][obj][6 + m.layer - 1]++;
    }

    // GeometryUtil.cc:3-23
    P3 strip_edge(const P3& h, uint32_t moddet, bool up) const {
        float phi = geo.ephi(moddet);
        float sign = up ? 1. : -1;
        float ex = sign * 2.5 * ::cos((double)phi);
        float ey = sign * 2.5 * ::sin((double)phi);
        float ez = 0;
        ex += h.x; ey += h.y; ez += h.z;
        return mk(ex, ey, ez);
    }

    // Event.cc:120-139
    void add_hit(float x, float y, float z, int idx, uint32_t d) {
        Hit h;
        h.p = mk(x, y, z);
        h.idx = idx;
        h.mod = module(d);
        const ModInfo& m = mods[h.mod];
        h.edge = m.subdet == kEndcap && m.type == kTwoS;
        if (h.edge) {
            h.hi = strip_edge(h.p, d, true);
            h.lo = strip_edge(h.p, d, false);
        }
        modHits[h.mod].push_back((int)hits.size());
        hits.push_back(h);
    }

    // MiniDoublet.cc:60-81
    int anchor_of(int lo, int up, const ModInfo& lm) const {
        if (lm.type == kPS) return lm.ltype == kPixel ? lo : up;
        return lo;
    }

    // MiniDoublet.cc:741-810
    float dphi_threshold(const P3& h, const ModInfo& m, float dPhi = 0, float dz = 1) const {
        static const float mulsB[6] = {0.0052f, 0.0038f, 0.0034f, 0.0034f, 0.0032f, 0.0034f};
        static const float mulsE[5] = {0.006f, 0.006f, 0.006f, 0.006f, 0.006f};
        static const float rB[6] = {21.8f, 34.6f, 49.6f, 67.4f, 87.6f, 106.8f};
        static const float rE[5] = {131.4f, 156.2f, 185.6f, 220.3f, 261.5f};
        const float ptCut = 1;
        const float sinAlphaMax = 0.95;
        const float rt = h.rt;
        const unsigned iL = m.layer - 1;
        const float miniSlope = f_asin(fmin_ref(rt * k2Rinv1GeVf / ptCut, sinAlphaMax));
        const float rLay = m.subdet == kBarrel ? rB[iL] : rE[iL];
        const float miniPVoff = 0.1 / rLay;
        const float miniMuls = m.subdet == kBarrel ? mulsB[iL] * 3.f / ptCut : mulsE[iL] * 3.f / ptCut;
        const bool isTilted = m.subdet == kBarrel && m.side != kCenter;
        const float pitch = 0.15;
        const uint32_t detid = m.ltype == kPixel ? m.partner : m.detid;
        const float drdz = geo.drdz(detid);
        const float miniTilt = isTilted ? 0.5f * pitch * drdz / ::sqrt((double)(1.f + drdz * drdz)) / gap_size(m) : 0;
        const float deltaZLum = 15.f;
        const float miniLum = iabs(trunc_i32(dPhi * deltaZLum / dz));
        if (m.subdet == kBarrel && m.side == kCenter)
            return miniSlope + ::sqrt(::pow(miniMuls, 2) + ::pow(miniPVoff, 2));
        if (m.subdet == kBarrel)
            return miniSlope + ::sqrt(::pow(miniMuls, 2) + ::pow(miniPVoff, 2) + ::pow(miniTilt * miniSlope, 2));
        return miniSlope + ::sqrt(::pow(miniMuls, 2) + ::pow(miniPVoff, 2) + ::pow(miniLum, 2));
    }

    // MiniDoublet.cc:989-1209
    void shift_strip(const P3& lo, const P3& up, const ModInfo& lm, float& xn, float& yn, float& zn) const {
        const P3* pix;
        const P3* str;
        uint32_t detid;
        if (lm.type == kPS) {
            if (lm.ltype == kPixel) { pix = &lo; str = &up; detid = lm.partner; }
            else { pix = &up; str = &lo; detid = lm.detid; }
        } else {
            pix = &lo; str = &up; detid = lm.detid;
        }
        const bool isEndcap = lm.subdet == kEndcap;
        float angleA = ::fabs((double)f_atan(pix->rt / pix->z));
        float angleB = isEndcap ? kPi / 2. : (double)f_atan(geo.drdz(detid));
        float sep = gap_size(lm);
        if (lm.type == kPS && lm.ltype != kPixel) sep *= -1;
        float drprime = (sep / f_sin(angleA + angleB)) * f_sin(angleA);
        float slope = 0;
        if (lm.subdet == kEndcap) slope = geo.eslope(detid);
        if (lm.subdet == kBarrel) slope = geo.tslope(detid);
        float absArctanSlope = (slope != kSdlInf) ? ::fabs((double)f_atan(slope)) : kPi / 2;
        float xp = pix->x, yp = pix->y;
        float angleM;
        if (xp > 0 && yp > 0) angleM = absArctanSlope;
        else if (xp > 0 && yp < 0) angleM = kPi - absArctanSlope;
        else if (xp < 0 && yp < 0) angleM = kPi + absArctanSlope;
        else angleM = 2 * kPi - absArctanSlope;
        float dx = drprime * f_sin(angleM);
        float dy = drprime * f_cos(angleM);
        float xa = xp + dx, ya = yp + dy;
        float xo = str->x, yo = str->y;
        if (slope == kSdlInf) { xn = xa; yn = yo; }
        else if (slope == 0) { xn = xo; yn = ya; }
        else {
            xn = (slope * xa + (1.f / slope) * xo - ya + yo) / (slope + (1.f / slope));
            yn = (xn - xa) * slope + ya;
        }
        float absdzprime = ::fabs((double)(sep / f_sin(angleA + angleB) * f_cos(angleA)));
        float abszn;
        if (lm.ltype == kPixel) abszn = ::fabs((double)pix->z) + absdzprime;
        else abszn = ::fabs((double)pix->z) - absdzprime;
        zn = abszn * ((pix->z > 0) ? 1 : -1);
    }

    // MiniDoublet.cc:243-447
    bool md_barrel(const P3& lo, const P3& up, const ModInfo& lm, MD& md) const {
        md.dz = lo.z - up.z;
        const float dz = md.dz;
        const float dzCut = lm.type == kPS ? 2.f : 10.f;
        const float sign = ((dz > 0) - (dz < 0)) * ((lo.z > 0) - (lo.z < 0));
        const float inverted = (iabs(trunc_i32(dz)) > 2) * sign;
        if (!CUT(std::abs(dz) < dzCut && inverted <= 0, std::abs(dz), -kNoBound, dzCut)) return false;
        const float miniCut = lm.ltype == kPixel ? dphi_threshold(lo, lm) : dphi_threshold(up, lm);
        float xn = 0, yn = 0, zn = 0;
        P3 shifted;
        if (lm.side != kCenter) {
            shift_strip(lo, up, lm, xn, yn, zn);
            if (lm.ltype == kPixel) { shifted = mk(xn, yn, up.z); md.dphi = dphi(lo, shifted); }
            else { shifted = mk(xn, yn, lo.z); md.dphi = dphi(shifted, up); }
        } else {
            md.dphi = dphi(lo, up);
        }
        if (!CUT(std::abs(md.dphi) < miniCut, std::abs(md.dphi), -kNoBound, miniCut)) return false;
        if (lm.side != kCenter) {
            if (lm.ltype == kPixel)
                md.dphichange = lo.rt < shifted.rt ? dphichange(lo, shifted) : dphichange(shifted, lo);
            else
                md.dphichange = shifted.rt < up.rt ? dphichange(shifted, up) : dphichange(up, shifted);
        } else {
            md.dphichange = dphichange(lo, up);
        }
        return CUT(std::abs(md.dphichange) < miniCut, std::abs(md.dphichange), -kNoBound, miniCut);
    }

    // MiniDoublet.cc:449-684
    bool md_endcap(const P3& lo, const P3& up, const ModInfo& lm, MD& md) const {
        md.dz = lo.z - up.z;
        float dz = md.dz;
        const float dzCut = 10.f;  // side() is never SubDet::Endcap (MiniDoublet.cc:470)
        if (!CUT(std::abs(dz) < dzCut, std::abs(dz), -kNoBound, dzCut)) return false;
        const float drtCut = lm.type == kPS ? 2.f : 10.f;
        float drt = std::abs(lo.rt - up.rt);
        if (!CUT(drt < drtCut, drt, -kNoBound, drtCut)) return false;
        float xn = 0, yn = 0, zn = 0;
        shift_strip(lo, up, lm, xn, yn, zn);
        P3 shifted;
        if (lm.type == kPS) {
            if (lm.ltype == kPixel) { shifted = mk(xn, yn, up.z); md.dphi = dphi(lo, shifted); }
            else { shifted = mk(xn, yn, lo.z); md.dphi = dphi(shifted, up); }
        } else {
            shifted = mk(xn, yn, up.z);
            md.dphi = dphi(lo, shifted);
        }
        if (lm.type == kPS) {
            md.shiftedDz = lm.ltype == kPixel ? lo.z - zn : up.z - zn;
            dz = md.shiftedDz;
        }
        const float miniCut = lm.ltype == kPixel ? dphi_threshold(lo, lm, md.dphi, dz)
                                                 : dphi_threshold(up, lm, md.dphi, dz);
        if (!CUT(std::abs(md.dphi) < miniCut, std::abs(md.dphi), -kNoBound, miniCut)) return false;
        float dzFrac = std::abs(dz) / ::fabs((double)lo.z);
        md.dphichange = md.dphi / dzFrac * (1.f + dzFrac);
        return CUT(std::abs(md.dphichange) < miniCut, std::abs(md.dphichange), -kNoBound, miniCut);
    }

    // Event.cc:245-305
    void create_mds(int algo) {
        const std::vector<int> lower = lowerMods;  // copy, as getLowerModulePtrs() returns one
        for (int li : lower) {
            const ModInfo lm = mods[li];
            int ui = module(lm.partner);
            for (int lh : modHits[li]) {
                for (int uh : modHits[ui]) {
                    count(0, 0, lm);
                    MD md;
                    md.lo = lh; md.up = uh; md.mod = li;
                    md.dz = 0; md.shiftedDz = 0; md.dphi = 0; md.dphichange = 0;
                    bool pass;
                    if (algo == 1) pass = true;
                    else if (lm.subdet == kBarrel) pass = md_barrel(hits[lh].p, hits[uh].p, lm, md);
                    else pass = md_endcap(hits[lh].p, hits[uh].p, lm, md);
                    if (!pass) continue;
                    count(0, 1, lm);
                    md.anchor = anchor_of(lh, uh, lm);
                    int id = (int)mds.size();
                    mds.push_back(md);
                    modMDs[li].push_back(id);
                    layerMDs[{lm.subdet, lm.layer}].push_back(id);
                }
            }
        }
    }

    // Segment.cc:886-994
    void dalpha_threshold(const MD& imd, const MD& omd, float th[3]) const {
        static const float mulsB[6] = {0.0052f, 0.0038f, 0.0034f, 0.0034f, 0.0032f, 0.0034f};
        static const float mulsE[5] = {0.006f, 0.006f, 0.006f, 0.006f, 0.006f};
        const ModInfo& im = mods[imd.mod];
        const ModInfo& om = mods[omd.mod];
        const float ptCut = 1.0;
        const float sinAlphaMax = 0.95;
        float sdMuls = im.subdet == kBarrel ? mulsB[im.layer - 1] * 3.f / ptCut : mulsE[im.layer - 1] * 3.f / ptCut;
        const P3& ia = hits[imd.anchor].p;
        const P3& oa = hits[omd.anchor].p;
        float segmentDr = ::sqrt(::pow(oa.y - ia.y, 2) + ::pow(oa.x - ia.x, 2));
        const float dAlpha_Bfield = f_asin(fmin_ref(segmentDr * k2Rinv1GeVf / ptCut, sinAlphaMax));
        const float pitch = 0.15;
        const bool inTilt = im.subdet == kBarrel && im.side != kCenter;
        const bool outTilt = om.subdet == kBarrel && om.side != kCenter;
        const uint32_t idet = im.ltype == kPixel ? im.partner : im.detid;
        const uint32_t odet = om.ltype == kPixel ? om.partner : om.detid;
        const float drdzi = geo.drdz(idet);
        const float drdzo = geo.drdz(odet);
        const float iTilt = inTilt ? (0.5f * pitch * drdzi / ::sqrt((double)(1.f + drdzi * drdzi)) / gap_size(im)) : 0;
        const float oTilt = outTilt ? (0.5f * pitch * drdzo / ::sqrt((double)(1.f + drdzo * drdzo)) / gap_size(om)) : 0;
        float miniDelta = gap_size(im);
        float lumIn, lumOut;
        if (im.subdet == kBarrel) lumIn = iTilt * dAlpha_Bfield;
        else if (im.type == kPS) lumIn = imd.dphi * 15.0 / imd.shiftedDz;
        else lumIn = imd.dphi * 15.0 / imd.dz;
        if (om.subdet == kBarrel) lumOut = oTilt * dAlpha_Bfield;
        else if (om.type == kPS) lumOut = omd.dphi * 15.0 / omd.shiftedDz;
        else lumOut = omd.dphi * 15.0 / omd.dz;
        float resIn = 0.02f / miniDelta * (im.subdet == kBarrel ? 1.0f : std::abs(ia.z / ia.rt));
        float resOut = 0.02f / miniDelta * (om.subdet == kBarrel ? 1.0f : std::abs(oa.z / oa.rt));
        float res = resIn + resOut;
        if (im.subdet == kBarrel && im.side == kCenter)
            th[0] = dAlpha_Bfield + ::sqrt(::pow(res, 2) + ::pow(sdMuls, 2));
        else
            th[0] = dAlpha_Bfield + ::sqrt(::pow(res, 2) + ::pow(sdMuls, 2) + ::pow(lumIn, 2));
        if (om.subdet == kBarrel && om.side == kCenter)
            th[1] = dAlpha_Bfield + ::sqrt(::pow(res, 2) + ::pow(sdMuls, 2));
        else
            th[1] = dAlpha_Bfield + ::sqrt(::pow(res, 2) + ::pow(sdMuls, 2) + ::pow(lumOut, 2));
        th[2] = dAlpha_Bfield + ::sqrt(::pow(res, 2) + ::pow(sdMuls, 2));
    }

    bool dalpha_cuts(const MD& imd, const MD& omd, float sg_alpha) const {
        float th[3];
        dalpha_threshold(imd, omd, th);
        if (!CUT(std::abs(imd.dphichange - sg_alpha) < th[0], std::abs(imd.dphichange - sg_alpha), -kNoBound, th[0])) return false;
        if (!CUT(std::abs(omd.dphichange - sg_alpha) < th[1], std::abs(omd.dphichange - sg_alpha), -kNoBound, th[1])) return false;
        return CUT(std::abs(omd.dphichange - imd.dphichange) < th[2], std::abs(omd.dphichange - imd.dphichange), -kNoBound, th[2]);
    }

    // Segment.cc:364-599
    bool sg_barrel(const MD& imd, const MD& omd, SG& sg) const {
        static const float mulsB[6] = {0.0052f, 0.0038f, 0.0034f, 0.0034f, 0.0032f, 0.0034f};
        const ModInfo& im = mods[imd.mod];
        const float sdMuls = mulsB[im.layer - 1] * 3.f / kPtCut;
        const P3& ia = hits[imd.anchor].p;
        const P3& oa = hits[omd.anchor].p;
        float rtIn = ia.rt, rtOut = oa.rt, zIn = ia.z, zOut = oa.z;
        const float sdSlope = f_asin(fmin_ref(rtOut * k2Rinv1GeVf / kPtCut, kSinAlphaMax));
        const float sdPVoff = 0.1f / rtOut;
        const float dzDrtScale = f_tan(sdSlope) / sdSlope;
        const float zGeom = im.layer <= 2 ? 2.f * kPixelPSZpitch : 2.f * kStrip2SZpitch;
        float zLo = zIn + (zIn - kDeltaZLum) * (rtOut / rtIn - 1.f) * (zIn > 0.f ? 1.f : dzDrtScale) - zGeom;
        float zHi = zIn + (zIn + kDeltaZLum) * (rtOut / rtIn - 1.f) * (zIn < 0.f ? 1.f : dzDrtScale) + zGeom;
        if (!CUT(zOut >= zLo && zOut <= zHi, zOut, zLo, zHi)) return false;
        const float sdCut = sdSlope + ::sqrt((double)(sdMuls * sdMuls + sdPVoff * sdPVoff));
        const float deltaPhi = dphi(ia, oa);
        if (!CUT(std::abs(deltaPhi) <= sdCut, std::abs(deltaPhi), -kNoBound, sdCut)) return false;
        sg.dphichange = dphichange(ia, oa);
        if (!CUT(std::abs(sg.dphichange) <= sdCut, std::abs(sg.dphichange), -kNoBound, sdCut)) return false;
        return dalpha_cuts(imd, omd, sg.dphichange);
    }

    // Segment.cc:601-859
    bool sg_endcap(const MD& imd, const MD& omd, SG& sg) const {
        const ModInfo& im = mods[imd.mod];
        const ModInfo& om = mods[omd.mod];
        bool found = false;
        for (uint32_t d : geo.connected(im.detid))
            if (om.detid == d) { found = true; break; }
        bool l2r123 = (im.ring == 1 || im.ring == 2 || im.ring == 3) && im.layer == 2;
        if (!CUT(found || l2r123, 0.f, -kNoBound, kNoBound)) return false;
        const Hit& iah = hits[imd.anchor];
        const Hit& oah = hits[omd.anchor];
        const P3& ia = iah.p;
        const P3& oa = oah.p;
        const bool out2S = om.type == kTwoS && om.subdet == kEndcap;
        const P3& oHi = out2S ? oah.hi : oa;
        const P3& oLo = out2S ? oah.lo : oa;
        float rtIn = ia.rt, rtOut = oa.rt, zIn = ia.z, zOut = oa.z;
        const float sdSlope = f_asin(fmin_ref(rtOut * k2Rinv1GeVf / kPtCut, kSinAlphaMax));
        const float disks2SMinRadius = 60.f;
        const float rtGeom = (rtIn < disks2SMinRadius && rtOut < disks2SMinRadius) ? (2.f * kPixelPSZpitch)
                           : ((rtIn < disks2SMinRadius || rtOut < disks2SMinRadius) ? (kPixelPSZpitch + kStrip2SZpitch)
                           : (2.f * kStrip2SZpitch));
        if (!CUT(!(zIn * zOut < 0), zIn * zOut, 0.f, kNoBound)) return false;
        const float dz = zOut - zIn;
        const float dLum = std::copysign(kDeltaZLum, zIn);
        const float drtDzScale = sdSlope / f_tan(sdSlope);
        float rtLo = fmax_ref(rtIn * (1.f + dz / (zIn + dLum) * drtDzScale) - rtGeom, rtIn - 0.5f * rtGeom);
        float rtHi = rtIn * (zOut - dLum) / (zIn - dLum) + rtGeom;
        if (!CUT(rtOut >= rtLo && rtOut <= rtHi, rtOut, rtLo, rtHi)) return false;
        const float dPhiPos = dphi(ia, oa);
        const float sdCut = sdSlope;
        const float hiP = dphi(ia, oHi);
        const float loP = dphi(ia, oLo);
        const bool hiBigger = iabs(trunc_i32(hiP)) > iabs(trunc_i32(loP));
        sg.dphi = dPhiPos;
        sg.dphimax = hiBigger ? hiP : loP;
        sg.dphimin = hiBigger ? loP : hiP;
        if (!CUT(std::abs(dPhiPos) <= sdCut, std::abs(dPhiPos), -kNoBound, sdCut)) return false;
        const float dzFrac = dz / zIn;
        sg.dphichange = dPhiPos / dzFrac * (1.f + dzFrac);
        sg.dphiminchange = sg.dphimin / dzFrac * (1.f + dzFrac);
        sg.dphimaxchange = sg.dphimax / dzFrac * (1.f + dzFrac);
        if (!CUT(std::abs(sg.dphichange) <= sdCut, std::abs(sg.dphichange), -kNoBound, sdCut)) return false;
        return dalpha_cuts(imd, omd, sg.dphichange);
    }

    // Segment.cc:296-362
    bool run_sg(int a, int b, int algo, SG& sg) const {
        sg.imd = a; sg.omd = b; sg.mod = mds[a].mod;
        sg.dphi = sg.dphimin = sg.dphimax = sg.dphichange = sg.dphiminchange = sg.dphimaxchange = 0;
        if (algo == 1) return true;
        const ModInfo& im = mods[mds[a].mod];
        const ModInfo& om = mods[mds[b].mod];
        if (im.subdet == kBarrel) {
            if (om.subdet == kBarrel) return sg_barrel(mds[a], mds[b], sg);
            return sg_endcap(mds[a], mds[b], sg);
        }
        if (om.subdet == kEndcap) return sg_endcap(mds[a], mds[b], sg);
        return sg_barrel(mds[a], mds[b], sg);
    }

    void add_sg(const SG& sg) {
        int id = (int)sgs.size();
        sgs.push_back(sg);
        const ModInfo& im = mods[sg.mod];
        modSGs[sg.mod].push_back(id);
        layerSGs[{im.subdet, im.layer}].push_back(id);
    }

    // Event.cc:445-522
    void create_sgs_map(int algo) {
        const std::vector<int> lower = lowerMods;
        for (int m1 : lower) {
            const ModInfo m1i = mods[m1];
            for (int a : modMDs[m1]) {
                for (uint32_t d2 : geo.connected(m1i.detid)) {
                    if (!has(d2)) continue;
                    int m2 = modIndex.at(d2);
                    for (int b : modMDs[m2]) {
                        SG sg;
                        bool pass = run_sg(a, b, algo, sg);
                        count(1, 0, m1i);
                        if (pass) {
                            count(1, 1, m1i);
                            add_sg(sg);
                        }
                    }
                }
            }
        }
    }

    // Event.cc:432-443, 793-821 and the pair table Layer.cc:32-50
    void create_sgs_layer(int algo) {
        static const int pairs[16][4] = {
            {kBarrel, 1, kBarrel, 2}, {kBarrel, 2, kBarrel, 3}, {kBarrel, 3, kBarrel, 4},
            {kBarrel, 4, kBarrel, 5}, {kBarrel, 5, kBarrel, 6}, {kBarrel, 1, kEndcap, 1},
            {kBarrel, 2, kEndcap, 1}, {kBarrel, 3, kEndcap, 1}, {kBarrel, 4, kEndcap, 1},
            {kBarrel, 5, kEndcap, 1}, {kEndcap, 1, kEndcap, 2}, {kEndcap, 2, kEndcap, 3},
            {kEndcap, 2, kEndcap, 4}, {kEndcap, 2, kEndcap, 5}, {kEndcap, 3, kEndcap, 4},
            {kEndcap, 4, kEndcap, 5}};
        for (auto& p : pairs) {
            const std::vector<int> inner = layerMDs[{p[0], p[1]}];
            const std::vector<int> outer = layerMDs[{p[2], p[3]}];
            for (int a : inner)
                for (int b : outer) {
                    SG sg;
                    if (run_sg(a, b, algo, sg)) add_sg(sg);
                }
        }
    }

    // ------------------------------------------------------------ tracklets
    struct Quad {
        const Hit *inLo, *inUp, *outLo, *outUp;
        const ModInfo *mInLo, *mInUp, *mOutLo, *mOutUp;
        const SG *isg, *osg;
    };

    // Tracklet.cc:3181-3324
    static void delta_beta_iterations(float& betaIn, float& betaOut, float& betaAv, float& pt_beta, float sdIn_dr,
                                      float sdOut_dr, float dr, int lIn, float pt_betaMax) {
        const float sinAlphaMax = 0.95;
        if (betaIn * betaOut > 0.f &&
            (std::abs(pt_beta) < 4.f * pt_betaMax || (lIn >= 11 && std::abs(pt_beta) < 8.f * pt_betaMax))) {
            const float betaInUpd = betaIn + ::copysign((double)f_asin(fmin_ref(sdIn_dr * k2Rinv1GeVf / std::abs(pt_beta), sinAlphaMax)), (double)betaIn);
            const float betaOutUpd = betaOut + ::copysign((double)f_asin(fmin_ref(sdOut_dr * k2Rinv1GeVf / std::abs(pt_beta), sinAlphaMax)), (double)betaOut);
            betaAv = 0.5f * (betaInUpd + betaOutUpd);
            pt_beta = dr * k2Rinv1GeVf / ::sin((double)betaAv);
            betaIn += ::copysign((double)f_asin(fmin_ref(sdIn_dr * k2Rinv1GeVf / std::abs(pt_beta), sinAlphaMax)), (double)betaIn);
            betaOut += ::copysign((double)f_asin(fmin_ref(sdOut_dr * k2Rinv1GeVf / std::abs(pt_beta), sinAlphaMax)), (double)betaOut);
            betaAv = 0.5f * (betaIn + betaOut);
            pt_beta = dr * k2Rinv1GeVf / ::sin((double)betaAv);
        } else if (lIn < 11 && std::abs(betaOut) < 0.2 * std::abs(betaIn) && std::abs(pt_beta) < 12.f * pt_betaMax) {
            const float pt_betaIn = dr * k2Rinv1GeVf / ::sin((double)betaIn);
            const float betaInUpd = betaIn + ::copysign((double)f_asin(fmin_ref(sdIn_dr * k2Rinv1GeVf / std::abs(pt_betaIn), sinAlphaMax)), (double)betaIn);
            const float betaOutUpd = betaOut + ::copysign((double)f_asin(fmin_ref(sdOut_dr * k2Rinv1GeVf / std::abs(pt_betaIn), sinAlphaMax)), (double)betaIn);
            betaAv = (std::abs(betaOut) > 0.2f * std::abs(betaIn)) ? (0.5f * (betaInUpd + betaOutUpd)) : betaInUpd;
            pt_beta = dr * k2Rinv1GeVf / ::sin((double)betaAv);
            betaIn += ::copysign((double)f_asin(fmin_ref(sdIn_dr * k2Rinv1GeVf / std::abs(pt_beta), sinAlphaMax)), (double)betaIn);
            betaOut += ::copysign((double)f_asin(fmin_ref(sdOut_dr * k2Rinv1GeVf / std::abs(pt_beta), sinAlphaMax)), (double)betaIn);
            betaAv = 0.5f * (betaIn + betaOut);
            pt_beta = dr * k2Rinv1GeVf / ::sin((double)betaAv);
        }
    }

    // the common tail of the three algorithms: dBeta cut (returns pass)
    bool dbeta_cut(float betaIn, float betaOut, float dBetaCut2) const {
        const float dBeta = betaIn - betaOut;
        if (!CUT(dBeta * dBeta <= dBetaCut2, dBeta * dBeta, -kNoBound, dBetaCut2)) return tlMode == 1;
        return true;
    }

    // Tracklet.cc:902-1538
    bool tl_bbbb(const Quad& q) const {
        const float pt_betaMax = 7.0f;
        const bool isPS_InLo = q.mInLo->type == kPS;
        const bool isPS_OutLo = q.mOutLo->type == kPS;
        const float rt_InLo = q.inLo->p.rt, rt_OutLo = q.outLo->p.rt;
        const float z_InLo = q.inLo->p.z, z_OutLo = q.outLo->p.z;
        const float alpha1GeV_OutLo = f_asin(fmin_ref(rt_OutLo * k2Rinv1GeVf / kPtCut, kSinAlphaMax));
        const float rtRatio = rt_OutLo / rt_InLo;
        const float dzDrtScale = ::tan((double)alpha1GeV_OutLo) / alpha1GeV_OutLo;
        const float zpitch_InLo = isPS_InLo ? kPixelPSZpitch : kStrip2SZpitch;
        const float zpitch_OutLo = isPS_OutLo ? kPixelPSZpitch : kStrip2SZpitch;
        const float zHi = z_InLo + (z_InLo + kDeltaZLum) * (rtRatio - 1.f) * (z_InLo < 0.f ? 1.f : dzDrtScale) + (zpitch_InLo + zpitch_OutLo);
        const float zLo = z_InLo + (z_InLo - kDeltaZLum) * (rtRatio - 1.f) * (z_InLo > 0.f ? 1.f : dzDrtScale) - (zpitch_InLo + zpitch_OutLo);
        if (!CUT(z_OutLo >= zLo && z_OutLo <= zHi, z_OutLo, zLo, zHi)) return false;
        const float drt_OutLo_InLo = rt_OutLo - rt_InLo;
        const float r3_InLo = ::sqrt((double)(z_InLo * z_InLo + rt_InLo * rt_InLo));
        const float drt_InSeg = q.inUp->p.rt - q.inLo->p.rt;
        const float dz_InSeg = q.inUp->p.z - q.inLo->p.z;
        const float dr3_InSeg = q.inUp->p.r3 - q.inLo->p.r3;
        const float coshEta = dr3_InSeg / drt_InSeg;
        float dzErr = (zpitch_InLo + zpitch_OutLo) * (zpitch_InLo + zpitch_OutLo) * 2.f;
        const float sdlThetaMulsF = 0.015f * ::sqrt(0.1f + 0.2 * (rt_OutLo - rt_InLo) / 50.f) * ::sqrt((double)(r3_InLo / rt_InLo));
        const float sdlMuls = sdlThetaMulsF * 3.f / kPtCut * 4.f;
        dzErr += sdlMuls * sdlMuls * drt_OutLo_InLo * drt_OutLo_InLo / 3.f * coshEta * coshEta;
        dzErr = ::sqrt((double)dzErr);
        const float dzMean = dz_InSeg / drt_InSeg * drt_OutLo_InLo;
        const float zWindow = dzErr / drt_InSeg * drt_OutLo_InLo + (zpitch_InLo + zpitch_OutLo);
        const float zLoPointed = z_InLo + dzMean * (z_InLo > 0.f ? 1.f : dzDrtScale) - zWindow;
        const float zHiPointed = z_InLo + dzMean * (z_InLo < 0.f ? 1.f : dzDrtScale) + zWindow;
        if (!CUT(z_OutLo >= zLoPointed && z_OutLo <= zHiPointed, z_OutLo, zLoPointed, zHiPointed)) return false;
        const float sdlPVoff = 0.1f / rt_OutLo;
        const float sdlCut = alpha1GeV_OutLo + ::sqrt((double)(sdlMuls * sdlMuls + sdlPVoff * sdlPVoff));
        const P3& hInUp = q.inUp->p;
        const P3& hOutUp = q.outUp->p;
        const P3& hInLo = q.inLo->p;
        const P3& hOutLo = q.outLo->p;
        float deltaPhiPos = dphi(hInUp, hOutUp);
        if (!CUT(std::abs(deltaPhiPos) <= sdlCut, std::abs(deltaPhiPos), -kNoBound, sdlCut)) return false;
        const P3 mid = midpoint(hInLo, hOutLo);
        const float dPhi = dphi(mid, sub(hOutLo, hInLo));
        if (!CUT(std::abs(dPhi) <= sdlCut, std::abs(dPhi), -kNoBound, sdlCut)) return false;
        const float alpha_InLo = q.isg->dphichange;
        const bool isEC_lastLayer = q.mOutUp->subdet == kEndcap && q.mOutUp->type == kTwoS;
        const P3 hiE = isEC_lastLayer ? strip_edge(hOutUp, q.mOutUp->detid, true) : hOutUp;
        const P3 loE = isEC_lastLayer ? strip_edge(hOutUp, q.mOutUp->detid, false) : hOutUp;
        const float alpha_OutUp = dphi(hOutUp, sub(hOutUp, hOutLo));
        const float alpha_OutUp_hi = dphi(hiE, sub(hiE, hOutLo));
        const float alpha_OutUp_lo = dphi(loE, sub(loE, hOutLo));
        const P3 tl_axis = sub(hOutUp, hInLo);
        const P3 tl_axis_hi = sub(hiE, hInLo);
        const P3 tl_axis_lo = sub(loE, hInLo);
        float betaIn = alpha_InLo - dphi(hInLo, tl_axis);
        float betaInRHmin = betaIn, betaInRHmax = betaIn;
        float betaOut = -alpha_OutUp + dphi(hOutUp, tl_axis);
        float betaOutRHmin = -alpha_OutUp_hi + dphi(hiE, tl_axis_hi);
        float betaOutRHmax = -alpha_OutUp_lo + dphi(loE, tl_axis_lo);
        const float drt_tl_axis = tl_axis.rt;
        const float corrF = 1.f;
        const float rt_InSeg = sub(hInUp, hInLo).rt;
        const float betaIn_cut = f_asin(fmin_ref((-rt_InSeg * corrF + drt_tl_axis) * k2Rinv1GeVf / kPtCut, kSinAlphaMax)) + (0.02f / drt_InSeg);
        if (!CUT(std::abs(betaInRHmin) < betaIn_cut, std::abs(betaInRHmin), -kNoBound, betaIn_cut)) return false;
        float betaAv = 0.5f * (betaIn + betaOut);
        float pt_beta = drt_tl_axis * k2Rinv1GeVf / ::sin((double)betaAv);
        const int lIn = 5;
        const int lOut = isEC_lastLayer ? 11 : 5;
        const float sdOut_dr = sub(hOutUp, hOutLo).rt;
        const float sdOut_d = hOutUp.rt - hOutLo.rt;
        delta_beta_iterations(betaIn, betaOut, betaAv, pt_beta, rt_InSeg, sdOut_dr, drt_tl_axis, lIn, pt_betaMax);
        const float betaInMMSF = (std::abs(betaInRHmin + betaInRHmax) > 0) ? (2.f * betaIn / std::abs(betaInRHmin + betaInRHmax)) : 0.;
        const float betaOutMMSF = (std::abs(betaOutRHmin + betaOutRHmax) > 0) ? (2.f * betaOut / std::abs(betaOutRHmin + betaOutRHmax)) : 0.;
        betaInRHmin *= betaInMMSF; betaInRHmax *= betaInMMSF;
        betaOutRHmin *= betaOutMMSF; betaOutRHmax *= betaOutMMSF;
        const float dBetaMuls = sdlThetaMulsF * 4.f / fmin_ref(std::abs(pt_beta), pt_betaMax);
        const float sdIn_rt = hInLo.rt, sdOut_rt = hOutLo.rt, sdIn_z = hInLo.z, sdOut_z = hOutLo.z;
        const float alpha_OutLo = q.osg->dphichange;
        const float alphaInAbsReg = fmax_ref(std::abs(alpha_InLo), f_asin(fmin_ref(sdIn_rt * k2Rinv1GeVf / 3.0f, kSinAlphaMax)));
        const float alphaOutAbsReg = fmax_ref(std::abs(alpha_OutLo), f_asin(fmin_ref(sdOut_rt * k2Rinv1GeVf / 3.0f, kSinAlphaMax)));
        const float dBetaInLum = lIn < 11 ? 0.0f : std::abs(alphaInAbsReg * kDeltaZLum / sdIn_z);
        const float dBetaOutLum = lOut < 11 ? 0.0f : std::abs(alphaOutAbsReg * kDeltaZLum / sdOut_z);
        const float dBetaLum2 = (dBetaInLum + dBetaOutLum) * (dBetaInLum + dBetaOutLum);
        const float sinDPhi = f_sin(dPhi);
        const float dBetaRIn2 = 0;
        const float dBetaROut2 = ::pow((double)((hiE.rt - loE.rt) * sinDPhi / drt_tl_axis), 2);
        const float betaOut_cut = f_asin(fmin_ref(drt_tl_axis * k2Rinv1GeVf / kPtCut, kSinAlphaMax)) + (0.02f / sdOut_d) + ::sqrt((double)(dBetaLum2 + dBetaMuls * dBetaMuls));
        if (!CUT(std::abs(betaOut) < betaOut_cut, std::abs(betaOut), -kNoBound, betaOut_cut)) return false;
        const float dBetaRes = 0.02f / fmin_ref(sdOut_d, drt_InSeg);
        const float dBetaCut2 = (dBetaRes * dBetaRes * 2.0f + dBetaMuls * dBetaMuls + dBetaLum2 + dBetaRIn2 + dBetaROut2 +
                                 0.25 * ::pow((double)(std::abs(betaInRHmin - betaInRHmax) + std::abs(betaOutRHmin - betaOutRHmax)), 2));
        return dbeta_cut(betaIn, betaOut, dBetaCut2);
    }

    // Tracklet.cc:1540-2016
    bool tl_bbee(const Quad& q) const {
        const float pt_betaMax = 7.0f;
        const float zGeom = (q.mInLo->type == kPS ? kPixelPSZpitch : kStrip2SZpitch) + (q.mOutLo->type == kPS ? kPixelPSZpitch : kStrip2SZpitch);
        const float rtIn = q.inLo->p.rt, rtOut = q.outLo->p.rt, zIn = q.inLo->p.z, zOut = q.outLo->p.z;
        const float sdlSlope = f_asin(fmin_ref(rtOut * k2Rinv1GeVf / kPtCut, kSinAlphaMax));
        const float dzDrtScale = ::tan((double)sdlSlope) / sdlSlope;
        if (!CUT(zIn * zOut > 0, zIn * zOut, 0.f, kNoBound)) return false;
        const float dLum = std::copysign(kDeltaZLum, zIn);
        const bool isOutSgInnerMDPS = q.mOutLo->type == kPS;
        const float rtGeom1 = isOutSgInnerMDPS ? kPixelPSZpitch : kStrip2SZpitch;
        const float zGeom1 = std::copysign(zGeom, zIn);
        const float rtLo = rtIn * (1.f + (zOut - zIn - zGeom1) / (zIn + zGeom1 + dLum) / dzDrtScale) - rtGeom1;
        if (!CUT(rtOut >= rtLo, rtOut, rtLo, kNoBound)) return false;
        float zInForHi = zIn - zGeom1 - dLum;
        if (zInForHi * zIn < 0) zInForHi = std::copysign(0.1f, zIn);
        const float rtHi = rtIn * (1.f + (zOut - zIn + zGeom1) / zInForHi) + rtGeom1;
        if (!CUT(rtOut >= rtLo && rtOut <= rtHi, rtOut, rtLo, rtHi)) return false;
        const float rIn = ::sqrt((double)(zIn * zIn + rtIn * rtIn));
        const float drtSDIn = q.inUp->p.rt - q.inLo->p.rt;
        const float dzSDIn = q.inUp->p.z - q.inLo->p.z;
        const float dr3SDIn = q.inUp->p.r3 - q.inLo->p.r3;
        const float coshEta = dr3SDIn / drtSDIn;
        const float dzOutInAbs = std::abs(zOut - zIn);
        const float multDzDr = dzOutInAbs * coshEta / (coshEta * coshEta - 1.f);
        const float zGeom1_another = kPixelPSZpitch;
        const float kZ = (zOut - zIn) / dzSDIn;
        float drtErr = zGeom1_another * zGeom1_another * drtSDIn * drtSDIn / dzSDIn / dzSDIn * (1.f - 2.f * kZ + 2.f * kZ * kZ);
        const float sdlThetaMulsF = 0.015f * ::sqrt(0.1f + 0.2 * (rtOut - rtIn) / 50.f) * ::sqrt((double)(rIn / rtIn));
        const float sdlMuls = sdlThetaMulsF * 3.f / kPtCut * 4.f;
        drtErr += sdlMuls * sdlMuls * multDzDr * multDzDr / 3.f * coshEta * coshEta;
        drtErr = ::sqrt((double)drtErr);
        if (!CUT(kZ >= 0 && rtOut >= rtLo && rtOut <= rtHi, rtOut, rtLo, rtHi)) return false;
        const float sdlPVoff = 0.1f / rtOut;
        const float sdlCut = sdlSlope + ::sqrt((double)(sdlMuls * sdlMuls + sdlPVoff * sdlPVoff));
        const P3& hInUp = q.inUp->p;
        const P3& hOutUp = q.outUp->p;
        const P3& hInLo = q.inLo->p;
        const P3& hOutLo = q.outLo->p;
        float deltaPhiPos = dphi(hInUp, hOutUp);
        if (!CUT(std::abs(deltaPhiPos) <= sdlCut, std::abs(deltaPhiPos), -kNoBound, sdlCut)) return false;
        const P3 mid = midpoint(hInLo, hOutLo);
        const float dPhi = dphi(mid, sub(hOutLo, hInLo));
        if (!CUT(std::abs(dPhi) <= sdlCut, std::abs(dPhi), -kNoBound, sdlCut)) return false;
        const float sdIn_alpha = q.isg->dphichange;
        const float sdOut_alpha = q.isg->dphichange;  // (sic) Tracklet.cc:1790
        const float sdOut_alphaOut = dphi(hOutUp, sub(hOutUp, hOutLo));
        const float sdOut_alphaOut_min = phi_mpi_pi(q.osg->dphiminchange - q.osg->dphimin);
        const float sdOut_alphaOut_max = phi_mpi_pi(q.osg->dphimaxchange - q.osg->dphimax);
        const P3 dr3 = sub(hOutUp, hInLo);
        float betaIn = sdIn_alpha - dphi(hInLo, dr3);
        float betaOut = -sdOut_alphaOut + dphi(hOutUp, dr3);
        // isEC_secondLayer compares subdet() with ModuleType::TwoS: always false (Tracklet.cc:1798)
        float betaInRHmin = betaIn;
        float betaInRHmax = betaIn;
        float betaOutRHmin = betaOut - sdOut_alphaOut_min + sdOut_alphaOut;
        float betaOutRHmax = betaOut - sdOut_alphaOut_max + sdOut_alphaOut;
        if (std::abs(betaOutRHmin) > std::abs(betaOutRHmax)) std::swap(betaOutRHmax, betaOutRHmin);
        if (std::abs(betaInRHmin) > std::abs(betaInRHmax)) std::swap(betaInRHmax, betaInRHmin);
        const float sdIn_dr = sub(hInUp, hInLo).rt;
        const float sdIn_d = hInUp.rt - hInLo.rt;
        const float dr = dr3.rt;
        const float corrF = 1.f;
        const float betaIn_cut = f_asin(fmin_ref((-sdIn_dr * corrF + dr) * k2Rinv1GeVf / kPtCut, kSinAlphaMax)) + (0.02f / sdIn_d);
        if (!CUT(std::abs(betaInRHmin) < betaIn_cut, std::abs(betaInRHmin), -kNoBound, betaIn_cut)) return false;
        float betaAv = 0.5f * (betaIn + betaOut);
        float pt_beta = dr * k2Rinv1GeVf / ::sin((double)betaAv);
        const int lIn = 5, lOut = 11;
        const float sdOut_dr = sub(hOutUp, hOutLo).rt;
        const float sdOut_d = hOutUp.rt - hOutLo.rt;
        delta_beta_iterations(betaIn, betaOut, betaAv, pt_beta, sdIn_dr, sdOut_dr, dr, lIn, pt_betaMax);
        const float betaInMMSF = (std::abs(betaInRHmin + betaInRHmax) > 0) ? 2.f * betaIn / std::abs(betaInRHmin + betaInRHmax) : 0.;
        const float betaOutMMSF = (std::abs(betaOutRHmin + betaOutRHmax) > 0) ? 2.f * betaOut / std::abs(betaOutRHmin + betaOutRHmax) : 0.;
        betaInRHmin *= betaInMMSF; betaInRHmax *= betaInMMSF;
        betaOutRHmin *= betaOutMMSF; betaOutRHmax *= betaOutMMSF;
        const float dBetaMuls = sdlThetaMulsF * 4.f / fmin_ref(std::abs(pt_beta), pt_betaMax);
        const float sdIn_rt = hInLo.rt, sdOut_rt = hOutLo.rt, sdIn_z = hInLo.z, sdOut_z = hOutLo.z;
        const float alphaInAbsReg = fmax_ref(std::abs(sdIn_alpha), f_asin(fmin_ref(sdIn_rt * k2Rinv1GeVf / 3.0f, kSinAlphaMax)));
        const float alphaOutAbsReg = fmax_ref(std::abs(sdOut_alpha), f_asin(fmin_ref(sdOut_rt * k2Rinv1GeVf / 3.0f, kSinAlphaMax)));
        const float dBetaInLum = lIn < 11 ? 0.0f : std::abs(alphaInAbsReg * kDeltaZLum / sdIn_z);
        const float dBetaOutLum = lOut < 11 ? 0.0f : std::abs(alphaOutAbsReg * kDeltaZLum / sdOut_z);
        const float dBetaLum2 = (dBetaInLum + dBetaOutLum) * (dBetaInLum + dBetaOutLum);
        const float sinDPhi = f_sin(dPhi);
        const bool out2S = q.mOutUp->type == kTwoS;
        const P3& hiE = out2S ? q.outUp->hi : hOutUp;
        const P3& loE = out2S ? q.outUp->lo : hOutUp;
        const float dBetaRIn2 = 0;
        const float dBetaROut2 = ::pow((double)((hiE.rt - loE.rt) * sinDPhi / dr), 2);
        const float betaOut_cut = f_asin(fmin_ref(dr * k2Rinv1GeVf / kPtCut, kSinAlphaMax)) + (0.02f / sdOut_d) + ::sqrt((double)(dBetaLum2 + dBetaMuls * dBetaMuls));
        if (!CUT(std::abs(betaOut) < betaOut_cut, std::abs(betaOut), -kNoBound, betaOut_cut)) return false;
        const float dBetaRes = 0.02f / fmin_ref(sdOut_d, sdIn_d);
        const float dBetaCut2 = (dBetaRes * dBetaRes * 2.0f + dBetaMuls * dBetaMuls + dBetaLum2 + dBetaRIn2 + dBetaROut2 +
                                 0.25 * ::pow((double)(std::abs(betaInRHmin - betaInRHmax) + std::abs(betaOutRHmin - betaOutRHmax)), 2));
        return dbeta_cut(betaIn, betaOut, dBetaCut2);
    }

    // Tracklet.cc:2018-2665
    bool tl_eeee(const Quad& q) const {
        const float pt_betaMax = 7.0f;
        const float zGeom = (q.mInLo->type == kPS ? kPixelPSZpitch : kStrip2SZpitch) + (q.mOutLo->type == kPS ? kPixelPSZpitch : kStrip2SZpitch);
        (void)zGeom;
        const float rtIn = q.inLo->p.rt, rtOut = q.outLo->p.rt, zIn = q.inLo->p.z, zOut = q.outLo->p.z;
        const float sdlSlope = f_asin(fmin_ref(rtOut * k2Rinv1GeVf / kPtCut, kSinAlphaMax));
        const float dzDrtScale = ::tan((double)sdlSlope) / sdlSlope;
        if (!CUT(zIn * zOut > 0, zIn * zOut, 0.f, kNoBound)) return false;
        const float dLum = std::copysign(kDeltaZLum, zIn);
        const bool isOutSgInnerMDPS = q.mOutLo->type == kPS;
        const bool isInSgInnerMDPS = q.mInLo->type == kPS;
        const float rtGeom = (isInSgInnerMDPS && isOutSgInnerMDPS) ? 2.f * kPixelPSZpitch
                           : (isInSgInnerMDPS || isOutSgInnerMDPS) ? (kPixelPSZpitch + kStrip2SZpitch) : 2.f * kStrip2SZpitch;
        const float dz = zOut - zIn;
        const float rtLo = rtIn * (1.f + dz / (zIn + dLum) / dzDrtScale) - rtGeom;
        if (!CUT(rtOut >= rtLo, rtOut, rtLo, kNoBound)) return false;
        const float rtHi = rtIn * (1.f + dz / (zIn - dLum)) + rtGeom;
        if (!CUT(rtOut >= rtLo && rtOut <= rtHi, rtOut, rtLo, rtHi)) return false;
        const bool isInSgOuterMDPS = q.mInUp->type == kPS;
        const float drtSDIn = q.inUp->p.rt - q.inLo->p.rt;
        const float dzSDIn = q.inUp->p.z - q.inLo->p.z;
        const float dr3SDIn = q.inUp->p.r3 - q.inLo->p.r3;
        const float coshEta = dr3SDIn / drtSDIn;
        const float dzOutInAbs = std::abs(zOut - zIn);
        const float multDzDr = dzOutInAbs * coshEta / (coshEta * coshEta - 1.f);
        const float kZ = (zOut - zIn) / dzSDIn;
        const float sdlThetaMulsF = 0.015f * ::sqrt(0.1f + 0.2 * (rtOut - rtIn) / 50.f);
        const float sdlMuls = sdlThetaMulsF * 3.f / kPtCut * 4.f;
        float drtErr = kPixelPSZpitch * kPixelPSZpitch * 2.f / dzSDIn / dzSDIn * dzOutInAbs * dzOutInAbs;
        drtErr += sdlMuls * sdlMuls * multDzDr * multDzDr / 3.f * coshEta * coshEta;
        drtErr = ::sqrt((double)drtErr);
        const float drtMean = drtSDIn * dzOutInAbs / std::abs(dzSDIn);
        const float rtWindow = drtErr + rtGeom;
        const float rtLo_point = rtIn + drtMean / dzDrtScale - rtWindow;
        const float rtHi_point = rtIn + drtMean + rtWindow;
        if (isInSgInnerMDPS && isInSgOuterMDPS) {
            if (!CUT(kZ >= 0 && rtOut >= rtLo_point && rtOut <= rtHi_point, rtOut, rtLo_point, rtHi_point)) return false;
        }
        const float sdlPVoff = 0.1f / rtOut;
        const float sdlCut = sdlSlope + ::sqrt((double)(sdlMuls * sdlMuls + sdlPVoff * sdlPVoff));
        const P3& hInUp = q.inUp->p;
        const P3& hOutUp = q.outUp->p;
        const P3& hInLo = q.inLo->p;
        const P3& hOutLo = q.outLo->p;
        float deltaPhiPos = dphi(hInUp, hOutUp);
        if (!CUT(std::abs(deltaPhiPos) <= sdlCut, std::abs(deltaPhiPos), -kNoBound, sdlCut)) return false;
        const P3 mid = midpoint(hInLo, hOutLo);
        const float dPhi = dphi(mid, sub(hOutLo, hInLo));
        if (!CUT(std::abs(dPhi) <= sdlCut, std::abs(dPhi), -kNoBound, sdlCut)) return false;
        const float sdIn_alpha = q.isg->dphichange;
        const float sdOut_alpha = q.isg->dphichange;  // (sic)
        float sdOut_dPhiPos = dphi(hOutLo, hOutUp);
        float sdOut_dPhiChange = q.osg->dphichange;
        float sdOut_dPhiChange_min = q.osg->dphiminchange;
        float sdOut_dPhiChange_max = q.osg->dphimaxchange;
        float sdOut_alphaOutRHmin = phi_mpi_pi(sdOut_dPhiChange_min - sdOut_dPhiPos);
        float sdOut_alphaOutRHmax = phi_mpi_pi(sdOut_dPhiChange_max - sdOut_dPhiPos);
        float sdOut_alphaOut = phi_mpi_pi(sdOut_dPhiChange - sdOut_dPhiPos);
        const P3 dr3 = sub(hOutUp, hInLo);
        float betaIn = sdIn_alpha - dphi(hInLo, dr3);
        float betaOut = -sdOut_alphaOut + dphi(hOutUp, dr3);
        float sdIn_alphaRHmin = q.isg->dphiminchange;
        float sdIn_alphaRHmax = q.isg->dphimaxchange;
        float betaInRHmin = betaIn + sdIn_alphaRHmin - sdIn_alpha;
        float betaInRHmax = betaIn + sdIn_alphaRHmax - sdIn_alpha;
        if (std::abs(betaInRHmin) > std::abs(betaInRHmax)) std::swap(betaInRHmax, betaInRHmin);
        float betaOutRHmin = betaOut - sdOut_alphaOutRHmin + sdOut_alphaOut;
        float betaOutRHmax = betaOut - sdOut_alphaOutRHmax + sdOut_alphaOut;
        if (std::abs(betaOutRHmin) > std::abs(betaOutRHmax)) std::swap(betaOutRHmax, betaOutRHmin);
        const float sdIn_dr = sub(hInUp, hInLo).rt;
        const float sdIn_d = hInUp.rt - hInLo.rt;
        const float dr = dr3.rt;
        // Cut #6 (betaIn) does not reject in this algorithm (Tracklet.cc:2327-2336)
        float betaAv = 0.5f * (betaIn + betaOut);
        float pt_beta = dr * k2Rinv1GeVf / ::sin((double)betaAv);
        const int lIn = 11, lOut = 13;
        const float sdOut_dr = sub(hOutUp, hOutLo).rt;
        const float sdOut_d = hOutUp.rt - hOutLo.rt;
        delta_beta_iterations(betaIn, betaOut, betaAv, pt_beta, sdIn_dr, sdOut_dr, dr, lIn, pt_betaMax);
        const float betaInMMSF = (std::abs(betaInRHmin + betaInRHmax) > 0) ? (2.f * betaIn / std::abs(betaInRHmin + betaInRHmax)) : 0.;
        const float betaOutMMSF = (std::abs(betaOutRHmin + betaOutRHmax) > 0) ? (2.f * betaOut / std::abs(betaOutRHmin + betaOutRHmax)) : 0.;
        betaInRHmin *= betaInMMSF; betaInRHmax *= betaInMMSF;
        betaOutRHmin *= betaOutMMSF; betaOutRHmax *= betaOutMMSF;
        const float dBetaMuls = sdlThetaMulsF * 4.f / fmin_ref(std::abs(pt_beta), pt_betaMax);
        const float sdIn_rt = hInLo.rt, sdOut_rt = hOutLo.rt, sdIn_z = hInLo.z, sdOut_z = hOutLo.z;
        const float alphaInAbsReg = fmax_ref(std::abs(sdIn_alpha), f_asin(fmin_ref(sdIn_rt * k2Rinv1GeVf / 3.0f, kSinAlphaMax)));
        const float alphaOutAbsReg = fmax_ref(std::abs(sdOut_alpha), f_asin(fmin_ref(sdOut_rt * k2Rinv1GeVf / 3.0f, kSinAlphaMax)));
        const float dBetaInLum = lIn < 11 ? 0.0f : std::abs(alphaInAbsReg * kDeltaZLum / sdIn_z);
        const float dBetaOutLum = lOut < 11 ? 0.0f : std::abs(alphaOutAbsReg * kDeltaZLum / sdOut_z);
        const float dBetaLum2 = (dBetaInLum + dBetaOutLum) * (dBetaInLum + dBetaOutLum);
        const float dBetaRIn2 = 0;
        const float dBetaROut2 = 0;
        const float betaOut_cut = f_asin(fmin_ref(dr * k2Rinv1GeVf / kPtCut, kSinAlphaMax)) + (0.02f / sdOut_d) + ::sqrt((double)(dBetaLum2 + dBetaMuls * dBetaMuls));
        if (!CUT(std::abs(betaOut) < betaOut_cut, std::abs(betaOut), -kNoBound, betaOut_cut)) return false;
        const float dBetaRes = 0.02f / fmin_ref(sdOut_d, sdIn_d);
        const float dBetaCut2 = (dBetaRes * dBetaRes * 2.0f + dBetaMuls * dBetaMuls + dBetaLum2 + dBetaRIn2 + dBetaROut2 +
                                 0.25 * ::pow((double)(std::abs(betaInRHmin - betaInRHmax) + std::abs(betaOutRHmin - betaOutRHmax)), 2));
        return dbeta_cut(betaIn, betaOut, dBetaCut2);
    }

    // Tracklet.cc:144-296
    bool run_tl(int si, int so, int algo) const {
        if (algo == 2) return true;  // AllComb
        const SG& a = sgs[si];
        const SG& b = sgs[so];
        Quad q;
        q.isg = &a; q.osg = &b;
        q.inLo = &hits[mds[a.imd].anchor]; q.inUp = &hits[mds[a.omd].anchor];
        q.outLo = &hits[mds[b.imd].anchor]; q.outUp = &hits[mds[b.omd].anchor];
        q.mInLo = &mods[q.inLo->mod]; q.mInUp = &mods[q.inUp->mod];
        q.mOutLo = &mods[q.outLo->mod]; q.mOutUp = &mods[q.outUp->mod];
        const bool b1 = q.mInLo->subdet == kBarrel, b2 = q.mInUp->subdet == kBarrel;
        const bool b3 = q.mOutLo->subdet == kBarrel, b4 = q.mOutUp->subdet == kBarrel;
        const bool e1 = q.mInLo->subdet == kEndcap, e2 = q.mInUp->subdet == kEndcap;
        const bool e3 = q.mOutLo->subdet == kEndcap, e4 = q.mOutUp->subdet == kEndcap;
        if (b1 && b2 && b3 && b4) return tl_bbbb(q);
        if (b1 && b2 && e3 && e4) return tl_bbee(q);
        if (b1 && b2 && b3 && e4) return tl_bbbb(q);
        if (b1 && e2 && e3 && e4) return tl_bbee(q);
        if (e1 && e2 && e3 && e4) return tl_eeee(q);
        return false;
    }

    void add_tl(int si, int so, bool toModule) {
        int id = (int)tls.size();
        tls.push_back({si, so});
        const ModInfo& m = mods[sgs[si].mod];
        if (toModule) modTLs[sgs[si].mod].push_back(id);
        layerTLs[{m.subdet, m.layer}].push_back(id);
    }

    // Event.cc:611-693
    void create_tls_map(int algo) {
        const std::vector<int> lower = lowerMods;
        for (int m1 : lower) {
            const ModInfo m1i = mods[m1];
            for (int si : modSGs[m1]) {
                const ModInfo& m2 = mods[mds[sgs[si].omd].mod];
                for (uint32_t d3 : geo.connected(m2.detid)) {
                    if (!has(d3)) continue;
                    int m3 = modIndex.at(d3);
                    for (int so : modSGs[m3]) {
                        count(2, 0, m1i);
                        if (run_tl(si, so, algo)) {
                            count(2, 1, m1i);
                            add_tl(si, so, true);
                        }
                    }
                }
            }
        }
    }

    // Event.cc:694-751: inner segment x segments leaving its outer MD x
    // segments leaving their outer MD (MiniDoublet.cc:40-58: every segment is
    // listed at its inner MD as outward); counted and stored at the inner
    // segment's lower module
    void create_tls_nav(int algo) {
        std::vector<std::vector<int>> outward(mds.size());
        for (size_t s = 0; s < sgs.size(); ++s) outward[sgs[s].imd].push_back((int)s);
        const std::vector<int> lower = lowerMods;
        for (int m1 : lower) {
            const ModInfo m1i = mods[m1];
            for (int si : modSGs[m1])
                for (int sc : outward[sgs[si].omd])
                    for (int so : outward[sgs[sc].omd]) {
                        count(2, 0, m1i);
                        if (run_tl(si, so, algo)) {
                            count(2, 1, m1i);
                            add_tl(si, so, true);
                        }
                    }
        }
    }

    // Event.cc:599-609, 755-790 and Layer.cc:19-24
    void create_tls_layer(int algo) {
        static const int pairs[3][2] = {{1, 3}, {2, 4}, {3, 5}};
        for (auto& p : pairs) {
            const std::vector<int> inner = layerSGs[{kBarrel, p[0]}];
            const std::vector<int> outer = layerSGs[{kBarrel, p[1]}];
            for (int si : inner)
                for (int so : outer) {
                    cnt[2][0][p[0] - 1]++;
                    if (run_tl(si, so, algo)) {
                        cnt[2][1][p[0] - 1]++;
                        add_tl(si, so, false);
                    }
                }
        }
    }

    // identity of objects by hit idx (Hit.cc:175-182, MiniDoublet.cc:686-693, Segment.cc:868-875)
    uint64_t md_key(int m) const {
        return ((uint64_t)(uint32_t)hits[mds[m].lo].idx << 32) | (uint32_t)hits[mds[m].up].idx;
    }

    // Event.cc:524-597 with Triplet.cc:50-122.  The all-pairs idx comparison
    // is evaluated as an equi-join on the shared MD's (lower, upper) idx.
    void create_tps(int algo) {
        const std::vector<int> lower = lowerMods;
        for (int m1 : lower) {
            const ModInfo m1i = mods[m1];
            if (modSGs[m1].empty()) continue;
            std::unordered_map<uint64_t, std::vector<int>> byInner;
            std::vector<int> cands;
            for (uint32_t d2 : geo.connected(m1i.detid)) {
                if (!has(d2)) continue;
                int m2 = modIndex.at(d2);
                for (int so : modSGs[m2]) {
                    cands.push_back(so);
                    byInner[md_key(sgs[so].imd)].push_back(so);
                }
            }
            for (int si : modSGs[m1]) {
                cnt[3][0][(m1i.subdet == kBarrel ? 0 : 6) + m1i.layer - 1] += (uint32_t)cands.size();
                if (algo == 1) {
                    for (int so : cands) { tps.push_back({si, so}); modTPs[m1].push_back((int)tps.size() - 1); count(3, 1, m1i); }
                    continue;
                }
                auto it = byInner.find(md_key(sgs[si].omd));
                if (it == byInner.end()) continue;
                for (int so : it->second) {
                    count(3, 1, m1i);
                    modTPs[m1].push_back((int)tps.size());
                    tps.push_back({si, so});
                }
            }
        }
    }

    uint64_t sg_hash(int s) const { return md_key(sgs[s].imd) * 1000003ULL ^ md_key(sgs[s].omd); }
    bool sg_match(int a, int b) const {
        return md_key(sgs[a].imd) == md_key(sgs[b].imd) && md_key(sgs[a].omd) == md_key(sgs[b].omd);
    }

    // Event.cc:823-872 with TrackCandidate.cc:143-226: barrel layer 1
    // tracklets x barrel layer 3 tracklets; pass iff the inner tracklet's outer
    // segment idx-matches the outer tracklet's inner segment (the radius check
    // never rejects).  Evaluated as an equi-join on the segment's four idx.
    void create_tcs(int algo) {
        const std::vector<int> inner = layerTLs[{kBarrel, 1}];
        const std::vector<int> outer = layerTLs[{kBarrel, 3}];
        cnt[4][0][0] += (uint32_t)(inner.size() * outer.size());
        if (algo == 1) {
            for (int a : inner) for (int b : outer) { tcs.push_back({a, b}); cnt[4][1][0]++; }
            return;
        }
        std::unordered_map<uint64_t, std::vector<int>> byInnerSG;
        for (int b : outer) byInnerSG[sg_hash(tls[b].in)].push_back(b);
        for (int a : inner) {
            auto it = byInnerSG.find(sg_hash(tls[a].out));
            if (it == byInnerSG.end()) continue;
            for (int b : it->second)
                if (sg_match(tls[a].out, tls[b].in)) {
                    tcs.push_back({a, b});
                    cnt[4][1][0]++;
                }
        }
    }

    // Event.cc:984-1062 with TrackCandidate.cc:143-226: every module's
    // tracklets x the tracklets of the modules connected to the module of the
    // inner segment's outer MD (repeated connections repeat them); pass iff
    // the inner tracklet's outer segment idx-matches the outer tracklet's
    // inner segment
    void create_tcs_from_tls(int algo) {
        const std::vector<int> lower = lowerMods;
        for (int m1 : lower) {
            const ModInfo m1i = mods[m1];
            for (int a : modTLs[m1]) {
                const ModInfo& m2 = mods[mds[sgs[tls[a].in].omd].mod];
                for (uint32_t d3 : geo.connected(m2.detid)) {
                    if (!has(d3)) continue;
                    for (int b : modTLs[modIndex.at(d3)]) {
                        count(4, 0, m1i);
                        if (algo == 1 || sg_match(tls[a].out, tls[b].in)) {
                            count(4, 1, m1i);
                            tcs.push_back({a, b});
                        }
                    }
                }
            }
        }
    }

    // Event.cc:874-982: every module's triplets x the triplets of the modules
    // connected to the module of the triplet's outermost MD; pass iff the
    // segment from that MD to the outer triplet's innermost MD passes the
    // segment algorithm and the tracklet (that segment, the outer triplet's
    // outer segment) passes the tracklet algorithm.  The trial segment is not
    // kept.
    void create_tcs_from_tps(int algo) {
        const std::vector<int> lower = lowerMods;
        for (int m1 : lower) {
            const ModInfo m1i = mods[m1];
            for (int a : modTPs[m1]) {
                const int mdA = sgs[tps[a].out].omd;
                const ModInfo& mo = mods[mds[mdA].mod];
                for (uint32_t d3 : geo.connected(mo.detid)) {
                    if (!has(d3)) continue;
                    for (int b : modTPs[modIndex.at(d3)]) {
                        count(4, 0, m1i);
                        SG trial;
                        if (!run_sg(mdA, sgs[tps[b].in].imd, 0, trial)) continue;
                        // run_tl reads segments by index; the tracklet algorithm
                        // is the default one here (Event.cc:947-951)
                        sgs.push_back(trial);
                        const int keep = tlMode;
                        tlMode = 0;
                        const bool pass = run_tl((int)sgs.size() - 1, tps[b].out, 0);
                        tlMode = keep;
                        sgs.pop_back();
                        if (!pass) continue;
                        (void)algo;
                        count(4, 1, m1i);
                        tcsTP.push_back({a, b});
                    }
                }
            }
        }
    }

    // ---------------------------------------------------------- output
    void push_md(std::vector<int32_t>& v, int m) const { v.push_back(hits[mds[m].lo].idx); v.push_back(hits[mds[m].up].idx); }
    void push_sg(std::vector<int32_t>& v, int s) const { push_md(v, sgs[s].imd); push_md(v, sgs[s].omd); }
    void push_tl(std::vector<int32_t>& v, const Pair& p) const { push_sg(v, p.in); push_sg(v, p.out); }

    void emit(Result& r) const {
        for (size_t i = 0; i < mds.size(); ++i) {
            push_md(r.t[0], (int)i);
            const MD& m = mds[i];
            r.vals[0].insert(r.vals[0].end(), {m.dz, m.shiftedDz, m.dphi, m.dphichange});
        }
        for (size_t i = 0; i < sgs.size(); ++i) {
            push_sg(r.t[1], (int)i);
            const SG& g = sgs[i];
            r.vals[1].insert(r.vals[1].end(), {g.dphi, g.dphimin, g.dphimax, g.dphichange, g.dphiminchange, g.dphimaxchange});
        }
        for (auto& p : tls) push_tl(r.t[2], p);
        for (auto& p : tps) push_tl(r.t[3], p);
        for (auto& p : tcs) { push_tl(r.t[4], tls[p.in]); push_tl(r.t[4], tls[p.out]); }
        for (auto& p : tcsTP) { push_tl(r.t[4], tps[p.in]); push_tl(r.t[4], tps[p.out]); }
        int k = 0;
        for (int s = 0; s < 5; ++s)
            for (int o = 0; o < 2; ++o)
                for (int l = 0; l < 11; ++l) r.counters[k++] = cnt[s][o][l];
    }
};

double now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// the chain on one event's hits, with the stage timings in r (may be NULL)
void run_chain(Event& ev, int64_t n, const float* x, const float* y, const float* z, const int32_t* idx,
               const uint32_t* detid, int mode, int stop_after, Result* r) {
    Result dummy;
    if (!r) r = &dummy;
    ev.tlMode = (mode & 4) ? 1 : 0;
    ev.hits.reserve(n);
    for (int64_t i = 0; i < n; ++i) ev.add_hit(x[i], y[i], z[i], idx[i], detid[i]);
    double t0 = now();
    ev.create_mds(0);
    r->seconds[0] = now() - t0;
    if (stop_after >= 1) {
        t0 = now();
        if (mode & 1) ev.create_sgs_layer(0); else ev.create_sgs_map(0);
        r->seconds[1] = now() - t0;
    }
    if (stop_after >= 2) {
        t0 = now();
        if (mode & 2) ev.create_tls_layer(0);
        else if (mode & 32) ev.create_tls_nav(0);
        else ev.create_tls_map(0);
        r->seconds[2] = now() - t0;
    }
    if (stop_after >= 3) {
        t0 = now();
        ev.create_tps(0);
        r->seconds[3] = now() - t0;
    }
    if (stop_after >= 4) {
        t0 = now();
        if (mode & 128) ev.create_tcs_from_tps(0);
        else if (mode & 64) ev.create_tcs_from_tls(0);
        else ev.create_tcs(0);
        r->seconds[4] = now() - t0;
    }
}

Result* run_event(const Geo& g, int64_t n, const float* x, const float* y, const float* z, const int32_t* idx,
                  const uint32_t* detid, int mode, int stop_after) {
    LibmScope libm;
    Result* r = new Result();
    std::memset(r->seconds, 0, sizeof(r->seconds));
    Event ev(g);
    run_chain(ev, n, x, y, z, idx, detid, mode, stop_after, r);
    ev.emit(*r);
    return r;
}

// ---------------------------------------------------------------- near-cut audit
// The chain is run twice on one event, with the reference's float libm
// (glibc) and with correctly rounded floats; every object that only one of
// the two runs makes is listed.  A "primary" flip is a candidate whose
// constituents both runs made but whose cuts decide differently: it is
// evaluated again in both runs with the cut trace on, and the cut that
// rejects it in one run is reported with its compared value and bounds in
// both (the distance to the cut).  A "secondary" flip only follows from a
// primary one (a missing constituent); triplets and track candidates, which
// are joins without float cuts, can only flip that way.
struct AuditRec {
    int32_t stage, accept_glibc, primary, pad;
    int32_t tuple[8];
    float g_value, g_lo, g_hi, r_value, r_lo, r_hi;
    char where[24];
    char cut[88];
};

using Key = std::array<int32_t, 8>;

Key key_of(const std::vector<int32_t>& t, size_t row, int w) {
    Key k;
    k.fill(INT32_MIN);
    for (int c = 0; c < w; ++c) k[c] = t[row * w + c];
    return k;
}

std::vector<CutRec> traced(int libm, const std::function<void()>& f) {
    std::vector<CutRec> t;
    const int keep = tl_libm;
    tl_libm = libm;
    tl_trace = &t;
    f();
    tl_trace = nullptr;
    tl_libm = keep;
    return t;
}

void audit_event(const Geo& g, int64_t n, const float* x, const float* y, const float* z, const int32_t* idx,
                 const uint32_t* detid, int mode, std::vector<AuditRec>& out, int64_t* summary20) {
    static const int w[3] = {2, 4, 8};
    Event ev[2] = {Event(g), Event(g)};
    Result res[2];
    for (int k = 0; k < 2; ++k) {
        const int keep = tl_libm;
        tl_libm = k == 0 ? kLibmGlibc : kLibmRounded;
        run_chain(ev[k], n, x, y, z, idx, detid, mode, 4, nullptr);
        tl_libm = keep;
        ev[k].emit(res[k]);
    }
    // object index of each key (first occurrence) per stage and run
    std::map<Key, std::vector<int>> obj[3][2];
    for (int k = 0; k < 2; ++k)
        for (int s = 0; s < 3; ++s) {
            const size_t nr = res[k].t[s].size() / w[s];
            for (size_t r = 0; r < nr; ++r) obj[s][k][key_of(res[k].t[s], r, w[s])].push_back((int)r);
        }
    for (int s = 0; s < 5; ++s) {
        summary20[s * 4 + 0] = (int64_t)res[0].t[s].size() / (s == 0 ? 2 : s == 1 ? 4 : s == 4 ? 16 : 8);
        summary20[s * 4 + 1] = (int64_t)res[1].t[s].size() / (s == 0 ? 2 : s == 1 ? 4 : s == 4 ? 16 : 8);
    }
    // triplets and track candidates: secondary flips only (multiset differences)
    for (int s = 3; s < 5; ++s) {
        const int ws = s == 4 ? 16 : 8;
        std::map<std::vector<int32_t>, int64_t> c;
        for (int k = 0; k < 2; ++k)
            for (size_t r = 0; r + ws <= res[k].t[s].size(); r += ws)
                c[std::vector<int32_t>(res[k].t[s].begin() + r, res[k].t[s].begin() + r + ws)] += k == 0 ? 1 : -1;
        int64_t d = 0;
        for (auto& kv : c) d += kv.second < 0 ? -kv.second : kv.second;
        summary20[s * 4 + 2] = 0;
        summary20[s * 4 + 3] = d;
    }
    for (int s = 0; s < 3; ++s) {
        int64_t prim = 0, sec = 0;
        for (int k = 0; k < 2; ++k) {
            const int o = 1 - k;  // the run that lacks the object
            for (auto& kv : obj[s][k]) {
                auto it = obj[s][o].find(kv.first);
                const size_t have = it == obj[s][o].end() ? 0 : it->second.size();
                if (kv.second.size() <= have) continue;
                const int64_t extra = (int64_t)(kv.second.size() - have);
                const Key& K = kv.first;
                // constituents in the run that lacks it
                int ci = -1, cj = -1;
                Event& eo = ev[o];
                Event& ek = ev[k];
                const int row = kv.second[0];
                if (s == 0) {
                    ci = ek.mds[row].lo;
                    cj = ek.mds[row].up;
                } else {
                    const Key a = [&] { Key q; q.fill(INT32_MIN); for (int c = 0; c < w[s - 1]; ++c) q[c] = K[c]; return q; }();
                    const Key b = [&] { Key q; q.fill(INT32_MIN); for (int c = 0; c < w[s - 1]; ++c) q[c] = K[w[s - 1] + c]; return q; }();
                    auto ia = obj[s - 1][o].find(a), ib = obj[s - 1][o].find(b);
                    if (ia != obj[s - 1][o].end() && ib != obj[s - 1][o].end()) {
                        ci = ia->second[0];
                        cj = ib->second[0];
                    }
                }
                if (s > 0 && ci < 0) {
                    sec += extra;
                    continue;
                }
                prim += extra;
                // evaluate the candidate in both runs with the trace on
                std::vector<CutRec> tr[2];
                for (int m = 0; m < 2; ++m) {
                    Event& e = ev[m];
                    const int libm = m == 0 ? kLibmGlibc : kLibmRounded;
                    if (s == 0) {
                        const int lh = m == k ? ek.mds[row].lo : ci, uh = m == k ? ek.mds[row].up : cj;
                        const ModInfo lm = e.mods[e.hits[lh].mod];
                        tr[m] = traced(libm, [&] {
                            MD md;
                            if (lm.subdet == kBarrel) e.md_barrel(e.hits[lh].p, e.hits[uh].p, lm, md);
                            else e.md_endcap(e.hits[lh].p, e.hits[uh].p, lm, md);
                        });
                    } else if (s == 1) {
                        const int a = m == k ? ek.sgs[row].imd : ci, b = m == k ? ek.sgs[row].omd : cj;
                        tr[m] = traced(libm, [&] {
                            SG sg;
                            e.run_sg(a, b, 0, sg);
                        });
                    } else {
                        const int a = m == k ? ek.tls[row].in : ci, b = m == k ? ek.tls[row].out : cj;
                        tr[m] = traced(libm, [&] { e.run_tl(a, b, e.tlMode); });
                    }
                }
                AuditRec rec{};
                rec.stage = s;
                rec.accept_glibc = k == 0;
                rec.primary = 1;
                for (int c = 0; c < 8; ++c) rec.tuple[c] = c < w[s] ? K[c] : -1;
                // the cut that rejects it in the run that lacks it, and the same cut in the other run
                const std::vector<CutRec>& rej = tr[o];
                const CutRec* rc = nullptr;
                for (const CutRec& c : rej)
                    if (!c.pass) { rc = &c; break; }
                if (rc) {
                    std::snprintf(rec.where, sizeof(rec.where), "%s", rc->where);
                    std::snprintf(rec.cut, sizeof(rec.cut), "%s", rc->cut);
                    const CutRec* ac = nullptr;
                    for (const CutRec& c : tr[k])
                        if (c.cut == rc->cut) ac = &c;
                    const CutRec* gc = o == 0 ? rc : ac;
                    const CutRec* cc = o == 0 ? ac : rc;
                    if (gc) { rec.g_value = gc->value; rec.g_lo = gc->lo; rec.g_hi = gc->hi; }
                    if (cc) { rec.r_value = cc->value; rec.r_lo = cc->lo; rec.r_hi = cc->hi; }
                }
                out.push_back(rec);
            }
        }
        summary20[s * 4 + 2] = prim;
        summary20[s * 4 + 3] = sec;
    }
}

// Order-independent digest of an object list (hit-index tuples of width w):
// the sum mod 2^64 of one 64-bit mix per row.  sdl_gb300/tuples.py computes
// the same digest in numpy for the GPU chain's objects.
inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
uint64_t multiset_digest(const std::vector<int32_t>& t, int w) {
    uint64_t s = 0;
    for (size_t r = 0; r + w <= t.size(); r += w) {
        uint64_t h = (uint64_t)w;
        for (int c = 0; c < w; ++c) h = mix64(h ^ (uint64_t)(uint32_t)t[r + c]);
        s += h;
    }
    return s;
}

}  // namespace

extern "C" {

void* sdlo_geometry_create(int64_t n_tilted, const uint32_t* t_detid, const float* t_vals, int64_t n_endcap,
                           const uint32_t* e_detid, const float* e_vals, int64_t n_keys, const uint32_t* keys,
                           const int64_t* off, const uint32_t* dst) {
    Geo* g = new Geo();
    for (int64_t i = 0; i < n_tilted; ++i) g->tilted[t_detid[i]] = {t_vals[2 * i], t_vals[2 * i + 1]};
    // EndcapGeometry.cc:55-58: slope lower is column 3; the 7th token is stored as the centroid phi
    for (int64_t i = 0; i < n_endcap; ++i) g->endcap[e_detid[i]] = {e_vals[8 * i + 2], e_vals[8 * i + 5]};
    for (int64_t k = 0; k < n_keys; ++k) g->conn[keys[k]] = std::vector<uint32_t>(dst + off[k], dst + off[k + 1]);
    return g;
}

void sdlo_geometry_free(void* geo) { delete static_cast<Geo*>(geo); }

void* sdlo_run(const void* geo, int64_t n, const float* x, const float* y, const float* z, const int32_t* idx,
               const uint32_t* detid, int mode, int stop_after) {
    return run_event(*static_cast<const Geo*>(geo), n, x, y, z, idx, detid, mode, stop_after);
}

int sdlo_width(int stage) {
    static const int w[5] = {2, 4, 8, 8, 16};
    return (stage >= 0 && stage < 5) ? w[stage] : 0;
}

int64_t sdlo_count(const void* res, int stage) {
    const Result* r = static_cast<const Result*>(res);
    return (int64_t)r->t[stage].size() / sdlo_width(stage);
}

void sdlo_copy(const void* res, int stage, int32_t* out) {
    const Result* r = static_cast<const Result*>(res);
    if (!r->t[stage].empty()) std::memcpy(out, r->t[stage].data(), r->t[stage].size() * 4);
}

void sdlo_vals(const void* res, int stage, float* out) {
    const Result* r = static_cast<const Result*>(res);
    if ((stage == 0 || stage == 1) && !r->vals[stage].empty())
        std::memcpy(out, r->vals[stage].data(), r->vals[stage].size() * sizeof(float));
}

void sdlo_counters(const void* res, uint32_t* out110) {
    std::memcpy(out110, static_cast<const Result*>(res)->counters, 110 * 4);
}

void sdlo_times(const void* res, double* out5) { std::memcpy(out5, static_cast<const Result*>(res)->seconds, 5 * 8); }

void sdlo_free(void* res) { delete static_cast<Result*>(res); }

void sdlo_libm_values(int fn, uint32_t start_bits, int64_t n, float* out, int n_threads) {
    auto one = [fn](float x) -> float {
        switch (fn) {
            case 0: return std::asin(x);
            case 1: return std::atan(x);
            case 2: return std::sin(x);
            case 3: return std::cos(x);
            default: return std::tan(x);
        }
    };
    std::atomic<int64_t> next(0);
    auto work = [&]() {
        for (;;) {
            const int64_t k0 = next.fetch_add(1 << 16);
            if (k0 >= n) break;
            const int64_t k1 = std::min<int64_t>(n, k0 + (1 << 16));
            for (int64_t k = k0; k < k1; ++k) {
                const uint32_t u = start_bits + (uint32_t)k;
                float x;
                std::memcpy(&x, &u, 4);
                out[k] = one(x);
            }
        }
    };
    std::vector<std::thread> th;
    for (int i = 0; i < std::max(1, n_threads); ++i) th.emplace_back(work);
    for (auto& t : th) t.join();
}

int64_t sdlo_audit(const void* geo, int64_t n, const float* x, const float* y, const float* z, const int32_t* idx,
                   const uint32_t* detid, int mode, void* out, int64_t cap, int64_t* summary20) {
    std::vector<AuditRec> recs;
    audit_event(*static_cast<const Geo*>(geo), n, x, y, z, idx, detid, mode, recs, summary20);
    const int64_t m = std::min<int64_t>(cap, (int64_t)recs.size());
    if (m > 0) std::memcpy(out, recs.data(), m * sizeof(AuditRec));
    return (int64_t)recs.size();
}

int sdlo_audit_record_size() { return (int)sizeof(AuditRec); }

void sdlo_set_libm(int mode) { g_libm_mode = (mode == kLibmRounded || mode == kLibmCount) ? mode : kLibmGlibc; }

void sdlo_libm_counts(uint64_t* out2, int reset) {
    out2[0] = g_libm_calls.load();
    out2[1] = g_libm_diff.load();
    if (reset) g_libm_calls = g_libm_diff = 0;
}

int64_t sdlo_run_many(const void* geo, int64_t n_events, const int64_t* ev_off, const float* x, const float* y,
                      const float* z, const int32_t* idx, const uint32_t* detid, int mode, int n_threads) {
    std::atomic<int64_t> next(0), total(0);
    auto work = [&]() {
        for (;;) {
            int64_t e = next.fetch_add(1);
            if (e >= n_events) break;
            int64_t b = ev_off[e], n = ev_off[e + 1] - b;
            Result* r = run_event(*static_cast<const Geo*>(geo), n, x + b, y + b, z + b, idx + b, detid + b, mode, 4);
            total += (int64_t)r->t[4].size() / 16;
            delete r;
        }
    };
    std::vector<std::thread> th;
    for (int i = 0; i < std::max(1, n_threads); ++i) th.emplace_back(work);
    for (auto& t : th) t.join();
    return total.load();
}

int64_t sdlo_run_many_digest(const void* geo, int64_t n_events, const int64_t* ev_off, const float* x, const float* y,
                             const float* z, const int32_t* idx, const uint32_t* detid, int mode, int n_threads,
                             int64_t* counts, uint64_t* digests, uint32_t* counters) {
    static const int w[5] = {2, 4, 8, 8, 16};
    std::atomic<int64_t> next(0), total(0);
    auto work = [&]() {
        for (;;) {
            int64_t e = next.fetch_add(1);
            if (e >= n_events) break;
            int64_t b = ev_off[e], n = ev_off[e + 1] - b;
            Result* r = run_event(*static_cast<const Geo*>(geo), n, x + b, y + b, z + b, idx + b, detid + b, mode, 4);
            for (int s = 0; s < 5; ++s) {
                counts[e * 5 + s] = (int64_t)r->t[s].size() / w[s];
                digests[e * 5 + s] = multiset_digest(r->t[s], w[s]);
            }
            std::memcpy(counters + e * 110, r->counters, 110 * sizeof(uint32_t));
            total += (int64_t)r->t[4].size() / 16;
            delete r;
        }
    };
    std::vector<std::thread> th;
    for (int i = 0; i < std::max(1, n_threads); ++i) th.emplace_back(work);
    for (auto& t : th) t.join();
    return total.load();
}

}  // extern "C"
