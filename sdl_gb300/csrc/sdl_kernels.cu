// Segment-linking kernels for sm_103a.
//
// Every stage follows the same pattern, batched over all events:
//   count  - per inner object, the number of candidate pairs the reference's
//            loop would test (Event.cc:257-301, 472-521, 635-691, ...);
//   scan   - exclusive prefix sum -> a flat candidate space [0, total);
//   enum   - a persistent, work-stealing grid: each warp takes 256
//            consecutive candidates, maps them back to (inner, outer) objects,
//            applies the reference's cuts and appends the survivors with a
//            warp-aggregated atomic, ranking each survivor inside its inner
//            module;
//   group  - per-module counts are scanned and the survivors scattered into
//            dense arrays grouped by inner module (objects of one event stay
//            contiguous).
// Triplets and track candidates are exact equi-joins on the shared
// mini-doublet / segment instead of the reference's all-pairs loops.
#include <cstdio>

#include "sdl_kernels.h"

namespace sdlg {

namespace {

// Bounds checks of every global-memory index (debug builds with
// -DSDL_DEVICE_CHECKS): a bad index is recorded in b.dbg (count, source line,
// index, limit) and the access is redirected to element 0 instead of faulting.
#ifdef SDL_DEVICE_CHECKS
__device__ __forceinline__ int64_t checked_idx(int64_t i, int64_t lim, int line, unsigned long long* dbg) {
    if (i >= 0 && i < lim) return i;
    if (atomicAdd(dbg, 1ull) == 0ull) {
        dbg[1] = (unsigned long long)line;
        dbg[2] = (unsigned long long)i;
        dbg[3] = (unsigned long long)lim;
    }
    return 0;
}
#define IX(i, lim) checked_idx((int64_t)(i), (int64_t)(lim), __LINE__, b.dbg)
#else
#define IX(i, lim) (i)
#endif
#define AT(arr, i, lim) (arr)[IX(i, lim)]

constexpr int kWarp = 32;
constexpr int kEnumThreads = 256;
constexpr int kTaskDefault = 256;  // candidates per warp task unless tuned
constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr int kScanBlock = kScanThreads * kScanItems;

__device__ __forceinline__ bool halted(const BatchDev& b) { return (*b.status & kStatusHalt) != 0; }

// add v to *addr with one atomic per group of lanes sharing the address;
// every lane of the warp must call it
__device__ __forceinline__ void warp_add(uint32_t* addr, uint32_t v, bool active) {
    const unsigned act = __ballot_sync(0xffffffffu, active);
    if (!active) return;
    const unsigned peers = __match_any_sync(act, (unsigned long long)(uintptr_t)addr);
    const uint32_t sum = __reduce_add_sync(peers, v);
    if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(addr, sum);
}

// largest i in [lo, hi] with off[i] <= c (off has `lim` entries)
__device__ __forceinline__ int find_obj(const BatchDev& b, const int64_t* off, int64_t lim, int lo, int hi, int64_t c) {
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (AT(off, mid, lim) <= c) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Bucket table of a stage's flat candidate space: bucket[k] is the inner
// object that holds candidate k * 2^kBucketShift, plus a last entry nobj - 1.
// A candidate c then lies in an inner object between bucket[c >> shift] and
// bucket[(c >> shift) + 1], so the enumerators search a few objects instead
// of all of them.  A table too small for the candidate space is not built
// and the search covers the whole range.
constexpr int kBucketShift = 8;

__device__ __forceinline__ bool buckets_ok(const BatchDev& b, int64_t total) {
    return ((total + (1ll << kBucketShift) - 1) >> kBucketShift) + 1 <= b.bucket_cap;
}

// search bounds of the inner objects of candidates c0 <= c1
__device__ __forceinline__ void obj_bounds(const BatchDev& b, int64_t nobj, int64_t total, int64_t c0, int64_t c1, int& lo,
                                           int& hi) {
    if (buckets_ok(b, total)) {
        lo = AT(b.bucket, c0 >> kBucketShift, b.bucket_cap);
        hi = AT(b.bucket, (c1 >> kBucketShift) + 1, b.bucket_cap);
    } else {
        lo = 0;
        hi = (int)nobj - 1;
    }
}

// ------------------------------------------------------------------ scan
struct ScanArgs {
    int64_t* data;      // cap + 1 entries
    const int64_t* n_ptr;
    int64_t cap;
    int64_t* blk;
    int64_t blk_cap;
    unsigned long long* dbg;
};

__global__ void k_scan_reduce(ScanArgs b) {
    const int64_t n = min(*b.n_ptr, b.cap);
    const int64_t base = (int64_t)blockIdx.x * kScanBlock;
    if (base >= n) return;
    int64_t s = 0;
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t i = base + (int64_t)k * kScanThreads + threadIdx.x;
        if (i < n) s += AT(b.data, i, b.cap + 1);
    }
    for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    __shared__ int64_t ws[32];  // one slot per lane of warp 0
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        int64_t v = threadIdx.x < kScanThreads / 32 ? ws[threadIdx.x] : 0;
        for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) AT(b.blk, blockIdx.x, b.blk_cap) = v;
    }
}

__global__ void k_scan_blocks(ScanArgs b) {
    const int64_t n = min(*b.n_ptr, b.cap);
    const int64_t nb = (n + kScanBlock - 1) / kScanBlock;
    __shared__ int64_t carry;
    __shared__ int64_t ws[32];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t base = 0; base < nb; base += blockDim.x) {
        const int64_t i = base + threadIdx.x;
        const int64_t v = i < nb ? AT(b.blk, i, b.blk_cap) : 0;
        int64_t x = v;
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) ws[w] = x;
        __syncthreads();
        if (w == 0) {
            int64_t t = lane < (int)(blockDim.x >> 5) ? ws[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                const int64_t y = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t += y;
            }
            ws[lane] = t;
        }
        __syncthreads();
        const int64_t incl = x + (w ? ws[w - 1] : 0);
        if (i < nb) AT(b.blk, i, b.blk_cap) = carry + incl - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) AT(b.data, n, b.cap + 1) = carry;
}

__global__ void k_scan_apply(ScanArgs b) {
    const int64_t n = min(*b.n_ptr, b.cap);
    const int64_t base = (int64_t)blockIdx.x * kScanBlock;
    if (base >= n) return;
    // each thread owns kScanItems consecutive elements
    int64_t v[kScanItems];
    int64_t s = 0;
    const int64_t my = base + (int64_t)threadIdx.x * kScanItems;
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = (my + k < n) ? AT(b.data, my + k, b.cap + 1) : 0;
        s += v[k];
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int64_t x = s;
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    __shared__ int64_t ws[32];  // one slot per lane of warp 0
    if (lane == 31) ws[w] = x;
    __syncthreads();
    if (w == 0) {
        int64_t t = lane < kScanThreads / 32 ? ws[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < kScanThreads / 32) ws[lane] = t;
    }
    __syncthreads();
    int64_t run = AT(b.blk, blockIdx.x, b.blk_cap) + x - s + (w ? ws[w - 1] : 0);
    for (int k = 0; k < kScanItems; ++k) {
        if (my + k < n) AT(b.data, my + k, b.cap + 1) = run;
        run += v[k];
    }
}

void scan(const BatchDev& bd, int64_t* data, const int64_t* n_ptr, int64_t cap, cudaStream_t s) {
    const int64_t nb = (cap + kScanBlock - 1) / kScanBlock;
    if (nb <= 0) return;
    ScanArgs a{data, n_ptr, cap, bd.scan_tmp, bd.scan_tmp_cap, bd.dbg};
    k_scan_reduce<<<(unsigned)nb, kScanThreads, 0, s>>>(a);
    k_scan_blocks<<<1, 1024, 0, s>>>(a);
    k_scan_apply<<<(unsigned)nb, kScanThreads, 0, s>>>(a);
}

// array sizes
__device__ __forceinline__ int64_t H(const BatchDev& b) { return b.n_hit_cap; }
__device__ __forceinline__ int64_t NG1(const BatchDev& b) { return (int64_t)b.n_gm + 1; }
// event and module of a global module index g = event * n_mod + module
// (0 <= g < 2^31): floor(g * ceil(2^64 / n) / 2^64) is floor(g / n) exactly
// for g and n = n_mod below 2^32 (the rounding-up error is below 2^-32 < 1 / n)
__device__ __forceinline__ int ev_of(const BatchDev& b, int64_t g) {
    return b.geo.n_mod == 1 ? (int)g : (int)__umul64hi((unsigned long long)g, b.geo.n_mod_inv);
}
__device__ __forceinline__ int mod_of(const BatchDev& b, int64_t g) {
    return (int)(g - (int64_t)ev_of(b, g) * b.geo.n_mod);
}
__device__ __forceinline__ int64_t NM(const BatchDev& b) { return b.geo.n_mod; }
__device__ __forceinline__ int64_t NC(const BatchDev& b) { return b.geo.n_conn > 0 ? b.geo.n_conn : 1; }
__device__ __forceinline__ int64_t NCP(const BatchDev& b) {
    const int64_t v = (int64_t)b.n_ev * b.geo.n_conn;
    return v > 0 ? v : 1;
}
__device__ __forceinline__ const ModDev& MOD(const BatchDev& b, int64_t m) { return AT(b.geo.mod, m, NM(b)); }

// ------------------------------------------------------------------ ingest
__global__ void k_hit_map(BatchDev b) {
    const int64_t n = *b.n_hit;
    for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < n; h += (int64_t)gridDim.x * blockDim.x) {
        int lo = 0, hi = b.n_ev;  // event: largest e with ev_off[e] <= h
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (AT(b.ev_off, mid, b.n_ev + 1) <= h) lo = mid;
            else hi = mid;
        }
        const int ev = lo;
        const uint32_t d = AT(b.in_det, h, H(b));
        int a = 0, c = b.geo.n_mod;  // first module with detid >= d
        while (a < c) {
            const int mid = (a + c) >> 1;
            if (AT(b.geo.detid, mid, NM(b)) < d) a = mid + 1;
            else c = mid;
        }
        int gm = -1, rank = 0;
        if (a < b.geo.n_mod && AT(b.geo.detid, a, NM(b)) == d) {
            gm = ev * b.geo.n_mod + a;
            rank = (int)atomicAdd((unsigned long long*)&AT(b.mod_hit, gm, NG1(b)), 1ull);
        } else {
            atomicOr(b.status, kStatusUnknownModule);
        }
        AT(b.hit_gm, h, H(b)) = gm;
        AT(b.hit_rank, h, H(b)) = rank;
    }
}

// sorted position of every input hit in a known module -> hit_perm
__global__ void k_hit_perm(BatchDev b) {
    const int64_t n = *b.n_hit;
    for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < n; h += (int64_t)gridDim.x * blockDim.x) {
        const int gm = AT(b.hit_gm, h, H(b));
        if (gm < 0) continue;
        AT(b.hit_perm, AT(b.mod_hit, gm, NG1(b)) + AT(b.hit_rank, h, H(b)), H(b)) = (int)h;
    }
}

// the sorted hit arrays, one thread per sorted position (coalesced writes;
// the input hit is gathered through hit_perm)
__global__ void k_hit_scatter(BatchDev b) {
    const int64_t n = min(AT(b.mod_hit, b.n_gm, NG1(b)), *b.n_hit);  // hits in known modules
    for (int64_t pos = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; pos < n; pos += (int64_t)gridDim.x * blockDim.x) {
        const int64_t h = AT(b.hit_perm, pos, H(b));
        const int gm = AT(b.hit_gm, h, H(b));
        const float x = AT(b.in_x, h, H(b)), y = AT(b.in_y, h, H(b)), z = AT(b.in_z, h, H(b));
        const P3 p = mk(x, y, z);
        AT(b.hx, pos, H(b)) = x; AT(b.hy, pos, H(b)) = y; AT(b.hz, pos, H(b)) = z;
        AT(b.hrt, pos, H(b)) = p.rt; AT(b.hphi, pos, H(b)) = p.phi; AT(b.hr3, pos, H(b)) = p.r3;
        const float a1 = g_asin(fmin_ref(p.rt * k2Rinv1GeVf / kPtCut, kSinAlphaMax));
        AT(b.ha1, pos, H(b)) = a1;
        AT(b.htf, pos, H(b)) = g_tan(a1);
        AT(b.htd, pos, H(b)) = f_tan_over(a1);
        AT(b.ha3, pos, H(b)) = g_asin(fmin_ref(p.rt * k2Rinv1GeVf / 3.0f, kSinAlphaMax));
        AT(b.hidx, pos, H(b)) = AT(b.in_idx, h, H(b));
        AT(b.hgm, pos, H(b)) = gm;
        // the strip shift of the mini-doublets this hit anchors
        const int m = mod_of(b, gm);
        const ModDev& M = MOD(b, m);
        const int lmi = M.lower ? m : M.partner;
        float xa = 0.f, ya = 0.f, zn = 0.f;
        if (lmi >= 0) {
            const ModDev& lm = MOD(b, lmi);
            if (md_shifts(lm) && (md_upper_anchors(lm) != (bool)M.lower)) shift_anchor(p, lm, xa, ya, zn);
        }
        AT(b.hsx, pos, H(b)) = xa; AT(b.hsy, pos, H(b)) = ya; AT(b.hsz, pos, H(b)) = zn;
    }
}

// ------------------------------------------------------------------ helpers
__device__ __forceinline__ P3 hit(const BatchDev& b, int64_t k) {
    P3 p;
    p.x = AT(b.hx, k, H(b)); p.y = AT(b.hy, k, H(b)); p.z = AT(b.hz, k, H(b));
    p.rt = AT(b.hrt, k, H(b)); p.phi = AT(b.hphi, k, H(b)); p.r3 = AT(b.hr3, k, H(b));
    return p;
}

__device__ __forceinline__ int md_anchor(const ModDev& lm, int lo, int up) {
    return (lm.type == kPS && lm.ltype != kPixel) ? up : lo;  // MiniDoublet.cc:60-81
}

// object arrays of stage st
__device__ __forceinline__ int OI(const BatchDev& b, int st, int64_t k) { return AT(b.obj[st].i, k, b.obj[st].cap); }
__device__ __forceinline__ int OJ(const BatchDev& b, int st, int64_t k) { return AT(b.obj[st].j, k, b.obj[st].cap); }
__device__ __forceinline__ int OG(const BatchDev& b, int st, int64_t k) { return AT(b.obj[st].g, k, b.obj[st].cap); }
__device__ __forceinline__ float OF(const BatchDev& b, int st, int f, int64_t k) {
    const Objs& O = b.obj[st];
    return AT(O.f, (int64_t)f * O.cap + k, O.cap * (O.nf > 0 ? O.nf : 1));
}
__device__ __forceinline__ int64_t OFF(const BatchDev& b, int st, int64_t g) { return AT(b.obj[st].mod_cnt, g, NG1(b)); }


// ------------------------------------------------------------------ stage functors
struct MDStage {
    static constexpr int kSt = kMD;
    __device__ static bool eval(const BatchDev& b, int gm, int64_t q, int& oi, int& oj, float* fv) {
        const int n_mod = b.geo.n_mod;
        const int ev = ev_of(b, gm);
        const ModDev lm = MOD(b, gm - ev * n_mod);
        const int pg = ev * n_mod + lm.partner;
        const int64_t nu = AT(b.mod_hit, pg + 1, NG1(b)) - AT(b.mod_hit, pg, NG1(b));
        if (nu <= 0) {
#ifdef SDL_DEVICE_CHECKS
            IX(-1, 0);
#endif
            return false;
        }
        const int64_t i = q / nu, j = q - i * nu;
        const int64_t lo = AT(b.mod_hit, gm, NG1(b)) + i, up = AT(b.mod_hit, pg, NG1(b)) + j;
        const P3 L = hit(b, lo), U = hit(b, up);
        const float pixAsin = lm.ltype == kPixel ? AT(b.ha1, lo, H(b)) : AT(b.ha1, up, H(b));
        const int64_t anc = md_upper_anchors(lm) ? up : lo;
        const float sh[3] = {AT(b.hsx, anc, H(b)), AT(b.hsy, anc, H(b)), AT(b.hsz, anc, H(b))};
        MDVals v;
        v.dz = 0.f; v.shiftedDz = 0.f; v.dphi = 0.f; v.dphichange = 0.f;
        const bool pass = lm.subdet == kBarrel ? md_barrel(L, U, pixAsin, lm, sh, v) : md_endcap(L, U, pixAsin, lm, sh, v);
        oi = (int)lo; oj = (int)up;
        fv[0] = v.dz; fv[1] = v.shiftedDz; fv[2] = v.dphi; fv[3] = v.dphichange;
        return pass;
    }
    __device__ static int group_of(const BatchDev& b, int gm) { return gm; }
};

// conn entry k of module m for the flat index q, given per-entry exclusive prefixes
__device__ __forceinline__ int conn_entry(const BatchDev& b, int ev, int m, int64_t q, int& pref) {
    const int k0 = AT(b.geo.conn_off, m, NM(b) + 1), k1 = AT(b.geo.conn_off, m + 1, NM(b) + 1);
    const int64_t base = (int64_t)ev * b.geo.n_conn;
    int lo = k0, hi = k1 - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (AT(b.conn_pref, base + mid, NCP(b)) <= q) lo = mid;
        else hi = mid - 1;
    }
    pref = AT(b.conn_pref, base + lo, NCP(b));
    return lo;
}

// One 64-byte record per mini-doublet for the segment stage (k_md_pack):
// the anchor hit with its derived quantities and asin / tan terms, the
// mini-doublet's four floats, the lower module and the anchor's module.
struct MDRec {
    MDView v;
    float a1, tf;  // asin(min(rt*k,.95)) and its float tan, of the anchor hit
    int anc_mod;   // module of the anchor hit
    float c0, c1;  // barrel: sdCut for the layer below (c0); endcap: strip-edge phis (hi, lo)
};
__device__ __forceinline__ MDRec md_rec(const BatchDev& b, int64_t a) {
    const float4* q = reinterpret_cast<const float4*>(&AT(b.mdpack, a * kMdPack, b.obj[kMD].cap * kMdPack));
    const float4 r0 = __ldg(q), r1 = __ldg(q + 1), r2 = __ldg(q + 2), r3 = __ldg(q + 3);
    MDRec r;
    r.v.a.x = r0.x; r.v.a.y = r0.y; r.v.a.z = r0.z; r.v.a.rt = r0.w;
    r.v.a.phi = r1.x; r.v.a.r3 = r1.y; r.a1 = r1.z; r.tf = r1.w;
    r.v.dz = r2.x; r.v.shiftedDz = r2.y; r.v.dphi = r2.z; r.v.dphichange = r2.w;
    r.v.m = &MOD(b, __float_as_int(r3.x));
    r.anc_mod = __float_as_int(r3.y);
    r.c0 = r3.z;
    r.c1 = r3.w;
    return r;
}

__global__ void k_md_pack(BatchDev b) {
    if (halted(b)) return;
    const int64_t n = min(OFF(b, kMD, b.n_gm), b.obj[kMD].cap);  // mini-doublets
    for (int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; a < n; a += (int64_t)gridDim.x * blockDim.x) {
        const int lm = mod_of(b, OG(b, kMD, a));
        const int anc = md_anchor(MOD(b, lm), OI(b, kMD, a), OJ(b, kMD, a));
        const P3 p = hit(b, anc);
        float4* q = reinterpret_cast<float4*>(&AT(b.mdpack, a * kMdPack, b.obj[kMD].cap * kMdPack));
        q[0] = make_float4(p.x, p.y, p.z, p.rt);
        q[1] = make_float4(p.phi, p.r3, AT(b.ha1, anc, H(b)), AT(b.htf, anc, H(b)));
        q[2] = make_float4(OF(b, kMD, 0, a), OF(b, kMD, 1, a), OF(b, kMD, 2, a), OF(b, kMD, 3, a));
        // what the segment algorithms compute from this mini-doublet alone as
        // the outer one: the barrel cut for the layer below, the endcap strip
        // edges' phi
        const ModDev& M = MOD(b, lm);
        const int am = mod_of(b, AT(b.hgm, anc, H(b)));
        float c0 = 0.f, c1 = 0.f;
        if (M.subdet == kBarrel) {
            if (M.layer >= 2) c0 = sg_barrel_cut(M.layer - 1, p.rt, AT(b.ha1, anc, H(b)));
        } else if (M.type == kTwoS) {
            c0 = strip_edge(p, MOD(b, am), true).phi;
            c1 = strip_edge(p, MOD(b, am), false).phi;
        } else {
            c0 = c1 = p.phi;
        }
        q[3] = make_float4(__int_as_float(lm), __int_as_float(am), c0, c1);
    }
}

// segment algorithm on inner MD a and outer MD bmd (Segment.cc:337-859);
// `connected`: the outer MD's module is in the inner module's connection list
// (the endcap algorithm's first requirement, Segment.cc:613-633)
// kOuter: 0 either algorithm, 1 only the barrel one (outer MD in the barrel),
// 2 only the endcap one (a kernel compiled for one keeps the other's code out
// of its instruction caches); a candidate of the other kind fails
template <bool kPre = false, int kOuter = 0>
__device__ __forceinline__ bool sg_pair_rec(const MDView& im, const MDRec& orec, bool connected, float* fv) {
    const MDView& om = orec.v;
    SGVals v;
    v.dphi = v.dphimin = v.dphimax = v.dphichange = v.dphiminchange = v.dphimaxchange = 0.f;
    bool pass = false;
    const bool ob = om.m->subdet == kBarrel;
    if (kOuter != 2 && ob) pass = sg_barrel<kPre>(im, om, orec.a1, orec.tf, orec.c0, v);
    else if (kOuter != 1 && !ob) pass = sg_endcap<kPre>(im, om, orec.a1, orec.tf, connected, orec.c0, orec.c1, v);
    fv[0] = v.dphi; fv[1] = v.dphimin; fv[2] = v.dphimax;
    fv[3] = v.dphichange; fv[4] = v.dphiminchange; fv[5] = v.dphimaxchange;
    return pass;
}
__device__ __forceinline__ bool sg_pair(const BatchDev& b, int a, int bmd, bool connected, float* fv) {
    return sg_pair_rec(md_rec(b, a).v, md_rec(b, bmd), connected, fv);
}

// segment candidates along the module map (Event.cc:445-522): candidate q of
// inner MD a is an MD of a connected module, in connection-list order; the
// outer mini-doublet of candidate q of inner MD a
__device__ __forceinline__ int sg_outer_md(const BatchDev& b, int a, int64_t q) {
    const int n_mod = b.geo.n_mod;
    const int g1 = OG(b, kMD, a);
    if (AT(b.toff, b.n_gm, NG1(b)) <= b.olist_cap) return AT(b.olist, AT(b.toff, g1, NG1(b)) + q, b.olist_cap);  // k_sg_olist_fill
    const int ev = ev_of(b, g1), m1 = g1 - ev * n_mod;
    int pref;
    const int k = conn_entry(b, ev, m1, q, pref);
    const int g2 = ev * n_mod + AT(b.geo.conn_idx, k, NC(b));
    return (int)(OFF(b, kMD, g2) + (q - pref));
}

// ------------------------------------------------------------------ layer pairs
// Layer.cc:32-50: the outer layer slots paired with inner slot si (barrel
// layers 1-5 -> the next barrel layer and endcap layer 1; endcap 1 -> 2;
// endcap 2 -> 3, 4, 5; endcap 3 -> 4; endcap 4 -> 5); -1 past the last
__device__ __forceinline__ int sg_layer_outer(int si, int k) {
    if (si <= 4) return k == 0 ? si + 1 : (k == 1 ? 6 : -1);
    if (si == 6) return k == 0 ? 7 : -1;
    if (si == 7) return k < 3 ? 8 + k : -1;
    if (si == 8 || si == 9) return k == 0 ? si + 1 : -1;
    return -1;
}

// Layer.cc:19-24: tracklet layer pairs are barrel (1,3), (2,4), (3,5)
__device__ __forceinline__ int tl_layer_outer(int si) { return si <= 2 ? si + 2 : -1; }

__device__ __forceinline__ int SR(const BatchDev& b, int k) { return AT(b.geo.slot_run, k, b.geo.n_slot_run); }

// objects of stage st in layer slot sl of event ev
__device__ __forceinline__ int64_t layer_count(const BatchDev& b, int st, int ev, int sl) {
    const int64_t base = (int64_t)ev * b.geo.n_mod;
    int64_t n = 0;
    for (int r = SR(b, sl); r < SR(b, sl + 1); ++r)
        n += OFF(b, st, base + SR(b, kNumSlots + 2 + 2 * r)) - OFF(b, st, base + SR(b, kNumSlots + 1 + 2 * r));
    return n;
}

// the q-th object of stage st in layer slot sl of event ev (q < layer_count)
__device__ __forceinline__ int layer_object(const BatchDev& b, int st, int ev, int sl, int64_t q) {
    const int64_t base = (int64_t)ev * b.geo.n_mod;
    for (int r = SR(b, sl); r < SR(b, sl + 1); ++r) {
        const int64_t o0 = OFF(b, st, base + SR(b, kNumSlots + 1 + 2 * r));
        const int64_t n = OFF(b, st, base + SR(b, kNumSlots + 2 + 2 * r)) - o0;
        if (q < n) return (int)(o0 + q);
        q -= n;
    }
#ifdef SDL_DEVICE_CHECKS
    (void)IX(-3, 0);
#endif
    return 0;
}

// segment candidates by layer pairs (Event.cc:432-443, 793-821): candidate q
// of inner MD a runs over the MDs of the paired outer layers, in table order
struct SGLayerStage {
    static constexpr int kSt = kSG;
    __device__ static bool eval(const BatchDev& b, int a, int64_t q, int& oi, int& oj, float* fv) {
        const int n_mod = b.geo.n_mod;
        const int g1 = OG(b, kMD, a);
        const int ev = ev_of(b, g1), m1 = g1 - ev * n_mod;
        const int si = MOD(b, m1).layer_slot;
        int bmd = -1;
        for (int k = 0; k < 3; ++k) {
            const int so = sg_layer_outer(si, k);
            if (so < 0) break;
            const int64_t n = layer_count(b, kMD, ev, so);
            if (q < n) {
                bmd = layer_object(b, kMD, ev, so, q);
                break;
            }
            q -= n;
        }
        oi = a; oj = bmd;
        if (bmd < 0) {
#ifdef SDL_DEVICE_CHECKS
            (void)IX(-4, 0);
#endif
            return false;
        }
        const int m2 = OG(b, kMD, bmd) - ev * n_mod;
        bool connected = false;
        if (MOD(b, m2).subdet == kEndcap) {
            const int k0 = AT(b.geo.conn_off, m1, NM(b) + 1), k1 = AT(b.geo.conn_off, m1 + 1, NM(b) + 1);
            for (int k = k0; k < k1 && !connected; ++k) connected = AT(b.geo.conn_idx, k, NC(b)) == m2;
        }
        return sg_pair(b, a, bmd, connected, fv);
    }
    __device__ static int group_of(const BatchDev& b, int a) { return OG(b, kMD, a); }
};

// tracklet candidate q of inner segment s -> outer segment (Event.cc:635-663)
__device__ __forceinline__ int tl_outer(const BatchDev& b, int s, int64_t q) {
    const int n_mod = b.geo.n_mod;
    // module of the outer mini-doublet, from the packed segment record
    const int g2 = __float_as_int(AT(b.sgpack, (int64_t)s * PK_N + PK_G2, b.obj[kSG].cap * PK_N));
    const int ev = ev_of(b, g2), m2 = g2 - ev * n_mod;
    int pref;
    const int k = conn_entry(b, ev, m2, q, pref);
    const int g3 = ev * n_mod + AT(b.geo.conn_idx, k, NC(b));
    return (int)(OFF(b, kSG, g3) + (q - pref));
}

// tracklet candidate q of inner segment s by layer pairs (Event.cc:755-790):
// the q-th segment of the paired outer barrel layer
__device__ __forceinline__ int tl_outer_layer(const BatchDev& b, int s, int64_t q) {
    const int n_mod = b.geo.n_mod;
    const int g1 = OG(b, kSG, s);
    const int ev = ev_of(b, g1);
    return layer_object(b, kSG, ev, tl_layer_outer(MOD(b, g1 - ev * n_mod).layer_slot), q);
}

// The triplets and track candidates are equi-joins on a mini-doublet: the
// join index lists the objects of stage st (segments, or tracklets) by their
// key mini-doublet (a segment's inner one; a tracklet's inner segment's inner
// one), so that each join visits only matching objects (joff: offsets per
// mini-doublet, jidx: the objects).
__device__ __forceinline__ int join_key(const BatchDev& b, int st, int64_t o) {
    return st == kSG ? OI(b, kSG, o) : OI(b, kSG, OI(b, st, o));  // tracklets, triplets: inner segment's inner MD
}
// the second index (the triplets by their innermost MD)
__device__ __forceinline__ int64_t join2_n(const BatchDev& b, int md) {
    return AT(b.joff2, md + 1, b.obj[kMD].cap + 1) - AT(b.joff2, md, b.obj[kMD].cap + 1);
}
__device__ __forceinline__ int join2_obj(const BatchDev& b, int md, int64_t k) {
    return AT(b.jidx2, AT(b.joff2, md, b.obj[kMD].cap + 1) + k, b.obj[kTP].cap);
}
__device__ __forceinline__ int64_t join_n(const BatchDev& b, int md) {
    return AT(b.joff, md + 1, b.obj[kMD].cap + 1) - AT(b.joff, md, b.obj[kMD].cap + 1);
}
__device__ __forceinline__ int join_obj(const BatchDev& b, int md, int64_t k) {
    return AT(b.jidx, AT(b.joff, md, b.obj[kMD].cap + 1) + k, max(b.obj[kSG].cap, b.obj[kTL].cap));
}

// triplet candidates (Event.cc:524-597 via Triplet.cc:55): candidate q of
// inner segment s1 is the (q mod n)-th segment starting at its outer
// mini-doublet; the multiplicity of the outer module in the connection list
// repeats each, as the reference's nested loops do (k_tp_count)
struct TPStage {
    static constexpr int kSt = kTP;
    __device__ static bool eval(const BatchDev& b, int s1, int64_t q, int& oi, int& oj, float* fv) {
        const int omd = OJ(b, kSG, s1);
        const int64_t n2 = join_n(b, omd);
        if (n2 <= 0) {
#ifdef SDL_DEVICE_CHECKS
            IX(-2, 0);
#endif
            return false;
        }
        oi = s1;
        oj = join_obj(b, omd, q % n2);
        (void)fv;
        return true;
    }
    __device__ static int group_of(const BatchDev& b, int s) { return OG(b, kSG, s); }
};

// track candidates (Event.cc:823-872, and 984-1062 for
// createTrackCandidatesFromTracklets, via TrackCandidate.cc:161): candidate q
// of inner tracklet t1 is the (q mod n)-th of the n tracklets whose inner
// segment starts at the inner mini-doublet of t1's outer segment (repeated
// connections repeat them, k_tc_count_tl); it matches when that segment's
// outer mini-doublet is the same too
struct TCStage {
    static constexpr int kSt = kTC;
    __device__ static bool eval(const BatchDev& b, int t1, int64_t q, int& oi, int& oj, float* fv) {
        const int sB = OJ(b, kTL, t1);
        const int mB = OI(b, kSG, sB);
        const int t2 = join_obj(b, mB, q % join_n(b, mB));  // n > 0 when t1 has candidates
        const int sC = OI(b, kTL, t2);
        oi = t1; oj = t2;
        (void)fv;
        return OI(b, kSG, sC) == OI(b, kSG, sB) && OJ(b, kSG, sC) == OJ(b, kSG, sB);  // TrackCandidate.cc:161
    }
    __device__ static int group_of(const BatchDev& b, int t) { return OG(b, kTL, t); }
};

// inner-object count of a stage (device), clamped to the inner capacity
__device__ __forceinline__ int64_t n_inner(const BatchDev& b, int st) {
    switch (st) {
        case kMD: return b.n_gm;
        case kSG: return min(OFF(b, kMD, b.n_gm), b.obj[kMD].cap);
        case kTL:
        case kTP: return min(OFF(b, kSG, b.n_gm), b.obj[kSG].cap);
        default:  // track candidates: tracklets, or triplets (createTrackCandidatesFromTriplets)
            return (b.flags & kFlagTCFromTP) ? min(OFF(b, kTP, b.n_gm), b.obj[kTP].cap)
                                             : min(OFF(b, kTL, b.n_gm), b.obj[kTL].cap);
    }
}

// bucket table of stage st's scanned candidate offsets
__global__ void k_cand_buckets(BatchDev b, int st) {
    if (halted(b)) return;
    const int64_t nobj = n_inner(b, st);
    if (nobj <= 0) return;
    const int64_t* off = b.cand[st];
    const int64_t offlim = b.cand_cap[st] + 1;
    const int64_t total = AT(off, nobj, offlim);
    if (!buckets_ok(b, total)) return;
    const int64_t nb = (total + (1ll << kBucketShift) - 1) >> kBucketShift;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid == 0) AT(b.bucket, nb, b.bucket_cap) = (int)(nobj - 1);
    for (int64_t s = tid; s < nobj; s += (int64_t)gridDim.x * blockDim.x) {
        const int64_t lo = AT(off, s, offlim), hi = AT(off, s + 1, offlim);
        for (int64_t k = (lo + (1ll << kBucketShift) - 1) >> kBucketShift; (k << kBucketShift) < hi; ++k)
            AT(b.bucket, k, b.bucket_cap) = (int)s;
    }
}

// A warp's accepted objects, collected in shared memory and appended to the
// stage's record list in batches of up to kRecBuf: one atomic on the list's
// count per batch instead of one per 32 candidates (atomics on one address
// serialise at its L2 slice), and coalesced record writes.  The ranks within
// the objects' modules are taken at the flush (atomics on distinct module
// counters, issued together).  Every lane of the warp calls rec_flush.
constexpr int kRecBuf = 64;
template <int kNF>
struct RecBuf {
    int (*e)[kRecBuf];  // this warp's [3 + kNF][kRecBuf] words: inner, outer, module, float values
    int n = 0;          // records held (warp-uniform)
};
template <int kNF>
__device__ __forceinline__ void rec_flush(const BatchDev& b, int st, RecBuf<kNF>& rb) {
    __syncwarp();
    const int lane = threadIdx.x & 31;
    const Recs& R = b.rec[st];
    const Objs& O = b.obj[st];
    unsigned long long p0 = 0;
    if (lane == 0 && rb.n) p0 = atomicAdd((unsigned long long*)(b.n_rec + st), (unsigned long long)rb.n);
    p0 = __shfl_sync(0xffffffffu, p0, 0);
    for (int k = lane; k < rb.n; k += kWarp) {
        const int64_t pos = (int64_t)p0 + k;
        if (pos < O.cap) {
            const int g = rb.e[2][k];
            AT(R.i, pos, O.cap) = rb.e[0][k];
            AT(R.j, pos, O.cap) = rb.e[1][k];
            AT(R.g, pos, O.cap) = g;
            AT(R.rank, pos, O.cap) = (int)atomicAdd((unsigned long long*)&AT(O.mod_cnt, g, NG1(b)), 1ull);
#pragma unroll
            for (int q = 0; q < kNF; ++q) AT(R.f, (int64_t)q * O.cap + pos, O.cap * kNF) = __int_as_float(rb.e[3 + q][k]);
        } else {
            atomicOr(b.status, 1u << st);
        }
    }
    __syncwarp();
    rb.n = 0;
}

template <class F>
__global__ void __launch_bounds__(kEnumThreads) k_enum(BatchDev b) {
    constexpr int st = F::kSt;
    constexpr int kNF = st == kMD ? 4 : (st == kSG ? 6 : 0);  // the stage's float values per object
    __shared__ int rbuf[kEnumThreads / kWarp][3 + kNF][kRecBuf];
    if (halted(b)) return;
    const int64_t nobj = n_inner(b, st);
    if (nobj <= 0) return;
    const int64_t* off = b.cand[st];
    const int64_t offlim = b.cand_cap[st] + 1;
    const int64_t total = AT(off, nobj, offlim);
    const int task = b.enum_task[st] > 0 ? b.enum_task[st] : kTaskDefault;
    const int64_t ntask = (total + task - 1) / task;
    const int lane = threadIdx.x & 31;
    RecBuf<kNF> rb{rbuf[threadIdx.x >> 5]};
    for (;;) {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(b.task + st, 1ull);
        t = __shfl_sync(0xffffffffu, t, 0);
        if ((int64_t)t >= ntask) break;
        const int64_t base = (int64_t)t * task;
        const int64_t end = min(base + task, total);
        int ilo = 0;
        if (lane < 2) {
            int lo, hi;
            obj_bounds(b, nobj, total, base, end - 1, lo, hi);
            ilo = find_obj(b, off, offlim, lo, hi, lane == 0 ? base : end - 1);
        }
        const int i0 = __shfl_sync(0xffffffffu, ilo, 0);
        const int i1 = __shfl_sync(0xffffffffu, ilo, 1);
        for (int64_t cb = base; cb < end; cb += kWarp) {
            const int64_t c = cb + lane;
            const bool valid = c < end;
            int oi = 0, oj = 0, g = 0;
            float fv[6];
            bool pass = false;
            if (valid) {
                const int i = (i0 == i1) ? i0 : find_obj(b, off, offlim, i0, i1, c);
                pass = F::eval(b, i, c - AT(off, i, offlim), oi, oj, fv);
                if (pass) g = F::group_of(b, i);
            }
            const unsigned m = __ballot_sync(0xffffffffu, pass);
            if (m) {
                const int c = __popc(m);
                if (rb.n + c > kRecBuf) rec_flush<kNF>(b, st, rb);
                if (pass) {
                    const int k = rb.n + __popc(m & ((1u << lane) - 1u));
                    rb.e[0][k] = oi;
                    rb.e[1][k] = oj;
                    rb.e[2][k] = g;
#pragma unroll
                    for (int q = 0; q < kNF; ++q) rb.e[3 + q][k] = __float_as_int(fv[q]);
                }
                rb.n += c;
            }
        }
    }
    rec_flush<kNF>(b, st, rb);
}


// One packed record per segment for the tracklet stage (the anchors of both
// mini-doublets, the segment's angles and the per-segment sub-expressions of
// Tracklet.cc that depend on one segment only).
// the packed record of the segment from mini-doublet im to mini-doublet om
// with the segment algorithm's six values f6 (dPhi, dPhiMin, dPhiMax,
// dPhiChange, dPhiMinChange, dPhiMaxChange)
__device__ __forceinline__ void sg_pack_record(const BatchDev& b, int im, int om, const float* f6, float* v) {
    const ModDev& ilm = MOD(b, mod_of(b, OG(b, kMD, im)));
    const ModDev& olm = MOD(b, mod_of(b, OG(b, kMD, om)));
    const int la = md_anchor(ilm, OI(b, kMD, im), OJ(b, kMD, im));
    const int ua = md_anchor(olm, OI(b, kMD, om), OJ(b, kMD, om));
    const P3 lo = hit(b, la), up = hit(b, ua);
    const ModDev& lam = MOD(b, mod_of(b, AT(b.hgm, la, H(b))));
    const ModDev& uam = MOD(b, mod_of(b, AT(b.hgm, ua, H(b))));
    uint32_t fl = 0;
    fl |= lam.subdet == kBarrel ? F_LO_B : 0u;
    fl |= lam.subdet == kEndcap ? F_LO_E : 0u;
    fl |= lam.type == kPS ? F_LO_PS : 0u;
    fl |= uam.subdet == kBarrel ? F_UP_B : 0u;
    fl |= uam.subdet == kEndcap ? F_UP_E : 0u;
    fl |= uam.type == kPS ? F_UP_PS : 0u;
    fl |= uam.type == kTwoS ? F_UP_2S : 0u;
    v[PK_LX] = lo.x; v[PK_LY] = lo.y; v[PK_LZ] = lo.z; v[PK_LRT] = lo.rt;
    v[PK_LPHI] = lo.phi; v[PK_LR3] = lo.r3; v[PK_LA1] = AT(b.ha1, la, H(b)); v[PK_LTD] = AT(b.htd, la, H(b));
    v[PK_LA3] = AT(b.ha3, la, H(b));
    v[PK_LR3Z] = __fsqrt_rn(lo.z * lo.z + lo.rt * lo.rt);
    v[PK_UX] = up.x; v[PK_UY] = up.y; v[PK_UZ] = up.z; v[PK_URT] = up.rt; v[PK_UPHI] = up.phi; v[PK_UR3] = up.r3;
    v[PK_DPC] = f6[3]; v[PK_DPMIN] = f6[1]; v[PK_DPMAX] = f6[2];
    v[PK_DPMINC] = f6[4]; v[PK_DPMAXC] = f6[5];
    v[PK_RTSEG] = rt_of_diff(up, lo);
    v[PK_ALPHAUP] = dphi(up, sub(up, lo));
    v[PK_DPHILU] = dphi(lo, up);
    v[PK_EX] = uam.edge_x; v[PK_EY] = uam.edge_y;
    v[PK_FLAGS] = __uint_as_float(fl);
    v[PK_G2] = __int_as_float(OG(b, kMD, om));
    // the inner role's per-segment terms of phase A (the same float
    // operations as there)
    v[PK_S0] = (up.z - lo.z) / (up.rt - lo.rt);
    v[PK_S1] = (up.r3 - lo.r3) / (up.rt - lo.rt);
    const float q = v[PK_LR3Z] / lo.rt;
    if (q > 0x1p-60f && q < 0x1p60f) {
        const ffm::ff sq = ffm::sqrt_ff(ffm::ff{q, 0.f});
        v[PK_S2] = sq.hi;
        v[PK_S3] = sq.lo;
    } else {
        v[PK_S2] = v[PK_S3] = __int_as_float(0x7fc00000);  // NaN: muls takes its double path
    }
}

__global__ void k_sg_pack(BatchDev b) {
    if (halted(b)) return;
    const int64_t n = n_inner(b, kTL);
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
        float f6[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) f6[k] = OF(b, kSG, k, s);
        float v[PK_N];
        sg_pack_record(b, OI(b, kSG, s), OJ(b, kSG, s), f6, v);
        const uint32_t fl = __float_as_uint(v[PK_FLAGS]);
        const int64_t C = b.obj[kSG].cap;
        const int fo[10] = {PK_LRT, PK_LZ, PK_LTD, PK_LA1, PK_UPHI, PK_FLAGS, -1, PK_LX, PK_LY, PK_UX};
#pragma unroll
        for (int k = 0; k < 10; ++k)
            if (k != 6) AT(b.sgouter, k * C + s, 11 * C) = v[fo[k]];
        AT(b.sgouter, 6 * C + s, 11 * C) = 0.1f / v[PK_LRT];  // the PV-offset term of an outer segment
        AT(b.sgouter, 10 * C + s, 11 * C) = v[PK_UY];
        float4* dst = reinterpret_cast<float4*>(&AT(b.sgpack, s * PK_N, b.obj[kSG].cap * PK_N));
        for (int k = 0; k < PK_N / 4; ++k) dst[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
        // the pre-filter's feature records (inner role, outer role)
        const float lz = v[PK_LZ], lrt = v[PK_LRT], uz = v[PK_UZ], urt = v[PK_URT];
        const float drIn = urt - lrt;
        const float slope = (uz - lz) / (fabsf(drIn) > 1e-3f ? drIn : copysignf(1e-3f, drIn));
        const float scode = ((fl & F_LO_E) ? 1.f : 0.f) + ((fl & F_LO_PS) ? 0.25f : 0.f);
        const float tcode = ((fl & F_UP_E) ? 0.5f : 0.f) + ((fl & F_UP_2S) ? 0.125f : 0.f);
        float4* fd = reinterpret_cast<float4*>(&AT(b.sgfeat, s * kFeatN, b.obj[kSG].cap * kFeatN));
        fd[0] = make_float4(v[PK_LX], v[PK_LY], lz, lrt);
        fd[1] = make_float4(v[PK_LPHI], v[PK_DPC], slope, scode);
        fd[2] = make_float4(v[PK_UX], v[PK_UY], uz, urt);
        fd[3] = make_float4(v[PK_UPHI], v[PK_ALPHAUP], tcode, 0.f);
    }
}

// createTrackCandidatesFromTriplets (Event.cc:874-982): candidate q of inner
// triplet p1 is a triplet p2 of a module connected to the module of p1's
// outermost MD (connection-list order, as the segment candidates); it passes
// when the trial segment from that MD to p2's innermost MD passes the segment
// algorithm and the tracklet (trial segment, p2's outer segment) passes the
// default tracklet algorithm.  The trial segment is not kept.
struct TCTPStage {
    static constexpr int kSt = kTC;
    __device__ static bool eval(const BatchDev& b, int p1, int64_t q, int& oi, int& oj, float* fv) {
        const int n_mod = b.geo.n_mod;
        const int mdA = OJ(b, kSG, OJ(b, kTP, p1));
        const int gA = OG(b, kMD, mdA);
        const int ev = ev_of(b, gA), mA = gA - ev * n_mod;
        int pref;
        const int k = conn_entry(b, ev, mA, q, pref);
        const int g3 = ev * n_mod + AT(b.geo.conn_idx, k, NC(b));
        const int p2 = (int)(OFF(b, kTP, g3) + (q - pref));
        oi = p1;
        oj = p2;
        (void)fv;
        const int mdB = OI(b, kSG, OI(b, kTP, p2));
        float f6[6];
        if (!sg_pair(b, mdA, mdB, true, f6)) return false;
        float v[PK_N];
        sg_pack_record(b, mdA, mdB, f6, v);
        const SGV S = sgv_from(v);
        const int so = OJ(b, kTP, p2);
        const SGV T = load_sgv(b.sgpack, so);
        float cut, muls;
        const int algo = tl_phaseA(S, T, cut, muls);
        if (algo == kAlgoNone || !tl_phaseB1_sgv(algo, S, T, cut)) return false;
        return tl_phaseB2_sgv<kB2All>(algo, S, T, muls, false);
    }
    __device__ static int group_of(const BatchDev& b, int p) { return OG(b, kTP, p); }
};

// createTrackCandidatesFromTriplets after module-map segments: the trial
// segment (mdA, mdB) passes the segment algorithm exactly when the segment
// stage made it, and it made it once per occurrence of mdB's module in the
// connection list of mdA's module, which is also how often the reference's
// loop (over that list) reaches each outer triplet starting at mdB.  So the
// candidates are: the segments leaving p1's outermost MD mdA (the join index)
// x the triplets starting at each one's outer MD (the second index); the
// tracklet algorithm then runs on that segment's packed record and p2's outer
// segment.  Same track candidates as TCTPStage, without the trial segments.
struct TCTPMapStage {
    static constexpr int kSt = kTC;
    __device__ static bool eval(const BatchDev& b, int p1, int64_t q, int& oi, int& oj, float* fv) {
        const int mdA = OJ(b, kSG, OJ(b, kTP, p1));
        const int64_t ns = join_n(b, mdA);
        int sx = 0, p2 = -1;
        for (int64_t k = 0; k < ns; ++k) {
            sx = join_obj(b, mdA, k);
            const int64_t n = join2_n(b, OJ(b, kSG, sx));
            if (q < n) {
                p2 = join2_obj(b, OJ(b, kSG, sx), q);
                break;
            }
            q -= n;
        }
        oi = p1;
        oj = p2;
        (void)fv;
        if (p2 < 0) return false;  // not reached: q is below the count (k_tc_count_tp)
        const int so = OJ(b, kTP, p2);
        float cut, muls;
        const int algo = tl_phaseA(load_sgv(b.sgpack, sx), load_sgv(b.sgpack, so), cut, muls);
        if (algo == kAlgoNone || !tl_phaseB1(algo, b.sgpack, sx, so, cut)) return false;
        return tl_phaseB2<kB2All>(algo, b.sgpack, sx, so, muls, false);
    }
    __device__ static int group_of(const BatchDev& b, int p) { return OG(b, kTP, p); }
};

// outer segment of flat tracklet candidate c of inner segment s
// tracklet candidate q of inner segment s by navigation (Event.cc:694-751):
// over the segments leaving s's outer MD, the segments leaving their outer MD
// (both lists from the join index of segments by inner MD)
__device__ __forceinline__ int tl_outer_nav(const BatchDev& b, int s, int64_t q) {
    const int m = OJ(b, kSG, s);
    const int64_t nc = join_n(b, m);
    for (int64_t k = 0; k < nc; ++k) {
        const int mc = OJ(b, kSG, join_obj(b, m, k));
        const int64_t n = join_n(b, mc);
        if (q < n) return join_obj(b, mc, q);
        q -= n;
    }
#ifdef SDL_DEVICE_CHECKS
    IX(-3, 0);
#endif
    return 0;  // q is below the candidate count (k_tl_count_nav)
}

// the tracklet variant of a run: 0 module map, 1 layer pairs, 2 navigation
__device__ __forceinline__ int tl_variant(const BatchDev& b) {
    return (b.flags & kFlagTLLayers) ? 1 : ((b.flags & kFlagTLNav) ? 2 : 0);
}
__device__ __forceinline__ int tl_outer_of(const BatchDev& b, int var, int s, int64_t q) {
    return var == 1 ? tl_outer_layer(b, s, q) : (var == 2 ? tl_outer_nav(b, s, q) : tl_outer(b, s, q));
}

// Phases A and B1 of a candidate from the single-precision decisions, with
// tl_phaseA where the first cannot decide: returns the algorithm (kAlgoNone:
// rejected by phase A or B1) and sets b1 when phase B1 passed already (0:
// phase B1 is left to k_tl_b1); exact tells whether an exact evaluation was
// needed.  txy: the outer segment's anchors (load_sgo_xy).  The exact cut
// values are computed again in phase B1.
__device__ __forceinline__ int tl_ab1_decide(const SGV& S, const SGOuter& T, float4 txy, int& b1, bool& exact) {
    float cut;
    int algo = tl_phaseA_quick(S, T, cut);
    exact = algo == kAlgoUnsure;
    if (exact) {
        float muls;
        algo = tl_phaseA(S, T, cut, muls);
    }
    b1 = 0;
    if (algo == kAlgoNone) return algo;
    const int q = tl_phaseB1_quick(algo, S, txy, cut);
    if (q == 0) return kAlgoNone;
    b1 = q > 0;
    exact = exact || q < 0;
    return algo;
}

// A warp's phase-A survivors, collected in shared memory and appended to
// the survivor list in batches of up to kPassBuf: one atomic on the list's
// count per batch instead of one per 32 candidates (atomics on one address
// serialise at its L2 slice, a few per nanosecond at most).  Positions past
// the list's capacity are not written and flag the overflow (the count keeps
// growing, so it holds the capacity needed).  Every lane of the warp calls
// passbuf_add and passbuf_flush.
constexpr int kPassBuf = 128;
constexpr int kPbBuf = 64;  // the phase-B2 (and segment first-pass) list's per-warp buffers
struct PassBuf {
    int4* e;    // this warp's kPassBuf entries in shared memory
    int n = 0;  // entries held (warp-uniform)
};
__device__ __forceinline__ void passbuf_flush(const BatchDev& b, PassBuf& pb) {
    __syncwarp();
    const int lane = threadIdx.x & 31;
    unsigned long long p0 = 0;
    if (lane == 0 && pb.n) p0 = atomicAdd(b.n_kept, (unsigned long long)pb.n);
    p0 = __shfl_sync(0xffffffffu, p0, 0);
    for (int i = lane; i < pb.n; i += kWarp) {
        const int64_t pos = (int64_t)p0 + i;
        if (pos < b.kept_cap) AT(b.passa, pos, b.kept_cap) = pb.e[i];
        else atomicOr(b.status, kStatusOverflowKept);
    }
    __syncwarp();
    pb.n = 0;
}
__device__ __forceinline__ void passbuf_add(const BatchDev& b, PassBuf& pb, int algo, int s, int tt, int b1) {
    const int lane = threadIdx.x & 31;
    const bool pass = algo != kAlgoNone;
    const unsigned m = __ballot_sync(0xffffffffu, pass);
    if (!m) return;
    const int c = __popc(m);
    if (pb.n + c > kPassBuf) passbuf_flush(b, pb);
    if (pass) pb.e[pb.n + __popc(m & ((1u << lane) - 1u))] = make_int4(s, tt, algo, b1);
    pb.n += c;
}

// Tracklet candidates (Event.cc:611-693 with Tracklet.cc:144-2665) in three
// kernels: the enumeration (k_tl_enum_a here: tasks of consecutive
// candidates from a shared counter; k_tl_enum_tiles below for the module
// map) runs phase A (the float cuts) and, for its survivors, the
// single-precision decision of phase B1 on each candidate and lists the
// survivors, marking those through phase B1 already; k_tl_b1 and k_tl_b2 run
// the two parts of phase B on compacted lists and append the tracklets.  The
// survivor list shares the pre-filter's capacity and overflow handling (its
// count is n_kept).
__global__ void __launch_bounds__(kEnumThreads) k_tl_enum_a(BatchDev b) {
    __shared__ int4 pbuf[kEnumThreads / kWarp][kPassBuf];
    if (halted(b)) return;
    const int64_t nobj = n_inner(b, kTL);
    if (nobj <= 0) return;
    const int64_t* off = b.cand[kTL];
    const int64_t offlim = b.cand_cap[kTL] + 1;
    const int64_t total = AT(off, nobj, offlim);
    const int task = b.enum_task[kTL] > 0 ? b.enum_task[kTL] : kTaskDefault;
    const int64_t ntask = (total + task - 1) / task;
    const int lane = threadIdx.x & 31;
    const int lay = tl_variant(b);
    PassBuf pb{pbuf[threadIdx.x >> 5]};
    for (;;) {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(b.task + kTL, 1ull);
        t = __shfl_sync(0xffffffffu, t, 0);
        if ((int64_t)t >= ntask) break;
        const int64_t base = (int64_t)t * task;
        const int64_t end = min(base + task, total);
        int ilo = 0;
        if (lane < 2) {
            int lo, hi;
            obj_bounds(b, nobj, total, base, end - 1, lo, hi);
            ilo = find_obj(b, off, offlim, lo, hi, lane == 0 ? base : end - 1);
        }
        const int i0 = __shfl_sync(0xffffffffu, ilo, 0);
        const int i1 = __shfl_sync(0xffffffffu, ilo, 1);
        for (int64_t cb = base; cb < end; cb += kWarp) {
            const int64_t c = cb + lane;
            int algo = kAlgoNone, s = 0, tt = 0, b1 = 0;
            if (c < end) {
                s = (i0 == i1) ? i0 : find_obj(b, off, offlim, i0, i1, c);
                tt = tl_outer_of(b, lay, s, c - AT(off, s, offlim));
                (void)IX(s, b.obj[kSG].cap);
                (void)IX(tt, b.obj[kSG].cap);
                const int64_t C = b.obj[kSG].cap;
                bool exact;
                algo = tl_ab1_decide(load_sgv(b.sgpack, s), load_sgo(b.sgouter, C, tt), load_sgo_xy(b.sgouter, C, tt), b1, exact);
            }
            passbuf_add(b, pb, algo, s, tt, b1);
        }
    }
    passbuf_flush(b, pb);
}

// Module-map tracklet candidates in module-pair tiles.  The outer segments of
// an inner segment are those of the modules connected to the module of its
// outer mini-doublet (Event.cc:611-693), so all inner segments ending in one
// module g share one list of outer segments, and g's candidates are the
// product (segments ending in g) x (segments of g's connected modules, in
// connection-list order).  A warp task is a tile of that product: up to
// kTileA inner segments x 32 outer segments.  Each lane decodes and loads its
// outer segment once per tile, and the inner segments' records are
// warp-uniform loads.  The candidates, and so the survivor list as a set, are
// those k_tl_enum_a enumerates.
#ifndef SDLG_TILE_A
#define SDLG_TILE_A 24
#endif
// inner segments per module-pair tile (a multiple of 4, at most 32); 24
// measured fastest on the 128-event PU 150-300 batch (enumeration 14.47 ms,
// against 14.82 at 16 and 14.60 at 32)
constexpr int kTileA = SDLG_TILE_A;
static_assert(kTileA % 4 == 0 && kTileA <= 32, "tile rows");

__device__ __forceinline__ int64_t tile_count(int64_t na, int64_t nb) {
    return (na > 0 && nb > 0) ? ((na + kTileA - 1) / kTileA) * ((nb + kWarp - 1) / kWarp) : 0;
}

// tiles per global module (eoff still holds the counts of segments ending there)
__global__ void k_tl_tile_count(BatchDev b) {
    if (halted(b)) return;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < b.n_gm; g += (int64_t)gridDim.x * blockDim.x)
        AT(b.toff, g, NG1(b)) = tile_count(AT(b.eoff, g, NG1(b)), AT(b.conn_sum, g, b.n_gm));
}

// the segments by the global module of their outer mini-doublet (eoff scanned)
__global__ void k_sg_end_scatter(BatchDev b) {
    if (halted(b)) return;
    const int64_t n = n_inner(b, kTL);
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
        const int g2 = OG(b, kMD, OJ(b, kSG, s));
        const int64_t pos = AT(b.eoff, g2, NG1(b)) + atomicAdd(&AT(b.ecur, g2, b.n_gm), 1);
        AT(b.eidx, pos, b.obj[kSG].cap) = (int)s;
    }
}

// the global module holding tile t: the largest g < n_gm with toff[g] <= t
// (toff[0] = 0 <= t), by a 32-way search; every lane calls it with the same t
__device__ __forceinline__ int tile_module(const BatchDev& b, int64_t t) {
    const int lane = threadIdx.x & 31;
    int lo = 0, hi = b.n_gm - 1;  // toff[lo] <= t, and the answer is in [lo, hi]
    while (hi - lo >= kWarp) {
        const int64_t span = (int64_t)(hi - lo) + 1;
        const int p = lo + (int)((span * lane) >> 5);  // probes lo = p_0 < p_1 < ... < p_31 <= hi
        const unsigned m = __ballot_sync(0xffffffffu, AT(b.toff, p, NG1(b)) <= t);
        const int j = 31 - __clz(m);  // bit 0 is set, and the set bits are a prefix
        if (j < 31) hi = lo + (int)((span * (j + 1)) >> 5) - 1;
        lo += (int)((span * j) >> 5);
    }
    const int p = lo + lane;
    const unsigned m = __ballot_sync(0xffffffffu, p <= hi && AT(b.toff, p, NG1(b)) <= t);
    return lo + 31 - __clz(m);
}

// tile -> global module map of the module-pair tiles (toff scanned); not
// built when the tiles exceed its capacity (the enumeration then searches toff)
__global__ void k_tile_map(BatchDev b) {
    if (halted(b)) return;
    const int64_t ntile = AT(b.toff, b.n_gm, NG1(b));
    if (ntile > b.tile_cap) return;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < b.n_gm; g += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t1 = AT(b.toff, g + 1, NG1(b));
        for (int64_t t = AT(b.toff, g, NG1(b)); t < t1; ++t) AT(b.tile_gm, t, b.tile_cap) = (int)g;
    }
}

// The outer object of lane q - q0 of a tile whose outer block starts at entry
// q0 of global module g's outer list (the objects of g's connected modules in
// connection-list order; module m of event ev, connection entries [k0, k1)),
// from the entries' prefix sums and first objects (k_conn_sum).  While g has
// at most 32 connections, lane j loads entry k0 + j and each lane finds its
// entry among them (the last one whose prefix sum is <= its q); otherwise
// each lane searches.  Every lane of the warp calls it; lanes with has false
// get an unspecified value.
__device__ __forceinline__ int tile_outer(const BatchDev& b, int ev, int m, int k0, int k1, int64_t q0, bool has) {
    const int lane = threadIdx.x & 31;
    const int64_t q = q0 + lane;
    const int64_t pbase = (int64_t)ev * b.geo.n_conn;
    if (k1 - k0 <= kWarp) {
        int pj = 0x7fffffff, fj = 0;
        if (lane < k1 - k0) {
            pj = AT(b.conn_pref, pbase + k0 + lane, NCP(b));
            fj = AT(b.conn_first, pbase + k0 + lane, NCP(b));
        }
        // entry 0 has prefix sum 0 <= q0
        int j = 31 - __clz(__ballot_sync(0xffffffffu, pj <= q0));
        for (int jj = j + 1; jj < k1 - k0; ++jj) {
            const int pjj = __shfl_sync(0xffffffffu, pj, jj);
            if (pjj > q0 + (kWarp - 1)) break;
            if (pjj <= q) j = jj;
        }
        const int pref = __shfl_sync(0xffffffffu, pj, j);
        const int first = __shfl_sync(0xffffffffu, fj, j);
        return first + (int)(q - pref);
    }
    if (!has) return 0;
    int pref;
    const int k = conn_entry(b, ev, m, q, pref);
    return (int)(AT(b.conn_first, pbase + k, NCP(b)) + (q - pref));
}

// Each warp takes tiles from a shared counter (the next index is fetched
// while the current tile runs).  Per tile, the loads come in a few dependent
// rounds: the module (tile map), its offsets and connection-list range, the
// inner segments' indices with the connection entries' prefix sums and first
// segments (one entry per lane while the module has at most 32 connections),
// then the inner segments' records (staged in shared memory, read there as
// warp-uniform values) with the lanes' outer-segment fields.
// CTAs per SM the module-pair enumeration is compiled for (register budget;
// 3, with 78 registers and no spill, measured 15.7 against 14.5 ms)
#ifndef SDLG_ENUM_MIN_BLOCKS
#define SDLG_ENUM_MIN_BLOCKS 4
#endif
__global__ void __launch_bounds__(kEnumThreads, SDLG_ENUM_MIN_BLOCKS) k_tl_enum_tiles(BatchDev b) {
    __shared__ __align__(16) float4 srec[kEnumThreads / kWarp][kTileA * (PK_N / 4)];
    __shared__ int sidx[kEnumThreads / kWarp][kTileA];
    __shared__ int4 pbuf[kEnumThreads / kWarp][kPassBuf];
    __shared__ float4 sxy[kEnumThreads / kWarp][kWarp];  // the lanes' outer anchors (phase B1)
    if (halted(b) || b.n_gm <= 0) return;
    const int64_t ntile = AT(b.toff, b.n_gm, NG1(b));
    const bool mapped = ntile <= b.tile_cap;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int n_mod = b.geo.n_mod;
    const int64_t sgcap = b.obj[kSG].cap;
    PassBuf pb{pbuf[w]};
    unsigned long long next = 0;
    if (lane == 0) next = atomicAdd(b.task + kTL, 1ull);
    for (;;) {
        const int64_t t = (int64_t)__shfl_sync(0xffffffffu, next, 0);
        if (t >= ntile) break;
        if (lane == 0) next = atomicAdd(b.task + kTL, 1ull);
        const int g = mapped ? AT(b.tile_gm, t, b.tile_cap) : tile_module(b, t);
        const int ev = ev_of(b, g), m2 = g - ev * n_mod;
        const int64_t a0 = AT(b.eoff, g, NG1(b));
        const int64_t na = AT(b.eoff, g + 1, NG1(b)) - a0;
        const int64_t nb = AT(b.conn_sum, g, b.n_gm);
        const int k0 = AT(b.geo.conn_off, m2, NM(b) + 1), k1 = AT(b.geo.conn_off, m2 + 1, NM(b) + 1);
        const int64_t nbb = (nb + kWarp - 1) / kWarp;
        const int64_t local = t - AT(b.toff, g, NG1(b));
        const int64_t ab = local / nbb, bb = local - ab * nbb;
        const int64_t abase = ab * kTileA;
        const int nat = (int)min((int64_t)kTileA, na - abase);
        // this lane's outer segment: entry q of g's outer list
        const int64_t q0 = bb * kWarp;
        const bool has = q0 + lane < nb;
        __syncwarp();  // the previous tile's records have been read
        if (lane < nat) sidx[w][lane] = AT(b.eidx, a0 + abase + lane, sgcap);
        const int tt = tile_outer(b, ev, m2, k0, k1, q0, has);
        SGOuter T{};
        if (has) {
            (void)IX(tt, sgcap);
            T = load_sgo(b.sgouter, sgcap, tt);
            sxy[w][lane] = load_sgo_xy(b.sgouter, sgcap, tt);
        }
        __syncwarp();
        // stage the tile's inner-segment records (nat x 8 float4)
#pragma unroll
        for (int r = 0; r < kTileA * (PK_N / 4) / kWarp; ++r) {
            const int e = lane + r * kWarp;
            if (e < nat * (PK_N / 4)) {
                const int sr = sidx[w][e / (PK_N / 4)];
                (void)IX(sr, sgcap);
                srec[w][e] = __ldg(reinterpret_cast<const float4*>(b.sgpack + (int64_t)sr * PK_N) + e % (PK_N / 4));
            }
        }
        __syncwarp();
        for (int r = 0; r < nat; ++r) {
            const int sr = sidx[w][r];
            int algo = kAlgoNone, b1 = 0;
            if (has) {
                bool exact;
                algo = tl_ab1_decide(sgv_from(reinterpret_cast<const float*>(&srec[w][r * (PK_N / 4)])), T, sxy[w][lane], b1,
                                     exact);
            }
            passbuf_add(b, pb, algo, sr, tt, b1);
        }
    }
    passbuf_flush(b, pb);
}

// CTAs per SM the segment second pass is compiled for (register budget: 64
// registers and no spill at 4, 40 and about 100 bytes of spills at 6).  With
// the pass split by algorithm, 4 measured fastest on the 128-event PU 150-300
// batch: segment stage 7.21 ms against 7.23 at 5 and 7.57 at 6
#ifndef SDLG_SGB_MIN_BLOCKS
#define SDLG_SGB_MIN_BLOCKS 4
#endif
constexpr int kSgbMinBlocks = SDLG_SGB_MIN_BLOCKS;

// Module-map segment candidates in two passes (Event.cc:445-522 with
// Segment.cc:337-859): k_sg_enum_a takes tasks of consecutive candidates
// like k_enum, runs the algorithm's first cuts (sg_pair_rec<true>: the same
// float code as the whole algorithm up to its phi cut) and lists the
// survivors in the passa list; k_sg_b runs the whole algorithm on the list on
// full warps and appends the segments.  The first cuts reject most
// candidates, so the expensive rest (the direction-change and dAlpha cuts)
// no longer runs beside idle lanes.
// A warp's segment first-pass survivors appended to the spare list pb:
// candidates with a barrel outer MD at its front (count n_pb[0]), the others
// at its back (n_pb[1]), so that the second pass runs each algorithm in its
// own kernel.  n_kept counts both and reserves their room: a batch that would
// take the two parts past kept_cap is not written and flags the overflow (the
// count keeps growing, so it holds the capacity needed).
__device__ __forceinline__ void sg_list_flush(const BatchDev& b, int4* buf, int& n, bool front) {
    __syncwarp();
    const int lane = threadIdx.x & 31;
    unsigned long long p0 = 0;
    int ok = 1;
    if (lane == 0 && n) {
        const unsigned long long tot = atomicAdd(b.n_kept, (unsigned long long)n);
        ok = tot + (unsigned long long)n <= (unsigned long long)b.kept_cap;
        if (ok) p0 = atomicAdd(b.n_pb + (front ? 0 : 1), (unsigned long long)n);
        else atomicOr(b.status, kStatusOverflowKept);
    }
    p0 = __shfl_sync(0xffffffffu, p0, 0);
    ok = __shfl_sync(0xffffffffu, ok, 0);
    if (ok)
        for (int k = lane; k < n; k += kWarp) {
            const int64_t q = (int64_t)p0 + k;
            AT(b.pb, front ? q : b.kept_cap - 1 - q, b.kept_cap) = buf[k];
        }
    __syncwarp();
    n = 0;
}

__global__ void __launch_bounds__(kEnumThreads) k_sg_enum_a(BatchDev b) {
    __shared__ int4 sbuf[kEnumThreads / kWarp][2][kPbBuf];
    if (halted(b)) return;
    const int64_t nobj = n_inner(b, kSG);
    if (nobj <= 0) return;
    const int64_t* off = b.cand[kSG];
    const int64_t offlim = b.cand_cap[kSG] + 1;
    const int64_t total = AT(off, nobj, offlim);
    const int task = b.enum_task[kSG] > 0 ? b.enum_task[kSG] : kTaskDefault;
    const int64_t ntask = (total + task - 1) / task;
    const int lane = threadIdx.x & 31;
    int4* fb = sbuf[threadIdx.x >> 5][0];
    int4* bb = sbuf[threadIdx.x >> 5][1];
    int nf = 0, nb = 0;
    for (;;) {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(b.task + kSG, 1ull);
        t = __shfl_sync(0xffffffffu, t, 0);
        if ((int64_t)t >= ntask) break;
        const int64_t base = (int64_t)t * task;
        const int64_t end = min(base + task, total);
        int ilo = 0;
        if (lane < 2) {
            int lo, hi;
            obj_bounds(b, nobj, total, base, end - 1, lo, hi);
            ilo = find_obj(b, off, offlim, lo, hi, lane == 0 ? base : end - 1);
        }
        const int i0 = __shfl_sync(0xffffffffu, ilo, 0);
        const int i1 = __shfl_sync(0xffffffffu, ilo, 1);
        for (int64_t cb = base; cb < end; cb += kWarp) {
            const int64_t c = cb + lane;
            int a = 0, bmd = 0;
            bool pass = false, ob = false;
            if (c < end) {
                a = (i0 == i1) ? i0 : find_obj(b, off, offlim, i0, i1, c);
                bmd = sg_outer_md(b, a, c - AT(off, a, offlim));
                (void)IX(bmd, b.obj[kMD].cap);
                float fv[6];
                const MDRec orec = md_rec(b, bmd);
                ob = orec.v.m->subdet == kBarrel;
                pass = sg_pair_rec<true>(md_rec(b, a).v, orec, true, fv);
            }
            const unsigned lt = (1u << lane) - 1u;
            const unsigned mf = __ballot_sync(0xffffffffu, pass && ob), mb = __ballot_sync(0xffffffffu, pass && !ob);
            if (nf + __popc(mf) > kPbBuf) sg_list_flush(b, fb, nf, true);
            if (nb + __popc(mb) > kPbBuf) sg_list_flush(b, bb, nb, false);
            if (pass && ob) fb[nf + __popc(mf & lt)] = make_int4(a, bmd, 1, 0);
            if (pass && !ob) bb[nb + __popc(mb & lt)] = make_int4(a, bmd, 2, 0);
            nf += __popc(mf);
            nb += __popc(mb);
        }
    }
    sg_list_flush(b, fb, nf, true);
    sg_list_flush(b, bb, nb, false);
}

template <int kOuter>
__global__ void __launch_bounds__(kEnumThreads, kSgbMinBlocks) k_sg_b(BatchDev b) {
    __shared__ int rbuf[kEnumThreads / kWarp][3 + 6][kRecBuf];
    if (halted(b)) return;
    // kOuter 1: the barrel part of the first pass's list (front), 2: the endcap part (back)
    const int64_t nfront = min((int64_t)b.n_pb[0], b.kept_cap);
    const int64_t n = kOuter == 1 ? nfront : min((int64_t)b.n_pb[1], b.kept_cap - nfront);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t nwarp = (int64_t)gridDim.x * (kEnumThreads / 32);
    RecBuf<6> rb{rbuf[w]};
    for (int64_t base = ((int64_t)blockIdx.x * (kEnumThreads / 32) + w) * kWarp; base < n; base += nwarp * kWarp) {
        const int64_t i = base + lane;
        bool pass = false;
        int a = 0, bmd = 0;
        float fv[6];
        if (i < n) {
            const int4 e = AT(b.pb, kOuter == 1 ? i : b.kept_cap - 1 - i, b.kept_cap);
            a = e.x;
            bmd = e.y;
            pass = sg_pair_rec<false, kOuter>(md_rec(b, a).v, md_rec(b, bmd), true, fv);
        }
        const unsigned m = __ballot_sync(0xffffffffu, pass);
        if (!m) continue;
        if (rb.n + __popc(m) > kRecBuf) rec_flush<6>(b, kSG, rb);
        if (pass) {
            const int k = rb.n + __popc(m & ((1u << lane) - 1u));
            rb.e[0][k] = a;
            rb.e[1][k] = bmd;
            rb.e[2][k] = OG(b, kMD, a);
#pragma unroll
            for (int q = 0; q < 6; ++q) rb.e[3 + q][k] = __float_as_int(fv[q]);
        }
        rb.n += __popc(m);
    }
    rec_flush<6>(b, kSG, rb);
}

// Learned pre-filter of the tracklet candidates (no counterpart in the
// reference).  It scores the enumeration's survivor list (n_kept entries:
// through phase A, and through phase B1 or undecided there) in tiles of 128
// entries on the tensor cores; the entries whose logit reaches the threshold
// go to the kept list (n_kept2 entries), which k_tl_b1 and k_tl_b2 judge.  A
// candidate that fails phase A or B1 gives no tracklet, so the tracklets are
// those of the plain chain among the candidates the network keeps; the
// network only sees phase-A survivors, the candidates it was trained on.
// Each CTA takes every gridDim.x-th tile; while the tensor cores run a
// tile's first layer, the CTA loads the next tile's entries and features.
// Control flow around the tile is uniform over the CTA.

// one tile's kept entries: written once the atomic that reserved their
// positions (issued by lane `leader`, raw value there) has returned
struct PfPending {
    unsigned m = 0u;
    unsigned long long raw = 0ull;
    int leader = 0;
    int4 e = make_int4(0, 0, 0, 0);  // (inner, outer, algorithm, 0)
};

__device__ __forceinline__ void pf_flush(const BatchDev& b, const PfPending& p) {
    if (p.m == 0u) return;
    const unsigned long long p0 = __shfl_sync(0xffffffffu, p.raw, p.leader);
    const int lane = threadIdx.x & 31;
    if (!((p.m >> lane) & 1u)) return;
    const int64_t pos = (int64_t)p0 + __popc(p.m & ((1u << lane) - 1u));  // below the list length <= kept_cap
    AT(b.kept, pos, b.kept_cap) = p.e;
}

// CTAs per SM: shared memory (33.4 KB per CTA) leaves room for 6; 6 and 8
// CTAs measured the same before the second layer took b2 into its MMA
constexpr int kPfCtasPerSm = 6;
__global__ void __launch_bounds__(kMlpTile, kPfCtasPerSm) k_tl_prefilter(BatchDev b) {
    __shared__ MlpSmem sm;
    if (halted(b)) return;
    const int64_t n = min((int64_t)*b.n_kept, b.kept_cap);
    const int64_t ntile = (n + kMlpTile - 1) / kMlpTile;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const int64_t nobj = n_inner(b, kTL);
        const int64_t cand = nobj > 0 ? AT(b.cand[kTL], nobj, b.cand_cap[kTL] + 1) : 0;
        atomicAdd(&b.mlp_stats->candidates, (unsigned long long)cand);
    }
    if ((int64_t)blockIdx.x >= ntile) return;
    const int lane = threadIdx.x & 31;
    mlp_setup(sm, b.mlp_pack);
    const float thr = reinterpret_cast<const float*>(sm.w + kPackB3)[1];
    MlpThread st;
    if (b.flags & kFlagTestMlpGiveUp) st.polls = 0;
    unsigned n_scored = 0, n_kept = 0;
    // Three tiles in the pipeline of each thread: the list entry of tile
    // t + 2G (G = gridDim.x) is loaded, the two segment records of tile t + G
    // are loaded with the entry loaded one iteration earlier, and the features
    // of tile t are computed from the records loaded one iteration earlier,
    // so that every load has a tile's MMAs and epilogue to complete in.
    const int64_t G = gridDim.x;
    auto entry = [&](int64_t tt, int4& e) -> bool {
        const int64_t i = tt * kMlpTile + threadIdx.x;
        const bool valid = tt < ntile && i < n;
        if (valid) e = AT(b.passa, i, b.kept_cap);
        return valid;
    };
    int64_t t = blockIdx.x;
    PfPending cur, pend;
    int4 e1 = make_int4(0, 0, 0, 0), e2 = make_int4(0, 0, 0, 0);
    bool valid = entry(t, cur.e);
    bool v1 = entry(t + G, e1);
    FeatS rs{};
    FeatT rt{};
    if (valid) {
        rs = feat_s(b.sgfeat, cur.e.x);
        rt = feat_t(b.sgfeat, cur.e.y);
    }
    while (t < ntile) {
        float f[kMlpIn];
        if (valid) {
            tl_features(rs, rt, f);
        } else {
#pragma unroll
            for (int k = 0; k < kMlpIn; ++k) f[k] = 0.f;
        }
        mlp_tile_begin(sm, f, st);
        const bool v2 = entry(t + 2 * G, e2);
        if (v1) {
            rs = feat_s(b.sgfeat, e1.x);
            rt = feat_t(b.sgfeat, e1.y);
        }
        pf_flush(b, pend);
        const float z = mlp_tile_end(sm, st);
        const bool keep = valid && z >= thr;
        n_scored += valid;
        n_kept += keep;
        cur.m = __ballot_sync(0xffffffffu, keep);
        if (cur.m) {
            cur.leader = __ffs(cur.m) - 1;
            if (lane == cur.leader) cur.raw = atomicAdd(b.n_kept2, (unsigned long long)__popc(cur.m));
        }
        pend = cur;
        cur.e = e1;
        valid = v1;
        e1 = e2;
        v1 = v2;
        t += G;
    }
    pf_flush(b, pend);
    n_scored = __reduce_add_sync(0xffffffffu, n_scored);
    n_kept = __reduce_add_sync(0xffffffffu, n_kept);
    if (lane == 0) {
        atomicAdd(&b.mlp_stats->scored, (unsigned long long)n_scored);
        atomicAdd(&b.mlp_stats->kept, (unsigned long long)n_kept);
    }
    if (st.abort && threadIdx.x == 0) {
        atomicAdd(&b.mlp_stats->timeouts, 1ull);
        atomicOr(b.status, kStatusMlpTimeout);
    }
    mlp_teardown(sm, st);
}

// Self-check of tl_b2_quick (no counterpart in the reference): every entry of
// the last run's phase-A survivor list judged by the filter and by the exact
// phases B1 and B2.  out[10]: entries; through exact phase B1; through exact
// phases B1 and B2; rejected by the filter; rejected by the filter but
// through the exact phases (must be 0); rejected by the filter among those
// through exact phase B1; the largest |filter value - exact value| / the
// filter's bound for deltaBeta, dBetaCut2 and betaOut (float bits; below 1
// when the bounds hold); entries the filter left before reaching the cuts;
// entries it finds through phase B2; of those, entries through exact phase B1
// but not exact phase B2 (must be 0).
__global__ void __launch_bounds__(256) k_tl_b2q_check(BatchDev b, unsigned long long* out) {
    const int64_t n = min((int64_t)*b.n_kept, b.kept_cap);
    unsigned long long c[6] = {0, 0, 0, 0, 0, 0}, inc = 0, acc = 0, acc_bad = 0;
    float rmax[3] = {0.f, 0.f, 0.f};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int4 e = AT(b.passa, i, b.kept_cap);
        (void)IX(e.x, b.obj[kSG].cap);
        (void)IX(e.y, b.obj[kSG].cap);
        const SGV S = load_sgv(b.sgpack, e.x), T = load_sgv(b.sgpack, e.y);
        float cut, muls;
        tl_cut_values(e.z, S, T, cut, muls);
        const bool p1 = tl_phaseB1_sgv(e.z, S, T, cut);
        float rec[kTLVarN];
        rec[kTLVarDBeta] = __int_as_float(0x7fc00000);
        const bool p2 = p1 && tl_phaseB2_sgv<kB2All>(e.z, S, T, muls, false, rec);
        B2Quick q;
        const int f = tl_b2_quick(e.z, S, T, &q);
        c[0] += 1;
        c[1] += p1;
        c[2] += p2;
        c[3] += f == 0;
        c[4] += f == 0 && p2;
        c[5] += f == 0 && p1;
        inc += f != 0 && !q.complete;
        acc += f == 3;
        acc_bad += f == 3 && p1 && !p2;
        if (p1 && q.complete && rec[kTLVarDBeta] == rec[kTLVarDBeta]) {
            rmax[0] = fmaxf(rmax[0], fabsf(q.dbeta - rec[kTLVarDBeta]) / q.e_dbeta);
            rmax[1] = fmaxf(rmax[1], fabsf(q.cut2 - rec[kTLVarDBetaCut2]) / q.e_cut2);
            rmax[2] = fmaxf(rmax[2], fabsf(q.bout - rec[kTLVarBetaOut]) / q.e_bout);
        }
    }
    for (int k = 0; k < 6; ++k) atomicAdd(out + k, c[k]);
    for (int k = 0; k < 3; ++k) atomicMax(out + 6 + k, (unsigned long long)__float_as_uint(rmax[k]));
    atomicAdd(out + 9, inc);
    atomicAdd(out + 10, acc);
    atomicAdd(out + 11, acc_bad);
}

// Phase B1 on a survivor list of phase A (count entries of list/muls); the candidates
// through it go to the phase-B2 list, BBBB ones from the front and the others
// from the back, so that phase B2's warps mostly run one algorithm.  Front
// and back never meet: together they hold at most count <= kept_cap entries.
// Each warp collects its BBBB and its other survivors in two shared-memory
// buffers and appends each with one atomic per batch (as passbuf_add).
__device__ __forceinline__ void pb_flush(const BatchDev& b, int4* buf, int& n, bool front) {
    __syncwarp();
    const int lane = threadIdx.x & 31;
    unsigned long long p0 = 0;
    if (lane == 0 && n) p0 = atomicAdd(b.n_pb + (front ? 0 : 1), (unsigned long long)n);
    p0 = __shfl_sync(0xffffffffu, p0, 0);
    for (int k = lane; k < n; k += kWarp) {
        const int64_t q = (int64_t)p0 + k;  // below the list length <= kept_cap
        AT(b.pb, front ? q : b.kept_cap - 1 - q, b.kept_cap) = buf[k];
    }
    __syncwarp();
    n = 0;
}

// Phase B2's single-precision decision (tl_b2_quick, no counterpart in the
// reference) on a survivor list (in / n_in: the enumeration's, or the
// pre-filter's kept list): the entries it cannot reject go to the filtered
// list (n_keptf entries, same format), which phase B1 reads.  Exact phase B2
// passes about one in thirteen of the enumeration's entries, so the filter
// spares the exact phases (float-float arithmetic and the host libm's
// functions) most of their work; the tracklets do not change.  Each warp
// takes blocks of 32 consecutive entries (one tile's survivors are
// consecutive, so their segment records are shared in L1) and appends its
// kept entries in batches.  Pass 0 evaluates the common case (BBBB without a
// 2S endcap outer anchor) and defers the entries of the long branches to the
// phase-B2 list pb (unused until phase B1): BBEE entries to its front, EEEE
// and the 2S endcap BBBB entries to its back; passes 1 and 2 evaluate the
// front and the back, so that each pass's warps mostly run one branch.  An
// entry the filter finds through phase B2 by more than its bounds, whose
// phase B1 the enumeration decided already (passed), is a tracklet: it is
// appended here as k_tl_b2 would, and the exact phases skip it.
template <int kPass>
__global__ void __launch_bounds__(kEnumThreads) k_tl_b2f(BatchDev b, const int4* __restrict__ in,
                                                        const unsigned long long* n_in) {
    constexpr bool kDefer = kPass == 0;
    __shared__ int4 fbuf[kEnumThreads / kWarp][kPassBuf];
    __shared__ int4 dbuf[kDefer ? kEnumThreads / kWarp : 1][2][kPbBuf];
    __shared__ int tbuf[kEnumThreads / kWarp][3][kRecBuf];
    if (halted(b)) return;
    int64_t n;
    if (kPass == 0) {
        n = min((int64_t)*n_in, b.kept_cap);
    } else {
        const int64_t nf = min((int64_t)b.n_pb[0], b.kept_cap);
        n = kPass == 1 ? nf : min((int64_t)b.n_pb[1], b.kept_cap - nf);
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int4* buf = fbuf[w];
    int4* dfront = dbuf[kDefer ? w : 0][0];
    int4* dback = dbuf[kDefer ? w : 0][1];
    RecBuf<0> tl{tbuf[w]};
    int nb = 0, nf = 0, nk = 0;
    // p0 + nb <= the input length <= kept_cap: the filtered list cannot overflow
    auto flush = [&]() {
        __syncwarp();
        unsigned long long p0 = 0;
        if (lane == 0 && nb) p0 = atomicAdd(b.n_keptf, (unsigned long long)nb);
        p0 = __shfl_sync(0xffffffffu, p0, 0);
        for (int i = lane; i < nb; i += kWarp) AT(b.passf, (int64_t)p0 + i, b.kept_cap) = buf[i];
        __syncwarp();
        nb = 0;
    };
    const int64_t warps = (int64_t)gridDim.x * (kEnumThreads / kWarp);
    for (int64_t base = ((int64_t)blockIdx.x * (kEnumThreads / kWarp) + w) * kWarp; base < n; base += warps * kWarp) {
        const int64_t i = base + lane;
        int r = 0;
        int4 e = make_int4(0, 0, 0, 0);
        if (i < n) {
            e = kPass == 0 ? AT(in, i, b.kept_cap) : AT(b.pb, kPass == 1 ? i : b.kept_cap - 1 - i, b.kept_cap);
            (void)IX(e.x, b.obj[kSG].cap);
            (void)IX(e.y, b.obj[kSG].cap);
            r = tl_b2_quick<kDefer>(e.z, load_sgv(b.sgpack, e.x), load_sgv(b.sgpack, e.y));
            if (r == 3) r = e.w ? 4 : 1;  // (phase B1 undecided: both exact phases run)
        }
        const unsigned lt = (1u << lane) - 1u;
        const unsigned mt = __ballot_sync(0xffffffffu, r == 4);
        if (mt) {
            if (tl.n + __popc(mt) > kRecBuf) rec_flush<0>(b, kTL, tl);
            if (r == 4) {
                const int k = tl.n + __popc(mt & lt);
                tl.e[0][k] = e.x;
                tl.e[1][k] = e.y;
                tl.e[2][k] = OG(b, kSG, e.x);
            }
            tl.n += __popc(mt);
        }
        const unsigned m = __ballot_sync(0xffffffffu, r == 1);
        if (nb + __popc(m) > kPassBuf) flush();
        if (r == 1) buf[nb + __popc(m & lt)] = e;
        nb += __popc(m);
        if (kDefer) {
            // (the deferred entries fit: together at most the input length <= kept_cap)
            const bool front = e.z == kAlgoBBEE;
            const unsigned mf = __ballot_sync(0xffffffffu, r == 2 && front);
            const unsigned mk = __ballot_sync(0xffffffffu, r == 2 && !front);
            if (nf + __popc(mf) > kPbBuf) pb_flush(b, dfront, nf, true);
            if (nk + __popc(mk) > kPbBuf) pb_flush(b, dback, nk, false);
            if (r == 2 && front) dfront[nf + __popc(mf & lt)] = e;
            if (r == 2 && !front) dback[nk + __popc(mk & lt)] = e;
            nf += __popc(mf);
            nk += __popc(mk);
        }
    }
    flush();
    rec_flush<0>(b, kTL, tl);
    if (kDefer) {
        pb_flush(b, dfront, nf, true);
        pb_flush(b, dback, nk, false);
    }
}

__global__ void __launch_bounds__(kEnumThreads) k_tl_b1(BatchDev b, const int4* __restrict__ list,
                                                         const unsigned long long* count) {
    __shared__ int4 fbuf[kEnumThreads / kWarp][kPbBuf], bbuf[kEnumThreads / kWarp][kPbBuf];
    if (halted(b)) return;
    const int64_t n = min((int64_t)*count, b.kept_cap);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int nfb = 0, nbb = 0;  // entries held in this warp's buffers
    const int64_t nwarp = (int64_t)gridDim.x * (kEnumThreads / 32);
    for (int64_t base = ((int64_t)blockIdx.x * (kEnumThreads / 32) + w) * kWarp; base < n; base += nwarp * kWarp) {
        const int64_t i = base + lane;
        bool pass = false;
        int4 p = make_int4(0, 0, kAlgoNone, 0);
        float muls = 0.f;
        if (i < n) {
            p = AT(list, i, b.kept_cap);
            if (p.w) {  // phase B1 passed in the enumeration
                pass = true;
                muls = tl_muls_entry(p.z, b.sgpack, p.x, p.y);
            } else {
                const B1Result r = tl_phaseB1_entry(p.z, b.sgpack, p.x, p.y);
                pass = r.pass;
                muls = r.muls;
            }
        }
        const bool front = pass && p.z == kAlgoBBBB;
        const unsigned mf = __ballot_sync(0xffffffffu, front);
        const unsigned mb = __ballot_sync(0xffffffffu, pass && !front);
        if (!(mf | mb)) continue;
        if (nfb + __popc(mf) > kPbBuf) pb_flush(b, fbuf[w], nfb, true);
        if (nbb + __popc(mb) > kPbBuf) pb_flush(b, bbuf[w], nbb, false);
        if (pass) {
            const unsigned below = (1u << lane) - 1u;
            const int4 e = make_int4(p.x, p.y, p.z, __float_as_int(muls));
            if (front) fbuf[w][nfb + __popc(mf & below)] = e;
            else bbuf[w][nbb + __popc(mb & below)] = e;
        }
        nfb += __popc(mf);
        nbb += __popc(mb);
    }
    pb_flush(b, fbuf[w], nfb, true);
    pb_flush(b, bbuf[w], nbb, false);
}

// CTAs per SM the phase-B2 kernels are compiled for (register budget; 4
// measured fastest on the 128-event PU 150-300 batch: phase B1+B2 8.1 ms
// against 9.7 ms at 1, plain chain's B2 54.9 ms against 58.5 ms)
#ifndef SDLG_B2_MIN_BLOCKS
#define SDLG_B2_MIN_BLOCKS 4
#endif
constexpr int kB2MinBlocks = SDLG_B2_MIN_BLOCKS;

// Phase B2 on one part of the phase-B2 list (kSet kB2BBBB: the front, BBBB
// entries; kB2Others: the back, BBEE and EEEE entries); appends the tracklets.
template <int kSet>
__global__ void __launch_bounds__(kEnumThreads, kB2MinBlocks) k_tl_b2(BatchDev b) {
    __shared__ int rbuf[kEnumThreads / kWarp][3][kRecBuf];
    if (halted(b)) return;
    const int64_t nf = min((int64_t)b.n_pb[0], b.kept_cap);
    const int64_t n = kSet == kB2BBBB ? nf : min((int64_t)b.n_pb[1], b.kept_cap - nf);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const bool nm1 = (b.flags & kFlagTLNm1) != 0;
    const int64_t nwarp = (int64_t)gridDim.x * (kEnumThreads / 32);
    RecBuf<0> rb{rbuf[w]};
    for (int64_t base = ((int64_t)blockIdx.x * (kEnumThreads / 32) + w) * kWarp; base < n; base += nwarp * kWarp) {
        const int64_t i = base + lane;
        bool pass = false;
        int s = 0, tt = 0;
        if (i < n) {
            const int64_t k = kSet == kB2BBBB ? i : b.kept_cap - 1 - i;
            const int4 p = AT(b.pb, k, b.kept_cap);
            s = p.x;
            tt = p.y;
            pass = tl_phaseB2<kSet>(p.z, b.sgpack, s, tt, __int_as_float(p.w), nm1);
        }
        const unsigned m = __ballot_sync(0xffffffffu, pass);
        if (!m) continue;
        if (rb.n + __popc(m) > kRecBuf) rec_flush<0>(b, kTL, rb);
        if (pass) {
            const int k = rb.n + __popc(m & ((1u << lane) - 1u));
            rb.e[0][k] = s;
            rb.e[1][k] = tt;
            rb.e[2][k] = OG(b, kSG, s);
        }
        rb.n += __popc(m);
    }
    rec_flush<0>(b, kTL, rb);
}

__device__ __forceinline__ float hash_unit(unsigned long long c, unsigned long long seed) {
    // splitmix64 finaliser (Steele, Lea, Flood 2014)
    unsigned long long z = c + seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (float)(z >> 40) * (1.0f / 16777216.0f);
}

// Training samples for the learned pre-filter: the features of every
// tracklet candidate of the last run that passes phase A, labelled by phase
// B (the plain chain's accept / reject); rejected ones are kept with
// probability neg_keep.
__global__ void k_tl_collect(BatchDev b, MlpCollect col) {
    if (halted(b)) return;
    const int64_t nobj = n_inner(b, kTL);
    if (nobj <= 0) return;
    const int64_t* off = b.cand[kTL];
    const int64_t offlim = b.cand_cap[kTL] + 1;
    const int64_t total = AT(off, nobj, offlim);
    const int lay = tl_variant(b);
    const int lane = threadIdx.x & 31;
    for (int64_t c0 = (int64_t)blockIdx.x * blockDim.x; c0 < total; c0 += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = c0 + threadIdx.x;
        bool keep = false;
        float label = 0.f;
        float f[kMlpIn];
        if (c < total) {
            int lo, hi;
            obj_bounds(b, nobj, total, c, c, lo, hi);
            const int s = find_obj(b, off, offlim, lo, hi, c);
            const int tt = tl_outer_of(b, lay, s, c - AT(off, s, offlim));
            const SGV S = load_sgv(b.sgpack, s);
            const SGV T = load_sgv(b.sgpack, tt);
            float cut = 0.f, muls = 0.f;
            const int algo = tl_phaseA(S, T, cut, muls);
            if (algo != kAlgoNone) {
                const bool pass = tl_phaseB(algo, b.sgpack, s, tt, cut, muls, false);
                label = pass ? 1.f : 0.f;
                keep = pass || hash_unit((unsigned long long)c, col.seed) < col.neg_keep;
                if (keep) tl_features(feat_s(b.sgfeat, s), feat_t(b.sgfeat, tt), f);
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (!m) continue;
        const int leader = __ffs(m) - 1;
        unsigned long long p0 = 0;
        if (lane == leader) p0 = atomicAdd(col.n, (unsigned long long)__popc(m));
        p0 = __shfl_sync(0xffffffffu, p0, leader);
        const int64_t pos = (int64_t)p0 + __popc(m & ((1u << lane) - 1u));
        if (keep && pos < col.cap) {
#pragma unroll
            for (int k = 0; k < kMlpIn; ++k) col.x[pos * kMlpIn + k] = f[k];
            col.y[pos] = label;
        }
    }
}

// Self-check of the enumeration's single-precision decisions (tl_ab1_decide:
// phase A, then phase B1 for its survivors) over the tracklet candidates of
// the last run, against the exact phase A and B1 on the packed records:
// out[0] candidates, out[1] settled by the approximations alone, out[2] that
// needed an exact evaluation, out[3] settled wrongly (0 when the margins
// hold): rejected although both phases pass, accepted with another
// algorithm or although phase A fails, or marked as through phase B1 although
// it fails.
__global__ void k_tl_quick_check(BatchDev b, unsigned long long* out) {
    if (halted(b)) return;
    const int64_t nobj = n_inner(b, kTL);
    if (nobj <= 0) return;
    const int64_t* off = b.cand[kTL];
    const int64_t offlim = b.cand_cap[kTL] + 1;
    const int64_t total = AT(off, nobj, offlim);
    const int lay = tl_variant(b);
    unsigned long long n[4] = {0ull, 0ull, 0ull, 0ull};
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < total; c += (int64_t)gridDim.x * blockDim.x) {
        int lo, hi;
        obj_bounds(b, nobj, total, c, c, lo, hi);
        const int s = find_obj(b, off, offlim, lo, hi, c);
        const int tt = tl_outer_of(b, lay, s, c - AT(off, s, offlim));
        const SGV S = load_sgv(b.sgpack, s), Tv = load_sgv(b.sgpack, tt);
        const int64_t C = b.obj[kSG].cap;
        int b1;
        bool exact;
        const int q = tl_ab1_decide(S, load_sgo(b.sgouter, C, tt), load_sgo_xy(b.sgouter, C, tt), b1, exact);
        float cut, muls;
        const int e = tl_phaseA(S, Tv, cut, muls);
        const bool eb1 = e != kAlgoNone && tl_phaseB1_sgv(e, S, Tv, cut);
        const bool bad = q == kAlgoNone ? eb1 : (q != e || (b1 && !eb1));
        n[0] += 1;
        n[1] += !exact;
        n[2] += exact;
        n[3] += bad;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        unsigned long long v = n[k];
        for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd(out + k, v);
    }
}

// per-module object counts of a stage -> layer counters (before the scan)
__global__ void k_obj_counters(BatchDev b, int st) {
    if (halted(b)) return;
    const int n_mod = b.geo.n_mod;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g - threadIdx.x < b.n_gm; g += (int64_t)gridDim.x * blockDim.x) {
        const bool in = g < b.n_gm;
        uint32_t v = 0;
        int ev = 0, slot = 0;
        if (in) {
            v = (uint32_t)OFF(b, st, g);
            ev = ev_of(b, g);
            slot = MOD(b, g - (int64_t)ev * n_mod).layer_slot;
        }
        const bool act = in && v != 0;
        warp_add(act ? &AT(b.counters, (int64_t)ev * 110 + st * 22 + 11 + slot, (int64_t)b.n_ev * 110) : b.counters, v, act);
    }
}

__global__ void k_scatter(BatchDev b, int st) {
    if (halted(b)) return;
    const Recs& R = b.rec[st];
    const Objs& O = b.obj[st];
    const int64_t n = min(b.n_rec[st], O.cap);
    const int64_t flim = O.cap * (O.nf > 0 ? O.nf : 1);
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const int g = AT(R.g, r, O.cap);
        const int64_t pos = OFF(b, st, g) + AT(R.rank, r, O.cap);
        if (pos >= O.cap) continue;
        AT(O.i, pos, O.cap) = AT(R.i, r, O.cap);
        AT(O.j, pos, O.cap) = AT(R.j, r, O.cap);
        AT(O.g, pos, O.cap) = g;
        for (int k = 0; k < O.nf; ++k) AT(O.f, (int64_t)k * O.cap + pos, flim) = AT(R.f, (int64_t)k * O.cap + r, flim);
    }
}

// ------------------------------------------------------------------ counts
__device__ __forceinline__ uint32_t* counter_at(const BatchDev& b, int ev, int st, int kind, int slot) {
    return &AT(b.counters, (int64_t)ev * 110 + st * 22 + kind * 11 + slot, (int64_t)b.n_ev * 110);
}

__global__ void k_md_count(BatchDev b) {
    const int n_mod = b.geo.n_mod;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g - threadIdx.x < b.n_gm; g += (int64_t)gridDim.x * blockDim.x) {
        const bool in = g < b.n_gm;
        int64_t c = 0;
        int ev = 0, slot = 0;
        if (in) {
            ev = ev_of(b, g);
            const ModDev& m = MOD(b, g - (int64_t)ev * n_mod);
            if (m.lower && m.partner >= 0) {
                const int64_t pg = (int64_t)ev * n_mod + m.partner;
                c = (AT(b.mod_hit, g + 1, NG1(b)) - AT(b.mod_hit, g, NG1(b))) *
                    (AT(b.mod_hit, pg + 1, NG1(b)) - AT(b.mod_hit, pg, NG1(b)));
            }
            slot = m.layer_slot;
            AT(b.cand[kMD], g, b.cand_cap[kMD] + 1) = c;
        }
        const bool act = in && c != 0;
        warp_add(act ? counter_at(b, ev, kMD, 0, slot) : b.counters, (uint32_t)c, act);
    }
}

// per lower module: running sums of the object counts of its connected
// modules (stage src) -> conn_pref per entry and conn_sum per module; the
// reference's candidate counters of stage cst get n_obj(g) * conn_sum(g).
__global__ void k_conn_sum(BatchDev b, int src, int cst) {
    if (halted(b)) return;
    const int n_mod = b.geo.n_mod;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g - threadIdx.x < b.n_gm; g += (int64_t)gridDim.x * blockDim.x) {
        const bool in = g < b.n_gm;
        int64_t sum = 0, cand = 0;
        int ev = 0, slot = 0;
        if (in) {
            ev = ev_of(b, g);
            const int m = (int)(g - (int64_t)ev * n_mod);
            const int k0 = AT(b.geo.conn_off, m, NM(b) + 1), k1 = AT(b.geo.conn_off, m + 1, NM(b) + 1);
            const int64_t pbase = (int64_t)ev * b.geo.n_conn;
            const int64_t ebase = (int64_t)ev * n_mod;
            for (int k = k0; k < k1; ++k) {
                AT(b.conn_pref, pbase + k, NCP(b)) = (int32_t)sum;
                const int64_t g2 = ebase + AT(b.geo.conn_idx, k, NC(b));
                const int64_t o2 = OFF(b, src, g2);
                AT(b.conn_first, pbase + k, NCP(b)) = (int32_t)o2;
                sum += OFF(b, src, g2 + 1) - o2;
            }
            AT(b.conn_sum, g, b.n_gm) = sum;
            cand = (OFF(b, src, g + 1) - OFF(b, src, g)) * sum;
            slot = MOD(b, m).layer_slot;
        }
        const bool act = in && cand != 0 && cst >= 0;
        warp_add(act ? counter_at(b, ev, cst, 0, slot) : b.counters, (uint32_t)cand, act);
    }
}

// The outer lists of the segment candidates, written out: for every global
// module g holding mini-doublets, the mini-doublets of g's connected modules
// in connection-list order (entry q of g's list at olist[toff[g] + q]), so
// that a candidate finds its outer mini-doublet with one load.  toff holds
// the list lengths, then (scanned) the offsets; the lists are not written
// when they exceed olist_cap (the candidates then search the connection list).
__global__ void k_sg_olist_count(BatchDev b) {
    if (halted(b)) return;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < b.n_gm; g += (int64_t)gridDim.x * blockDim.x)
        AT(b.toff, g, NG1(b)) = OFF(b, kMD, g + 1) > OFF(b, kMD, g) ? AT(b.conn_sum, g, b.n_gm) : 0;
}
__global__ void k_sg_olist_fill(BatchDev b) {
    if (halted(b) || AT(b.toff, b.n_gm, NG1(b)) > b.olist_cap) return;
    const int n_mod = b.geo.n_mod;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < b.n_gm; g += (int64_t)gridDim.x * blockDim.x) {
        int64_t o = AT(b.toff, g, NG1(b));
        if (AT(b.toff, g + 1, NG1(b)) == o) continue;
        const int ev = ev_of(b, g), m = (int)(g - (int64_t)ev * n_mod);
        const int k0 = AT(b.geo.conn_off, m, NM(b) + 1), k1 = AT(b.geo.conn_off, m + 1, NM(b) + 1);
        for (int k = k0; k < k1; ++k) {
            const int64_t g2 = (int64_t)ev * n_mod + AT(b.geo.conn_idx, k, NC(b));
            const int64_t e = OFF(b, kMD, g2 + 1);
            for (int64_t md = OFF(b, kMD, g2); md < e; ++md) AT(b.olist, o++, b.olist_cap) = (int)md;
        }
    }
}

__global__ void k_sg_count(BatchDev b) {
    if (halted(b)) return;
    const int64_t n = n_inner(b, kSG);
    for (int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; a < n; a += (int64_t)gridDim.x * blockDim.x)
        AT(b.cand[kSG], a, b.cand_cap[kSG] + 1) = AT(b.conn_sum, OG(b, kMD, a), b.n_gm);
}

__global__ void k_tl_count(BatchDev b) {
    if (halted(b)) return;
    const int n_mod = b.geo.n_mod;
    const int64_t n = n_inner(b, kTL);
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s - threadIdx.x < n; s += (int64_t)gridDim.x * blockDim.x) {
        const bool in = s < n;
        int64_t c = 0;
        int ev = 0, slot = 0;
        if (in) {
            const int g2 = OG(b, kMD, OJ(b, kSG, s));
            c = AT(b.conn_sum, g2, b.n_gm);
            AT(b.cand[kTL], s, b.cand_cap[kTL] + 1) = c;
            atomicAdd((unsigned long long*)&AT(b.eoff, g2, NG1(b)), 1ull);  // segments ending in g2
            const int g1 = OG(b, kSG, s);
            ev = ev_of(b, g1);
            slot = MOD(b, g1 - ev * n_mod).layer_slot;
        }
        const bool act = in && c != 0;
        warp_add(act ? counter_at(b, ev, kTL, 0, slot) : b.counters, (uint32_t)c, act);
    }
}

// layer-pair segment candidates of every MD (Event.cc:805-818 loops over
// inner-layer MDs x outer-layer MDs); the reference counts none of them
__global__ void k_sg_count_layers(BatchDev b) {
    if (halted(b)) return;
    const int n_mod = b.geo.n_mod;
    const int64_t n = n_inner(b, kSG);
    for (int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; a < n; a += (int64_t)gridDim.x * blockDim.x) {
        const int g1 = OG(b, kMD, a);
        const int ev = ev_of(b, g1);
        const int si = MOD(b, g1 - ev * n_mod).layer_slot;
        int64_t c = 0;
        for (int k = 0; k < 3; ++k) {
            const int so = sg_layer_outer(si, k);
            if (so < 0) break;
            c += layer_count(b, kMD, ev, so);
        }
        AT(b.cand[kSG], a, b.cand_cap[kSG] + 1) = c;
    }
}

// layer-pair tracklet candidates of every segment (Event.cc:762-787), counted
// per inner layer like the module-map variant
__global__ void k_tl_count_layers(BatchDev b) {
    if (halted(b)) return;
    const int n_mod = b.geo.n_mod;
    const int64_t n = n_inner(b, kTL);
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s - threadIdx.x < n; s += (int64_t)gridDim.x * blockDim.x) {
        const bool in = s < n;
        int64_t c = 0;
        int ev = 0, slot = 0;
        if (in) {
            const int g1 = OG(b, kSG, s);
            ev = ev_of(b, g1);
            slot = MOD(b, g1 - ev * n_mod).layer_slot;
            const int so = tl_layer_outer(slot);
            c = so >= 0 ? layer_count(b, kSG, ev, so) : 0;
            AT(b.cand[kTL], s, b.cand_cap[kTL] + 1) = c;
        }
        const bool act = in && c != 0;
        warp_add(act ? counter_at(b, ev, kTL, 0, slot) : b.counters, (uint32_t)c, act);
    }
}

// objects of stage st per key mini-doublet, then their positions
__global__ void k_join_count(BatchDev b, int st, bool second) {
    if (halted(b)) return;
    int64_t* off = second ? b.joff2 : b.joff;
    const int64_t n = min(OFF(b, st, b.n_gm), b.obj[st].cap);
    for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < n; o += (int64_t)gridDim.x * blockDim.x)
        atomicAdd((unsigned long long*)&AT(off, join_key(b, st, o), b.obj[kMD].cap + 1), 1ull);
}
__global__ void k_join_scatter(BatchDev b, int st, bool second) {
    if (halted(b)) return;
    const int64_t* off = second ? b.joff2 : b.joff;
    int32_t* cur = second ? b.jcur2 : b.jcur;
    int32_t* idx = second ? b.jidx2 : b.jidx;
    const int64_t cap = second ? b.obj[kTP].cap : max(b.obj[kSG].cap, b.obj[kTL].cap);
    const int64_t n = min(OFF(b, st, b.n_gm), b.obj[st].cap);
    for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < n; o += (int64_t)gridDim.x * blockDim.x) {
        const int k = join_key(b, st, o);
        const int64_t pos = AT(off, k, b.obj[kMD].cap + 1) + atomicAdd(&AT(cur, k, b.obj[kMD].cap), 1);
        AT(idx, pos, cap) = (int)o;
    }
}

__global__ void k_tp_count(BatchDev b) {
    if (halted(b)) return;
    const int n_mod = b.geo.n_mod;
    const int64_t n = n_inner(b, kTP);
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
        const int g1 = OG(b, kSG, s);
        const int ev = ev_of(b, g1), m1 = g1 - ev * n_mod;
        const int g2 = OG(b, kMD, OJ(b, kSG, s));
        const int m2 = g2 - ev * n_mod;
        int mult = 0;
        const int k0 = AT(b.geo.conn_off, m1, NM(b) + 1), k1 = AT(b.geo.conn_off, m1 + 1, NM(b) + 1);
        for (int k = k0; k < k1; ++k) mult += AT(b.geo.conn_idx, k, NC(b)) == m2;
        AT(b.cand[kTP], s, b.cand_cap[kTP] + 1) = (int64_t)mult * join_n(b, OJ(b, kSG, s));
    }
}

__global__ void k_tc_count(BatchDev b) {
    if (halted(b)) return;
    const int64_t n = n_inner(b, kTC);
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t c = 0;
        const int g1 = OG(b, kTL, t);
        const ModDev& m1 = MOD(b, mod_of(b, g1));
        if (m1.subdet == kBarrel && m1.layer == 1) {
            const int g3 = OG(b, kSG, OJ(b, kTL, t));
            const ModDev& m3 = MOD(b, mod_of(b, g3));
            if (m3.subdet == kBarrel && m3.layer == 3) c = join_n(b, OI(b, kSG, OJ(b, kTL, t)));
        }
        AT(b.cand[kTC], t, b.cand_cap[kTC] + 1) = c;
    }
}

// navigation tracklet candidates of every segment (Event.cc:694-751) and the
// reference's candidate counters
__global__ void k_tl_count_nav(BatchDev b) {
    if (halted(b)) return;
    const int n_mod = b.geo.n_mod;
    const int64_t n = n_inner(b, kTL);
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s - threadIdx.x < n; s += (int64_t)gridDim.x * blockDim.x) {
        const bool in = s < n;
        int64_t c = 0;
        int ev = 0, slot = 0;
        if (in) {
            const int m = OJ(b, kSG, s);
            const int64_t nc = join_n(b, m);
            for (int64_t k = 0; k < nc; ++k) c += join_n(b, OJ(b, kSG, join_obj(b, m, k)));
            AT(b.cand[kTL], s, b.cand_cap[kTL] + 1) = c;
            const int g1 = OG(b, kSG, s);
            ev = ev_of(b, g1);
            slot = MOD(b, g1 - ev * n_mod).layer_slot;
        }
        const bool act = in && c != 0;
        warp_add(act ? counter_at(b, ev, kTL, 0, slot) : b.counters, (uint32_t)c, act);
    }
}

// createTrackCandidatesFromTracklets (Event.cc:984-1062): the reference's
// candidates of tracklet t are the tracklets of the modules connected to the
// module of its inner segment's outer MD (conn_sum over tracklet counts); the
// matching ones are the tracklets whose inner segment matches t's outer
// segment, which all lie in the module of that segment's inner MD and come
// once per occurrence of that module in the connection list.  Layer-pair
// tracklets are listed by no module (Event.cc:785 via
// addTrackletToLowerLayer), so after them there are no candidates.
__global__ void k_tc_count_tl(BatchDev b) {
    if (halted(b)) return;
    const int n_mod = b.geo.n_mod;
    const int64_t n = n_inner(b, kTC);
    const bool none = (b.flags & kFlagTLLayers) != 0;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t - threadIdx.x < n; t += (int64_t)gridDim.x * blockDim.x) {
        const bool in = t < n;
        int64_t cref = 0;
        int ev = 0, slot = 0;
        if (in) {
            const int gA2 = OG(b, kMD, OJ(b, kSG, OI(b, kTL, t)));
            ev = ev_of(b, gA2);
            const int mA2 = gA2 - ev * n_mod;
            cref = none ? 0 : AT(b.conn_sum, gA2, b.n_gm);
            const int mB = OI(b, kSG, OJ(b, kTL, t));
            const int mB1 = OG(b, kMD, mB) - ev * n_mod;
            int mult = 0;
            const int k0 = AT(b.geo.conn_off, mA2, NM(b) + 1), k1 = AT(b.geo.conn_off, mA2 + 1, NM(b) + 1);
            for (int k = k0; k < k1; ++k) mult += AT(b.geo.conn_idx, k, NC(b)) == mB1;
            AT(b.cand[kTC], t, b.cand_cap[kTC] + 1) = none ? 0 : (int64_t)mult * join_n(b, mB);
            slot = MOD(b, OG(b, kTL, t) - ev * n_mod).layer_slot;
        }
        const bool act = in && cref != 0;
        warp_add(act ? counter_at(b, ev, kTC, 0, slot) : b.counters, (uint32_t)cref, act);
    }
}

// createTrackCandidatesFromTriplets (Event.cc:874-982): candidates of triplet
// p = the triplets of the modules connected to the module of its outermost MD
// (conn_sum over triplet counts), with the reference's candidate counters
__global__ void k_tc_count_tp(BatchDev b) {
    if (halted(b)) return;
    const int n_mod = b.geo.n_mod;
    const int64_t n = n_inner(b, kTC);
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p - threadIdx.x < n; p += (int64_t)gridDim.x * blockDim.x) {
        const bool in = p < n;
        int64_t c = 0;
        int ev = 0, slot = 0;
        if (in) {
            const int mdA = OJ(b, kSG, OJ(b, kTP, p));
            c = AT(b.conn_sum, OG(b, kMD, mdA), b.n_gm);
            int64_t e = c;  // the trial-segment enumeration: every reference candidate
            if (!(b.flags & kFlagSGLayers)) {  // TCTPMapStage: segments leaving mdA x triplets at their outer MD
                e = 0;
                const int64_t ns = join_n(b, mdA);
                for (int64_t k = 0; k < ns; ++k) e += join2_n(b, OJ(b, kSG, join_obj(b, mdA, k)));
            }
            AT(b.cand[kTC], p, b.cand_cap[kTC] + 1) = e;
            const int g1 = OG(b, kTP, p);
            ev = ev_of(b, g1);
            slot = MOD(b, g1 - ev * n_mod).layer_slot;
        }
        const bool act = in && c != 0;
        warp_add(act ? counter_at(b, ev, kTC, 0, slot) : b.counters, (uint32_t)c, act);
    }
}

// Event.cc:835: track-candidate candidates are barrel-layer-1 x barrel-layer-3 tracklets
__global__ void k_tc_cand_counter(BatchDev b) {
    for (int ev = blockIdx.x * blockDim.x + threadIdx.x; ev < b.n_ev; ev += gridDim.x * blockDim.x) {
        const uint32_t n1 = *counter_at(b, ev, kTL, 1, 0), n3 = *counter_at(b, ev, kTL, 1, 2);
        *counter_at(b, ev, kTC, 0, 0) += n1 * n3;
    }
}

// ------------------------------------------------------------------ output
__device__ __forceinline__ void put_md(const BatchDev& b, int a, int32_t* o) {
    o[0] = AT(b.hidx, OI(b, kMD, a), H(b));
    o[1] = AT(b.hidx, OJ(b, kMD, a), H(b));
}
__device__ __forceinline__ void put_sg(const BatchDev& b, int s, int32_t* o) {
    put_md(b, OI(b, kSG, s), o);
    put_md(b, OJ(b, kSG, s), o + 2);
}
__device__ __forceinline__ void put_tl(const BatchDev& b, int st, int t, int32_t* o) {
    put_sg(b, OI(b, st, t), o);
    put_sg(b, OJ(b, st, t), o + 4);
}

// one row of W hit indices, built in registers, stored with 8- or 16-byte
// stores when the output is 16-byte aligned
template <int W>
__device__ __forceinline__ void store_row(int32_t* o, const int32_t* v, bool vec) {
    if (vec) {
        if constexpr (W == 2) {
            *reinterpret_cast<int2*>(o) = make_int2(v[0], v[1]);
        } else {
#pragma unroll
            for (int i = 0; i < W; i += 4) *reinterpret_cast<int4*>(o + i) = make_int4(v[i], v[i + 1], v[i + 2], v[i + 3]);
        }
    } else {
#pragma unroll
        for (int i = 0; i < W; ++i) o[i] = v[i];
    }
}

template <int kSt>
__global__ void k_materialize(BatchDev b, int64_t first, int64_t n, int32_t* out) {
    constexpr int W = kSt == kMD ? 2 : kSt == kSG ? 4 : kSt == kTC ? 16 : 8;
    const bool vec = (reinterpret_cast<uintptr_t>(out) & 15) == 0;
    const int ist = (b.flags & kFlagTCFromTP) ? kTP : kTL;  // track candidates: two tracklets or two triplets
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int o = (int)(first + k);
        int32_t v[W];
        if constexpr (kSt == kMD) {
            put_md(b, o, v);
        } else if constexpr (kSt == kSG) {
            put_sg(b, o, v);
        } else if constexpr (kSt == kTC) {
            put_tl(b, ist, OI(b, kTC, o), v);
            put_tl(b, ist, OJ(b, kTC, o), v + 8);
        } else {
            put_tl(b, kSt, o, v);
        }
        store_row<W>(out + (int64_t)W * k, v, vec);
    }
}

// The object graph of stage st for objects [first, first + n) of one event:
// constituents as indices into the event's lists of the stage below (hits:
// their position in the event's input order), the inner lower module within
// the event, and the floats the stage keeps per object.  lo_first: the
// event's first object of the stage below (its first input hit for
// mini-doublets); gm0: the event's first global module.
__global__ void k_links(BatchDev b, int st, int64_t first, int64_t n, int64_t lo_first, int64_t gm0, int32_t* links,
                        int32_t* module, float* vals) {
    const int nf = b.obj[st].nf;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t o = first + k;
        int64_t a = OI(b, st, o), c = OJ(b, st, o);
        if (st == kMD) {  // sorted hit positions -> input hits
            a = AT(b.hit_perm, a, H(b));
            c = AT(b.hit_perm, c, H(b));
        }
        if (links) {
            links[2 * k] = (int32_t)(a - lo_first);
            links[2 * k + 1] = (int32_t)(c - lo_first);
        }
        if (module) module[k] = (int32_t)(OG(b, st, o) - gm0);
        if (vals)
            for (int f = 0; f < nf; ++f) vals[k * nf + f] = OF(b, st, f, o);
    }
}

// the host libm's float functions as the chain evaluates them, on the float
// bit patterns start .. start + n - 1 (the self-check of the libm tables)
__global__ void k_libm_eval(int fn, uint32_t start, int64_t n, float* out) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const float x = __uint_as_float(start + (uint32_t)k);
        float v;
        switch (fn) {
            case kLmAsin: v = g_asin(x); break;
            case kLmAtan: v = g_atan(x); break;
            case kLmSin: v = g_sin(x); break;
            case kLmCos: v = g_cos(x); break;
            default: v = g_tan(x); break;
        }
        out[k] = v;
    }
}

unsigned grid_for(int64_t n, int threads, int cap_blocks) {
    int64_t g = (n + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > cap_blocks) g = cap_blocks;
    return (unsigned)g;
}

inline void rec_event(cudaEvent_t e, cudaStream_t s) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(s, &st);
    if (st == cudaStreamCaptureStatusActive) cudaEventRecordWithFlags(e, s, cudaEventRecordExternal);
    else cudaEventRecord(e, s);
}

void scan_h(const BatchDev& b, int64_t* data, const int64_t* n_ptr, int64_t cap, cudaStream_t s, Hooks* h) {
    scan(b, data, n_ptr, cap, s);
    if (h) h->launches += 3;
}

int enum_grid(const BatchDev& b, int st) { return b.enum_grid[st] > 0 ? b.enum_grid[st] : 8; }

template <class F>
void enum_and_group(const BatchDev& b, cudaStream_t s, Hooks* h, bool layer_counters = true) {
    constexpr int st = F::kSt;
    const int64_t* ninner_ptr = nullptr;
    switch (st) {
        case kMD: ninner_ptr = b.n_gm_dev; break;
        case kSG: ninner_ptr = b.obj[kMD].mod_cnt + b.n_gm; break;
        case kTL:
        case kTP: ninner_ptr = b.obj[kSG].mod_cnt + b.n_gm; break;
        default: ninner_ptr = ((b.flags & kFlagTCFromTP) ? b.obj[kTP] : b.obj[kTL]).mod_cnt + b.n_gm;
    }
    scan_h(b, b.cand[st], ninner_ptr, b.cand_cap[st], s, h);
    k_cand_buckets<<<b.n_sm * 8, 256, 0, s>>>(b, st);
    if (h) h->launches += 1;
    if (h && h->timed) rec_event(h->enum_start[st], s);
    k_enum<F><<<b.n_sm * enum_grid(b, st), kEnumThreads, 0, s>>>(b);
    if (h && h->timed) rec_event(h->enum_stop[st], s);
    if (layer_counters) k_obj_counters<<<grid_for(b.n_gm, 256, b.n_sm * 16), 256, 0, s>>>(b, st);
    scan_h(b, b.obj[st].mod_cnt, b.n_gm_dev, b.n_gm, s, h);
    k_scatter<<<b.n_sm * 8, 256, 0, s>>>(b, st);
    if (h) h->launches += layer_counters ? 3 : 2;
}

// device-to-device copies of 4-byte words (job blockIdx.y), 16 bytes at a
// time where both buffers are 16-byte aligned
__global__ void __launch_bounds__(256) k_copy_words(CopyJobs j) {
    const int q = blockIdx.y;
    if (q >= j.count) return;
    const uint32_t* __restrict__ src = j.src[q];
    uint32_t* __restrict__ dst = j.dst[q];
    const int64_t n = j.n[q];
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t done = 0;
    if (((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15u) == 0) {
        const int64_t n4 = n / 4;
        const uint4* s4 = reinterpret_cast<const uint4*>(src);
        uint4* d4 = reinterpret_cast<uint4*>(dst);
        for (int64_t i = t; i < n4; i += stride) d4[i] = __ldg(s4 + i);
        done = n4 * 4;
    }
    for (int64_t i = done + t; i < n; i += stride) dst[i] = __ldg(src + i);
}

}  // namespace

void launch_ingest(const BatchDev& b, cudaStream_t s, Hooks* h) {
    const unsigned g = grid_for(b.n_hit_cap, 256, b.n_sm * 16);
    k_hit_map<<<g, 256, 0, s>>>(b);
    scan_h(b, b.mod_hit, b.n_gm_dev, b.n_gm, s, h);
    k_hit_perm<<<g, 256, 0, s>>>(b);
    k_hit_scatter<<<g, 256, 0, s>>>(b);
    if (h) h->launches += 3;
}

void launch_md(const BatchDev& b, cudaStream_t s, Hooks* h) {
    k_md_count<<<grid_for(b.n_gm, 256, b.n_sm * 16), 256, 0, s>>>(b);
    if (h) h->launches += 1;
    enum_and_group<MDStage>(b, s, h);
}

void launch_sg(const BatchDev& b, cudaStream_t s, Hooks* h) {
    k_md_pack<<<b.n_sm * 8, 256, 0, s>>>(b);
    if (h) h->launches += 1;
    if (b.flags & kFlagSGLayers) {
        // Event.cc:793-821 increments no per-layer counter
        k_sg_count_layers<<<b.n_sm * 8, 256, 0, s>>>(b);
        if (h) h->launches += 1;
        enum_and_group<SGLayerStage>(b, s, h, false);
        return;
    }
    k_conn_sum<<<grid_for(b.n_gm, 256, b.n_sm * 16), 256, 0, s>>>(b, kMD, kSG);
    k_sg_count<<<b.n_sm * 8, 256, 0, s>>>(b);
    k_sg_olist_count<<<grid_for(b.n_gm, 256, b.n_sm * 16), 256, 0, s>>>(b);
    scan_h(b, b.toff, b.n_gm_dev, b.n_gm, s, h);
    k_sg_olist_fill<<<grid_for(b.n_gm, 256, b.n_sm * 16), 256, 0, s>>>(b);
    scan_h(b, b.cand[kSG], b.obj[kMD].mod_cnt + b.n_gm, b.cand_cap[kSG], s, h);
    k_cand_buckets<<<b.n_sm * 8, 256, 0, s>>>(b, kSG);
    if (h) h->launches += 5;
    // first cuts -> survivor list -> whole algorithm (k_sg_enum_a, k_sg_b)
    if (h && h->timed) rec_event(h->enum_start[kSG], s);
    cudaMemsetAsync(b.n_kept, 0, sizeof(unsigned long long), s);
    cudaMemsetAsync(b.n_pb, 0, 2 * sizeof(unsigned long long), s);
    k_sg_enum_a<<<b.n_sm * enum_grid(b, kSG), kEnumThreads, 0, s>>>(b);
    k_sg_b<1><<<b.n_sm * enum_grid(b, kSG), kEnumThreads, 0, s>>>(b);
    k_sg_b<2><<<b.n_sm * enum_grid(b, kSG), kEnumThreads, 0, s>>>(b);
    if (h && h->timed) rec_event(h->enum_stop[kSG], s);
    k_obj_counters<<<grid_for(b.n_gm, 256, b.n_sm * 16), 256, 0, s>>>(b, kSG);
    scan_h(b, b.obj[kSG].mod_cnt, b.n_gm_dev, b.n_gm, s, h);
    k_scatter<<<b.n_sm * 8, 256, 0, s>>>(b, kSG);
    if (h) h->launches += 5;
}

// the join index of stage st's objects (segments or tracklets), keyed by
// mini-doublet; second = true builds the second index (triplets)
static void join_index(const BatchDev& b, int st, cudaStream_t s, Hooks* h, bool second = false) {
    int64_t* off = second ? b.joff2 : b.joff;
    cudaMemsetAsync(off, 0, (b.obj[kMD].cap + 1) * sizeof(int64_t), s);
    cudaMemsetAsync(second ? b.jcur2 : b.jcur, 0, b.obj[kMD].cap * sizeof(int32_t), s);
    k_join_count<<<b.n_sm * 8, 256, 0, s>>>(b, st, second);
    scan_h(b, off, b.obj[kMD].mod_cnt + b.n_gm, b.obj[kMD].cap, s, h);
    k_join_scatter<<<b.n_sm * 8, 256, 0, s>>>(b, st, second);
    if (h) h->launches += 2;
}

void launch_tl(const BatchDev& b, cudaStream_t s, Hooks* h) {
    // conn sums over segment counts serve the tracklet enumeration and the
    // triplet candidate counters (Event.cc:547-596 loops over the same lists)
    k_sg_pack<<<b.n_sm * 8, 256, 0, s>>>(b);
    k_conn_sum<<<grid_for(b.n_gm, 256, b.n_sm * 16), 256, 0, s>>>(b, kSG, kTP);
    if (b.flags & kFlagTLLayers) {
        k_tl_count_layers<<<b.n_sm * 8, 256, 0, s>>>(b);
    } else if (b.flags & kFlagTLNav) {
        join_index(b, kSG, s, h);  // segments by inner MD: the outward lists
        k_tl_count_nav<<<b.n_sm * 8, 256, 0, s>>>(b);
    } else {
        cudaMemsetAsync(b.eoff, 0, (b.n_gm + 1) * sizeof(int64_t), s);
        cudaMemsetAsync(b.ecur, 0, b.n_gm * sizeof(int32_t), s);
        k_tl_count<<<b.n_sm * 8, 256, 0, s>>>(b);
    }
    if (h) h->launches += 3;
    scan_h(b, b.cand[kTL], b.obj[kSG].mod_cnt + b.n_gm, b.cand_cap[kTL], s, h);
    k_cand_buckets<<<b.n_sm * 8, 256, 0, s>>>(b, kTL);
    if (h) h->launches += 1;
    // module-map candidates: the module-pair tiles (k_tl_enum_tiles)
    const bool tiles = !(b.flags & (kFlagTLLayers | kFlagTLNav));
    if (tiles) {
        k_tl_tile_count<<<grid_for(b.n_gm, 256, b.n_sm * 16), 256, 0, s>>>(b);
        scan_h(b, b.eoff, b.n_gm_dev, b.n_gm, s, h);
        scan_h(b, b.toff, b.n_gm_dev, b.n_gm, s, h);
        k_sg_end_scatter<<<b.n_sm * 8, 256, 0, s>>>(b);
        k_tile_map<<<grid_for(b.n_gm, 256, b.n_sm * 16), 256, 0, s>>>(b);
        if (h) h->launches += 3;
    }
    if (h && h->timed) rec_event(h->enum_start[kTL], s);
    // enumeration + phase A -> survivor list (-> the pre-filter -> kept list)
    // -> phase B1 -> phase B2
    cudaMemsetAsync(b.n_kept, 0, sizeof(unsigned long long), s);
    if (tiles) k_tl_enum_tiles<<<b.n_sm * enum_grid(b, kTL), kEnumThreads, 0, s>>>(b);
    else k_tl_enum_a<<<b.n_sm * enum_grid(b, kTL), kEnumThreads, 0, s>>>(b);
    if (h && h->timed) rec_event(h->tl_mid[0], s);
    // the list phase B1 reads: the enumeration's, the pre-filter's kept
    // entries, then what phase B2's single-precision filter leaves of it (not
    // with DefaultNm1, whose phase B2 keeps what fails the deltaBeta cut)
    int4* list = b.passa;
    unsigned long long* count = b.n_kept;
    const bool mlp = (b.flags & kFlagMLP) != 0;
    if (mlp) {
        cudaMemsetAsync(b.n_kept2, 0, sizeof(unsigned long long), s);
        k_tl_prefilter<<<b.n_sm * kPfCtasPerSm, kMlpTile, 0, s>>>(b);
        list = b.kept;
        count = b.n_kept2;
    }
    if (h && h->timed) rec_event(h->tl_mid[1], s);
    const bool filt = !(b.flags & (kFlagTLNm1 | kFlagNoB2Filter));
    if (filt) {
        cudaMemsetAsync(b.n_keptf, 0, sizeof(unsigned long long), s);
        cudaMemsetAsync(b.n_pb, 0, 2 * sizeof(unsigned long long), s);
        k_tl_b2f<0><<<b.n_sm * enum_grid(b, kTL), kEnumThreads, 0, s>>>(b, list, count);
        k_tl_b2f<1><<<b.n_sm * enum_grid(b, kTL), kEnumThreads, 0, s>>>(b, nullptr, nullptr);
        k_tl_b2f<2><<<b.n_sm * enum_grid(b, kTL), kEnumThreads, 0, s>>>(b, nullptr, nullptr);
        list = b.passf;
        count = b.n_keptf;
    }
    if (h && h->timed) rec_event(h->tl_mid[2], s);
    cudaMemsetAsync(b.n_pb, 0, 2 * sizeof(unsigned long long), s);
    k_tl_b1<<<b.n_sm * enum_grid(b, kTL), kEnumThreads, 0, s>>>(b, list, count);
    k_tl_b2<kB2BBBB><<<b.n_sm * enum_grid(b, kTL), kEnumThreads, 0, s>>>(b);
    k_tl_b2<kB2Others><<<b.n_sm * enum_grid(b, kTL), kEnumThreads, 0, s>>>(b);
    if (h) h->launches += 3 + (mlp ? 1 : 0) + (filt ? 3 : 0);
    if (h && h->timed) rec_event(h->enum_stop[kTL], s);
    k_obj_counters<<<grid_for(b.n_gm, 256, b.n_sm * 16), 256, 0, s>>>(b, kTL);
    scan_h(b, b.obj[kTL].mod_cnt, b.n_gm_dev, b.n_gm, s, h);
    k_scatter<<<b.n_sm * 8, 256, 0, s>>>(b, kTL);
    if (h) h->launches += 3;
}


void launch_tp(const BatchDev& b, cudaStream_t s, Hooks* h) {
    join_index(b, kSG, s, h);
    k_tp_count<<<b.n_sm * 8, 256, 0, s>>>(b);
    if (h) h->launches += 1;
    enum_and_group<TPStage>(b, s, h);
}

void launch_tc(const BatchDev& b, cudaStream_t s, Hooks* h) {
    if (b.flags & kFlagTCFromTP) {
        const bool map = !(b.flags & kFlagSGLayers);
        if (map) {
            join_index(b, kSG, s, h);        // segments by inner MD
            join_index(b, kTP, s, h, true);  // triplets by innermost MD
        }
        k_conn_sum<<<grid_for(b.n_gm, 256, b.n_sm * 16), 256, 0, s>>>(b, kTP, -1);
        k_tc_count_tp<<<b.n_sm * 8, 256, 0, s>>>(b);
        if (h) h->launches += 2;
        if (map) enum_and_group<TCTPMapStage>(b, s, h);
        else enum_and_group<TCTPStage>(b, s, h);
        return;
    }
    join_index(b, kTL, s, h);
    if (b.flags & kFlagTCFromTL) {
        k_conn_sum<<<grid_for(b.n_gm, 256, b.n_sm * 16), 256, 0, s>>>(b, kTL, -1);
        k_tc_count_tl<<<b.n_sm * 8, 256, 0, s>>>(b);
    } else {
        k_tc_count<<<b.n_sm * 8, 256, 0, s>>>(b);
        k_tc_cand_counter<<<grid_for(b.n_ev, 128, 1024), 128, 0, s>>>(b);
    }
    if (h) h->launches += 2;
    enum_and_group<TCStage>(b, s, h);
}

// ------------------------------------------------------------------ self-check
// The float-float fast paths of the cut arithmetic against the double
// evaluation they stand for: every input whose fast path succeeds must give
// the same float bit for bit.  Inputs are either all float bit patterns of a
// range (unary functions) or hashed pseudo-random values.
__device__ __forceinline__ float hash_log(unsigned long long h, float lo_exp, float hi_exp) {
    const float u = (float)((h >> 11) & 0xffffffull) * (1.f / 16777216.f);
    const float m = 1.f + (float)((h >> 35) & 0x7fffffull) * (1.f / 8388608.f);
    return ldexpf(m, (int)floorf(lo_exp + u * (hi_exp - lo_exp)));
}
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void k_math_check(int fn, int exhaustive, unsigned long long start, long long n, unsigned long long seed,
                             unsigned long long* out) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float a = 0.f, b = 0.f, c = 0.f, d = 0.f;
        if (exhaustive) {
            a = __uint_as_float((unsigned)(start + (unsigned long long)i));
        } else {
            const unsigned long long h1 = mix64(seed * 0x9E3779B97F4A7C15ull + (unsigned long long)i);
            const unsigned long long h2 = mix64(h1 + 0x632BE59BD9B4E019ull);
            const unsigned long long h3 = mix64(h2 + 0x632BE59BD9B4E019ull);
            const unsigned long long h4 = mix64(h3 + 0x632BE59BD9B4E019ull);
            const float sa = (h1 & 1) ? -1.f : 1.f, sb = (h2 & 1) ? -1.f : 1.f;
            switch (fn) {
                case 1: case 2: case 16: case 20:  // coordinates: magnitudes 2^-12..2^9, a fraction on axes and diagonals
                    a = sa * hash_log(h1, -12.f, 9.f);
                    b = sb * hash_log(h2, -12.f, 9.f);
                    if ((h3 & 15) == 0) b = sb * fabsf(a) * (1.f + (float)((h4 >> 40) & 0xff) * 0x1p-20f);
                    if ((h3 & 15) == 1) b = a * 0x1p-20f;
                    break;
                case 3:
                    a = sa * hash_log(h1, -20.f, 4.f);
                    b = hash_log(h2, -40.f, 6.f);
                    break;
                case 7:  // (dr k, beta): |beta| below 0.5
                    a = hash_log(h1, -8.f, 1.f);
                    b = sa * hash_log(h2, -24.f, -1.f);
                    break;
                case 8: case 15:  // (rtOut - rtIn, r3/rt)
                    a = hash_log(h1, -10.f, 8.f);
                    b = 1.f + hash_log(h2, -12.f, 2.f);
                    break;
                case 9:  // (head, t)
                    a = hash_log(h1, -30.f, 2.f);
                    b = hash_log(h2, -16.f, 2.f);
                    break;
                case 13:  // coordinate differences
                    a = sa * hash_log(h1, -12.f, 8.f);
                    b = sb * hash_log(h2, -12.f, 8.f);
                    break;
                case 14:  // (dphi, dz)
                    a = sa * hash_log(h1, -24.f, 1.f);
                    b = sb * hash_log(h2, -8.f, 4.f);
                    break;
                case 4:
                    a = hash_log(h1, -10.f, 1.f);
                    b = hash_log(h2, -14.f, 1.f);
                    c = hash_log(h3, -14.f, 1.f);
                    d = (h4 & 3) == 0 ? 0.f : hash_log(h4, -14.f, 3.f);
                    break;
                default:
                    a = sa * hash_log(h1, -30.f, 0.f);
            }
        }
        float f = 0.f, ref = 0.f;
        bool ok = false;
        switch (fn) {
            case 0: ok = f_asin_fast(a, f); if (ok) ref = f_asin_d(a); break;
            case 1: ok = atan2_fast(a, b, f); if (ok) ref = atan2_d(a, b); break;
            case 2: {
                f = phi_of(a, b);
                ref = phi_of_d(a, b);
                ok = true;
                break;
            }
            case 3: ok = add_dsqrt_fast(a, b, f); if (ok) ref = add_dsqrt_d(a, b); break;
            case 4: ok = add_dsqrt3_fast(a, b, c, d, f); if (ok) ref = add_dsqrt3_d(a, b, c, d); break;
            case 5: ok = phi_mpi_pi_fast(a, f); if (ok) ref = phi_mpi_pi_d(a); break;
            case 6: ok = add_pi_fast(a, f); if (ok) ref = (float)(kPi + (double)a); break;
            case 7: ok = pt_from_fast(a, b, f); if (ok) ref = pt_from_d(a, b); break;
            case 8: ok = muls_fast(a, b, true, f); if (ok) ref = muls_d(a, b, true); break;
            case 9: ok = add_quarter_sq_fast(a, b, f); if (ok) ref = add_quarter_sq_d(a, b); break;
            case 10: ok = f_sincos_fast(a, 0, f); if (ok) ref = f_sin_d(a); break;
            case 11: ok = f_sincos_fast(a, 1, f); if (ok) ref = f_cos_d(a); break;
            case 12: ok = f_atan_fast(a, f); if (ok) ref = f_atan_d(a); break;
            case 13: ok = hypot_fast(a, b, f); if (ok) ref = hypot_d(a, b); break;
            case 14: ok = times15_over_fast(a, b, f); if (ok) ref = times15_over_d(a, b); break;
            case 15: ok = muls_fast(a, b, false, f); if (ok) ref = muls_d(a, b, false); break;
            case 16: ok = phi_approx(a, b, f); if (ok) ref = phi_of(a, b); break;
            case 17: ok = fabsf(a) <= kSinAlphaMax; if (ok) { f = asinf(a); ref = f_asin(a); } break;
            case 18: ok = f_tan_fast(a, false, f); if (ok) ref = f_tan(a); break;
            case 19: ok = f_tan_fast(a, true, f); if (ok) ref = f_tan_over_d(a); break;
            case 20: ok = phi_fast(a, b, f); if (ok) ref = phi_of(a, b); break;
            default: break;
        }
        // functions 16, 17 and 20 are the approximations of phase B1: within
        // 2e-6 (16, 17) and 2.5e-6 (20) of the exact value (directions compared
        // modulo 2 pi); the others must match the double evaluation bit for bit
        const bool approx = fn == 16 || fn == 17 || fn == 20;
        const float tol = fn == 20 ? 2.5e-6f : 2e-6f;
        const bool bad = approx ? ok && !(fabsf(fn == 17 ? f - ref : wrap_approx(f - ref)) <= tol)
                                : ok && __float_as_uint(f) != __float_as_uint(ref) && !(isnan(f) && isnan(ref));
        const unsigned m_ok = __ballot_sync(__activemask(), ok);
        const unsigned m_bad = __ballot_sync(__activemask(), bad);
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(out + 0, (unsigned long long)__popc(m_ok));
            if (m_bad) atomicAdd(out + 1, (unsigned long long)__popc(m_bad));
        }
        if (bad && atomicCAS(out + 2, 0ull, 1ull) == 0ull) {
            out[3] = __float_as_uint(a);
            out[4] = __float_as_uint(b);
            out[5] = __float_as_uint(c);
            out[6] = __float_as_uint(f);
            out[7] = __float_as_uint(ref);
        }
    }
}

void launch_math_check(int fn, int exhaustive, unsigned long long start, long long n, unsigned long long seed,
                       unsigned long long* out, int n_sm, cudaStream_t s) {
    k_math_check<<<n_sm * 16, 256, 0, s>>>(fn, exhaustive, start, n, seed, out);
}

void launch_tl_collect(const BatchDev& b, const MlpCollect& c, cudaStream_t s) {
    // the bucket table holds the last stage that ran: rebuild the tracklet one
    k_cand_buckets<<<b.n_sm * 8, 256, 0, s>>>(b, kTL);
    k_tl_collect<<<b.n_sm * 8, 256, 0, s>>>(b, c);
}

void launch_tl_b2q_check(const BatchDev& b, unsigned long long* out, cudaStream_t s) {
    k_tl_b2q_check<<<b.n_sm * 8, 256, 0, s>>>(b, out);
}

void launch_tl_quick_check(const BatchDev& b, unsigned long long* out, cudaStream_t s) {
    k_cand_buckets<<<b.n_sm * 8, 256, 0, s>>>(b, kTL);
    k_tl_quick_check<<<b.n_sm * 8, 256, 0, s>>>(b, out);
}

// the final cut variables of tracklets [first, first + n) (kTLVarN floats
// each, NaN for a pair phase A does not accept): phase A for the algorithm
// and the factors, then phase B2 with its record.  The reference's BBEE
// algorithm records none of them (Tracklet.cc:1540-2016 only resets them to
// -999 at its start), so BBEE tracklets report -999 as the reference does.
__global__ void k_tl_vars(BatchDev b, int64_t first, int64_t n, float* out) {
    const bool nm1 = (b.flags & kFlagTLNm1) != 0;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t o = first + k;
        const SGV S = load_sgv(b.sgpack, OI(b, kTL, o));
        const SGV T = load_sgv(b.sgpack, OJ(b, kTL, o));
        float cut, muls, rec[kTLVarN];
#pragma unroll
        for (int j = 0; j < kTLVarN; ++j) rec[j] = __int_as_float(0x7fc00000);
        const int algo = tl_phaseA(S, T, cut, muls);
        if (algo == kAlgoBBEE) {
#pragma unroll
            for (int j = 0; j < kTLVarN; ++j) rec[j] = -999.f;
        } else if (algo != kAlgoNone) {
            (void)tl_phaseB2_sgv<kB2All>(algo, S, T, muls, nm1, rec);
        }
#pragma unroll
        for (int j = 0; j < kTLVarN; ++j) out[k * kTLVarN + j] = rec[j];
    }
}

void launch_tl_vars(const BatchDev& b, int64_t first, int64_t n, float* out, cudaStream_t s) {
    if (n <= 0) return;
    k_tl_vars<<<grid_for(n, 128, b.n_sm * 8), 128, 0, s>>>(b, first, n, out);
}

void launch_links(const BatchDev& b, int st, int64_t first, int64_t n, int64_t lo_first, int64_t gm0, int32_t* links,
                  int32_t* module, float* vals, cudaStream_t s) {
    if (n <= 0) return;
    k_links<<<grid_for(n, 256, b.n_sm * 16), 256, 0, s>>>(b, st, first, n, lo_first, gm0, links, module, vals);
}

cudaError_t set_libm_tables(const LibmTab* t) { return cudaMemcpyToSymbol(c_libm, t, sizeof(LibmTab) * kLmCount); }

void launch_libm_eval(int fn, uint32_t start, int64_t n, float* out, int n_sm, cudaStream_t s) {
    if (n <= 0) return;
    k_libm_eval<<<grid_for(n, 256, n_sm * 16), 256, 0, s>>>(fn, start, n, out);
}

void launch_copy_words(const CopyJobs& j, int n_sm, cudaStream_t s) {
    if (j.count <= 0) return;
    k_copy_words<<<dim3((unsigned)(n_sm * 2), (unsigned)j.count), 256, 0, s>>>(j);
}

void launch_materialize(const BatchDev& b, int st, int64_t first, int64_t n, int32_t* out, cudaStream_t s) {
    if (n <= 0) return;
    const unsigned g = grid_for(n, 256, b.n_sm * 16);
    switch (st) {
        case kMD: k_materialize<kMD><<<g, 256, 0, s>>>(b, first, n, out); break;
        case kSG: k_materialize<kSG><<<g, 256, 0, s>>>(b, first, n, out); break;
        case kTL: k_materialize<kTL><<<g, 256, 0, s>>>(b, first, n, out); break;
        case kTP: k_materialize<kTP><<<g, 256, 0, s>>>(b, first, n, out); break;
        default: k_materialize<kTC><<<g, 256, 0, s>>>(b, first, n, out);
    }
}

}  // namespace sdlg
