// Host side of the GB300 segment-linking chain: context, geometry tables,
// device buffers and the C ABI declared in include/sdl_gpu.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/sdl_gpu.h"
#include "sdl_kernels.h"
#include "sdl_mlp.h"

using namespace sdlg;

namespace {

// ------------------------------------------------------------------ detId decoding (Module.cc:159-358)
struct Decoded {
    uint16_t subdet, side, layer, rod, ring, module;
    bool lower, inverted;
    uint8_t type, ltype;
    uint32_t partner;
};

Decoded decode(uint32_t d) {
    Decoded m{};
    m.subdet = (d >> 25) & 7;
    const bool ec = m.subdet == kEndcap, br = m.subdet == kBarrel;
    m.side = ec ? (d >> 23) & 3 : br ? (d >> 18) & 3 : 0;
    m.layer = ec ? (d >> 18) & 7 : br ? (d >> 20) & 7 : 0;
    m.rod = br ? (d >> 10) & 127 : 0;
    m.ring = ec ? (d >> 12) & 15 : 0;
    m.module = (d >> 2) & 127;
    bool inv = false;
    if (ec) inv = m.side == kNegZ ? (m.module % 2 == 1) : m.side == kPosZ ? (m.module % 2 == 0) : false;
    else if (br) {
        if (m.side == kCenter) inv = m.layer <= 3 ? (m.module % 2 == 1) : (m.module % 2 == 0);
        else if (m.side == kNegZ || m.side == kPosZ) inv = m.layer <= 2 ? (m.module % 2 == 1) : m.layer == 3 ? (m.module % 2 == 0) : false;
    }
    m.inverted = inv;
    m.lower = inv ? !(d & 1) : (d & 1);
    m.partner = m.lower ? (inv ? d - 1 : d + 1) : (inv ? d + 1 : d - 1);
    if (br) m.type = m.layer <= 3 ? kPS : kTwoS;
    else m.type = (m.layer <= 2 ? m.ring <= 10 : m.ring <= 7) ? kPS : kTwoS;
    m.ltype = m.type == kTwoS ? kStrip : (inv ? (m.lower ? kStrip : kPixel) : (m.lower ? kPixel : kStrip));
    return m;
}

bool valid_module(const Decoded& m) {
    if (m.subdet == kBarrel) return m.layer >= 1 && m.layer <= 6;
    if (m.subdet == kEndcap) return m.layer >= 1 && m.layer <= 5 && m.ring >= 1 && m.ring <= 15;
    return false;
}

// MiniDoublet.cc:1242-1332 (sensor gap of a module)
float gap_size(const Decoded& m) {
    const bool b = m.subdet == kBarrel;
    const bool tighter = (b && m.side != kCenter && m.layer == 3) || (b && m.side == kNegZ && m.layer == 2 && m.rod > 5) ||
                         (b && m.side == kPosZ && m.layer == 2 && m.rod < 8) || (b && m.side == kNegZ && m.layer == 1 && m.rod > 9) ||
                         (b && m.side == kPosZ && m.layer == 1 && m.rod < 4);
    static const float flat[6] = {0.26f, 0.16f, 0.16f, 0.18f, 0.18f, 0.18f};
    const int iL = m.layer - 1;
    if (b && m.side == kCenter) return flat[iL];
    if (tighter) return 0.26f;
    if (m.subdet == kEndcap) {
        const int lim = iL <= 1 ? 10 : iL <= 3 ? 8 : 9;
        return (m.ring - 1) < lim ? 0.4f : 0.18f;
    }
    return 0.4f;
}

struct HostGeometry {
    std::map<uint32_t, std::pair<float, float>> tilted;  // drdz, slope
    std::map<uint32_t, std::pair<float, float>> endcap;  // slope lower, centroid phi (7th column)
    std::map<uint32_t, std::vector<uint32_t>> conn;
};

template <class T>
struct DevBuf {
    T* p = nullptr;
    int64_t n = 0;
};

}  // namespace

struct sdlg_ctx {
    int device = 0;
    int n_sm = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    bool have_geo = false;
    HostGeometry hg;
    std::vector<uint32_t> detids;  // sorted module table
    std::vector<ModDev> mods;
    std::vector<int32_t> conn_off, conn_idx;
    // device geometry
    uint32_t* d_detid = nullptr;
    ModDev* d_mod = nullptr;
    int32_t* d_conn_off = nullptr;
    int32_t* d_conn_idx = nullptr;
    std::vector<int32_t> slot_run;
    int32_t* d_slot_run = nullptr;
    // learned tracklet pre-filter: parameters, packed weights, training state
    struct {
        float* params = nullptr;        // FP32 master parameters (kMlpParams)
        unsigned char* pack = nullptr;  // packed inference weights + threshold (kPackBytes)
        MlpStats* stats = nullptr;
        float *grad = nullptr, *m = nullptr, *v = nullptr;
        double* loss = nullptr;
        unsigned int* status = nullptr;
        unsigned long long* found = nullptr;
        int64_t adam_t = 0;
        float thr = 0.f;
        bool have = false;
        float *x = nullptr, *y = nullptr;  // training samples
        int64_t n = 0, cap = 0;
        int32_t* order = nullptr;
        int64_t order_cap = 0;
    } mlp;
    // batch
    int64_t n_ev = 0, n_hit = 0;
    std::vector<int64_t> ev_off;
    BatchDev b{};
    std::vector<void*> allocs;  // batch allocations
    int64_t cap_hit = 0, cap_ev = 0;
    int64_t cap_obj[kNumStages] = {0, 0, 0, 0, 0};
    int64_t cap_kept = 0;  // tracklet candidates the pre-filter may keep per run
    int64_t cap_init[kNumStages + 1] = {0, 0, 0, 0, 0, 0};  // starting capacities (0: from the hit count)
    int tune_task[kNumStages] = {0, 0, 0, 0, 0};  // tuned launch shapes (0: default)
    int tune_grid[kNumStages] = {0, 0, 0, 0, 0};
    bool buffers_ok = false;
    // pinned staging
    void* pinned = nullptr;
    int64_t pinned_bytes = 0;
    // device scratch for results on their way to host memory, two buffers
    // (kept between calls: allocating a gigabyte afresh costs more than
    // copying it); the synchronous readbacks use the first
    void* scratch[2] = {nullptr, nullptr};
    int64_t scratch_bytes[2] = {0, 0};
    // asynchronous readback: a kernel on the gather stream writes the tuples
    // into the next scratch buffer once the run that made the objects is
    // complete (ev_mat) and that buffer's previous copy has read it
    // (ev_copy[k]), then the copy stream copies them to the host.  ev_read:
    // the objects have been read, so a new run may overwrite them.  The
    // gathering never waits behind the previous readback's copy.
    cudaStream_t copy_stream = nullptr, gather_stream = nullptr;
    cudaEvent_t ev_mat = nullptr, ev_read = nullptr, ev_copy[2] = {nullptr, nullptr};
    bool copy_pending[2] = {false, false}, read_pending = false;
    int next_scratch = 0;
    int64_t* h_small = nullptr;   // pinned: n_rec[5], status
    // the next batch, copied to the device while a run may still be going
    // (sdlg_stage_events) and installed by the next run from the hits: one
    // device allocation of x, y, z, idx, detid (hits each) and the offsets
    // (events + 1), copied on its own stream (ev_in: the copy is done;
    // ev_used: the install's copies have read it); a batch that does not fit
    // the current buffers waits on the host (host_*) for the next run
    struct {
        char* dev = nullptr;
        int64_t hits = 0, evs = 0;  // capacity of dev
        int64_t* h_off = nullptr;   // pinned offsets on their way to dev
        int64_t h_off_cap = 0;
        int64_t n_ev = 0, n_hit = 0;
        std::vector<int64_t> ev_off;
        bool pending = false, on_host = false, used_pending = false;
        std::vector<float> host_f[3];
        std::vector<int32_t> host_idx;
        std::vector<uint32_t> host_det;
        cudaStream_t stream = nullptr;
        cudaEvent_t ev_in = nullptr, ev_used = nullptr;
    } stage;
    // graph
    cudaGraphExec_t graph = nullptr;
    int graph_stop = -1, graph_flags = -1;
    // timing
    cudaEvent_t ev[8];
    Hooks hooks;
    int launches_per_run = 0;
    int last_stop = -1, last_flags = 0;
    bool ran = false;
};

namespace {

int fail(sdlg_ctx* c, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    return code;
}

#define CK(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) return fail(ctx, SDLG_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

int set_events_impl(sdlg_ctx* ctx, int64_t n_events, const int64_t* ev_off, const float* x, const float* y, const float* z,
                    const int32_t* idx, const uint32_t* detid);

// a new run (or freed buffers) must not overwrite objects that an
// asynchronous readback still reads: its kernel runs on the copy stream
void wait_readback(sdlg_ctx* ctx) {
    if (!ctx->read_pending) return;
    cudaStreamWaitEvent(ctx->stream, ctx->ev_read, 0);
    ctx->read_pending = false;
}

void free_batch(sdlg_ctx* ctx) {
    if (ctx->read_pending) {
        cudaStreamSynchronize(ctx->gather_stream);
        ctx->read_pending = false;
    }
    if (ctx->graph) {
        cudaGraphExecDestroy(ctx->graph);
        ctx->graph = nullptr;
    }
    for (void* p : ctx->allocs) cudaFree(p);
    ctx->allocs.clear();
    ctx->buffers_ok = false;
}

// ctx->scratch[k] grown to at least `bytes` (with a quarter of headroom)
int ensure_scratch(sdlg_ctx* ctx, int k, size_t bytes, void** p) {
    if (ctx->scratch_bytes[k] < (int64_t)bytes) {
        if (ctx->scratch[k]) {
            cudaStreamSynchronize(ctx->stream);
            cudaStreamSynchronize(ctx->gather_stream);
            cudaStreamSynchronize(ctx->copy_stream);
            ctx->copy_pending[0] = ctx->copy_pending[1] = false;
            ctx->read_pending = false;
            cudaFree(ctx->scratch[k]);
        }
        ctx->scratch[k] = nullptr;
        ctx->scratch_bytes[k] = 0;
        const size_t want = bytes + bytes / 4 + 256;
        cudaError_t e = cudaMalloc(&ctx->scratch[k], want);
        if (e != cudaSuccess) return fail(ctx, SDLG_ERR_CAPACITY, "cudaMalloc(%zu): %s", want, cudaGetErrorString(e));
        ctx->scratch_bytes[k] = (int64_t)want;
    }
    *p = ctx->scratch[k];
    return SDLG_OK;
}

template <class T>
int dalloc(sdlg_ctx* ctx, T** p, int64_t n) {
    void* q = nullptr;
    const size_t bytes = (size_t)std::max<int64_t>(n, 1) * sizeof(T);
    cudaError_t e = cudaMalloc(&q, bytes);
    if (e != cudaSuccess) return fail(ctx, SDLG_ERR_CAPACITY, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
    ctx->allocs.push_back(q);
    *p = static_cast<T*>(q);
    return SDLG_OK;
}

int build_module_table(sdlg_ctx* ctx, const std::vector<uint32_t>& extra) {
    std::vector<uint32_t> ids;
    for (auto& kv : ctx->hg.tilted) ids.push_back(kv.first);
    for (auto& kv : ctx->hg.endcap) ids.push_back(kv.first);
    for (auto& kv : ctx->hg.conn) {
        ids.push_back(kv.first);
        for (uint32_t d : kv.second) ids.push_back(d);
    }
    ids.insert(ids.end(), ctx->detids.begin(), ctx->detids.end());
    ids.insert(ids.end(), extra.begin(), extra.end());
    std::vector<uint32_t> valid;
    for (uint32_t d : ids) {
        const Decoded m = decode(d);
        if (!valid_module(m)) continue;
        valid.push_back(d);
        valid.push_back(m.partner);
    }
    std::sort(valid.begin(), valid.end());
    valid.erase(std::unique(valid.begin(), valid.end()), valid.end());
    ctx->detids = valid;
    const int n = (int)valid.size();
    auto index_of = [&](uint32_t d) -> int {
        auto it = std::lower_bound(valid.begin(), valid.end(), d);
        return (it != valid.end() && *it == d) ? (int)(it - valid.begin()) : -1;
    };
    auto tget = [&](uint32_t d, int k) -> float {
        auto it = ctx->hg.tilted.find(d);
        return it == ctx->hg.tilted.end() ? 0.f : (k ? it->second.second : it->second.first);
    };
    auto eget = [&](uint32_t d, int k) -> float {
        auto it = ctx->hg.endcap.find(d);
        return it == ctx->hg.endcap.end() ? 0.f : (k ? it->second.second : it->second.first);
    };
    ctx->mods.assign(n, ModDev{});
    for (int i = 0; i < n; ++i) {
        const uint32_t d = valid[i];
        const Decoded m = decode(d);
        ModDev& o = ctx->mods[i];
        o.detid = d;
        o.partner = index_of(m.partner);
        o.subdet = (uint8_t)m.subdet; o.side = (uint8_t)m.side; o.layer = (uint8_t)m.layer; o.ring = (uint8_t)m.ring;
        o.rod = (uint8_t)m.rod; o.module = (uint8_t)m.module; o.lower = m.lower; o.inverted = m.inverted;
        o.type = m.type; o.ltype = m.ltype;
        o.layer_slot = (uint8_t)(m.subdet == kBarrel ? m.layer - 1 : 6 + m.layer - 1);
        o.gap = gap_size(m);
        // the strip sensor of the pair keys the tilted / endcap lookups (MiniDoublet.cc:781,1040-1053)
        const uint32_t strip = m.ltype == kPixel ? m.partner : d;
        o.drdz_s = tget(strip, 0);
        o.slope_s = m.subdet == kEndcap ? eget(strip, 0) : tget(strip, 1);
        // GeometryUtil.cc:12-16: the edge offset along this sensor's centroid phi
        const float phi = eget(d, 1);
        o.edge_x = (float)(2.5 * std::cos((double)phi));
        o.edge_y = (float)(2.5 * std::sin((double)phi));
        // MiniDoublet.cc:781-783 / Segment.cc:920-928: the tilt term depends on the module only
        const float half_pitch_drdz = 0.5f * 0.15f * o.drdz_s;
        const float one_plus = 1.f + o.drdz_s * o.drdz_s;
        o.tilt = (float)((double)half_pitch_drdz / std::sqrt((double)one_plus) / (double)o.gap);
        // the strip shift's module-only terms (MiniDoublet.cc:1260-1332), with
        // the host's float functions as the reference calls them
        o.sh_angle_b = m.subdet == kEndcap ? (float)(M_PI / 2.) : std::atan(o.drdz_s);
        const float abs_atan_slope = (o.slope_s != kSdlInf) ? std::fabs(std::atan(o.slope_s)) : (float)(M_PI / 2);
        const float angle_m[4] = {abs_atan_slope, (float)(M_PI - (double)abs_atan_slope),
                                  (float)(M_PI + (double)abs_atan_slope), (float)(2 * M_PI - (double)abs_atan_slope)};
        for (int q = 0; q < 4; ++q) {
            o.sh_sin[q] = std::sin(angle_m[q]);
            o.sh_cos[q] = std::cos(angle_m[q]);
        }
    }
    ctx->conn_off.assign(n + 1, 0);
    ctx->conn_idx.clear();
    for (int i = 0; i < n; ++i) {
        auto it = ctx->hg.conn.find(valid[i]);
        if (it != ctx->hg.conn.end())
            for (uint32_t d : it->second) {
                const int k = index_of(d);
                if (k >= 0) ctx->conn_idx.push_back(k);
            }
        ctx->conn_off[i + 1] = (int32_t)ctx->conn_idx.size();
    }
    // layers as runs of consecutive module indices (Layer.cc:3-50 pairs layers)
    std::vector<std::vector<int32_t>> runs(kNumSlots);
    for (int i = 0; i < n; ++i) {
        auto& r = runs[ctx->mods[i].layer_slot];
        if (!r.empty() && r.back() == i) r.back() = i + 1;
        else { r.push_back(i); r.push_back(i + 1); }
    }
    ctx->slot_run.assign(kNumSlots + 1, 0);
    for (int sl = 0; sl < kNumSlots; ++sl) ctx->slot_run[sl + 1] = ctx->slot_run[sl] + (int32_t)runs[sl].size() / 2;
    for (int sl = 0; sl < kNumSlots; ++sl) ctx->slot_run.insert(ctx->slot_run.end(), runs[sl].begin(), runs[sl].end());
    // upload
    free_batch(ctx);
    cudaFree(ctx->d_detid); cudaFree(ctx->d_mod); cudaFree(ctx->d_conn_off); cudaFree(ctx->d_conn_idx);
    cudaFree(ctx->d_slot_run);
    ctx->d_detid = nullptr; ctx->d_mod = nullptr; ctx->d_conn_off = nullptr; ctx->d_conn_idx = nullptr;
    ctx->d_slot_run = nullptr;
    CK(cudaMalloc(&ctx->d_detid, std::max(1, n) * sizeof(uint32_t)));
    CK(cudaMalloc(&ctx->d_mod, std::max(1, n) * sizeof(ModDev)));
    CK(cudaMalloc(&ctx->d_conn_off, (n + 1) * sizeof(int32_t)));
    CK(cudaMalloc(&ctx->d_conn_idx, std::max<size_t>(1, ctx->conn_idx.size()) * sizeof(int32_t)));
    CK(cudaMemcpy(ctx->d_detid, valid.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_mod, ctx->mods.data(), n * sizeof(ModDev), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_conn_off, ctx->conn_off.data(), (n + 1) * sizeof(int32_t), cudaMemcpyHostToDevice));
    if (!ctx->conn_idx.empty())
        CK(cudaMemcpy(ctx->d_conn_idx, ctx->conn_idx.data(), ctx->conn_idx.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    CK(cudaMalloc(&ctx->d_slot_run, ctx->slot_run.size() * sizeof(int32_t)));
    CK(cudaMemcpy(ctx->d_slot_run, ctx->slot_run.data(), ctx->slot_run.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    ctx->have_geo = true;
    return SDLG_OK;
}

// (re)allocate the batch buffers for the current event sizes and capacities
int ensure_buffers(sdlg_ctx* ctx) {
    const int n_mod = (int)ctx->detids.size();
    const int64_t n_gm = ctx->n_ev * n_mod;
    if (ctx->buffers_ok && ctx->n_hit <= ctx->cap_hit && ctx->n_ev == ctx->cap_ev) return SDLG_OK;
    free_batch(ctx);
    ctx->cap_hit = std::max<int64_t>(ctx->n_hit, ctx->cap_hit);
    ctx->cap_ev = ctx->n_ev;
    const int64_t H = std::max<int64_t>(ctx->cap_hit, 1024);
    const int64_t mult[kNumStages] = {1, 2, 3, 4, 2};
    for (int s = 0; s < kNumStages; ++s)
        ctx->cap_obj[s] = std::max<int64_t>(ctx->cap_obj[s], ctx->cap_init[s] > 0 ? ctx->cap_init[s] : H * mult[s] + 4096);
    ctx->cap_kept = std::max<int64_t>(ctx->cap_kept, ctx->cap_init[kNumStages] > 0 ? ctx->cap_init[kNumStages] : 8 * H + 4096);
    BatchDev& b = ctx->b;
    b = BatchDev{};
    b.geo.n_mod = n_mod;
    b.geo.n_mod_inv = n_mod > 1 ? UINT64_MAX / (uint64_t)n_mod + 1 : 0;  // ceil(2^64 / n_mod)
    b.geo.n_conn = (int)ctx->conn_idx.size();
    b.geo.detid = ctx->d_detid;
    b.geo.mod = ctx->d_mod;
    b.geo.conn_off = ctx->d_conn_off;
    b.geo.conn_idx = ctx->d_conn_idx;
    b.geo.slot_run = ctx->d_slot_run;
    b.geo.n_slot_run = (int)ctx->slot_run.size();
    b.n_ev = (int)ctx->n_ev;
    b.n_gm = (int)n_gm;
    b.n_hit_cap = H;
    b.n_sm = ctx->n_sm;
    b.mlp_pack = ctx->mlp.pack;
    b.mlp_stats = ctx->mlp.stats;
    for (int st = 0; st < kNumStages; ++st) {
        b.enum_task[st] = ctx->tune_task[st];
        b.enum_grid[st] = ctx->tune_grid[st];
    }
    int rc;
#define AL(ptr, n) if ((rc = dalloc(ctx, &(ptr), (n))) != SDLG_OK) return rc
    int64_t* small;
    AL(small, 2 + kNumStages);
    b.n_hit = small;
    b.n_gm_dev = small + 1;
    b.n_rec = small + 2;
    float* fx; float* fy; float* fz; int32_t* fi; uint32_t* fd; int64_t* eo;
    AL(fx, H); AL(fy, H); AL(fz, H); AL(fi, H); AL(fd, H); AL(eo, ctx->n_ev + 1);
    b.in_x = fx; b.in_y = fy; b.in_z = fz; b.in_idx = fi; b.in_det = fd; b.ev_off = eo;
    AL(b.hit_gm, H); AL(b.hit_rank, H); AL(b.hit_perm, H); AL(b.mod_hit, n_gm + 1);
    AL(b.hx, H); AL(b.hy, H); AL(b.hz, H); AL(b.hrt, H); AL(b.hphi, H); AL(b.hr3, H);
    AL(b.ha1, H); AL(b.htf, H); AL(b.htd, H); AL(b.ha3, H); AL(b.hidx, H); AL(b.hgm, H);
    AL(b.hsx, H); AL(b.hsy, H); AL(b.hsz, H);
    const int nf[kNumStages] = {4, 6, 0, 0, 0};
    for (int s = 0; s < kNumStages; ++s) {
        const int64_t C = ctx->cap_obj[s];
        Objs& O = b.obj[s];
        Recs& R = b.rec[s];
        O.cap = C; O.nf = nf[s]; R.nf = nf[s];
        AL(O.i, C); AL(O.j, C); AL(O.g, C); AL(O.f, C * std::max(1, nf[s])); AL(O.mod_cnt, n_gm + 1);
        AL(R.i, C); AL(R.j, C); AL(R.g, C); AL(R.rank, C); AL(R.f, C * std::max(1, nf[s]));
    }
    b.cand_cap[kMD] = n_gm;
    b.cand_cap[kSG] = ctx->cap_obj[kMD];
    b.cand_cap[kTL] = ctx->cap_obj[kSG];
    b.cand_cap[kTP] = ctx->cap_obj[kSG];
    b.cand_cap[kTC] = std::max(ctx->cap_obj[kTL], ctx->cap_obj[kTP]);  // tracklets, or triplets (SDLG_FLAG_TC_FROM_TP)
    for (int s = 0; s < kNumStages; ++s) AL(b.cand[s], b.cand_cap[s] + 1);
    AL(b.conn_pref, std::max<int64_t>(1, ctx->n_ev * (int64_t)ctx->conn_idx.size()));
    AL(b.conn_first, std::max<int64_t>(1, ctx->n_ev * (int64_t)ctx->conn_idx.size()));
    AL(b.conn_sum, n_gm);
    b.bucket_cap = (int64_t)1 << 24;  // covers 2^32 candidates of one stage
    AL(b.bucket, b.bucket_cap);
    b.kept_cap = ctx->cap_kept;
    AL(b.n_kept, 1);
    AL(b.passa, b.kept_cap);
    AL(b.kept, b.kept_cap);
    AL(b.n_kept2, 1);
    AL(b.passf, b.kept_cap);
    AL(b.n_keptf, 1);
    AL(b.pb, b.kept_cap);
    AL(b.n_pb, 2);
    AL(b.sgpack, ctx->cap_obj[kSG] * PK_N);
    AL(b.sgouter, ctx->cap_obj[kSG] * 11);
    AL(b.sgfeat, ctx->cap_obj[kSG] * kFeatN);
    AL(b.mdpack, ctx->cap_obj[kMD] * kMdPack);
    AL(b.counters, ctx->n_ev * 110);
    AL(b.status, 1);
    AL(b.task, kNumStages);
    AL(b.dbg, 8);
    int64_t mx = n_gm;
    for (int s = 0; s < kNumStages; ++s) mx = std::max(mx, ctx->cap_obj[s]);
    b.scan_tmp_cap = mx / 4096 + 16;
    AL(b.scan_tmp, b.scan_tmp_cap);
    AL(b.joff, ctx->cap_obj[kMD] + 1);
    AL(b.jcur, ctx->cap_obj[kMD]);
    AL(b.jidx, std::max(ctx->cap_obj[kSG], ctx->cap_obj[kTL]));
    AL(b.joff2, ctx->cap_obj[kMD] + 1);
    AL(b.jcur2, ctx->cap_obj[kMD]);
    AL(b.jidx2, ctx->cap_obj[kTP]);
    AL(b.eoff, n_gm + 1);
    AL(b.ecur, n_gm);
    AL(b.eidx, ctx->cap_obj[kSG]);
    AL(b.toff, n_gm + 1);
    b.tile_cap = 2 * std::max<int64_t>(ctx->cap_obj[kSG], n_gm);
    AL(b.tile_gm, b.tile_cap);
    b.olist_cap = 4 * std::max<int64_t>(ctx->cap_obj[kSG], n_gm);
    AL(b.olist, b.olist_cap);
#undef AL
    CK(cudaMemcpyAsync(b.n_gm_dev, &n_gm, sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->buffers_ok = true;
    return SDLG_OK;
}

// events recorded while a stream is captured must become graph nodes
inline void record(cudaEvent_t e, cudaStream_t s) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(s, &st);
    if (st == cudaStreamCaptureStatusActive) cudaEventRecordWithFlags(e, s, cudaEventRecordExternal);
    else cudaEventRecord(e, s);
}

// the full chain, enqueued on the context stream (also the body of the CUDA graph)
void enqueue_chain(sdlg_ctx* ctx, int stop_after) {
    BatchDev& b = ctx->b;
    cudaStream_t s = ctx->stream;
    const int64_t n_gm = b.n_gm;
    record(ctx->ev[0], s);
    cudaMemsetAsync(b.status, 0, sizeof(uint32_t), s);
    cudaMemsetAsync(b.dbg, 0, 8 * sizeof(unsigned long long), s);
    cudaMemsetAsync(b.n_rec, 0, kNumStages * sizeof(int64_t), s);
    cudaMemsetAsync(b.task, 0, kNumStages * sizeof(unsigned long long), s);
    cudaMemsetAsync(b.counters, 0, b.n_ev * 110 * sizeof(uint32_t), s);
    cudaMemsetAsync(b.mod_hit, 0, (n_gm + 1) * sizeof(int64_t), s);
    for (int st = 0; st < kNumStages; ++st) cudaMemsetAsync(b.obj[st].mod_cnt, 0, (n_gm + 1) * sizeof(int64_t), s);
    cudaMemsetAsync(b.mlp_stats, 0, sizeof(MlpStats), s);
    Hooks* h = &ctx->hooks;
    h->timed = true;
    h->launches = 0;
    launch_ingest(b, s, h);
    record(ctx->ev[1], s);
    if (stop_after >= kMD) launch_md(b, s, h);
    record(ctx->ev[2], s);
    if (stop_after >= kSG) launch_sg(b, s, h);
    record(ctx->ev[3], s);
    if (stop_after >= kTL) launch_tl(b, s, h);
    record(ctx->ev[4], s);
    if (stop_after >= kTP) launch_tp(b, s, h);
    record(ctx->ev[5], s);
    if (stop_after >= kTC) launch_tc(b, s, h);
    record(ctx->ev[6], s);
    ctx->launches_per_run = h->launches;
    // status word and attempted appends for the host's overflow check
    cudaMemcpyAsync(ctx->h_small, b.n_rec, kNumStages * sizeof(int64_t), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(ctx->h_small + kNumStages, b.status, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(ctx->h_small + kNumStages + 1, b.n_kept, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
}

// stages first..last only (first >= 1), on the objects the previous run left
// for the stages below first; no graph
void enqueue_stages(sdlg_ctx* ctx, int first, int last) {
    BatchDev& b = ctx->b;
    cudaStream_t s = ctx->stream;
    const int64_t n_gm = b.n_gm;
    const int ns = last - first + 1;
    record(ctx->ev[0], s);
    cudaMemsetAsync(b.status, 0, sizeof(uint32_t), s);
    cudaMemsetAsync(b.dbg, 0, 8 * sizeof(unsigned long long), s);
    cudaMemsetAsync(b.n_rec + first, 0, ns * sizeof(int64_t), s);
    cudaMemsetAsync(b.task + first, 0, ns * sizeof(unsigned long long), s);
    // the counters these stages write (22 per stage in each event's 110:
    // candidates, then objects): the triplet candidates are counted by the
    // tracklet stage (Event.cc:547-596 loops over the segment lists)
    auto zero_counters = [&](int at, int n) {
        cudaMemset2DAsync(b.counters + at, 110 * sizeof(uint32_t), 0, n * sizeof(uint32_t), b.n_ev, s);
    };
    for (int st = first; st <= last; ++st) {
        if (st == kTP) zero_counters(kTP * 22 + 11, 11);
        else zero_counters(st * 22, 22);
    }
    if (first <= kTL && last >= kTL) zero_counters(kTP * 22, 11);
    for (int st = first; st <= last; ++st) cudaMemsetAsync(b.obj[st].mod_cnt, 0, (n_gm + 1) * sizeof(int64_t), s);
    if (first <= kTL && last >= kTL) cudaMemsetAsync(b.mlp_stats, 0, sizeof(MlpStats), s);
    Hooks* h = &ctx->hooks;
    h->timed = true;
    h->launches = 0;
    record(ctx->ev[1], s);
    void (*fns[5])(const BatchDev&, cudaStream_t, Hooks*) = {launch_md, launch_sg, launch_tl, launch_tp, launch_tc};
    for (int st = 0; st < kNumStages; ++st) {
        if (st >= first && st <= last) fns[st](b, s, h);
        record(ctx->ev[2 + st], s);
    }
    cudaMemcpyAsync(ctx->h_small, b.n_rec, kNumStages * sizeof(int64_t), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(ctx->h_small + kNumStages, b.status, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(ctx->h_small + kNumStages + 1, b.n_kept, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
}

#ifdef SDL_DEVICE_CHECKS
// debug builds: run stage by stage, synchronising after each, and report the
// first out-of-bounds index the device checks recorded
int check_stage(sdlg_ctx* ctx, const char* what) {
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return fail(ctx, SDLG_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    unsigned long long d[4];
    CK(cudaMemcpy(d, ctx->b.dbg, sizeof(d), cudaMemcpyDeviceToHost));
    if (d[0]) return fail(ctx, SDLG_ERR_CUDA, "%s: %llu bad indices, first at sdl_kernels.cu:%llu index %lld limit %lld", what,
                          d[0], d[1], (long long)d[2], (long long)d[3]);
    return SDLG_OK;
}

int launch_checked(sdlg_ctx* ctx, int stop_after) {
    BatchDev& b = ctx->b;
    cudaStream_t s = ctx->stream;
    const int64_t n_gm = b.n_gm;
    cudaMemsetAsync(b.status, 0, sizeof(uint32_t), s);
    cudaMemsetAsync(b.dbg, 0, 8 * sizeof(unsigned long long), s);
    cudaMemsetAsync(b.n_rec, 0, kNumStages * sizeof(int64_t), s);
    cudaMemsetAsync(b.task, 0, kNumStages * sizeof(unsigned long long), s);
    cudaMemsetAsync(b.counters, 0, b.n_ev * 110 * sizeof(uint32_t), s);
    cudaMemsetAsync(b.mod_hit, 0, (n_gm + 1) * sizeof(int64_t), s);
    for (int st = 0; st < kNumStages; ++st) cudaMemsetAsync(b.obj[st].mod_cnt, 0, (n_gm + 1) * sizeof(int64_t), s);
    cudaMemsetAsync(b.mlp_stats, 0, sizeof(MlpStats), s);
    int rc;
    record(ctx->ev[0], s);
    Hooks* h = &ctx->hooks;
    h->timed = true;
    h->launches = 0;
    launch_ingest(b, s, h);
    if ((rc = check_stage(ctx, "ingest"))) return rc;
    record(ctx->ev[1], s);
    void (*fns[5])(const BatchDev&, cudaStream_t, Hooks*) = {launch_md, launch_sg, launch_tl, launch_tp, launch_tc};
    static const char* names[5] = {"MD", "SG", "TL", "TP", "TC"};
    for (int st = 0; st < 5; ++st) {
        if (stop_after >= st) fns[st](b, s, h);
        if ((rc = check_stage(ctx, names[st]))) return rc;
        record(ctx->ev[2 + st], s);
    }
    cudaMemcpyAsync(ctx->h_small, b.n_rec, kNumStages * sizeof(int64_t), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(ctx->h_small + kNumStages, b.status, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(ctx->h_small + kNumStages + 1, b.n_kept, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
    return SDLG_OK;
}
#endif

int launch(sdlg_ctx* ctx, int stop_after, int flags) {
    ctx->b.flags = flags;
    ctx->ran = true;
    wait_readback(ctx);
#ifdef SDL_DEVICE_CHECKS
    return launch_checked(ctx, stop_after);
#endif
    const bool use_graph = !(flags & SDLG_FLAG_NO_GRAPH);
    if (!use_graph) {
        enqueue_chain(ctx, stop_after);
        CK(cudaGetLastError());
        return SDLG_OK;
    }
    if (!ctx->graph || ctx->graph_stop != stop_after || ctx->graph_flags != flags) {
        if (ctx->graph) {
            cudaGraphExecDestroy(ctx->graph);
            ctx->graph = nullptr;
        }
        cudaGraph_t g;
        CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        enqueue_chain(ctx, stop_after);
        CK(cudaStreamEndCapture(ctx->stream, &g));
        cudaError_t e = cudaGraphInstantiate(&ctx->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(ctx, SDLG_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
        ctx->graph_stop = stop_after;
        ctx->graph_flags = flags;
    }
    CK(cudaGraphLaunch(ctx->graph, ctx->stream));
    return SDLG_OK;
}

// wait for a run; grow overflowing capacities and re-run until clean
int finish(sdlg_ctx* ctx) {
    for (int attempt = 0; attempt < 16; ++attempt) {  // one overflowing stage per attempt at worst
        CK(cudaStreamSynchronize(ctx->stream));
        const uint32_t status = (uint32_t)(ctx->h_small[kNumStages] & 0xffffffffu);
        if (status & kStatusUnknownModule) {
            // new detIds: extend the module table and re-run (modules created on
            // demand, Event.cc:54-78)
            std::vector<uint32_t> hd(ctx->n_hit);
            CK(cudaMemcpy(hd.data(), ctx->b.in_det, ctx->n_hit * sizeof(uint32_t), cudaMemcpyDeviceToHost));
            std::vector<float> keep[3];
            std::vector<int32_t> ki(ctx->n_hit);
            for (int k = 0; k < 3; ++k) keep[k].resize(ctx->n_hit);
            CK(cudaMemcpy(keep[0].data(), ctx->b.in_x, ctx->n_hit * 4, cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(keep[1].data(), ctx->b.in_y, ctx->n_hit * 4, cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(keep[2].data(), ctx->b.in_z, ctx->n_hit * 4, cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(ki.data(), ctx->b.in_idx, ctx->n_hit * 4, cudaMemcpyDeviceToHost));
            for (uint32_t d : hd)
                if (!valid_module(decode(d))) return fail(ctx, SDLG_ERR_DETID, "detId %u is not a barrel or endcap module", d);
            const std::vector<int64_t> off = ctx->ev_off;
            int rc = build_module_table(ctx, hd);
            if (rc) return rc;
            rc = set_events_impl(ctx, ctx->n_ev, off.data(), keep[0].data(), keep[1].data(), keep[2].data(), ki.data(), hd.data());
            if (rc) return rc;
            rc = launch(ctx, ctx->last_stop, ctx->last_flags);
            if (rc) return rc;
            continue;
        }
        if (status & kStatusMlpTimeout)
            return fail(ctx, SDLG_ERR_CUDA, "tracklet pre-filter: a tensor-core wait gave up; results discarded");
        if (!(status & kStatusHalt)) return SDLG_OK;
        // grow every stage that overflowed (the attempted-append counters hold
        // the exact need of the first overflowing stage)
        bool grew = false;
        for (int s = 0; s < kNumStages; ++s) {
            if (status & (1u << s)) {
                ctx->cap_obj[s] = std::max<int64_t>(ctx->cap_obj[s] * 2, ctx->h_small[s] + ctx->h_small[s] / 4 + 4096);
                grew = true;
            }
        }
        if (status & kStatusOverflowKept) {
            const int64_t need = ctx->h_small[kNumStages + 1];
            ctx->cap_kept = std::max<int64_t>(ctx->cap_kept * 2, need + need / 4 + 4096);
            grew = true;
        }
        if (!grew) return fail(ctx, SDLG_ERR_CAPACITY, "inconsistent status %u", status);
        ctx->buffers_ok = false;
        const std::vector<int64_t> off = ctx->ev_off;
        // keep the inputs: copy them back, reallocate, upload again
        std::vector<float> x(ctx->n_hit), y(ctx->n_hit), z(ctx->n_hit);
        std::vector<int32_t> idx(ctx->n_hit);
        std::vector<uint32_t> det(ctx->n_hit);
        CK(cudaMemcpy(x.data(), ctx->b.in_x, ctx->n_hit * 4, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(y.data(), ctx->b.in_y, ctx->n_hit * 4, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(z.data(), ctx->b.in_z, ctx->n_hit * 4, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(idx.data(), ctx->b.in_idx, ctx->n_hit * 4, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(det.data(), ctx->b.in_det, ctx->n_hit * 4, cudaMemcpyDeviceToHost));
        int rc = set_events_impl(ctx, ctx->n_ev, off.data(), x.data(), y.data(), z.data(), idx.data(), det.data());
        if (rc) return rc;
        rc = launch(ctx, ctx->last_stop, ctx->last_flags);
        if (rc) return rc;
    }
    return fail(ctx, SDLG_ERR_CAPACITY, "capacity did not converge");
}

int parse_file(const char* path, int kind, HostGeometry& hg) {
    std::ifstream f(path);
    if (!f.is_open()) return SDLG_ERR_IO;
    std::string line;
    while (std::getline(f, line)) {
        std::stringstream ss(line);
        unsigned int d;
        if (kind == 0) {  // TiltedGeometry.cc:28-40
            float drdz, slope;
            ss >> d >> drdz >> slope;
            hg.tilted[d] = {drdz, slope};
        } else if (kind == 1) {  // EndcapGeometry.cc:36-59
            float avgr2, yl, sl, yh, sh, c7, c8, cz;
            ss >> d >> avgr2 >> yl >> sl >> yh >> sh >> c7 >> c8 >> cz;
            hg.endcap[d] = {sl, c7};
        } else {  // ModuleConnectionMap.cc:28-45
            int n;
            ss >> d >> n;
            std::vector<uint32_t> v;
            for (int k = 0; k < n; ++k) {
                unsigned int e;
                ss >> e;
                v.push_back(e);
            }
            hg.conn[d] = v;
        }
    }
    return SDLG_OK;
}

}  // namespace

namespace {

// ------------------------------------------------------------------ pre-filter
uint64_t splitmix64(uint64_t& state) {
    uint64_t z = (state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

int mlp_repack(sdlg_ctx* ctx) {
    launch_mlp_pack(ctx->mlp.params, ctx->mlp.pack, ctx->mlp.thr, ctx->stream);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(ctx->stream));
    return SDLG_OK;
}

// grow the training-sample buffers to hold `need` samples, keeping the first n
int mlp_reserve(sdlg_ctx* ctx, int64_t need) {
    auto& M = ctx->mlp;
    if (need <= M.cap) return SDLG_OK;
    const int64_t cap = std::max<int64_t>(need, M.cap * 2 + 65536);
    float *x = nullptr, *y = nullptr;
    CK(cudaMalloc(&x, cap * kMlpIn * sizeof(float)));
    if (cudaMalloc(&y, cap * sizeof(float)) != cudaSuccess) {
        cudaFree(x);
        return fail(ctx, SDLG_ERR_CAPACITY, "no device memory for %lld training samples", (long long)cap);
    }
    if (M.n) {
        CK(cudaMemcpy(x, M.x, M.n * kMlpIn * sizeof(float), cudaMemcpyDeviceToDevice));
        CK(cudaMemcpy(y, M.y, M.n * sizeof(float), cudaMemcpyDeviceToDevice));
    }
    cudaFree(M.x);
    cudaFree(M.y);
    M.x = x;
    M.y = y;
    M.cap = cap;
    return SDLG_OK;
}

// device copy of a host array (caller frees)
template <class T>
int to_device(sdlg_ctx* ctx, const T* h, int64_t n, T** d) {
    *d = nullptr;
    CK(cudaMalloc(d, std::max<int64_t>(n, 1) * sizeof(T)));
    if (n) CK(cudaMemcpy(*d, h, n * sizeof(T), cudaMemcpyHostToDevice));
    return SDLG_OK;
}

}  // namespace

extern "C" {

int sdlg_create(sdlg_ctx** out, int device) {
    if (!out) return SDLG_ERR_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return SDLG_ERR_NO_DEVICE;
    if (device < 0 || device >= n) return SDLG_ERR_ARG;
    sdlg_ctx* ctx = new sdlg_ctx();
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->n_sm, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->gather_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stage.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->stage.ev_in, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->stage.ev_used, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_mat, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_read, cudaEventDisableTiming);
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) e = cudaEventCreateWithFlags(&ctx->ev_copy[k], cudaEventDisableTiming);
    for (int k = 0; k < 8 && e == cudaSuccess; ++k) e = cudaEventCreate(&ctx->ev[k]);
    for (int k = 0; k < kNumStages && e == cudaSuccess; ++k) {
        e = cudaEventCreate(&ctx->hooks.enum_start[k]);
        if (e == cudaSuccess) e = cudaEventCreate(&ctx->hooks.enum_stop[k]);
    }
    for (int k = 0; k < 3; ++k)
        if (e == cudaSuccess) e = cudaEventCreate(&ctx->hooks.tl_mid[k]);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&ctx->h_small, 16 * sizeof(int64_t));
    // the host libm's float functions for the cut arithmetic (once per process / device)
    const char* lm_err = nullptr;
    if (e == cudaSuccess && libm_setup(device, &lm_err) != 0) e = cudaErrorMemoryAllocation;
    // pre-filter state is small and allocated once, so device pointers captured
    // in the launch graph never change
    auto& M = ctx->mlp;
    if (e == cudaSuccess) e = cudaMalloc(&M.params, kMlpParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&M.grad, kMlpParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&M.m, kMlpParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&M.v, kMlpParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&M.pack, kPackBytes);
    if (e == cudaSuccess) e = cudaMalloc(&M.stats, sizeof(MlpStats));
    if (e == cudaSuccess) e = cudaMalloc(&M.loss, sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&M.status, sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMalloc(&M.found, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(M.grad, 0, kMlpParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(M.pack, 0, kPackBytes);
    if (e == cudaSuccess) e = cudaMemset(M.stats, 0, sizeof(MlpStats));
    if (e != cudaSuccess) {
        void* ps[] = {M.params, M.pack, M.stats, M.grad, M.m, M.v, M.loss, M.status, M.found};
        for (void* p : ps) cudaFree(p);
        delete ctx;
        return SDLG_ERR_CUDA;
    }
    *out = ctx;
    return SDLG_OK;
}

int sdlg_destroy(sdlg_ctx* ctx) {
    if (!ctx) return SDLG_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->gather_stream) cudaStreamSynchronize(ctx->gather_stream);
    if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
    if (ctx->stage.stream) cudaStreamSynchronize(ctx->stage.stream);
    free_batch(ctx);
    if (ctx->stage.dev) cudaFree(ctx->stage.dev);
    if (ctx->stage.h_off) cudaFreeHost(ctx->stage.h_off);
    if (ctx->stage.ev_in) cudaEventDestroy(ctx->stage.ev_in);
    if (ctx->stage.ev_used) cudaEventDestroy(ctx->stage.ev_used);
    if (ctx->stage.stream) cudaStreamDestroy(ctx->stage.stream);
    cudaFree(ctx->d_detid); cudaFree(ctx->d_mod); cudaFree(ctx->d_conn_off); cudaFree(ctx->d_conn_idx);
    cudaFree(ctx->d_slot_run);
    {
        auto& M = ctx->mlp;
        void* ps[] = {M.params, M.pack, M.stats, M.grad, M.m, M.v, M.loss, M.status, M.found, M.x, M.y, M.order};
        for (void* p : ps) cudaFree(p);
    }
    if (ctx->pinned) cudaFreeHost(ctx->pinned);
    for (int k = 0; k < 2; ++k)
        if (ctx->scratch[k]) cudaFree(ctx->scratch[k]);
    if (ctx->ev_mat) cudaEventDestroy(ctx->ev_mat);
    if (ctx->ev_read) cudaEventDestroy(ctx->ev_read);
    for (int k = 0; k < 2; ++k)
        if (ctx->ev_copy[k]) cudaEventDestroy(ctx->ev_copy[k]);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    if (ctx->gather_stream) cudaStreamDestroy(ctx->gather_stream);
    if (ctx->h_small) cudaFreeHost(ctx->h_small);
    for (int k = 0; k < 8; ++k) if (ctx->ev[k]) cudaEventDestroy(ctx->ev[k]);
    for (int k = 0; k < kNumStages; ++k) {
        if (ctx->hooks.enum_start[k]) cudaEventDestroy(ctx->hooks.enum_start[k]);
        if (ctx->hooks.enum_stop[k]) cudaEventDestroy(ctx->hooks.enum_stop[k]);
    }
    for (int k = 0; k < 3; ++k)
        if (ctx->hooks.tl_mid[k]) cudaEventDestroy(ctx->hooks.tl_mid[k]);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return SDLG_OK;
}

const char* sdlg_last_error(const sdlg_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int sdlg_geometry_load_files(sdlg_ctx* ctx, const char* tilted_path, const char* endcap_path, const char* map_path) {
    if (!ctx) return SDLG_ERR_ARG;
    cudaSetDevice(ctx->device);
    HostGeometry hg;
    const char* paths[3] = {tilted_path, endcap_path, map_path};
    for (int k = 0; k < 3; ++k)
        if (paths[k] && parse_file(paths[k], k, hg) != SDLG_OK) return fail(ctx, SDLG_ERR_IO, "cannot read %s", paths[k]);
    ctx->hg = hg;
    ctx->detids.clear();
    return build_module_table(ctx, {});
}

// ---- binary geometry: the host tables in one file (format in sdl_gpu.h)
namespace {
const char kGeoMagic[8] = {'S', 'D', 'L', 'G', 'E', 'O', '1', 0};

bool write_geometry(const HostGeometry& hg, const char* path) {
    std::FILE* f = std::fopen(path, "wb");
    if (!f) return false;
    bool ok = std::fwrite(kGeoMagic, 1, 8, f) == 8;
    auto u64 = [&](uint64_t v) { ok = ok && std::fwrite(&v, 8, 1, f) == 1; };
    auto row = [&](uint32_t d, float a, float c) {
        ok = ok && std::fwrite(&d, 4, 1, f) == 1 && std::fwrite(&a, 4, 1, f) == 1 && std::fwrite(&c, 4, 1, f) == 1;
    };
    u64(hg.tilted.size());
    for (const auto& kv : hg.tilted) row(kv.first, kv.second.first, kv.second.second);
    u64(hg.endcap.size());
    for (const auto& kv : hg.endcap) row(kv.first, kv.second.first, kv.second.second);
    u64(hg.conn.size());
    for (const auto& kv : hg.conn) {
        const uint32_t n = (uint32_t)kv.second.size();
        ok = ok && std::fwrite(&kv.first, 4, 1, f) == 1 && std::fwrite(&n, 4, 1, f) == 1;
    }
    for (const auto& kv : hg.conn)
        if (!kv.second.empty()) ok = ok && std::fwrite(kv.second.data(), 4, kv.second.size(), f) == kv.second.size();
    return std::fclose(f) == 0 && ok;
}

bool read_geometry(const char* path, HostGeometry& hg) {
    std::FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    char magic[8];
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kGeoMagic, 8) == 0;
    auto u64 = [&]() {
        uint64_t v = 0;
        ok = ok && std::fread(&v, 8, 1, f) == 1 && v < (1ull << 32);
        return ok ? v : 0ull;
    };
    for (int table = 0; table < 2 && ok; ++table) {
        const uint64_t n = u64();
        for (uint64_t i = 0; i < n && ok; ++i) {
            uint32_t d;
            float a, c;
            ok = std::fread(&d, 4, 1, f) == 1 && std::fread(&a, 4, 1, f) == 1 && std::fread(&c, 4, 1, f) == 1;
            if (ok) (table == 0 ? hg.tilted : hg.endcap)[d] = {a, c};
        }
    }
    const uint64_t nk = u64();
    std::vector<std::pair<uint32_t, uint32_t>> keys;
    for (uint64_t k = 0; k < nk && ok; ++k) {
        uint32_t d, n;
        ok = std::fread(&d, 4, 1, f) == 1 && std::fread(&n, 4, 1, f) == 1;
        if (ok) keys.push_back({d, n});
    }
    for (const auto& kn : keys) {
        if (!ok) break;
        std::vector<uint32_t> v(kn.second);
        ok = kn.second == 0 || std::fread(v.data(), 4, kn.second, f) == kn.second;
        hg.conn[kn.first] = std::move(v);
    }
    std::fclose(f);
    return ok;
}
}  // namespace

int sdlg_geometry_convert(const char* tilted_path, const char* endcap_path, const char* map_path, const char* out_path) {
    if (!out_path) return SDLG_ERR_ARG;
    HostGeometry hg;
    const char* paths[3] = {tilted_path, endcap_path, map_path};
    for (int k = 0; k < 3; ++k)
        if (paths[k] && parse_file(paths[k], k, hg) != SDLG_OK) return SDLG_ERR_IO;
    return write_geometry(hg, out_path) ? SDLG_OK : SDLG_ERR_IO;
}

int sdlg_geometry_load_binary(sdlg_ctx* ctx, const char* path) {
    if (!ctx || !path) return SDLG_ERR_ARG;
    cudaSetDevice(ctx->device);
    HostGeometry hg;
    if (!read_geometry(path, hg)) return fail(ctx, SDLG_ERR_IO, "cannot read binary geometry %s", path);
    ctx->hg = hg;
    ctx->detids.clear();
    return build_module_table(ctx, {});
}

int sdlg_geometry_upload(sdlg_ctx* ctx, int64_t n_tilted, const uint32_t* t_detid, const float* t_vals, int64_t n_endcap,
                         const uint32_t* e_detid, const float* e_vals, int64_t n_keys, const uint32_t* keys,
                         const int64_t* off, const uint32_t* dst) {
    if (!ctx || n_tilted < 0 || n_endcap < 0 || n_keys < 0) return SDLG_ERR_ARG;
    if ((n_tilted && (!t_detid || !t_vals)) || (n_endcap && (!e_detid || !e_vals)) || (n_keys && (!keys || !off)))
        return fail(ctx, SDLG_ERR_ARG, "null table pointer");
    cudaSetDevice(ctx->device);
    HostGeometry hg;
    for (int64_t i = 0; i < n_tilted; ++i) hg.tilted[t_detid[i]] = {t_vals[2 * i], t_vals[2 * i + 1]};
    for (int64_t i = 0; i < n_endcap; ++i) hg.endcap[e_detid[i]] = {e_vals[8 * i + 2], e_vals[8 * i + 5]};
    for (int64_t k = 0; k < n_keys; ++k) {
        if (off[k + 1] < off[k]) return fail(ctx, SDLG_ERR_ARG, "map offsets not monotone");
        hg.conn[keys[k]] = std::vector<uint32_t>(dst + off[k], dst + off[k + 1]);
    }
    ctx->hg = hg;
    ctx->detids.clear();
    return build_module_table(ctx, {});
}

int64_t sdlg_num_modules(const sdlg_ctx* ctx) { return ctx ? (int64_t)ctx->detids.size() : -1; }

}  // extern "C"

namespace {

// the checks of sdlg_set_events and sdlg_stage_events; n: the batch's hits
int check_events(sdlg_ctx* ctx, int64_t n_events, const int64_t* ev_off, const float* x, const float* y, const float* z,
                 const int32_t* idx, const uint32_t* detid, int64_t* n_out) {
    if (!ctx || n_events <= 0 || !ev_off) return SDLG_ERR_ARG;
    if (!ctx->have_geo) return fail(ctx, SDLG_ERR_NO_GEOMETRY, "no geometry loaded");
    if (ev_off[0] != 0) return fail(ctx, SDLG_ERR_ARG, "ev_off[0] must be 0");
    for (int64_t e = 0; e < n_events; ++e)
        if (ev_off[e + 1] < ev_off[e]) return fail(ctx, SDLG_ERR_ARG, "event offsets not monotone");
    const int64_t n = ev_off[n_events];
    if (n > 0 && (!x || !y || !z || !idx || !detid)) return fail(ctx, SDLG_ERR_ARG, "null hit array");
    if (n > INT32_MAX / 4) return fail(ctx, SDLG_ERR_ARG, "too many hits in one batch");
    *n_out = n;
    return SDLG_OK;
}

// the staged device batch's layout: x, y, z, idx, detid (S.hits each, every
// array 16-byte aligned), then the offsets (S.evs + 1) and the hit count,
// 256-byte aligned
size_t stage_stride(int64_t hits) { return (size_t)((hits + 3) / 4) * 16; }
size_t stage_off_pos(int64_t hits) { return (5 * stage_stride(hits) + 255) / 256 * 256; }

int set_events_impl(sdlg_ctx* ctx, int64_t n_events, const int64_t* ev_off, const float* x, const float* y, const float* z,
                    const int32_t* idx, const uint32_t* detid) {
    int64_t n = 0;
    int rc0 = check_events(ctx, n_events, ev_off, x, y, z, idx, detid, &n);
    if (rc0) return rc0;
    cudaSetDevice(ctx->device);
    // wait for any run still reading the inputs
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->n_ev = n_events;
    ctx->n_hit = n;
    ctx->ev_off.assign(ev_off, ev_off + n_events + 1);
    int rc = ensure_buffers(ctx);
    if (rc) return rc;
    BatchDev& b = ctx->b;
    cudaStream_t s = ctx->stream;
    const void* src[5] = {x, y, z, idx, detid};
    void* dstp[5] = {(void*)b.in_x, (void*)b.in_y, (void*)b.in_z, (void*)b.in_idx, (void*)b.in_det};
    const size_t bytes = (size_t)n * 4;
    // pinned callers are copied directly; others through the pinned staging buffer
    bool all_pinned = true;
    for (int k = 0; k < 5 && n > 0; ++k) {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, src[k]) != cudaSuccess || a.type != cudaMemoryTypeHost) {
            cudaGetLastError();
            all_pinned = false;
        }
    }
    if (n > 0 && all_pinned) {
        for (int k = 0; k < 5; ++k) CK(cudaMemcpyAsync(dstp[k], src[k], bytes, cudaMemcpyHostToDevice, s));
    } else if (n > 0) {
        if (ctx->pinned_bytes < (int64_t)(bytes * 5)) {
            if (ctx->pinned) cudaFreeHost(ctx->pinned);
            ctx->pinned = nullptr;
            ctx->pinned_bytes = 0;
            CK(cudaMallocHost(&ctx->pinned, bytes * 5));
            ctx->pinned_bytes = (int64_t)bytes * 5;
        }
        char* p = static_cast<char*>(ctx->pinned);
        for (int k = 0; k < 5; ++k) {
            std::memcpy(p + k * bytes, src[k], bytes);
            CK(cudaMemcpyAsync(dstp[k], p + k * bytes, bytes, cudaMemcpyHostToDevice, s));
        }
    }
    int64_t* hsm = ctx->h_small + 8;
    hsm[0] = n;
    CK(cudaMemcpyAsync(const_cast<int64_t*>(b.n_hit), hsm, sizeof(int64_t), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(const_cast<int64_t*>(b.ev_off), ev_off, (n_events + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, s));
    // the host offsets may be pageable: make the copy complete before returning
    CK(cudaStreamSynchronize(s));
    ctx->ran = false;
    return SDLG_OK;
}

}  // namespace

extern "C" {

int sdlg_set_events(sdlg_ctx* ctx, int64_t n_events, const int64_t* ev_off, const float* x, const float* y, const float* z,
                    const int32_t* idx, const uint32_t* detid) {
    if (!ctx) return SDLG_ERR_ARG;
    // these events replace a staged batch
    auto& S = ctx->stage;
    S.pending = false;
    S.on_host = false;
    for (auto& v : S.host_f) std::vector<float>().swap(v);
    std::vector<int32_t>().swap(S.host_idx);
    std::vector<uint32_t>().swap(S.host_det);
    return set_events_impl(ctx, n_events, ev_off, x, y, z, idx, detid);
}

int sdlg_stage_events(sdlg_ctx* ctx, int64_t n_events, const int64_t* ev_off, const float* x, const float* y, const float* z,
                      const int32_t* idx, const uint32_t* detid) {
    int64_t n = 0;
    int rc = check_events(ctx, n_events, ev_off, x, y, z, idx, detid, &n);
    if (rc) return rc;
    cudaSetDevice(ctx->device);
    auto& S = ctx->stage;
    // the previous staging's copy may still read the pinned offsets
    CK(cudaStreamSynchronize(S.stream));
    S.pending = false;
    S.on_host = false;
    S.n_ev = n_events;
    S.n_hit = n;
    S.ev_off.assign(ev_off, ev_off + n_events + 1);
    if (!(ctx->buffers_ok && n_events == ctx->cap_ev && n <= ctx->cap_hit)) {
        // the batch needs other buffers: it waits on the host, and the next
        // run reallocates and uploads it (sdlg_set_events' path)
        S.host_f[0].assign(x, x + n);
        S.host_f[1].assign(y, y + n);
        S.host_f[2].assign(z, z + n);
        S.host_idx.assign(idx, idx + n);
        S.host_det.assign(detid, detid + n);
        S.on_host = true;
        S.pending = true;
        return SDLG_OK;
    }
    for (auto& v : S.host_f) std::vector<float>().swap(v);
    std::vector<int32_t>().swap(S.host_idx);
    std::vector<uint32_t>().swap(S.host_det);
    if (S.hits < ctx->cap_hit || S.evs < ctx->cap_ev) {
        // an install may still read the old allocation
        if (S.used_pending) CK(cudaEventSynchronize(S.ev_used));
        S.used_pending = false;
        if (S.dev) cudaFree(S.dev);
        S.dev = nullptr;
        S.hits = S.evs = 0;
        const size_t bytes = stage_off_pos(ctx->cap_hit) + (size_t)(ctx->cap_ev + 2) * sizeof(int64_t);
        cudaError_t e = cudaMalloc(&S.dev, bytes);
        if (e != cudaSuccess) return fail(ctx, SDLG_ERR_CAPACITY, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
        S.hits = ctx->cap_hit;
        S.evs = ctx->cap_ev;
    }
    if (S.h_off_cap < n_events + 2) {
        if (S.h_off) cudaFreeHost(S.h_off);
        S.h_off = nullptr;
        S.h_off_cap = 0;
        CK(cudaMallocHost((void**)&S.h_off, (n_events + 2) * sizeof(int64_t)));
        S.h_off_cap = n_events + 2;
    }
    std::memcpy(S.h_off, ev_off, (n_events + 1) * sizeof(int64_t));
    S.h_off[n_events + 1] = n;
    // the previous install's copies out of the staging come first
    if (S.used_pending) CK(cudaStreamWaitEvent(S.stream, S.ev_used, 0));
    const void* src[5] = {x, y, z, idx, detid};
    const size_t bytes = (size_t)n * 4;
    bool all_pinned = true;
    for (int k = 0; k < 5 && n > 0; ++k) {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, src[k]) != cudaSuccess || a.type != cudaMemoryTypeHost) {
            cudaGetLastError();
            all_pinned = false;
        }
    }
    if (n > 0 && !all_pinned) {
        // through the pinned host staging (free: its users wait for their copies)
        if (ctx->pinned_bytes < (int64_t)(bytes * 5)) {
            if (ctx->pinned) cudaFreeHost(ctx->pinned);
            ctx->pinned = nullptr;
            ctx->pinned_bytes = 0;
            CK(cudaMallocHost(&ctx->pinned, bytes * 5));
            ctx->pinned_bytes = (int64_t)bytes * 5;
        }
        char* p = static_cast<char*>(ctx->pinned);
        for (int k = 0; k < 5; ++k) {
            std::memcpy(p + k * bytes, src[k], bytes);
            src[k] = p + k * bytes;
        }
    }
    for (int k = 0; k < 5 && n > 0; ++k)
        CK(cudaMemcpyAsync(S.dev + k * stage_stride(S.hits), src[k], bytes, cudaMemcpyHostToDevice, S.stream));
    CK(cudaMemcpyAsync(S.dev + stage_off_pos(S.hits), S.h_off, (n_events + 2) * sizeof(int64_t), cudaMemcpyHostToDevice,
                       S.stream));
    CK(cudaEventRecord(S.ev_in, S.stream));
    // the caller's buffers are read when this returns
    CK(cudaEventSynchronize(S.ev_in));
    S.pending = true;
    return SDLG_OK;
}

}  // extern "C"

namespace {

// the staged batch becomes the context's events, at the start of a run from
// the hits: copies from the staging into the batch buffers on the context
// stream (after the staging's own copy), or sdlg_set_events' path for a
// batch that waits on the host or no longer fits
int install_staged(sdlg_ctx* ctx) {
    auto& S = ctx->stage;
    if (!S.pending) return SDLG_OK;
    S.pending = false;
    if (!S.on_host && !(ctx->buffers_ok && S.n_ev == ctx->cap_ev && S.n_hit <= ctx->cap_hit)) {
        // the buffers changed since the batch was staged: back through the host
        CK(cudaStreamSynchronize(S.stream));
        const size_t bytes = (size_t)S.n_hit * 4;
        S.host_f[0].resize(S.n_hit); S.host_f[1].resize(S.n_hit); S.host_f[2].resize(S.n_hit);
        S.host_idx.resize(S.n_hit); S.host_det.resize(S.n_hit);
        void* dst[5] = {S.host_f[0].data(), S.host_f[1].data(), S.host_f[2].data(), S.host_idx.data(), S.host_det.data()};
        for (int k = 0; k < 5 && S.n_hit > 0; ++k)
            CK(cudaMemcpy(dst[k], S.dev + k * stage_stride(S.hits), bytes, cudaMemcpyDeviceToHost));
        S.on_host = true;
    }
    if (S.on_host) {
        S.on_host = false;
        const int rc = set_events_impl(ctx, S.n_ev, S.ev_off.data(), S.host_f[0].data(), S.host_f[1].data(),
                                       S.host_f[2].data(), S.host_idx.data(), S.host_det.data());
        for (auto& v : S.host_f) std::vector<float>().swap(v);
        std::vector<int32_t>().swap(S.host_idx);
        std::vector<uint32_t>().swap(S.host_det);
        return rc;
    }
    BatchDev& b = ctx->b;
    cudaStream_t s = ctx->stream;
    CK(cudaStreamWaitEvent(s, S.ev_in, 0));
    // one copy kernel on the SMs: the copy engines may still be busy with the
    // previous batch's readback
    void* dstp[5] = {(void*)b.in_x, (void*)b.in_y, (void*)b.in_z, (void*)b.in_idx, (void*)b.in_det};
    const char* offs = S.dev + stage_off_pos(S.hits);
    CopyJobs j{};
    for (int k = 0; k < 5; ++k) {
        j.src[k] = reinterpret_cast<const uint32_t*>(S.dev + k * stage_stride(S.hits));
        j.dst[k] = static_cast<uint32_t*>(dstp[k]);
        j.n[k] = S.n_hit;
    }
    j.src[5] = reinterpret_cast<const uint32_t*>(offs);
    j.dst[5] = reinterpret_cast<uint32_t*>(const_cast<int64_t*>(b.ev_off));
    j.n[5] = (S.n_ev + 1) * 2;
    j.src[6] = reinterpret_cast<const uint32_t*>(offs + (S.n_ev + 1) * sizeof(int64_t));
    j.dst[6] = reinterpret_cast<uint32_t*>(const_cast<int64_t*>(b.n_hit));
    j.n[6] = 2;
    j.count = 7;
    launch_copy_words(j, ctx->n_sm, s);
    CK(cudaGetLastError());
    CK(cudaEventRecord(S.ev_used, s));
    S.used_pending = true;
    ctx->n_ev = S.n_ev;
    ctx->n_hit = S.n_hit;
    ctx->ev_off = S.ev_off;
    ctx->ran = false;
    return SDLG_OK;
}

}  // namespace

extern "C" {

int sdlg_run_async(sdlg_ctx* ctx, int stop_after, int flags) {
    if (!ctx) return SDLG_ERR_ARG;
    if (ctx->stage.pending) {
        cudaSetDevice(ctx->device);
        const int rc = install_staged(ctx);
        if (rc) return rc;
    }
    if (!ctx->have_geo) return fail(ctx, SDLG_ERR_NO_GEOMETRY, "no geometry loaded");
    if (!ctx->buffers_ok || ctx->n_ev <= 0) return fail(ctx, SDLG_ERR_NO_EVENTS, "no events set");
    if (stop_after < 0 || stop_after > 4) return fail(ctx, SDLG_ERR_ARG, "stop_after out of range");
    if ((flags & SDLG_FLAG_MLP) && !ctx->mlp.have) return fail(ctx, SDLG_ERR_ARG, "SDLG_FLAG_MLP without pre-filter parameters");
    cudaSetDevice(ctx->device);
    ctx->last_stop = stop_after;
    ctx->last_flags = flags;
    ctx->ran = true;
    return launch(ctx, stop_after, flags);
}

int sdlg_sync(sdlg_ctx* ctx) {
    if (!ctx) return SDLG_ERR_ARG;
    cudaSetDevice(ctx->device);
    return finish(ctx);
}

int sdlg_run(sdlg_ctx* ctx, int stop_after, int flags) {
    int rc = sdlg_run_async(ctx, stop_after, flags);
    if (rc) return rc;
    return sdlg_sync(ctx);
}

int sdlg_set_capacities(sdlg_ctx* ctx, const int64_t* caps6) {
    if (!ctx || !caps6) return SDLG_ERR_ARG;
    for (int k = 0; k <= kNumStages; ++k)
        if (caps6[k] < 0) return fail(ctx, SDLG_ERR_ARG, "negative capacity");
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    free_batch(ctx);
    for (int k = 0; k < kNumStages; ++k) {
        ctx->cap_init[k] = caps6[k];
        ctx->cap_obj[k] = caps6[k];
    }
    ctx->cap_init[kNumStages] = caps6[kNumStages];
    ctx->cap_kept = caps6[kNumStages];
    ctx->n_ev = 0;
    ctx->ran = false;
    return SDLG_OK;
}

int sdlg_get_capacities(const sdlg_ctx* ctx, int64_t* out6) {
    if (!ctx || !out6) return SDLG_ERR_ARG;
    for (int k = 0; k < kNumStages; ++k) out6[k] = ctx->cap_obj[k];
    out6[kNumStages] = ctx->cap_kept;
    return SDLG_OK;
}

int sdlg_run_stages(sdlg_ctx* ctx, int first, int last, int flags) {
    if (!ctx) return SDLG_ERR_ARG;
    if (first < 0 || last > 4 || first > last) return fail(ctx, SDLG_ERR_ARG, "stages %d..%d out of range", first, last);
    // a first stage right after the last run's final stage continues that
    // run; anything else (no run yet, new events, a stage run again) runs
    // from the hits
    if (first == 0 || !ctx->ran || !ctx->buffers_ok || ctx->last_stop != first - 1) return sdlg_run(ctx, last, flags);
    if ((flags & SDLG_FLAG_MLP) && !ctx->mlp.have) return fail(ctx, SDLG_ERR_ARG, "SDLG_FLAG_MLP without pre-filter parameters");
    cudaSetDevice(ctx->device);
    ctx->b.flags = flags;
    ctx->last_stop = last;
    ctx->last_flags = flags;
    wait_readback(ctx);
#ifdef SDL_DEVICE_CHECKS
    int rc = launch_checked(ctx, last);
    if (rc) return rc;
#else
    enqueue_stages(ctx, first, last);
    CK(cudaGetLastError());
#endif
    return finish(ctx);
}

static int event_range(sdlg_ctx* ctx, int stage, int64_t event, int64_t* first, int64_t* n) {
    if (!ctx->ran) return fail(ctx, SDLG_ERR_NO_EVENTS, "chain not run");
    if (stage < 0 || stage > ctx->last_stop) return fail(ctx, SDLG_ERR_ARG, "stage %d not run", stage);
    if (event >= ctx->n_ev) return fail(ctx, SDLG_ERR_ARG, "event out of range");
    const int64_t n_mod = (int64_t)ctx->detids.size();
    const int64_t a = event < 0 ? 0 : event * n_mod;
    const int64_t z = event < 0 ? ctx->n_ev * n_mod : (event + 1) * n_mod;
    int64_t v[2];
    CK(cudaMemcpyAsync(&v[0], ctx->b.obj[stage].mod_cnt + a, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(&v[1], ctx->b.obj[stage].mod_cnt + z, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    *first = v[0];
    *n = v[1] - v[0];
    return SDLG_OK;
}

int sdlg_get_counts(sdlg_ctx* ctx, int64_t event, int64_t* out5) {
    if (!ctx || !out5) return SDLG_ERR_ARG;
    cudaSetDevice(ctx->device);
    for (int s = 0; s < 5; ++s) {
        out5[s] = 0;
        if (s > ctx->last_stop) continue;
        int64_t f, n;
        int rc = event_range(ctx, s, event, &f, &n);
        if (rc) return rc;
        out5[s] = n;
    }
    return SDLG_OK;
}

int sdlg_get_objects(sdlg_ctx* ctx, int stage, int64_t event, int32_t* out, int64_t cap, int64_t* n_out) {
    if (!ctx || !n_out || cap < 0) return SDLG_ERR_ARG;
    cudaSetDevice(ctx->device);
    int64_t first, n;
    int rc = event_range(ctx, stage, event, &first, &n);
    if (rc) return rc;
    *n_out = n;
    if (n == 0 || !out) return SDLG_OK;  // a NULL out is a size query
    if (cap < n) return fail(ctx, SDLG_ERR_ARG, "output capacity %lld < %lld tuples", (long long)cap, (long long)n);
    static const int width[5] = {2, 4, 8, 8, 16};
    const size_t bytes = (size_t)n * width[stage] * 4;
    // through the device scratch and one copy (measured on the 1.06 GB of a
    // 128-event batch's track candidates: 9 ms, against 26 ms for the kernel
    // writing pinned host memory itself)
    void* tmp = nullptr;
    rc = ensure_scratch(ctx, 0, bytes, &tmp);
    if (rc) return rc;
    if (ctx->copy_pending[0]) CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_copy[0], 0));
    launch_materialize(ctx->b, stage, first, n, static_cast<int32_t*>(tmp), ctx->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, tmp, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SDLG_OK;
}

int sdlg_get_objects_async(sdlg_ctx* ctx, int stage, int64_t event, int32_t* out, int64_t cap, int64_t* n_out) {
    if (!ctx || !n_out || cap < 0) return SDLG_ERR_ARG;
    cudaSetDevice(ctx->device);
    int64_t first, n;
    int rc = event_range(ctx, stage, event, &first, &n);
    if (rc) return rc;
    *n_out = n;
    if (n == 0 || !out) return SDLG_OK;
    if (cap < n) return fail(ctx, SDLG_ERR_ARG, "output capacity %lld < %lld tuples", (long long)cap, (long long)n);
    static const int width[5] = {2, 4, 8, 8, 16};
    const size_t bytes = (size_t)n * width[stage] * 4;
    const int kb = ctx->next_scratch;
    void* tmp = nullptr;
    rc = ensure_scratch(ctx, kb, bytes, &tmp);
    if (rc) return rc;
    ctx->next_scratch ^= 1;
    // the tuples are written into scratch buffer kb on the gather stream,
    // after the run that made them (ev_mat) and after kb's previous copy, two
    // readbacks ago; the copy stream then copies them to the host.  The next
    // run waits for the kernel alone (ev_read, wait_readback), so that the
    // kernel overlaps the next batch's input copy and the copy overlaps the
    // next run
    CK(cudaEventRecord(ctx->ev_mat, ctx->stream));
    CK(cudaStreamWaitEvent(ctx->gather_stream, ctx->ev_mat, 0));
    if (ctx->copy_pending[kb]) CK(cudaStreamWaitEvent(ctx->gather_stream, ctx->ev_copy[kb], 0));
    launch_materialize(ctx->b, stage, first, n, static_cast<int32_t*>(tmp), ctx->gather_stream);
    CK(cudaGetLastError());
    CK(cudaEventRecord(ctx->ev_read, ctx->gather_stream));
    ctx->read_pending = true;
    CK(cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_read, 0));
    CK(cudaMemcpyAsync(out, tmp, bytes, cudaMemcpyDeviceToHost, ctx->copy_stream));
    CK(cudaEventRecord(ctx->ev_copy[kb], ctx->copy_stream));
    ctx->copy_pending[kb] = true;
    return SDLG_OK;
}

int sdlg_wait_objects(sdlg_ctx* ctx) {
    if (!ctx) return SDLG_ERR_ARG;
    cudaSetDevice(ctx->device);
    for (int k = 0; k < 2; ++k) {
        if (ctx->copy_pending[k]) {
            CK(cudaEventSynchronize(ctx->ev_copy[k]));
            ctx->copy_pending[k] = false;
        }
    }
    return SDLG_OK;
}

int sdlg_get_object_links(sdlg_ctx* ctx, int stage, int64_t event, int32_t* links, int32_t* module, float* vals,
                          int64_t cap, int64_t* n_out) {
    if (!ctx || !n_out || cap < 0) return SDLG_ERR_ARG;
    if (event < 0) return fail(ctx, SDLG_ERR_ARG, "object links are per event");
    cudaSetDevice(ctx->device);
    int64_t first, n;
    int rc = event_range(ctx, stage, event, &first, &n);
    if (rc) return rc;
    *n_out = n;
    if (n == 0 || (!links && !module && !vals)) return SDLG_OK;  // a size query
    if (cap < n) return fail(ctx, SDLG_ERR_ARG, "output capacity %lld < %lld objects", (long long)cap, (long long)n);
    // the list the constituents index: hits, mini-doublets, segments
    // (tracklets and triplets), tracklets or triplets (track candidates)
    int64_t lo_first = ctx->ev_off[event];
    if (stage != kMD) {
        const int lower = stage == kSG ? kMD : stage <= kTP ? kSG : ((ctx->b.flags & SDLG_FLAG_TC_FROM_TP) ? kTP : kTL);
        int64_t nl;
        rc = event_range(ctx, lower, event, &lo_first, &nl);
        if (rc) return rc;
    }
    const int nf = ctx->b.obj[stage].nf;
    const size_t b_links = (size_t)n * 2 * sizeof(int32_t), b_mod = (size_t)n * sizeof(int32_t);
    const size_t b_vals = (size_t)n * nf * sizeof(float);
    void* vtmp = nullptr;
    rc = ensure_scratch(ctx, 0, b_links + b_mod + b_vals + 16, &vtmp);
    if (rc) return rc;
    char* tmp = static_cast<char*>(vtmp);
    if (ctx->copy_pending[0]) CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_copy[0], 0));
    int32_t* d_links = links ? reinterpret_cast<int32_t*>(tmp) : nullptr;
    int32_t* d_mod = module ? reinterpret_cast<int32_t*>(tmp + b_links) : nullptr;
    float* d_vals = (vals && nf) ? reinterpret_cast<float*>(tmp + b_links + b_mod) : nullptr;
    launch_links(ctx->b, stage, first, n, lo_first, event * (int64_t)ctx->detids.size(), d_links, d_mod, d_vals,
                 ctx->stream);
    CK(cudaGetLastError());
    if (d_links) CK(cudaMemcpyAsync(links, d_links, b_links, cudaMemcpyDeviceToHost, ctx->stream));
    if (d_mod) CK(cudaMemcpyAsync(module, d_mod, b_mod, cudaMemcpyDeviceToHost, ctx->stream));
    if (d_vals) CK(cudaMemcpyAsync(vals, d_vals, b_vals, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SDLG_OK;
}

int sdlg_get_module_detids(const sdlg_ctx* ctx, uint32_t* out, int64_t cap, int64_t* n_out) {
    if (!ctx || !n_out || cap < 0) return SDLG_ERR_ARG;
    const int64_t n = (int64_t)ctx->detids.size();
    *n_out = n;
    if (!out) return SDLG_OK;
    if (cap < n) return SDLG_ERR_ARG;
    std::memcpy(out, ctx->detids.data(), n * sizeof(uint32_t));
    return SDLG_OK;
}

int sdlg_module_info(uint32_t detid, uint32_t* out11) {
    if (!out11) return SDLG_ERR_ARG;
    const Decoded m = decode(detid);
    const uint32_t v[11] = {m.subdet, m.side, m.layer, m.rod, m.ring, m.module, (uint32_t)m.lower,
                            (uint32_t)m.inverted, m.partner, m.type, m.ltype};
    std::memcpy(out11, v, sizeof(v));
    return valid_module(m) ? SDLG_OK : SDLG_ERR_DETID;
}

// Hit.cc:68-83 with MathUtil.cc:3-27, in the reference's types: float
// products and sums, double sqrt and atan2 rounded to float, Phi_mpi_pi's
// double comparisons, the float acosh (this file is compiled without
// multiply-add contraction)
int sdlg_hit_derived(int64_t n, const float* x, const float* y, const float* z, float* rt, float* phi, float* eta,
                     float* r3) {
    if (n < 0 || (n > 0 && (!x || !y || !z))) return SDLG_ERR_ARG;
    for (int64_t i = 0; i < n; ++i) {
        const float X = x[i], Y = y[i], Z = z[i];
        const float R3 = (float)std::sqrt((double)(X * X + Y * Y + Z * Z));
        const float RT = (float)std::sqrt((double)(X * X + Y * Y));
        float at;
        if (-X != 0) at = (float)std::atan2((double)-Y, (double)-X);
        else if (-Y == 0) at = 0.f;
        else if (-Y > 0) at = (float)(M_PI / 2);
        else at = (float)(-M_PI / 2);
        float p = (float)(M_PI + (double)at);
        if (!std::isnan(p)) {
            while (p >= M_PI) p = (float)((double)p - 2. * M_PI);
            while (p < -M_PI) p = (float)((double)p + 2. * M_PI);
        }
        if (rt) rt[i] = RT;
        if (r3) r3[i] = R3;
        if (phi) phi[i] = p;
        if (eta) eta[i] = (float)((Z > 0) - (Z < 0)) * std::acosh(R3 / RT);
    }
    return SDLG_OK;
}

int sdlg_libm_eval(sdlg_ctx* ctx, int fn, uint32_t start_bits, int64_t n, float* out) {
    if (!ctx || !out || n < 0 || fn < 0 || fn >= kLmCount) return SDLG_ERR_ARG;
    if ((uint64_t)start_bits + (uint64_t)n > (1ull << 32)) return fail(ctx, SDLG_ERR_ARG, "bit patterns past 2^32");
    cudaSetDevice(ctx->device);
    if (n == 0) return SDLG_OK;
    float* d = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&d, n * sizeof(float), ctx->stream);
    if (e != cudaSuccess) return fail(ctx, SDLG_ERR_CUDA, "cudaMallocAsync: %s", cudaGetErrorString(e));
    launch_libm_eval(fn, start_bits, n, d, ctx->n_sm, ctx->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, d, n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaFreeAsync(d, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SDLG_OK;
}

int sdlg_libm_stats(int fn, uint64_t* out3) {
    if (!out3 || fn < 0 || fn >= kLmCount) return SDLG_ERR_ARG;
    libm_stats(fn, out3);
    return SDLG_OK;
}

int sdlg_get_tracklet_vars(sdlg_ctx* ctx, int64_t event, float* out, int64_t cap, int64_t* n_out) {
    if (!ctx || !n_out || cap < 0) return SDLG_ERR_ARG;
    cudaSetDevice(ctx->device);
    int64_t first, n;
    int rc = event_range(ctx, kTL, event, &first, &n);
    if (rc) return rc;
    *n_out = n;
    if (n == 0 || !out) return SDLG_OK;  // a NULL out is a size query
    if (cap < n) return fail(ctx, SDLG_ERR_ARG, "output capacity %lld < %lld tracklets", (long long)cap, (long long)n);
    const size_t bytes = (size_t)n * 15 * sizeof(float);
    float* tmp = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&tmp, bytes, ctx->stream);
    if (e != cudaSuccess) return fail(ctx, SDLG_ERR_CUDA, "cudaMallocAsync: %s", cudaGetErrorString(e));
    launch_tl_vars(ctx->b, first, n, tmp, ctx->stream);
    CK(cudaMemcpyAsync(out, tmp, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaFreeAsync(tmp, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SDLG_OK;
}

int sdlg_tl_phase_a_check(sdlg_ctx* ctx, uint64_t* out4) {
    if (!ctx || !out4) return SDLG_ERR_ARG;
    if (!ctx->ran || ctx->last_stop < kTL) return fail(ctx, SDLG_ERR_ARG, "run the chain through the tracklet stage first");
    cudaSetDevice(ctx->device);
    unsigned long long* d = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&d, 4 * sizeof(unsigned long long), ctx->stream);
    if (e != cudaSuccess) return fail(ctx, SDLG_ERR_CUDA, "cudaMallocAsync: %s", cudaGetErrorString(e));
    CK(cudaMemsetAsync(d, 0, 4 * sizeof(unsigned long long), ctx->stream));
    launch_tl_quick_check(ctx->b, d, ctx->stream);
    CK(cudaGetLastError());
    unsigned long long h[4] = {0, 0, 0, 0};
    CK(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaFreeAsync(d, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    for (int k = 0; k < 4; ++k) out4[k] = h[k];
    return SDLG_OK;
}

int sdlg_get_counters(sdlg_ctx* ctx, int64_t event, uint32_t* out110) {
    if (!ctx || !out110 || event < 0 || event >= ctx->n_ev) return SDLG_ERR_ARG;
    if (!ctx->ran) return fail(ctx, SDLG_ERR_NO_EVENTS, "chain not run");
    cudaSetDevice(ctx->device);
    CK(cudaMemcpyAsync(out110, ctx->b.counters + event * 110, 110 * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SDLG_OK;
}

int sdlg_last_times(sdlg_ctx* ctx, float* out7) {
    if (!ctx || !out7) return SDLG_ERR_ARG;
    cudaSetDevice(ctx->device);
    CK(cudaEventSynchronize(ctx->ev[6]));
    for (int k = 0; k < 6; ++k) CK(cudaEventElapsedTime(&out7[k], ctx->ev[k], ctx->ev[k + 1]));
    CK(cudaEventElapsedTime(&out7[6], ctx->ev[0], ctx->ev[6]));
    return SDLG_OK;
}

int sdlg_last_kernel_times(sdlg_ctx* ctx, float* out5) {
    if (!ctx || !out5) return SDLG_ERR_ARG;
    if (!ctx->ran) return fail(ctx, SDLG_ERR_NO_EVENTS, "chain not run");
    cudaSetDevice(ctx->device);
    for (int k = 0; k < kNumStages; ++k) {
        out5[k] = 0.f;
        if (k > ctx->last_stop) continue;
        CK(cudaEventSynchronize(ctx->hooks.enum_stop[k]));
        CK(cudaEventElapsedTime(&out5[k], ctx->hooks.enum_start[k], ctx->hooks.enum_stop[k]));
    }
    return SDLG_OK;
}

int sdlg_autotune(sdlg_ctx* ctx, int stop_after, int flags, int32_t* out10) {
    if (!ctx) return SDLG_ERR_ARG;
    if (!ctx->have_geo) return fail(ctx, SDLG_ERR_NO_GEOMETRY, "no geometry loaded");
    if (!ctx->buffers_ok || ctx->n_ev <= 0) return fail(ctx, SDLG_ERR_NO_EVENTS, "no events set");
    if (stop_after < 0 || stop_after > 4) return fail(ctx, SDLG_ERR_ARG, "stop_after out of range");
    static const int kTasks[] = {128, 256, 512, 1024};
    static const int kGrids[] = {4, 8, 16};
    float best[kNumStages];
    int bt[kNumStages], bg[kNumStages];
    for (int st = 0; st < kNumStages; ++st) {
        best[st] = 3.4e38f;
        bt[st] = ctx->tune_task[st];
        bg[st] = ctx->tune_grid[st];
    }
    for (int task : kTasks) {
        for (int grid : kGrids) {
            for (int st = 0; st < kNumStages; ++st) {  // (a capacity regrow re-reads the context's values)
                ctx->tune_task[st] = ctx->b.enum_task[st] = task;
                ctx->tune_grid[st] = ctx->b.enum_grid[st] = grid;
            }
            float t[kNumStages];
            for (int rep = 0; rep < 2; ++rep) {  // the second run is timed
                int rc = sdlg_run(ctx, stop_after, flags | SDLG_FLAG_NO_GRAPH);
                if (rc) return rc;
                rc = sdlg_last_kernel_times(ctx, t);
                if (rc) return rc;
            }
            for (int st = 0; st <= stop_after; ++st)
                if (t[st] < best[st]) {
                    best[st] = t[st];
                    bt[st] = task;
                    bg[st] = grid;
                }
        }
    }
    for (int st = 0; st < kNumStages; ++st) {
        ctx->tune_task[st] = bt[st];
        ctx->tune_grid[st] = bg[st];
        ctx->b.enum_task[st] = bt[st];
        ctx->b.enum_grid[st] = bg[st];
        if (out10) {
            out10[st] = bt[st];
            out10[kNumStages + st] = bg[st];
        }
    }
    ctx->graph_stop = -1;  // the launch graph holds the old shapes
    return SDLG_OK;
}

int sdlg_last_tl_pass_times4(sdlg_ctx* ctx, float* out4) {
    if (!ctx || !out4) return SDLG_ERR_ARG;
    if (!ctx->ran) return fail(ctx, SDLG_ERR_NO_EVENTS, "chain not run");
    out4[0] = out4[1] = out4[2] = out4[3] = 0.f;
    if (ctx->last_stop < kTL) return SDLG_OK;
    cudaSetDevice(ctx->device);
    CK(cudaEventSynchronize(ctx->hooks.enum_stop[kTL]));
    CK(cudaEventElapsedTime(&out4[0], ctx->hooks.enum_start[kTL], ctx->hooks.tl_mid[0]));
    CK(cudaEventElapsedTime(&out4[1], ctx->hooks.tl_mid[0], ctx->hooks.tl_mid[1]));
    CK(cudaEventElapsedTime(&out4[2], ctx->hooks.tl_mid[1], ctx->hooks.tl_mid[2]));
    CK(cudaEventElapsedTime(&out4[3], ctx->hooks.tl_mid[2], ctx->hooks.enum_stop[kTL]));
    return SDLG_OK;
}

int sdlg_last_tl_pass_times(sdlg_ctx* ctx, float* out3) {
    if (!out3) return SDLG_ERR_ARG;
    float t[4];
    const int rc = sdlg_last_tl_pass_times4(ctx, t);
    if (rc) return rc;
    out3[0] = t[0];
    out3[1] = t[1] + t[2];
    out3[2] = t[3];
    return SDLG_OK;
}

int sdlg_last_tl_list_counts(sdlg_ctx* ctx, int64_t* out3) {
    if (!ctx || !out3) return SDLG_ERR_ARG;
    if (!ctx->ran) return fail(ctx, SDLG_ERR_NO_EVENTS, "chain not run");
    out3[0] = out3[1] = out3[2] = 0;
    if (ctx->last_stop < kTL) return SDLG_OK;
    cudaSetDevice(ctx->device);
    unsigned long long h[3] = {0, 0, 0};
    CK(cudaMemcpyAsync(&h[0], ctx->b.n_kept, 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(&h[1], ctx->b.n_keptf, 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(&h[2], ctx->b.n_kept2, 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    const bool filt = !(ctx->last_flags & (SDLG_FLAG_TL_NM1 | SDLG_FLAG_NO_B2_FILTER));
    const bool mlp = (ctx->last_flags & SDLG_FLAG_MLP) != 0;
    out3[0] = (int64_t)h[0];
    out3[1] = mlp ? (int64_t)h[2] : 0;
    out3[2] = filt ? (int64_t)h[1] : out3[mlp ? 1 : 0];
    return SDLG_OK;
}

int sdlg_tl_b2_filter_check(sdlg_ctx* ctx, uint64_t* out12) {
    if (!ctx || !out12) return SDLG_ERR_ARG;
    if (!ctx->ran || ctx->last_stop < kTL) return fail(ctx, SDLG_ERR_ARG, "run the chain through the tracklet stage first");
    cudaSetDevice(ctx->device);
    unsigned long long* d = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&d, 12 * sizeof(unsigned long long), ctx->stream);
    if (e != cudaSuccess) return fail(ctx, SDLG_ERR_CUDA, "cudaMallocAsync: %s", cudaGetErrorString(e));
    CK(cudaMemsetAsync(d, 0, 12 * sizeof(unsigned long long), ctx->stream));
    launch_tl_b2q_check(ctx->b, d, ctx->stream);
    CK(cudaGetLastError());
    unsigned long long h[12];
    CK(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaFreeAsync(d, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    for (int k = 0; k < 12; ++k) out12[k] = h[k];
    return SDLG_OK;
}

int64_t sdlg_last_launches(const sdlg_ctx* ctx) { return ctx ? ctx->launches_per_run : -1; }

int sdlg_math_check(sdlg_ctx* ctx, int fn, int exhaustive, uint64_t start, int64_t n, uint64_t seed, uint64_t* out8) {
    if (!ctx || !out8 || n < 0 || fn < 0 || fn > 20) return SDLG_ERR_ARG;
    cudaSetDevice(ctx->device);
    unsigned long long* d = nullptr;
    CK(cudaMalloc(&d, 8 * sizeof(unsigned long long)));
    cudaError_t e = cudaMemsetAsync(d, 0, 8 * sizeof(unsigned long long), ctx->stream);
    if (e == cudaSuccess) {
        launch_math_check(fn, exhaustive, (unsigned long long)start, (long long)n, (unsigned long long)seed, d, ctx->n_sm,
                          ctx->stream);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out8, d, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(d);
    if (e != cudaSuccess) return fail(ctx, SDLG_ERR_CUDA, "math check: %s", cudaGetErrorString(e));
    return SDLG_OK;
}

// ------------------------------------------------------------------ pre-filter
int sdlg_mlp_set_params(sdlg_ctx* ctx, const float* params, float threshold) {
    if (!ctx || !params) return SDLG_ERR_ARG;
    for (int k = 0; k < kMlpParams; ++k)
        if (!std::isfinite(params[k])) return fail(ctx, SDLG_ERR_ARG, "parameter %d is not finite", k);
    cudaSetDevice(ctx->device);
    auto& M = ctx->mlp;
    CK(cudaMemcpy(M.params, params, kMlpParams * sizeof(float), cudaMemcpyHostToDevice));
    CK(cudaMemset(M.m, 0, kMlpParams * sizeof(float)));
    CK(cudaMemset(M.v, 0, kMlpParams * sizeof(float)));
    CK(cudaMemset(M.grad, 0, kMlpParams * sizeof(float)));
    M.adam_t = 0;
    M.thr = threshold;
    M.have = true;
    return mlp_repack(ctx);
}

int sdlg_mlp_get_params(sdlg_ctx* ctx, float* params, float* threshold) {
    if (!ctx) return SDLG_ERR_ARG;
    if (!ctx->mlp.have) return fail(ctx, SDLG_ERR_ARG, "no pre-filter parameters");
    cudaSetDevice(ctx->device);
    if (params) CK(cudaMemcpy(params, ctx->mlp.params, kMlpParams * sizeof(float), cudaMemcpyDeviceToHost));
    if (threshold) *threshold = ctx->mlp.thr;
    return SDLG_OK;
}

int sdlg_mlp_set_threshold(sdlg_ctx* ctx, float threshold) {
    if (!ctx) return SDLG_ERR_ARG;
    if (!ctx->mlp.have) return fail(ctx, SDLG_ERR_ARG, "no pre-filter parameters");
    cudaSetDevice(ctx->device);
    ctx->mlp.thr = threshold;
    return mlp_repack(ctx);
}

int sdlg_mlp_init(sdlg_ctx* ctx, uint64_t seed) {
    if (!ctx) return SDLG_ERR_ARG;
    // uniform fan-in initialisation (He et al. 2015), zero biases
    std::vector<float> p(kMlpParams, 0.f);
    uint64_t st = seed;
    auto u = [&]() { return (double)(splitmix64(st) >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0; };
    const double a1 = std::sqrt(6.0 / kMlpIn), a2 = std::sqrt(6.0 / kMlpHid);
    for (int k = 0; k < kMlpHid * kMlpIn; ++k) p[kMlpW1 + k] = (float)(a1 * u());
    for (int k = 0; k < kMlpHid * kMlpHid; ++k) p[kMlpW2 + k] = (float)(a2 * u());
    for (int k = 0; k < kMlpHid; ++k) p[kMlpW3 + k] = (float)(a2 * u());
    return sdlg_mlp_set_params(ctx, p.data(), 0.f);
}

int sdlg_mlp_collect(sdlg_ctx* ctx, float neg_keep, uint64_t seed, int64_t* n_total) {
    if (!ctx || !(neg_keep >= 0.f && neg_keep <= 1.f)) return SDLG_ERR_ARG;
    if (!ctx->ran || ctx->last_stop < kTL) return fail(ctx, SDLG_ERR_ARG, "run the chain through the tracklet stage first");
    if (ctx->last_flags & SDLG_FLAG_MLP) return fail(ctx, SDLG_ERR_ARG, "collect after a run without SDLG_FLAG_MLP");
    cudaSetDevice(ctx->device);
    auto& M = ctx->mlp;
    for (int attempt = 0; attempt < 2; ++attempt) {
        int rc = mlp_reserve(ctx, M.n + 1);
        if (rc) return rc;
        CK(cudaMemsetAsync(M.found, 0, sizeof(unsigned long long), ctx->stream));
        MlpCollect c;
        c.x = M.x + M.n * kMlpIn;
        c.y = M.y + M.n;
        c.cap = M.cap - M.n;
        c.n = M.found;
        c.neg_keep = neg_keep;
        c.seed = seed;
        launch_tl_collect(ctx->b, c, ctx->stream);
        CK(cudaGetLastError());
        unsigned long long found = 0;
        CK(cudaMemcpyAsync(&found, M.found, sizeof(found), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        if ((int64_t)found <= c.cap) {
            M.n += (int64_t)found;
            if (n_total) *n_total = M.n;
            return SDLG_OK;
        }
        rc = mlp_reserve(ctx, M.n + (int64_t)found);  // the sampling is deterministic: collect again
        if (rc) return rc;
    }
    return fail(ctx, SDLG_ERR_CAPACITY, "sample collection did not fit");
}

int sdlg_mlp_add_samples(sdlg_ctx* ctx, int64_t n, const float* x, const float* y) {
    if (!ctx || n < 0 || (n && (!x || !y))) return SDLG_ERR_ARG;
    cudaSetDevice(ctx->device);
    auto& M = ctx->mlp;
    int rc = mlp_reserve(ctx, M.n + n);
    if (rc) return rc;
    if (n) {
        CK(cudaMemcpy(M.x + M.n * kMlpIn, x, n * kMlpIn * sizeof(float), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(M.y + M.n, y, n * sizeof(float), cudaMemcpyHostToDevice));
    }
    M.n += n;
    return SDLG_OK;
}

int sdlg_mlp_num_samples(sdlg_ctx* ctx, int64_t* n) {
    if (!ctx || !n) return SDLG_ERR_ARG;
    *n = ctx->mlp.n;
    return SDLG_OK;
}

int sdlg_mlp_get_samples(sdlg_ctx* ctx, float* x, float* y, int64_t cap, int64_t* n) {
    if (!ctx || cap < 0) return SDLG_ERR_ARG;
    cudaSetDevice(ctx->device);
    const int64_t k = std::min(cap, ctx->mlp.n);
    if (k && x) CK(cudaMemcpy(x, ctx->mlp.x, k * kMlpIn * sizeof(float), cudaMemcpyDeviceToHost));
    if (k && y) CK(cudaMemcpy(y, ctx->mlp.y, k * sizeof(float), cudaMemcpyDeviceToHost));
    if (n) *n = ctx->mlp.n;
    return SDLG_OK;
}

int sdlg_mlp_clear_samples(sdlg_ctx* ctx) {
    if (!ctx) return SDLG_ERR_ARG;
    ctx->mlp.n = 0;
    return SDLG_OK;
}

int sdlg_mlp_train(sdlg_ctx* ctx, int epochs, int batch, float lr, float pos_weight, uint64_t seed, float* epoch_loss) {
    if (!ctx || epochs < 0 || batch <= 0 || !(lr > 0.f) || !(pos_weight > 0.f)) return SDLG_ERR_ARG;
    auto& M = ctx->mlp;
    if (!M.have) return fail(ctx, SDLG_ERR_ARG, "no pre-filter parameters (sdlg_mlp_init or sdlg_mlp_set_params)");
    if (M.n <= 0) return fail(ctx, SDLG_ERR_ARG, "no training samples");
    if (M.n > INT32_MAX) return fail(ctx, SDLG_ERR_ARG, "too many training samples");
    cudaSetDevice(ctx->device);
    cudaStream_t s = ctx->stream;
    if (M.order_cap < M.n) {
        cudaFree(M.order);
        M.order = nullptr;
        CK(cudaMalloc(&M.order, M.n * sizeof(int32_t)));
        M.order_cap = M.n;
    }
    std::vector<int32_t> order(M.n);
    for (int64_t i = 0; i < M.n; ++i) order[i] = (int32_t)i;
    uint64_t st = seed;
    for (int ep = 0; ep < epochs; ++ep) {
        for (int64_t i = M.n - 1; i > 0; --i) std::swap(order[i], order[splitmix64(st) % (uint64_t)(i + 1)]);
        CK(cudaMemcpyAsync(M.order, order.data(), M.n * sizeof(int32_t), cudaMemcpyHostToDevice, s));
        CK(cudaMemsetAsync(M.loss, 0, sizeof(double), s));
        for (int64_t start = 0; start < M.n; start += batch) {
            const int64_t count = std::min<int64_t>(batch, M.n - start);
            cudaError_t e = launch_mlp_fwd_bwd(M.x, M.y, nullptr, M.order, start, count, pos_weight, 1.f / (float)count,
                                               M.params, M.grad, M.loss, s);
            if (e != cudaSuccess) return fail(ctx, SDLG_ERR_CUDA, "training step: %s", cudaGetErrorString(e));
            ++M.adam_t;
            const float c1 = (float)(1.0 - std::pow(0.9, (double)M.adam_t));
            const float c2 = (float)(1.0 - std::pow(0.999, (double)M.adam_t));
            launch_mlp_adam(M.params, M.grad, M.m, M.v, lr, c1, c2, s);
        }
        double loss = 0.0;
        CK(cudaMemcpyAsync(&loss, M.loss, sizeof(double), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));  // the host order buffer is reused next epoch
        if (epoch_loss) epoch_loss[ep] = (float)(loss / (double)M.n);
    }
    CK(cudaGetLastError());
    return mlp_repack(ctx);
}

int sdlg_mlp_gradient(sdlg_ctx* ctx, int64_t n, const float* x, const float* y, const float* w, float* grad, double* loss) {
    if (!ctx || n <= 0 || !x || !y || !w || !grad) return SDLG_ERR_ARG;
    if (!ctx->mlp.have) return fail(ctx, SDLG_ERR_ARG, "no pre-filter parameters");
    cudaSetDevice(ctx->device);
    auto& M = ctx->mlp;
    float *dx = nullptr, *dy = nullptr, *dw = nullptr;
    int rc = to_device(ctx, x, n * kMlpIn, &dx);
    if (!rc) rc = to_device(ctx, y, n, &dy);
    if (!rc) rc = to_device(ctx, w, n, &dw);
    cudaError_t e = cudaSuccess;
    double l = 0.0;
    if (!rc) {
        cudaMemsetAsync(M.grad, 0, kMlpParams * sizeof(float), ctx->stream);
        cudaMemsetAsync(M.loss, 0, sizeof(double), ctx->stream);
        e = launch_mlp_fwd_bwd(dx, dy, dw, nullptr, 0, n, 1.f, 1.f / (float)n, M.params, M.grad, M.loss, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(grad, M.grad, kMlpParams * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&l, M.loss, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(M.grad, 0, kMlpParams * sizeof(float), ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    }
    cudaFree(dx);
    cudaFree(dy);
    cudaFree(dw);
    if (rc) return rc;
    if (e != cudaSuccess) return fail(ctx, SDLG_ERR_CUDA, "gradient: %s", cudaGetErrorString(e));
    if (loss) *loss = l / (double)n;
    return SDLG_OK;
}

int sdlg_mlp_score(sdlg_ctx* ctx, int64_t n, const float* x, float* logits) {
    if (!ctx || n < 0 || (n && (!x || !logits))) return SDLG_ERR_ARG;
    if (!ctx->mlp.have) return fail(ctx, SDLG_ERR_ARG, "no pre-filter parameters");
    if (!n) return SDLG_OK;
    cudaSetDevice(ctx->device);
    float *dx = nullptr, *dz = nullptr;
    int rc = to_device(ctx, x, n * kMlpIn, &dx);
    if (!rc && cudaMalloc(&dz, n * sizeof(float)) != cudaSuccess) rc = fail(ctx, SDLG_ERR_CUDA, "cudaMalloc");
    cudaError_t e = cudaSuccess;
    unsigned int st = 0;
    if (!rc) {
        cudaMemsetAsync(ctx->mlp.status, 0, sizeof(unsigned int), ctx->stream);
        launch_mlp_score(dx, n, ctx->mlp.pack, dz, ctx->mlp.status, ctx->n_sm, ctx->stream);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(logits, dz, n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&st, ctx->mlp.status, sizeof(st), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    }
    cudaFree(dx);
    cudaFree(dz);
    if (rc) return rc;
    if (e != cudaSuccess) return fail(ctx, SDLG_ERR_CUDA, "score: %s", cudaGetErrorString(e));
    if (st) return fail(ctx, SDLG_ERR_CUDA, "score: a tensor-core wait gave up");
    return SDLG_OK;
}

int sdlg_mlp_stats(sdlg_ctx* ctx, int64_t* out4) {
    if (!ctx || !out4) return SDLG_ERR_ARG;
    cudaSetDevice(ctx->device);
    MlpStats h;
    CK(cudaMemcpy(&h, ctx->mlp.stats, sizeof(h), cudaMemcpyDeviceToHost));
    out4[0] = (int64_t)h.candidates;
    out4[1] = (int64_t)h.scored;
    out4[2] = (int64_t)h.kept;
    out4[3] = (int64_t)h.timeouts;
    return SDLG_OK;
}

}  // extern "C"

// read-only views of a context for sdl_static.cu
namespace sdlg {
bool ctx_geometry(const sdlg_ctx* ctx, Geometry* g, int* device, int* n_sm) {
    if (!ctx || !ctx->have_geo) return false;
    g->n_mod = (int)ctx->detids.size();
    g->n_mod_inv = g->n_mod > 1 ? UINT64_MAX / (uint64_t)g->n_mod + 1 : 0;  // ceil(2^64 / n_mod)
    g->n_conn = (int)ctx->conn_idx.size();
    g->detid = ctx->d_detid;
    g->mod = ctx->d_mod;
    g->conn_off = ctx->d_conn_off;
    g->conn_idx = ctx->d_conn_idx;
    g->slot_run = ctx->d_slot_run;
    g->n_slot_run = (int)ctx->slot_run.size();
    *device = ctx->device;
    *n_sm = ctx->n_sm;
    return true;
}
void* ctx_stream(const sdlg_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }
void ctx_set_error(sdlg_ctx* ctx, const char* msg) {
    if (ctx) ctx->err = msg;
}
}  // namespace sdlg

extern "C" {

int sdlg_host_alloc(sdlg_ctx* ctx, int64_t bytes, void** out) {
    if (!ctx || !out || bytes <= 0) return SDLG_ERR_ARG;
    cudaSetDevice(ctx->device);
    CK(cudaMallocHost(out, (size_t)bytes));
    return SDLG_OK;
}

int sdlg_host_free(sdlg_ctx* ctx, void* p) {
    if (!ctx) return SDLG_ERR_ARG;
    CK(cudaFreeHost(p));
    return SDLG_OK;
}

}  // extern "C"
