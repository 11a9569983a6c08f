// Mini-doublets of one event with no device allocation: the working memory
// lives in a fixed array compiled into the library instead of coming from
// cudaMalloc.
//
// Some callers cannot allocate device memory while they process events: a
// framework that hands out all device memory at start-up from its own pool
// and forbids allocation afterwards (online trigger farms run this way so
// that a busy node never stalls or fails in the middle of an event), and
// plugins whose host application owns the device allocator.
// sdlg_mini_doublets_static serves them: inputs and outputs are the caller's
// device buffers and everything else comes from the array below.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/sdl_gpu.h"
#include "sdl_kernels.h"

namespace sdlg {
bool ctx_geometry(const sdlg_ctx* ctx, Geometry* g, int* device, int* n_sm);
void* ctx_stream(const sdlg_ctx* ctx);
void ctx_set_error(sdlg_ctx* ctx, const char* msg);
}  // namespace sdlg

using namespace sdlg;

namespace {

// Limits of one call; the array size follows from them (kBytes = 18,875,496
// bytes, about 18 MiB, held on every GPU that loads this library until the
// process exits).
constexpr int64_t kMaxHits = SDLG_STATIC_MAX_HITS;
constexpr int64_t kMaxModules = SDLG_STATIC_MAX_MODULES;
constexpr int64_t kMaxMD = SDLG_STATIC_MAX_MINI_DOUBLETS;
constexpr int64_t kScanTmp = kMaxModules / 4096 + 16;

// Layout of the array, in 8-byte words.
constexpr int64_t kSmall = 0;                                   // n_hit, n_gm, n_rec[5]
constexpr int64_t kEvOff = 16;                                  // ev_off[2]
constexpr int64_t kModHit = kEvOff + 2;                         // kMaxModules + 1
constexpr int64_t kCandMD = kModHit + kMaxModules + 1;          // kMaxModules + 1
constexpr int64_t kModCnt = kCandMD + kMaxModules + 1;          // kMaxModules + 1
constexpr int64_t kScan = kModCnt + kMaxModules + 1;            // kScanTmp
constexpr int64_t kWords64 = (kScan + kScanTmp + 31) / 32 * 32;  // 256-byte multiple: the 4-byte regions start aligned
// 4-byte regions follow the 8-byte ones
constexpr int64_t kHitArrays = 18;                              // hit_gm, hit_rank, hit_perm and 15 sorted arrays
constexpr int64_t kObjWords = 3 + 4;                            // i, j, g, f[4]
constexpr int64_t kRecWords = 4 + 4;                            // i, j, g, rank, f[4]
constexpr int64_t kWords32Raw = kHitArrays * kMaxHits + (kObjWords + kRecWords) * kMaxMD + 110 + 1;
constexpr int64_t kWords32 = (kWords32Raw + 63) / 64 * 64;  // 256-byte multiple: the 8-byte tail starts aligned
constexpr int64_t kBytes = kWords64 * 8 + kWords32 * 4 + 8 * (5 + 8);
static_assert(kBytes == 18875496, "the documented size of the fixed array (include/sdl_gpu.h)");

static __device__ __align__(256) unsigned char g_scratch[kBytes];

std::mutex g_mu;
void* g_addr[128] = {};  // device address of g_scratch per device ordinal

// first call on a device: look up the array's device address (the host-side
// symbol is only a stand-in and must not be passed to kernels)
int scratch_address(int device, void** out) {
    if (device < 0 || device >= 128) return SDLG_ERR_ARG;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess || !p) return SDLG_ERR_CUDA;
        g_addr[device] = p;
    }
    *out = g_addr[device];
    return SDLG_OK;
}

__global__ void k_static_init(BatchDev b, int64_t n_hits) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        *const_cast<int64_t*>(b.n_hit) = n_hits;
        *b.n_gm_dev = b.n_gm;
        int64_t* eo = const_cast<int64_t*>(b.ev_off);
        eo[0] = 0;
        eo[1] = n_hits;
    }
}

// hit-index pairs of the mini-doublets into the caller's buffer, the count
// and the status word
__global__ void k_static_out(BatchDev b, int32_t* pairs, int64_t cap, int64_t* count, uint32_t* status) {
    const int64_t n = b.obj[kMD].mod_cnt[b.n_gm];
    const uint32_t st = *b.status;
    const bool ok = (st & 0x1fu) == 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *count = ok ? n : b.n_rec[kMD];
        *status = st;
    }
    if (!ok) return;
    const int64_t m = n < cap ? n : cap;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < m; k += (int64_t)gridDim.x * blockDim.x) {
        pairs[2 * k] = b.hidx[b.obj[kMD].i[k]];
        pairs[2 * k + 1] = b.hidx[b.obj[kMD].j[k]];
    }
}

}  // namespace

extern "C" int sdlg_mini_doublets_static(sdlg_ctx* ctx, int64_t n_hits, const float* d_x, const float* d_y,
                                         const float* d_z, const int32_t* d_idx, const uint32_t* d_detid,
                                         int32_t* d_pairs, int64_t pair_cap, int64_t* d_count, uint32_t* d_status,
                                         void* stream) {
    Geometry geo;
    int device = 0, n_sm = 0;
    if (!ctx) return SDLG_ERR_ARG;
    if (!ctx_geometry(ctx, &geo, &device, &n_sm)) {
        ctx_set_error(ctx, "no geometry loaded");
        return SDLG_ERR_NO_GEOMETRY;
    }
    if (n_hits < 0 || pair_cap < 0 || !d_count || !d_status || (n_hits > 0 && (!d_x || !d_y || !d_z || !d_idx || !d_detid)) ||
        (pair_cap > 0 && !d_pairs)) {
        ctx_set_error(ctx, "invalid argument");
        return SDLG_ERR_ARG;
    }
    char msg[256];
    if (n_hits > kMaxHits) {
        snprintf(msg, sizeof(msg), "%lld hits exceed the static limit of %lld per call", (long long)n_hits, (long long)kMaxHits);
        ctx_set_error(ctx, msg);
        return SDLG_ERR_CAPACITY;
    }
    if (geo.n_mod > kMaxModules) {
        snprintf(msg, sizeof(msg), "%d modules exceed the static limit of %lld", geo.n_mod, (long long)kMaxModules);
        ctx_set_error(ctx, msg);
        return SDLG_ERR_CAPACITY;
    }
    if (cudaSetDevice(device) != cudaSuccess) {
        ctx_set_error(ctx, "cudaSetDevice failed");
        return SDLG_ERR_CUDA;
    }
    void* base = nullptr;
    if (scratch_address(device, &base) != SDLG_OK) {
        ctx_set_error(ctx, "cudaGetSymbolAddress of the static scratch array failed");
        return SDLG_ERR_CUDA;
    }
    cudaStream_t s = stream ? (cudaStream_t)stream : (cudaStream_t)ctx_stream(ctx);
    // carve the array
    int64_t* w64 = static_cast<int64_t*>(base);
    int32_t* w32 = reinterpret_cast<int32_t*>(w64 + kWords64);
    float* f32 = reinterpret_cast<float*>(w32);
    const int64_t H = kMaxHits;
    BatchDev b{};
    b.geo = geo;
    b.n_ev = 1;
    b.n_gm = geo.n_mod;
    b.n_hit_cap = H;
    b.n_hit = w64 + kSmall;
    b.n_gm_dev = w64 + kSmall + 1;
    b.n_rec = w64 + kSmall + 2;
    b.ev_off = w64 + kEvOff;
    b.in_x = d_x; b.in_y = d_y; b.in_z = d_z; b.in_idx = d_idx; b.in_det = d_detid;
    b.mod_hit = w64 + kModHit;
    b.cand[kMD] = w64 + kCandMD;
    b.cand_cap[kMD] = geo.n_mod;
    b.scan_tmp = w64 + kScan;
    b.scan_tmp_cap = kScanTmp;
    int64_t o = 0;
    b.hit_gm = w32 + o; o += H;
    b.hit_rank = w32 + o; o += H;
    b.hit_perm = w32 + o; o += H;
    float** hf[13] = {&b.hx, &b.hy, &b.hz, &b.hrt, &b.hphi, &b.hr3, &b.ha1, &b.htf, &b.htd, &b.ha3, &b.hsx, &b.hsy, &b.hsz};
    for (float** f : hf) { *f = f32 + o; o += H; }
    b.hidx = w32 + o; o += H;
    b.hgm = w32 + o; o += H;
    Objs& O = b.obj[kMD];
    O.cap = kMaxMD; O.nf = 4;
    O.i = w32 + o; o += kMaxMD;
    O.j = w32 + o; o += kMaxMD;
    O.g = w32 + o; o += kMaxMD;
    O.f = f32 + o; o += 4 * kMaxMD;
    O.mod_cnt = w64 + kModCnt;
    Recs& R = b.rec[kMD];
    R.nf = 4;
    R.i = w32 + o; o += kMaxMD;
    R.j = w32 + o; o += kMaxMD;
    R.g = w32 + o; o += kMaxMD;
    R.rank = w32 + o; o += kMaxMD;
    R.f = f32 + o; o += 4 * kMaxMD;
    b.counters = reinterpret_cast<uint32_t*>(w32 + o); o += 110;
    b.status = reinterpret_cast<uint32_t*>(w32 + o); o += 1;
    unsigned long long* tail = reinterpret_cast<unsigned long long*>(reinterpret_cast<unsigned char*>(base) + kWords64 * 8 + kWords32 * 4);
    b.task = tail;
    b.dbg = tail + 5;
    b.n_sm = n_sm;
    b.flags = 0;
    // the array keeps the previous call's contents: zero what the kernels
    // accumulate into
    cudaMemsetAsync(b.status, 0, sizeof(uint32_t), s);
    cudaMemsetAsync(b.n_rec, 0, kNumStages * sizeof(int64_t), s);
    cudaMemsetAsync(b.task, 0, kNumStages * sizeof(unsigned long long), s);
    cudaMemsetAsync(b.dbg, 0, 8 * sizeof(unsigned long long), s);
    cudaMemsetAsync(b.counters, 0, 110 * sizeof(uint32_t), s);
    cudaMemsetAsync(b.mod_hit, 0, (geo.n_mod + 1) * sizeof(int64_t), s);
    cudaMemsetAsync(O.mod_cnt, 0, (geo.n_mod + 1) * sizeof(int64_t), s);
    k_static_init<<<1, 32, 0, s>>>(b, n_hits);
    launch_ingest(b, s, nullptr);
    launch_md(b, s, nullptr);
    k_static_out<<<n_sm * 4, 256, 0, s>>>(b, d_pairs, pair_cap, d_count, d_status);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        snprintf(msg, sizeof(msg), "launch failed: %s", cudaGetErrorString(e));
        ctx_set_error(ctx, msg);
        return SDLG_ERR_CUDA;
    }
    return SDLG_OK;
}
