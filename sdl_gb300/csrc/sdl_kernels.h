// Launchers for the segment-linking kernels (sm_103a).  The host code in
// sdl_capi.cu owns the buffers and calls these in stage order on one stream.
#pragma once
#include <cuda_runtime.h>

#include "sdl_mlp.cuh"
#include "sdl_types.h"

namespace sdlg {

struct BatchDev {
    Geometry geo;
    int n_ev;
    int n_gm;          // n_ev * n_mod
    int64_t n_hit_cap;
    const int64_t* n_hit;   // device scalar
    // inputs (concatenated events)
    const float *in_x, *in_y, *in_z;
    const int32_t* in_idx;
    const uint32_t* in_det;
    const int64_t* ev_off;   // n_ev + 1
    // ingest
    int32_t* hit_gm;
    int32_t* hit_rank;
    int32_t* hit_perm;       // sorted position -> input hit
    int64_t* mod_hit;        // n_gm + 1: counts -> offsets
    // sorted hits (SoA)
    float *hx, *hy, *hz, *hrt, *hphi, *hr3, *ha1, *htf, *htd, *ha3;
    float *hsx, *hsy, *hsz;  // the strip-shift anchor point of an anchoring hit (shift_anchor)
    int32_t *hidx, *hgm;
    // stages
    Objs obj[kNumStages];
    Recs rec[kNumStages];
    int64_t* cand[kNumStages];     // per inner object candidate counts -> offsets (cap_inner + 1)
    int64_t cand_cap[kNumStages];
    int64_t* n_rec;                // kNumStages attempted appends
    int64_t* n_gm_dev;             // device scalar = n_gm
    // connection-list prefix sums of per-module object counts
    int32_t* conn_pref;            // n_ev * n_conn
    int32_t* conn_first;           // n_ev * n_conn: offset of the entry's module's first object
    int64_t* conn_sum;             // n_gm
    float* sgpack;                 // segment cap * PK_N packed records for the tracklet stage
    float* sgouter;                // segment cap * 11, one array per field: what the enumeration reads of an
                                   //   outer segment (lrt, lz, ltd, la1, uphi, flags, 0.1/lrt: SGOuter;
                                   //   lx, ly, ux, uy: load_sgo_xy)
    float* sgfeat;                 // segment cap * kFeatN: the pre-filter's per-segment feature records
    float* mdpack;                 // mini-doublet cap * kMdPack: packed records for the segment stage
    uint32_t* counters;            // n_ev * 110
    uint32_t* status;
    unsigned long long* task;      // kNumStages work counters
    int64_t* scan_tmp;
    int64_t scan_tmp_cap;
    int32_t* bucket;               // first inner object of every 256 consecutive candidates of the running stage
    int64_t bucket_cap;
    int flags;                     // kFlag* bits
    // launch shape of each stage's candidate-evaluation kernel (autotuned):
    // candidates per warp task (a multiple of 32) and CTAs per SM
    int enum_task[kNumStages];
    int enum_grid[kNumStages];
    const unsigned char* mlp_pack; // packed pre-filter weights and threshold (kPackBytes)
    MlpStats* mlp_stats;           // pre-filter counts of the last run
    int4* passa;                   // tracklet candidates through phase A: (inner, outer, algorithm, 1 when
                                   //   phase B1 passed already, else 0)
    int64_t kept_cap;              // entries of each survivor list
    unsigned long long* n_kept;    // phase-A survivors found (can exceed kept_cap: overflow)
    int4* kept;                    // the phase-A survivors the pre-filter kept, as passa
    unsigned long long* n_kept2;
    int4* passf;                   // what phase B2's single-precision decision (tl_b2_quick) left of
                                   //   the enumeration's or the pre-filter's list, as passa
    unsigned long long* n_keptf;
    // join index (triplets, then track candidates): the segments by their inner
    // mini-doublet, then the tracklets by their inner segment's inner mini-doublet
    int64_t* joff;                 // mini-doublet cap + 1: counts -> offsets
    int32_t* jcur;                 // mini-doublet cap: fill cursors
    int32_t* jidx;                 // max(segment cap, tracklet cap): object indices
    int64_t* joff2;                // a second index (createTrackCandidatesFromTriplets: the triplets by their
    int32_t* jcur2;                //   innermost mini-doublet, beside the segments by inner mini-doublet)
    int32_t* jidx2;                // triplet cap
    // module-pair tiles of the module-map tracklet candidates: the segments by
    // the global module of their outer mini-doublet, and the tiles per module
    int64_t* eoff;                 // n_gm + 1: counts -> offsets
    int32_t* ecur;                 // n_gm: fill cursors
    int32_t* eidx;                 // segment cap: segment indices
    int64_t* toff;                 // n_gm + 1: tile counts -> offsets
    int32_t* tile_gm;              // tile_cap: the global module of each tile (when the tiles fit)
    int64_t tile_cap;
    int32_t* olist;                // olist_cap: the segment candidates' outer lists (k_sg_olist_fill; offsets in toff)
    int64_t olist_cap;
    int4* pb;                      // candidates through phase B1: (inner, outer, algorithm, muls bits), BBBB
                                   //   from the front, the others from the back
    unsigned long long* n_pb;      // [2]: BBBB entries, other entries (kept_cap in all)
    int n_sm;
    unsigned long long* dbg;       // bounds-check record (debug builds): count, line, index, limit
};

// Host-side instrumentation of the launches: events around each stage's
// candidate-evaluation kernel and a count of kernels launched.
struct Hooks {
    cudaEvent_t enum_start[kNumStages] = {};
    cudaEvent_t enum_stop[kNumStages] = {};
    cudaEvent_t tl_mid[3] = {};  // after phase A, after the pre-filter, after the B2 filter
    bool timed = false;
    int launches = 0;
};

// stage launchers (each enqueues its kernels on stream s)
void launch_ingest(const BatchDev& b, cudaStream_t s, Hooks* h);
void launch_md(const BatchDev& b, cudaStream_t s, Hooks* h);
void launch_sg(const BatchDev& b, cudaStream_t s, Hooks* h);
void launch_tl(const BatchDev& b, cudaStream_t s, Hooks* h);
void launch_tp(const BatchDev& b, cudaStream_t s, Hooks* h);
void launch_tc(const BatchDev& b, cudaStream_t s, Hooks* h);
// Training samples for the pre-filter from the last run's tracklet step
struct MlpCollect {
    float* x;                  // cap x kMlpIn features
    float* y;                  // cap labels (1: the tracklet cuts accept)
    int64_t cap;
    unsigned long long* n;     // samples found (can exceed cap; nothing past cap is written)
    float neg_keep;            // probability of keeping a rejected candidate
    unsigned long long seed;
};
void launch_tl_collect(const BatchDev& b, const MlpCollect& c, cudaStream_t s);
// self-check of the float-float fast paths (out[8]: see k_math_check)
void launch_math_check(int fn, int exhaustive, unsigned long long start, long long n, unsigned long long seed,
                       unsigned long long* out, int n_sm, cudaStream_t s);
// self-check of phase A's single-precision decision (out[4]: see k_tl_quick_check)
void launch_tl_b2q_check(const BatchDev& b, unsigned long long* out, cudaStream_t s);
void launch_tl_quick_check(const BatchDev& b, unsigned long long* out, cudaStream_t s);
// final cut variables of tracklets [first, first + n) (15 floats each, the kTLVar* order)
void launch_tl_vars(const BatchDev& b, int64_t first, int64_t n, float* out, cudaStream_t s);
// the host libm's float functions on the device (sdl_libm.cu): build the
// tables once per process, upload them once per device and point this
// module's kernels at them (call with the device current); the host tables'
// size, moved entries and exceptions of function fn; the device's values on
// consecutive float bit patterns; the constant-memory setter
int libm_setup(int device, const char** err);
void libm_stats(int fn, uint64_t* out3);
void launch_libm_eval(int fn, uint32_t start, int64_t n, float* out, int n_sm, cudaStream_t s);
cudaError_t set_libm_tables(const LibmTab* t);
// object graph of stage st for objects [first, first + n) of one event (see k_links)
void launch_links(const BatchDev& b, int st, int64_t first, int64_t n, int64_t lo_first, int64_t gm0, int32_t* links,
                  int32_t* module, float* vals, cudaStream_t s);
// hit-index tuples of stage st for objects [first, first + n) into out (width 2/4/8/8/16)
void launch_materialize(const BatchDev& b, int st, int64_t first, int64_t n, int32_t* out, cudaStream_t s);

// device-to-device copies of 4-byte words on the SMs, one kernel for up to
// kCopyJobs buffers (the copy engines may be busy with readbacks)
constexpr int kCopyJobs = 8;
struct CopyJobs {
    const uint32_t* src[kCopyJobs];
    uint32_t* dst[kCopyJobs];
    int64_t n[kCopyJobs];  // words
    int count;
};
void launch_copy_words(const CopyJobs& j, int n_sm, cudaStream_t s);

}  // namespace sdlg
