// Device buffer layout of one batch of events (host-visible struct of device
// pointers).  All per-module arrays are indexed by the global module index
// gm = event * n_mod + module, so every stage runs over all events of the
// batch in one launch and the objects of one event stay contiguous.
#pragma once
#include <cstdint>

#include "sdl_device.cuh"

namespace sdlg {

enum Stage { kMD = 0, kSG = 1, kTL = 2, kTP = 3, kTC = 4, kNumStages = 5 };

// staging records of one stage: the candidate (inner object i, outer object
// j), the inner object's module and the rank inside that module, plus the
// floats the next stages read.
struct Recs {
    int32_t* i;
    int32_t* j;
    int32_t* g;
    int32_t* rank;
    float* f;      // nf floats per record, SoA: f[k * cap + r]
    int nf;
};

// Dense object arrays grouped by inner module.
struct Objs {
    int32_t* i;    // MD: lower hit | SG: inner MD | TL/TP: inner SG | TC: inner TL
    int32_t* j;    // MD: upper hit | SG: outer MD | TL/TP: outer SG | TC: outer TL
    int32_t* g;    // inner module (gm)
    float* f;      // nf floats SoA (cap stride)
    int nf;
    int64_t* mod_cnt;  // n_gm + 1 counts, scanned in place to offsets
    int64_t cap;
};

struct Geometry {
    int n_mod;
    uint64_t n_mod_inv;      // ceil(2^64 / n_mod) (n_mod > 1): global module index -> event by a multiply-high
    int n_conn;
    const uint32_t* detid;   // sorted
    const ModDev* mod;
    const int32_t* conn_off; // n_mod + 1
    const int32_t* conn_idx;
    // Layers as module-index runs, for the layer-pair variants (Layer.cc:3-50):
    // slot_run[s] .. slot_run[s + 1] are the runs of layer slot s (0-5 barrel
    // layers 1-6, 6-10 endcap layers 1-5); run r spans module indices
    // [slot_run[kNumSlots + 1 + 2r], slot_run[kNumSlots + 2 + 2r]).  Barrel
    // layers are one run of the sorted detIds, endcap layers one run per side.
    const int32_t* slot_run;
    int n_slot_run;          // entries of slot_run
};

constexpr int kNumSlots = 11;

// Chain flags (the SDLG_FLAG_* values of the C ABI)
enum : int {
    kFlagSGLayers = 1,   // createSegments: layer-pair segments
    kFlagTLLayers = 2,   // createTracklets: layer-pair tracklets
    kFlagTLNm1 = 4,      // DefaultNm1_TLAlgo
    kFlagMLP = 16,       // learned pre-filter ahead of the tracklet cuts
    kFlagTLNav = 32,     // createTrackletsViaNavigation
    kFlagTCFromTL = 64,  // createTrackCandidatesFromTracklets
    kFlagTCFromTP = 128, // createTrackCandidatesFromTriplets
    kFlagNoB2Filter = 256,  // phase B2's single-precision filter off
    kFlagTestMlpGiveUp = 4096,  // self-test: the pre-filter's first tensor-core wait of each CTA gives up at once
};

// Per-stage status word bits
enum : uint32_t {
    kStatusOverflowMD = 1u << 0,
    kStatusOverflowSG = 1u << 1,
    kStatusOverflowTL = 1u << 2,
    kStatusOverflowTP = 1u << 3,
    kStatusOverflowTC = 1u << 4,
    kStatusUnknownModule = 1u << 8,
    kStatusPhiLoop = 1u << 9,
    kStatusMlpTimeout = 1u << 10,  // a tensor-core wait of the pre-filter gave up
    kStatusOverflowKept = 1u << 11,  // the pre-filter's list of kept candidates overflowed
    kStatusHalt = 0x1fu | kStatusOverflowKept,  // bits that stop the remaining kernels of a run
};

}  // namespace sdlg
