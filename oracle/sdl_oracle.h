/*
 * CPU restatement of the reference segment-linking chain -- TEST
 * INFRASTRUCTURE ONLY.  Nothing in the product links this; the GPU parity
 * tests, smoke() and the benchmark's CPU-baseline leg use it as the checker.
 *
 * It restates, in the reference's precision and operation order, the live
 * code of Hit.cc:68-183, MathUtil.cc:3-27, GeometryUtil.cc:3-23,
 * Module.cc:159-358, MiniDoublet.cc:60-81,228-684,741-810,989-1209,1242-1332,
 * Segment.cc:337-994, Tracklet.cc:144-301,902-2665,3181-3331,
 * Triplet.cc:50-122, TrackCandidate.cc:143-226 and the stage drivers of
 * Event.cc:120-139,245-305,432-872.  It is pinned against the compiled
 * reference (oracle/_ref) on the committed golden fixtures.
 *
 * Output: per stage (0 MD, 1 SG, 2 TL, 3 TP, 4 TC) a list of hit-index tuples
 * of width 2, 4, 8, 8, 16, and the reference's per-layer counters
 * (5 stages x {candidates, objects} x {barrel[6], endcap[5]}).
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Geometry: tilted rows (detid, drdz, slope); endcap rows (detid, 8 values in
 * file column order: avgr2 yl sl yh sh c7 c8 cz); connection map as CSR
 * (keys[nk], off[nk+1], dst[off[nk]]). Later rows win for repeated keys, as
 * the reference's load() does. */
void* sdlo_geometry_create(int64_t n_tilted, const uint32_t* t_detid, const float* t_vals,
                           int64_t n_endcap, const uint32_t* e_detid, const float* e_vals,
                           int64_t n_keys, const uint32_t* keys, const int64_t* off,
                           const uint32_t* dst);
void sdlo_geometry_free(void* geo);

/* mode bit 0: layer-pair segments (createSegments) instead of module map;
 * bit 1: layer-pair tracklets (createTracklets) instead of module map;
 * bit 2: DefaultNm1 tracklet algorithm (no deltaBeta rejection);
 * bit 5 (32): tracklets via navigation (createTrackletsViaNavigation);
 * bit 6 (64): track candidates from tracklets (createTrackCandidatesFromTracklets);
 * bit 7 (128): track candidates from triplets (createTrackCandidatesFromTriplets).
 * stop_after: last stage to run (0 MD .. 4 TC). */
void* sdlo_run(const void* geo, int64_t n, const float* x, const float* y, const float* z,
               const int32_t* idx, const uint32_t* detid, int mode, int stop_after);
int64_t sdlo_count(const void* res, int stage);
int sdlo_width(int stage);
void sdlo_copy(const void* res, int stage, int32_t* out);
void sdlo_counters(const void* res, uint32_t* out110);
/* per-object floats in tuple order: stage 0 (mini-doublets) dz, shiftedDz,
 * dphi, dphichange; stage 1 (segments) dphi, dphimin, dphimax, dphichange,
 * dphiminchange, dphimaxchange */
void sdlo_vals(const void* res, int stage, float* out);
void sdlo_times(const void* res, double* out5);
void sdlo_free(void* res);

/* Near-cut audit of one event: the chain with the reference's float libm
 * (glibc) and with correctly rounded floats; every object only one of them
 * makes is written to out (cap records of sdlo_audit_record_size() bytes:
 * int32 stage, accepted with glibc, primary, pad, tuple[8] (-1 padded),
 * float value, lo, hi of the rejecting cut with glibc, the same with rounded
 * floats, char where[24], char cut[88]); summary20 = per stage {objects with
 * glibc, objects rounded, primary flips, secondary flips}.  Returns the
 * number of records (may exceed cap). */
int64_t sdlo_audit(const void* geo, int64_t n, const float* x, const float* y, const float* z, const int32_t* idx,
                   const uint32_t* detid, int mode, void* out, int64_t cap, int64_t* summary20);
int sdlo_audit_record_size(void);

/* Float libm used for the reference's std::asin/atan/sin/cos/tan on floats
 * (process-wide, read at the start of each event): 0 glibc's float functions
 * (the reference's; the default), 1 the correctly rounded float (the double
 * function rounded once: the GPU chain's arithmetic), 2 glibc's values while
 * counting the calls whose correctly rounded value differs.
 * sdlo_libm_counts: out2 = {calls counted, calls that differ} since the last
 * reset (mode 2). */
void sdlo_set_libm(int mode);
/* The host libm's float function fn (0 asin, 1 atan, 2 sin, 3 cos, 4 tan)
 * on the n floats with bit patterns start_bits .. start_bits + n - 1. */
void sdlo_libm_values(int fn, uint32_t start_bits, int64_t n, float* out, int n_threads);
void sdlo_libm_counts(uint64_t* out2, int reset);

/* Thread-parallel helper for the CPU baseline: runs n_events independent
 * events (CSR over the concatenated hit arrays) on n_threads threads and
 * returns the total number of track candidates. */
int64_t sdlo_run_many(const void* geo, int64_t n_events, const int64_t* ev_off, const float* x,
                      const float* y, const float* z, const int32_t* idx, const uint32_t* detid,
                      int mode, int n_threads);

/* The same, keeping per event e and stage s the object count
 * counts[5e+s], an order-independent digest of the object multiset
 * digests[5e+s] (sum mod 2^64 of a 64-bit mix of each hit-index tuple; the
 * numpy twin is sdl_gb300/tuples.py) and the 110 per-layer counters
 * counters[110e..]. */
int64_t sdlo_run_many_digest(const void* geo, int64_t n_events, const int64_t* ev_off, const float* x,
                             const float* y, const float* z, const int32_t* idx, const uint32_t* detid,
                             int mode, int n_threads, int64_t* counts, uint64_t* digests, uint32_t* counters);

#ifdef __cplusplus
}
#endif
