/*
 * sdl_gpu.h - C ABI of the GB300 segment-linking chain (libsdlgpu.so).
 *
 * The reference library (bsathian/SDL) is a C++ class library with no FFI of
 * its own; a caller loads three geometry singletons, adds hits to an
 * SDL::Event and calls the create* stages.  Each entry point below replaces
 * one step of that call sequence (file:line of the reference interface in
 * brackets) with plain pointers and sizes, so it can be bound from C, C++
 * (see sdl_event.hpp), Python ctypes, or any other FFI.
 *
 * Conventions: every function returns SDLG_OK (0) or a negative SDLG_ERR_*
 * code and never throws; sdlg_last_error() describes the last failure of a
 * context.  A context owns one CUDA stream and all of its device memory; the
 * functions of one context must not be called concurrently.  Host buffers
 * are caller-owned and only read/written during the call.
 *
 * Objects are reported as hit-index tuples (the idx the caller gave each hit):
 *   mini-doublet (lower, upper)                               width 2
 *   segment      (inner MD, outer MD)                         width 4
 *   tracklet / triplet (inner segment, outer segment)         width 8
 *   track candidate (inner tracklet, outer tracklet)          width 16
 * which is the identity the reference's isIdxMatched() uses
 * (Hit.cc:175-182, MiniDoublet.cc:686-693, Segment.cc:868-875).
 */
#ifndef SDL_GPU_H
#define SDL_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SDLG_OK 0
#define SDLG_ERR_ARG (-1)          /* invalid argument */
#define SDLG_ERR_CUDA (-2)         /* CUDA runtime error (message in sdlg_last_error) */
#define SDLG_ERR_NO_GEOMETRY (-3)  /* sdlg_geometry_* not called yet */
#define SDLG_ERR_NO_EVENTS (-4)    /* sdlg_set_events not called yet */
#define SDLG_ERR_IO (-5)           /* geometry file unreadable */
#define SDLG_ERR_DETID (-6)        /* detId that does not decode to a barrel/endcap module */
#define SDLG_ERR_CAPACITY (-7)     /* object capacity could not be grown (device memory) */
#define SDLG_ERR_DUP_IDX (-8)      /* reserved */
#define SDLG_ERR_NO_DEVICE (-9)    /* no CUDA device */

/* stages (create* order) */
#define SDLG_STAGE_MD 0
#define SDLG_STAGE_SG 1
#define SDLG_STAGE_TL 2
#define SDLG_STAGE_TP 3
#define SDLG_STAGE_TC 4

/* run flags */
#define SDLG_FLAG_SG_LAYERS 1 /* segments by layer pairs: Event::createSegments (Event.cc:432-443,793-821;
                                 pair table Layer.cc:32-50) instead of createSegmentsWithModuleMap */
#define SDLG_FLAG_TL_LAYERS 2 /* tracklets by layer pairs: Event::createTracklets (Event.cc:599-609,755-790;
                                 pair table Layer.cc:3-30) instead of createTrackletsWithModuleMap */
#define SDLG_FLAG_TL_NM1 4   /* tracklets with DefaultNm1_TLAlgo (Algo.h:23-28) */
#define SDLG_FLAG_NO_GRAPH 8 /* launch stage by stage instead of replaying a CUDA graph */
#define SDLG_FLAG_MLP 16     /* learned pre-filter ahead of the tracklet cuts (no counterpart in the reference) */
#define SDLG_FLAG_TL_NAV 32  /* tracklets via navigation: Event::createTrackletsViaNavigation (Event.cc:694-751):
                                inner segment x segments leaving its outer MD x segments leaving theirs */
#define SDLG_FLAG_TC_FROM_TL 64  /* track candidates: Event::createTrackCandidatesFromTracklets (Event.cc:984-1062) */
#define SDLG_FLAG_TC_FROM_TP 128 /* track candidates from two triplets and a trial segment between them:
                                    Event::createTrackCandidatesFromTriplets (Event.cc:874-982); the objects
                                    of stage 4 are then pairs of triplets (hit tuples of width 16 as before) */
#define SDLG_FLAG_NO_B2_FILTER 256 /* the exact phases B1 and B2 judge every survivor of the enumeration (or
                                    * of the pre-filter), without the single-precision phase-B2 filter
                                    * ahead of them (the same tracklets; no counterpart in the reference) */
#define SDLG_FLAG_TEST_MLP_GIVE_UP 4096 /* self-test of a failure path (no counterpart in the reference): with
                                    SDLG_FLAG_MLP, the pre-filter's first tensor-core wait in each CTA gives up at
                                    once, as a wait that ran out of time would; the run fails with SDLG_ERR_CUDA,
                                    sdlg_mlp_stats counts the waits that gave up, the context stays usable */

typedef struct sdlg_ctx sdlg_ctx;

/* Create a context on CUDA device `device` (new SDL::Event's device state). */
int sdlg_create(sdlg_ctx** out, int device);
int sdlg_destroy(sdlg_ctx* ctx);
const char* sdlg_last_error(const sdlg_ctx* ctx);

/* Load the three geometry text files in the reference's formats:
 * replaces SDL::tiltedGeometry.load (TiltedGeometry.cc:18-41),
 * SDL::endcapGeometry.load (EndcapGeometry.cc:18-61; the 7th column is the
 * centroid phi) and SDL::moduleConnectionMap.load (ModuleConnectionMap.cc:18-47).
 * Any path may be NULL (empty table, as an unloaded singleton). */
int sdlg_geometry_load_files(sdlg_ctx* ctx, const char* tilted_path, const char* endcap_path,
                             const char* map_path);

/* Same tables as arrays: tilted rows (detid, drdz, slope); endcap rows
 * (detid, 8 floats in file column order avgr2 yl sl yh sh c7 c8 cz); the map
 * as CSR keys[n_keys], off[n_keys+1], dst[off[n_keys]].  Later rows win for
 * repeated keys, as in the reference's load(). */
int sdlg_geometry_upload(sdlg_ctx* ctx, int64_t n_tilted, const uint32_t* t_detid, const float* t_vals,
                         int64_t n_endcap, const uint32_t* e_detid, const float* e_vals, int64_t n_keys,
                         const uint32_t* keys, const int64_t* off, const uint32_t* dst);

/* Binary geometry (no counterpart in the reference): the three tables in one
 * file that loads without text parsing.  sdlg_geometry_convert parses the
 * text files (as sdlg_geometry_load_files; any path may be NULL) and writes
 * the binary file; it needs no context and no device.  Layout (little
 * endian): "SDLGEO1" and a zero byte; uint64 n, then n x {uint32 detid,
 * float drdz, float slope} (tilted); uint64 n, then n x {uint32 detid, float
 * slope lower, float centroid phi} (endcap); uint64 n_keys, then n_keys x
 * {uint32 detid, uint32 count}, then the uint32 connected detids of all keys
 * in key order.  Rows are in detid order. */
int sdlg_geometry_convert(const char* tilted_path, const char* endcap_path, const char* map_path, const char* out_path);
int sdlg_geometry_load_binary(sdlg_ctx* ctx, const char* path);

/* Starting object capacities (no counterpart in the reference): caps6 =
 * mini-doublets, segments, tracklets, triplets, track candidates, and
 * tracklet candidates through the enumeration's cuts; 0 = the default (a
 * multiple of the batch's hit count).  Capacities grow by themselves when a
 * run overflows them (the run is repeated), so small values only cost time;
 * they exist to exercise that path.  Frees the batch buffers: call
 * sdlg_set_events next.  sdlg_get_capacities: the current ones. */
int sdlg_set_capacities(sdlg_ctx* ctx, const int64_t* caps6);
int sdlg_get_capacities(const sdlg_ctx* ctx, int64_t* out6);

/* Straight-line module connection map on the GPU (no counterpart in the
 * reference, which reads its map from a text file, ModuleConnectionMap.cc:
 * 18-47; this builds one for a detector of barrel cylinders with modules
 * tiled in phi and z -- layers 1-3 tilted beyond |z| = flat_zmax_tilted when
 * has_tilt -- and endcap disks of rings tiled in phi, the detId layout of
 * Module.cc:159-358).  For every lower module, straight lines from five
 * vertex positions z0 in [-lum_z, lum_z] through a 3 x 3 grid of its points
 * (0 and +-98 % of its half extents) are extended to the next barrel layer,
 * or the first disk when they leave the barrel, or the next disk; each
 * crossing, also turned by +- the bend of a track of radius radius_1gev
 * between the two radii, connects the lower module that covers it.  Inputs:
 * n lower modules with detid, kind (0 flat barrel, 1 tilted barrel, 2
 * endcap) and 16 doubles of geometry each (centre xyz, in-plane tangential
 * axis xyz, in-plane long axis xyz, half width, half length, ring inner and
 * outer radius, centre phi, half phi width, tilt angle).  Output: the map as
 * CSR in detId order (keys[n_keys], off[n_keys + 1], dst[n_dst], the
 * connected detIds of each key sorted), the sdlg_geometry_upload layout;
 * all NULL: a size query.  Runs on CUDA device `device`; needs no context. */
typedef struct sdlg_line_map_layout {
    double barrel_r[6];
    int32_t barrel_nphi[6];
    double zmax, module_dz, flat_zmax_tilted, lum_z, radius_1gev;
    int32_t n_tilt_rings, has_tilt, has_endcap;
    double disk_z[5];
    int32_t disk_nrings[5];
    double ec_rmin, ec_rmax;
} sdlg_line_map_layout;
int sdlg_build_line_map(int device, const sdlg_line_map_layout* layout, int64_t n, const uint32_t* detid,
                        const int8_t* kind, const double* geom, int64_t cap_keys, int64_t cap_dst, uint32_t* keys,
                        int64_t* off, uint32_t* dst, int64_t* n_keys, int64_t* n_dst);

/* Number of modules in the device module table. */
int64_t sdlg_num_modules(const sdlg_ctx* ctx);

/* Set the hits of a batch of n_events events (replaces
 * SDL::Event::addHitToModule, Event.cc:120-139, for every hit).  Event e owns
 * hits [ev_off[e], ev_off[e+1]) of the concatenated arrays.  Host buffers; the
 * copy to the device is issued on the context stream (pinned buffers from
 * sdlg_host_alloc are copied directly, others through a pinned staging
 * buffer).  Hit idx values must be unique within an event. */
int sdlg_set_events(sdlg_ctx* ctx, int64_t n_events, const int64_t* ev_off, const float* x, const float* y,
                    const float* z, const int32_t* idx, const uint32_t* detid);

/* The next batch (arguments as sdlg_set_events; no counterpart in the
 * reference), copied to the device while a run of the current batch may
 * still be going: on its own stream into a device staging area, returning
 * once the host buffers have been read.  The next run from the hits
 * (sdlg_run, sdlg_run_async, sdlg_autotune, sdlg_run_stages from stage 0)
 * first copies it into the batch buffers on the device and takes it as its
 * events; until then the current batch's results stay readable.  A batch
 * whose event count differs from the current one, or whose hits exceed the
 * buffers, waits on the host and takes sdlg_set_events' path at that run.
 * sdlg_set_events drops a staged batch.  The streaming pattern: set the
 * first batch, then per batch sdlg_run_async, sdlg_stage_events of the next
 * one, sdlg_sync, sdlg_get_objects_async. */
int sdlg_stage_events(sdlg_ctx* ctx, int64_t n_events, const int64_t* ev_off, const float* x, const float* y,
                      const float* z, const int32_t* idx, const uint32_t* detid);

/* Run the chain createMiniDoublets -> createSegmentsWithModuleMap ->
 * createTrackletsWithModuleMap -> createTriplets -> createTrackCandidates
 * (Event.cc:245-305, 445-522, 611-693, 524-597, 823-872) on every event of
 * the batch, up to and including stage `stop_after`.  Synchronous: returns
 * when the results are on the device.  Object capacities grow automatically.
 * `flags` selects the variants: SDLG_FLAG_SG_LAYERS / SDLG_FLAG_TL_LAYERS
 * replace the module-map segment / tracklet steps by the layer-pair ones
 * (createSegments / createTracklets; these count no segment candidates or
 * segments in the per-layer counters, as in the reference), SDLG_FLAG_TL_NM1
 * selects DefaultNm1_TLAlgo, SDLG_FLAG_NO_GRAPH launches without a graph. */
int sdlg_run(sdlg_ctx* ctx, int stop_after, int flags);

/* Run stages first..last of the chain (0 MD .. 4 TC), one create* call at a
 * time, as the reference's Event::create* methods do (Event.cc:245-305,
 * 445-522, 611-693, 524-597, 823-872): when `first` is the stage right
 * after the last run's final stage, only stages first..last run, on the
 * objects that run left (so the five create* calls of an event cost one
 * chain run); otherwise (first == 0, new events, a stage run again) the
 * chain runs from the hits up to `last`.  `flags` are those of every stage
 * run so far (the segment variant, the tracklet variant, ...).  Synchronous,
 * with the capacity growth of sdlg_run (which re-runs from the hits). */
int sdlg_run_stages(sdlg_ctx* ctx, int first, int last, int flags);

/* Enqueue the same chain on the context stream without waiting (for callers
 * that overlap work or time the device); sdlg_sync() waits and resolves
 * capacity overflows by re-running. */
int sdlg_run_async(sdlg_ctx* ctx, int stop_after, int flags);
int sdlg_sync(sdlg_ctx* ctx);

/* Objects per stage for event `event` (or the whole batch when event < 0):
 * out5[stage] (getNumberOfMiniDoublets ... getNumberOfTrackCandidates,
 * Event.h:302-311). */
int sdlg_get_counts(sdlg_ctx* ctx, int64_t event, int64_t* out5);

/* Copy the hit-index tuples of one stage of one event (event < 0: all) into
 * out (capacity `cap` tuples); *n_out receives the number of tuples. */
int sdlg_get_objects(sdlg_ctx* ctx, int stage, int64_t event, int32_t* out, int64_t cap, int64_t* n_out);

/* The same tuples without waiting for the copy: a kernel on a gather stream
 * writes them into one of two device buffers (used in turn) once the run is
 * complete, and the copy to `out` follows on a copy stream while the caller
 * goes on (the next sdlg_set_events or sdlg_stage_events may follow at once;
 * the next run starts once the kernel has read the objects, without waiting
 * for the copy).  out must stay valid and untouched until
 * sdlg_wait_objects() returns, and should be pinned (sdlg_host_alloc) for the
 * copy to overlap the next run.  *n_out is known on return.  A later
 * readback into the same device buffer waits for this copy first. */
int sdlg_get_objects_async(sdlg_ctx* ctx, int stage, int64_t event, int32_t* out, int64_t cap, int64_t* n_out);
int sdlg_wait_objects(sdlg_ctx* ctx);

/* The object graph of one event, for the reference's pointer accessors
 * (Module::getMiniDoubletPtrs ... getTrackletPtrs, Module.h:273-277;
 * MiniDoublet::lowerHitPtr/upperHitPtr, getDz, getShiftedDz, getDeltaPhi,
 * getDeltaPhiChange, MiniDoublet.h:73-84; Segment::inner/outerMiniDoubletPtr,
 * getDeltaPhi, getDeltaPhiMin/Max, getDeltaPhiChange,
 * getDeltaPhiMin/MaxChange, Segment.h:110-127;
 * TrackletBase::inner/outerSegmentPtr, TrackletBase.h:49-50;
 * TrackCandidate::inner/outerTrackletBasePtr, TrackCandidate.h:91-96).
 * For the n objects of stage `stage` of event `event` (n_out), in the row
 * order of sdlg_get_objects:
 *   links[2k], links[2k+1]: the two constituents, as indices into the
 *     event's list of the stage below: mini-doublet -> the event's hits
 *     (lower, upper; their position in the order sdlg_set_events got them),
 *     segment -> mini-doublets (inner, outer), tracklet and triplet ->
 *     segments (inner, outer), track candidate -> tracklets, or triplets
 *     after SDLG_FLAG_TC_FROM_TP (inner, outer);
 *   module[k]: the object's inner lower module (index into
 *     sdlg_get_module_detids), the module the reference lists it in;
 *   vals[k*nv + v]: nv = 4 floats per mini-doublet (dz, shiftedDz, deltaPhi,
 *     deltaPhiChange), 6 per segment (deltaPhi, deltaPhiMin, deltaPhiMax,
 *     deltaPhiChange, deltaPhiMinChange, deltaPhiMaxChange), none otherwise.
 * Any output may be NULL (all NULL: a size query); cap is in objects. */
int sdlg_get_object_links(sdlg_ctx* ctx, int stage, int64_t event, int32_t* links, int32_t* module, float* vals,
                          int64_t cap, int64_t* n_out);

/* The device module table: the detIds of module indices 0 .. n-1. */
int sdlg_get_module_detids(const sdlg_ctx* ctx, uint32_t* out, int64_t cap, int64_t* n_out);

/* detId decoding of SDL::Module (Module.cc:159-358; no context or device):
 * out11 = subdet, side, layer, rod, ring, module, isLower, isInverted,
 * partnerDetId, moduleType (0 PS, 1 2S), moduleLayerType (0 pixel, 1 strip).
 * Returns SDLG_ERR_DETID (with out11 filled) when the detId is neither a
 * barrel layer 1-6 nor an endcap layer 1-5 ring 1-15 module. */
int sdlg_module_info(uint32_t detid, uint32_t* out11);

/* SDL::Hit's derived quantities (Hit.cc:68-83; no context or device) for n
 * points: rt, phi, eta, r3 (any output may be NULL). */
int sdlg_hit_derived(int64_t n, const float* x, const float* y, const float* z, float* rt, float* phi, float* eta,
                     float* r3);

/* Debug dump of the tracklets' final cut variables, as the reference records
 * them in each Tracklet's recovars map (Tracklet.cc:1440-1495 and the same
 * block of the BBEE and EEEE algorithms): 15 floats per tracklet of the event
 * (event < 0: all), in the row order of sdlg_get_objects(stage 2):
 * betaIn, betaInRHmin, betaInRHmax, betaOut, betaOutRHmin, betaOutRHmax,
 * betaAv, pt_beta, dBeta, dBetaCut2, dBetaLum2, dBetaMuls, dBetaRes, dBetaRIn2,
 * dBetaROut2.  Recomputed on demand from the last run's segments.  As in the
 * reference, BBEE tracklets report -999 (their algorithm records none of
 * these), and values that pass through the reference's float std::asin can
 * differ from it in the last bit (glibc's asinf is not always correctly
 * rounded; the cut decisions here use the correctly rounded value). */
int sdlg_get_tracklet_vars(sdlg_ctx* ctx, int64_t event, float* out, int64_t cap, int64_t* n_out);

/* The reference's per-layer counters for one event (Event.cc:1064-1344):
 * 5 stages x {candidates, objects} x {barrel layers 1-6, endcap layers 1-5}. */
int sdlg_get_counters(sdlg_ctx* ctx, int64_t event, uint32_t* out110);

/* Device time of the last run: [0] ingest, [1..5] MD..TC stages, [6] total (ms). */
int sdlg_last_times(sdlg_ctx* ctx, float* out7);

/* Device time of each stage's candidate-evaluation kernel in the last run (ms). */
int sdlg_last_kernel_times(sdlg_ctx* ctx, float* out5);

/* Autotuner (no counterpart in the reference): runs the chain on the current
 * batch with each of a grid of launch shapes for the stages' candidate
 * evaluation kernels (candidates per warp task 128-1024, 4-16 CTAs per SM),
 * keeps the fastest shape per stage for later runs of this context, and
 * returns it in out10 (tasks[5], CTAs per SM[5]; may be NULL).  Results do
 * not depend on the shapes.  Takes about 24 runs of the chain. */
int sdlg_autotune(sdlg_ctx* ctx, int stop_after, int flags, int32_t* out10);

/* Device time (ms) of the last run's tracklet passes (no counterpart in the
 * reference): the enumeration with the float part of the cuts, the filters
 * (with SDLG_FLAG_MLP the pre-filter, then phase B2's single-precision
 * decision), and the double-precision part of the cuts; zeros for a run that
 * stopped before the tracklets.  sdlg_last_tl_pass_times4 gives the two
 * filters apart: enumeration, pre-filter, phase-B2 filter, exact cuts. */
int sdlg_last_tl_pass_times(sdlg_ctx* ctx, float* out3);
int sdlg_last_tl_pass_times4(sdlg_ctx* ctx, float* out4);

/* Entries of the last run's tracklet candidate lists (no counterpart in the
 * reference): the enumeration's phase-A survivors, those the pre-filter kept
 * (0 without SDLG_FLAG_MLP), and what the single-precision phase-B2 filter
 * left of the list before it for the exact phases to judge (that list's length
 * without the filter; the entries the filter found through phase B2 are
 * tracklets already and not counted). */
int sdlg_last_tl_list_counts(sdlg_ctx* ctx, int64_t* out3);

/* Self-check of the float-float evaluations that stand for the reference's
 * double sub-expressions (no counterpart in the reference).  Function fn
 * (0 asin, 1 atan2, 2 hit phi, 3 x + sqrt(y), 4 s + sqrt(a^2+b^2+c^2),
 * 5 Phi_mpi_pi, 6 M_PI + x, 7 a / sin(b), 8 and 15 the tracklets' multiple
 * scattering factor with and without its second square root, 9 a + b^2/4,
 * 10 sin, 11 cos, 12 atan, 13 sqrt(a^2 + b^2), 14 15 a / b) is evaluated on
 * n inputs: the float bit patterns
 * start .. start+n-1 (exhaustive != 0, unary functions) or hashed pseudo-random
 * inputs from `seed`.  out8: inputs where the fast path answered, of those
 * the ones whose float differs from the double evaluation's (must be 0), a
 * flag, and the first differing inputs and results as bit patterns.
 * Functions 16 (direction of a point by atan2f) and 17 (asinf) are the
 * tracklet cuts' single-precision approximations: "differs" there means
 * more than 2e-6 away from the exact value.  Functions 18 and 19 are tan(x)
 * and tan(x) / x (the hits' tan of their asin angle).  Function 20 is the
 * polynomial direction of the tracklet enumeration's phase-B1 decision
 * ("differs": more than 2.5e-6 away). */
int sdlg_math_check(sdlg_ctx* ctx, int fn, int exhaustive, uint64_t start, int64_t n, uint64_t seed, uint64_t* out8);

/* The host C library's float functions on the device (no counterpart in
 * the reference, whose std::asin/atan/sin/cos/tan calls on floats are the
 * host libm's asinf, atanf, sinf, cosf, tanf).  Those are not correctly
 * rounded, and the cuts see the difference; the chain evaluates the
 * correctly rounded float and moves it to the host function's value with a
 * table built from the host's own functions when the first context of the
 * process is created (a few seconds; about 200 MB on each device).
 * sdlg_libm_eval: the device's values of function fn (0 asin, 1 atan, 2 sin,
 * 3 cos, 4 tan) on the n floats whose bit patterns are start_bits ..
 * start_bits + n - 1, into host memory (the self-check against the host's
 * functions).  sdlg_libm_stats: out3 = floats tabulated, floats whose host
 * value is not the correctly rounded one, and those more than one float
 * away (kept in an exception list); no context or device needed. */
int sdlg_libm_eval(sdlg_ctx* ctx, int fn, uint32_t start_bits, int64_t n, float* out);
int sdlg_libm_stats(int fn, uint64_t* out3);

/* Self-check of the tracklet enumeration's single-precision decisions (no
 * counterpart in the reference): after a run through the tracklet stage,
 * every tracklet candidate of the batch is judged both by the fast decisions
 * (the float cuts, then for their survivors the first part of the tracklet
 * cuts) and by the exact cuts.  out4: candidates, candidates the fast
 * decisions settled alone, candidates that needed an exact evaluation, and
 * candidates settled differently from the exact cuts (must be 0). */
int sdlg_tl_phase_a_check(sdlg_ctx* ctx, uint64_t* out4);

/* Self-check of the single-precision phase-B2 filter (no counterpart in the
 * reference): after a run through the tracklet stage, every entry of the
 * enumeration's survivor list is judged by the filter and by the exact phases
 * B1 and B2.  out12: entries; through exact phase B1; through exact phases B1
 * and B2; rejected by the filter; rejected by the filter but through the exact
 * phases (must be 0); rejected by the filter among those through exact phase
 * B1; the largest |filter value - exact value| / the filter's bound for
 * deltaBeta, dBetaCut2 and betaOut (as float bits; below 1 when the bounds
 * hold); entries the filter left before reaching the cuts; entries the filter
 * finds through phase B2; of those, entries through exact phase B1 but not
 * through exact phase B2 (must be 0). */
int sdlg_tl_b2_filter_check(sdlg_ctx* ctx, uint64_t* out12);

/* Number of kernels one run of the chain launches (as last enqueued). */
int64_t sdlg_last_launches(const sdlg_ctx* ctx);

/* Mini-doublets of one event with no device allocation (no counterpart in
 * the reference, whose only interface is the host class library).  It is for
 * callers that may not allocate device memory while they process events:
 * frameworks that hand out all device memory from their own pool at start-up
 * and forbid allocation afterwards, and plugins whose host owns the
 * allocator.  Inputs (n_hits hits: x, y, z, idx, detid) and outputs are the
 * caller's DEVICE buffers; the stage's working memory is a fixed array inside
 * the library (18,875,496 bytes, about 18 MiB, held on every GPU that loads
 * the library until the process exits).  Results: d_pairs receives up to
 * pair_cap (lower idx, upper idx) pairs (the first pair_cap when there are
 * more), *d_count the number of mini-doublets (or, if the array's capacity
 * overflowed, the number needed)
 * and *d_status the device status word (0 = clean; bit 0 = more than
 * SDLG_STATIC_MAX_MINI_DOUBLETS mini-doublets, nothing written; bit 8 = hits
 * in modules the geometry does not list, which are skipped).  Asynchronous on
 * `stream` (NULL: the context's stream); the geometry must be loaded.
 * Limits: n_hits <= SDLG_STATIC_MAX_HITS and at most SDLG_STATIC_MAX_MODULES
 * modules, else SDLG_ERR_CAPACITY.  The first call on a device looks up the
 * array's device address.  All calls share the one array: calls that overlap on the GPU (different
 * streams, contexts or threads without ordering) race and corrupt each
 * other's results. */
#define SDLG_STATIC_MAX_HITS 131072
#define SDLG_STATIC_MAX_MODULES 65536
#define SDLG_STATIC_MAX_MINI_DOUBLETS 131072
int sdlg_mini_doublets_static(sdlg_ctx* ctx, int64_t n_hits, const float* d_x, const float* d_y, const float* d_z,
                              const int32_t* d_idx, const uint32_t* d_detid, int32_t* d_pairs, int64_t pair_cap,
                              int64_t* d_count, uint32_t* d_status, void* stream);

/* ---- Learned tracklet pre-filter (no counterpart in the reference) ----
 * A 12-64-64-1 perceptron (ReLU, BF16 weights and first hidden layer, FP32
 * accumulation) scores every tracklet candidate (inner segment, outer
 * segment) from 12 float features; with SDLG_FLAG_MLP every candidate through
 * the float part of the reference's tracklet cuts and the first part of the
 * rest (the direction and betaIn cuts, where their single-precision decision
 * settles them) is scored, one whose logit is below the threshold is dropped,
 * and the rest of the cuts judge every other one.  The cuts and the network
 * judge each candidate on its own, so their order does not change the
 * result.  The pruned chain's tracklets,
 * triplets and track candidates are therefore subsets of the plain chain's.
 * Inference runs on the tensor cores inside the tracklet kernel; training
 * runs on the GPU with this library's kernels on samples labelled by the
 * plain chain's tracklet cuts.
 * Parameter vector (SDLG_MLP_PARAMS floats): W1[64][12], b1[64], W2[64][64],
 * b2[64], w3[64], b3; logit = b3 + w3 . relu(W2 relu(W1 x + b1) + b2). */
#define SDLG_MLP_FEATURES 12
#define SDLG_MLP_PARAMS 5057
int sdlg_mlp_set_params(sdlg_ctx* ctx, const float* params, float threshold);
int sdlg_mlp_get_params(sdlg_ctx* ctx, float* params, float* threshold);
int sdlg_mlp_set_threshold(sdlg_ctx* ctx, float threshold);
/* uniform fan-in initialisation from `seed`, zero biases, threshold 0 */
int sdlg_mlp_init(sdlg_ctx* ctx, uint64_t seed);
/* After a run through the tracklet stage without SDLG_FLAG_MLP: append the
 * features of every tracklet candidate that passes the float cuts to the
 * context's training set, labelled 1 if the tracklet cuts accept it and 0
 * otherwise; rejected candidates are kept with probability neg_keep (a
 * deterministic hash of the candidate and `seed`).  *n_total: samples held. */
int sdlg_mlp_collect(sdlg_ctx* ctx, float neg_keep, uint64_t seed, int64_t* n_total);
int sdlg_mlp_add_samples(sdlg_ctx* ctx, int64_t n, const float* x, const float* y);
int sdlg_mlp_num_samples(sdlg_ctx* ctx, int64_t* n);
int sdlg_mlp_get_samples(sdlg_ctx* ctx, float* x, float* y, int64_t cap, int64_t* n);
int sdlg_mlp_clear_samples(sdlg_ctx* ctx);
/* Adam (beta 0.9, 0.999) on the weighted logistic loss, positives weighted
 * pos_weight, mini-batches of `batch` in a fresh shuffle per epoch;
 * epoch_loss[e] (optional) receives each epoch's mean loss. */
int sdlg_mlp_train(sdlg_ctx* ctx, int epochs, int batch, float lr, float pos_weight, uint64_t seed, float* epoch_loss);
/* Gradient of mean_i w_i * (softplus(z_i) - y_i z_i) at the current
 * parameters over n samples (the training kernels), and the loss. */
int sdlg_mlp_gradient(sdlg_ctx* ctx, int64_t n, const float* x, const float* y, const float* w, float* grad, double* loss);
/* logits of n feature rows (n x 12) through the tensor-core kernel */
int sdlg_mlp_score(sdlg_ctx* ctx, int64_t n, const float* x, float* logits);
/* counts of the last run with SDLG_FLAG_MLP: tracklet candidates, those
 * through the float cuts and the enumeration's decision of the direction and
 * betaIn cuts (scored by the network), those kept (logit at or above the
 * threshold), tensor-core waits that gave up */
int sdlg_mlp_stats(sdlg_ctx* ctx, int64_t* out4);

/* Pinned host memory for zero-staging transfers. */
int sdlg_host_alloc(sdlg_ctx* ctx, int64_t bytes, void** out);
int sdlg_host_free(sdlg_ctx* ctx, void* p);

#ifdef __cplusplus
}
#endif

#endif /* SDL_GPU_H */
