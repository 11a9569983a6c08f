// sdl_event.hpp - the reference's C++ user interface (SDL::Event, SDL::Hit and
// the geometry singletons) on top of the C ABI in sdl_gpu.h.
//
// A caller of the reference writes (Event.h:210,239-300; TiltedGeometry.h,
// EndcapGeometry.h, ModuleConnectionMap.h):
//
//     SDL::tiltedGeometry.load("tilted.txt");
//     SDL::endcapGeometry.load("endcap.txt");
//     SDL::moduleConnectionMap.load("map.txt");
//     SDL::Event ev;
//     ev.addHitToModule(SDL::Hit(x, y, z, idx), detId);   // for every hit
//     ev.createMiniDoublets();
//     ev.createSegmentsWithModuleMap();
//     ev.createTrackletsWithModuleMap();
//     ev.createTriplets();
//     ev.createTrackCandidates();
//     ev.getNumberOfTrackCandidates();
//
// and the same lines compile against this header.  The object lists are
// returned as hit-index tuples (the idx given to each hit), which is how the
// reference identifies objects (isIdxMatched, Hit.cc:175-182).  Each create*
// call runs the chain on the GPU up to that stage.  Errors are reported as
// SDL::Error exceptions (the reference has no error reporting of its own;
// it silently reads 0 for missing geometry, which this layer does too).
#pragma once

#include <array>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "sdl_gpu.h"

namespace SDL {

enum MDAlgo { Default_MDAlgo = 0, AllComb_MDAlgo };
enum SGAlgo { Default_SGAlgo = 0, AllComb_SGAlgo };
enum TLAlgo { Default_TLAlgo = 0, DefaultNm1_TLAlgo, AllComb_TLAlgo };
enum TPAlgo { Default_TPAlgo = 0, AllComb_TPAlgo };
enum TCAlgo { Default_TCAlgo = 0, AllComb_TCAlgo };

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

class Hit {
  public:
    Hit() = default;
    Hit(float x, float y, float z, int idx = -1) : x_(x), y_(y), z_(z), idx_(idx) {}
    float x() const { return x_; }
    float y() const { return y_; }
    float z() const { return z_; }
    int idx() const { return idx_; }

  private:
    float x_ = 0, y_ = 0, z_ = 0;
    int idx_ = -1;
};

// Geometry singletons: load() records the file; every Event reads it.
struct GeometryFile {
    std::string path;
    void load(const std::string& p) { path = p; }
};
inline GeometryFile tiltedGeometry;       // TiltedGeometry.cc:3
inline GeometryFile endcapGeometry;       // EndcapGeometry.cc:3
inline GeometryFile moduleConnectionMap;  // ModuleConnectionMap.cc:3

class Event {
  public:
    explicit Event(int device = 0) {
        check(sdlg_create(&ctx_, device), "sdlg_create");
        const char* t = tiltedGeometry.path.empty() ? nullptr : tiltedGeometry.path.c_str();
        const char* e = endcapGeometry.path.empty() ? nullptr : endcapGeometry.path.c_str();
        const char* m = moduleConnectionMap.path.empty() ? nullptr : moduleConnectionMap.path.c_str();
        check(sdlg_geometry_load_files(ctx_, t, e, m), "geometry");
    }
    ~Event() {
        if (ctx_) sdlg_destroy(ctx_);
    }
    Event(const Event&) = delete;
    Event& operator=(const Event&) = delete;

    // Event.cc:120-139
    void addHitToModule(Hit hit, unsigned int detId) {
        x_.push_back(hit.x());
        y_.push_back(hit.y());
        z_.push_back(hit.z());
        idx_.push_back(hit.idx());
        det_.push_back(detId);
        dirty_ = true;
    }

    // Event.cc:245-305, 445-522, 611-693, 524-597, 823-872
    void createMiniDoublets(MDAlgo algo = Default_MDAlgo) { require(algo == Default_MDAlgo); run(SDLG_STAGE_MD); }
    void createSegmentsWithModuleMap(SGAlgo algo = Default_SGAlgo) {
        require(algo == Default_SGAlgo);
        sg_flags_ = 0;
        run(SDLG_STAGE_SG);
    }
    // Event.cc:432-443: segments from the layer pairs of Layer.cc:32-50
    void createSegments(SGAlgo algo = Default_SGAlgo) {
        require(algo == Default_SGAlgo);
        sg_flags_ = SDLG_FLAG_SG_LAYERS;
        run(SDLG_STAGE_SG);
    }
    void createTrackletsWithModuleMap(TLAlgo algo = Default_TLAlgo) {
        require(algo == Default_TLAlgo || algo == DefaultNm1_TLAlgo);
        tl_flags_ = algo == DefaultNm1_TLAlgo ? SDLG_FLAG_TL_NM1 : 0;
        run(SDLG_STAGE_TL);
    }
    // Event.cc:599-609: tracklets from the layer pairs of Layer.cc:3-30
    void createTracklets(TLAlgo algo = Default_TLAlgo) {
        require(algo == Default_TLAlgo || algo == DefaultNm1_TLAlgo);
        tl_flags_ = SDLG_FLAG_TL_LAYERS | (algo == DefaultNm1_TLAlgo ? SDLG_FLAG_TL_NM1 : 0);
        run(SDLG_STAGE_TL);
    }
    // Event.cc:694-751: tracklets along the segments that share mini-doublets
    void createTrackletsViaNavigation(TLAlgo algo = Default_TLAlgo) {
        require(algo == Default_TLAlgo || algo == DefaultNm1_TLAlgo);
        tl_flags_ = SDLG_FLAG_TL_NAV | (algo == DefaultNm1_TLAlgo ? SDLG_FLAG_TL_NM1 : 0);
        run(SDLG_STAGE_TL);
    }
    void createTriplets(TPAlgo algo = Default_TPAlgo) { require(algo == Default_TPAlgo); run(SDLG_STAGE_TP); }
    void createTrackCandidates(TCAlgo algo = Default_TCAlgo) {
        require(algo == Default_TCAlgo);
        tc_flags_ = 0;
        run(SDLG_STAGE_TC);
    }
    // Event.cc:984-1062
    void createTrackCandidatesFromTracklets(TCAlgo algo = Default_TCAlgo) {
        require(algo == Default_TCAlgo);
        tc_flags_ = SDLG_FLAG_TC_FROM_TL;
        run(SDLG_STAGE_TC);
    }
    // Event.cc:874-982
    void createTrackCandidatesFromTriplets(TCAlgo algo = Default_TCAlgo) {
        require(algo == Default_TCAlgo);
        tc_flags_ = SDLG_FLAG_TC_FROM_TP;
        run(SDLG_STAGE_TC);
    }

    // Event.h:302-311
    unsigned int getNumberOfHits() const { return (unsigned int)x_.size(); }
    unsigned int getNumberOfMiniDoublets() { return count(SDLG_STAGE_MD); }
    unsigned int getNumberOfSegments() { return count(SDLG_STAGE_SG); }
    unsigned int getNumberOfTracklets() { return count(SDLG_STAGE_TL); }
    unsigned int getNumberOfTriplets() { return count(SDLG_STAGE_TP); }
    unsigned int getNumberOfTrackCandidates() { return count(SDLG_STAGE_TC); }

    // per-layer counters (Event.cc:1064-1344); layer is 0-based as in the reference's arrays
    unsigned int getNumberOfMiniDoubletCandidatesByLayerBarrel(unsigned int i) { return counter(0, 0, i); }
    unsigned int getNumberOfMiniDoubletsByLayerBarrel(unsigned int i) { return counter(0, 1, i); }
    unsigned int getNumberOfSegmentCandidatesByLayerBarrel(unsigned int i) { return counter(1, 0, i); }
    unsigned int getNumberOfSegmentsByLayerBarrel(unsigned int i) { return counter(1, 1, i); }
    unsigned int getNumberOfTrackletCandidatesByLayerBarrel(unsigned int i) { return counter(2, 0, i); }
    unsigned int getNumberOfTrackletsByLayerBarrel(unsigned int i) { return counter(2, 1, i); }
    unsigned int getNumberOfTripletCandidatesByLayerBarrel(unsigned int i) { return counter(3, 0, i); }
    unsigned int getNumberOfTripletsByLayerBarrel(unsigned int i) { return counter(3, 1, i); }
    unsigned int getNumberOfTrackCandidateCandidatesByLayerBarrel(unsigned int i) { return counter(4, 0, i); }
    unsigned int getNumberOfTrackCandidatesByLayerBarrel(unsigned int i) { return counter(4, 1, i); }
    unsigned int getNumberOfMiniDoubletCandidatesByLayerEndcap(unsigned int i) { return counter(0, 0, 6 + i); }
    unsigned int getNumberOfMiniDoubletsByLayerEndcap(unsigned int i) { return counter(0, 1, 6 + i); }
    unsigned int getNumberOfSegmentCandidatesByLayerEndcap(unsigned int i) { return counter(1, 0, 6 + i); }
    unsigned int getNumberOfSegmentsByLayerEndcap(unsigned int i) { return counter(1, 1, 6 + i); }
    unsigned int getNumberOfTrackletCandidatesByLayerEndcap(unsigned int i) { return counter(2, 0, 6 + i); }
    unsigned int getNumberOfTrackletsByLayerEndcap(unsigned int i) { return counter(2, 1, 6 + i); }
    unsigned int getNumberOfTripletCandidatesByLayerEndcap(unsigned int i) { return counter(3, 0, 6 + i); }
    unsigned int getNumberOfTripletsByLayerEndcap(unsigned int i) { return counter(3, 1, 6 + i); }
    unsigned int getNumberOfTrackCandidateCandidatesByLayerEndcap(unsigned int i) { return counter(4, 0, 6 + i); }
    unsigned int getNumberOfTrackCandidatesByLayerEndcap(unsigned int i) { return counter(4, 1, 6 + i); }

    // object lists as hit-index tuples
    std::vector<std::array<int32_t, 2>> getMiniDoublets() { return objects<2>(SDLG_STAGE_MD); }
    std::vector<std::array<int32_t, 4>> getSegments() { return objects<4>(SDLG_STAGE_SG); }
    std::vector<std::array<int32_t, 8>> getTracklets() { return objects<8>(SDLG_STAGE_TL); }
    std::vector<std::array<int32_t, 8>> getTriplets() { return objects<8>(SDLG_STAGE_TP); }
    std::vector<std::array<int32_t, 16>> getTrackCandidates() { return objects<16>(SDLG_STAGE_TC); }

    sdlg_ctx* context() { return ctx_; }

  private:
    void check(int rc, const char* what) const {
        if (rc != SDLG_OK) throw Error(rc, std::string(what) + ": " + (ctx_ ? sdlg_last_error(ctx_) : "no context"));
    }
    static void require(bool ok) {
        if (!ok) throw Error(SDLG_ERR_ARG, "algorithm variant not available on the GPU chain");
    }
    void run(int stage) {
        if (x_.empty()) {
            ran_ = -1;
            stage_ = stage;
            return;
        }
        if (dirty_) {
            const int64_t off[2] = {0, (int64_t)x_.size()};
            check(sdlg_set_events(ctx_, 1, off, x_.data(), y_.data(), z_.data(), idx_.data(), det_.data()), "set_events");
            dirty_ = false;
        }
        // each call re-runs the chain up to `stage` with the variants chosen so far
        check(sdlg_run(ctx_, stage, sg_flags_ | tl_flags_ | tc_flags_), "run");
        ran_ = stage;
        stage_ = stage;
    }
    unsigned int count(int stage) {
        if (ran_ < stage) return 0;
        int64_t n[5];
        check(sdlg_get_counts(ctx_, 0, n), "counts");
        return (unsigned int)n[stage];
    }
    unsigned int counter(int stage, int kind, unsigned int slot) {
        if (ran_ < 0 || slot >= 11) return 0;
        uint32_t c[110];
        check(sdlg_get_counters(ctx_, 0, c), "counters");
        return c[stage * 22 + kind * 11 + slot];
    }
    template <int W>
    std::vector<std::array<int32_t, W>> objects(int stage) {
        std::vector<std::array<int32_t, W>> out;
        if (ran_ < stage) return out;
        int64_t n = 0;
        check(sdlg_get_objects(ctx_, stage, 0, nullptr, 0, &n), "objects");
        out.resize((size_t)n);
        if (n) check(sdlg_get_objects(ctx_, stage, 0, out.data()->data(), n, &n), "objects");
        return out;
    }

    sdlg_ctx* ctx_ = nullptr;
    std::vector<float> x_, y_, z_;
    std::vector<int32_t> idx_;
    std::vector<uint32_t> det_;
    bool dirty_ = false;
    int sg_flags_ = 0, tl_flags_ = 0, tc_flags_ = 0;
    int ran_ = -1;
    int stage_ = -1;
};

}  // namespace SDL
