// sdl_event.hpp - the reference's C++ user interface (SDL::Event, SDL::Hit,
// SDL::Module, SDL::Layer, the five object classes and the geometry
// singletons) on top of the C ABI in sdl_gpu.h.
//
// A caller of the reference writes (Event.h:197-300; TiltedGeometry.h,
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
//     for (SDL::Module* m : ev.getLowerModulePtrs())
//         for (SDL::Segment* sg : m->getSegmentPtrs())
//             sg->innerMiniDoubletPtr()->lowerHitPtr()->idx();
//
// and the same lines compile against this header.  Each create* call runs
// only its own stage on the GPU, on the objects the previous calls left
// there (sdlg_run_stages), so the five calls cost one chain run.  The object
// graph (modules, layers, mini-doublets ... track candidates and their
// pointer accessors) is built on the host from the device's index arrays
// (sdlg_get_object_links) the first time a caller walks a stage, and lives
// until the next create* call or the next hit: pointers handed out before
// that are invalidated, as the reference's are when its Event is destroyed.
// Within a module the objects come in the GPU's order, not in the order of
// the reference's loops; the lists hold the same objects.  Errors are
// reported as SDL::Error exceptions (the reference has no error reporting
// of its own; it silently reads 0 for missing geometry, which this layer
// does too); TrackCandidate::innerTrackletPtr() and its siblings throw
// std::logic_error as the reference's do (TrackCandidate.cc:38-86).
#pragma once

#include <array>
#include <cstdint>
#include <deque>
#include <map>
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

class Event;
class Module;
class Layer;
class MiniDoublet;
class Segment;
class TrackletBase;
class Tracklet;
class Triplet;
class TrackCandidate;

// Hit.h:19-91: a point with its derived quantities (Hit.cc:68-83, computed
// by the library with the reference's arithmetic)
class Hit {
  public:
    Hit() = default;
    Hit(float x, float y, float z, int idx = -1) : x_(x), y_(y), z_(z), idx_(idx) {
        sdlg_hit_derived(1, &x_, &y_, &z_, &rt_, &phi_, &eta_, &r3_);
    }
    const float& x() const { return x_; }
    const float& y() const { return y_; }
    const float& z() const { return z_; }
    const float& rt() const { return rt_; }
    const float& r3() const { return r3_; }
    const float& phi() const { return phi_; }
    const float& eta() const { return eta_; }
    const int& idx() const { return idx_; }
    // the module the hit was added to (Hit.h:67); only for an event's hits
    const Module& getModule() const {
        if (!module_) throw std::logic_error("Hit::getModule: the hit belongs to no event");
        return *module_;
    }
    bool isIdxMatched(const Hit& o) const { return idx_ == o.idx_; }  // Hit.cc:175-182

  private:
    friend class Event;
    float x_ = 0, y_ = 0, z_ = 0, rt_ = 0, phi_ = 0, eta_ = 0, r3_ = 0;
    int idx_ = -1;
    const Module* module_ = nullptr;
};

// Module.h:22-304: the decoded detId (Module.cc:159-358, decoded by the
// library) and the objects listed in the module
class Module {
  public:
    enum SubDet { Barrel = 5, Endcap = 4 };
    enum Side { NegZ = 1, PosZ = 2, Center = 3 };
    enum ModuleType { PS, TwoS };
    enum ModuleLayerType { Pixel, Strip };

    explicit Module(unsigned int detId = 0) { setDetId(detId); }

    const unsigned int& detId() const { return detId_; }
    const unsigned int& partnerDetId() const { return partnerDetId_; }
    const unsigned short& subdet() const { return subdet_; }
    const unsigned short& side() const { return side_; }
    const unsigned short& layer() const { return layer_; }
    const unsigned short& rod() const { return rod_; }
    const unsigned short& ring() const { return ring_; }
    const unsigned short& module() const { return module_; }
    const unsigned short& isLower() const { return isLower_; }
    const bool& isInverted() const { return isInverted_; }
    const ModuleType& moduleType() const { return moduleType_; }
    const ModuleLayerType& moduleLayerType() const { return moduleLayerType_; }

    const std::vector<Hit*>& getHitPtrs() const { return hits_; }
    inline const std::vector<MiniDoublet*>& getMiniDoubletPtrs() const;
    inline const std::vector<Segment*>& getSegmentPtrs() const;
    inline const std::vector<Triplet*>& getTripletPtrs() const;
    inline const std::vector<Tracklet*>& getTrackletPtrs() const;

    void setDetId(unsigned int d) {
        uint32_t v[11];
        sdlg_module_info(d, v);
        detId_ = d;
        subdet_ = (unsigned short)v[0];
        side_ = (unsigned short)v[1];
        layer_ = (unsigned short)v[2];
        rod_ = (unsigned short)v[3];
        ring_ = (unsigned short)v[4];
        module_ = (unsigned short)v[5];
        isLower_ = (unsigned short)v[6];
        isInverted_ = v[7] != 0;
        partnerDetId_ = v[8];
        moduleType_ = v[9] ? TwoS : PS;
        moduleLayerType_ = v[10] ? Strip : Pixel;
    }

  private:
    friend class Event;
    unsigned int detId_ = 0, partnerDetId_ = 0;
    unsigned short subdet_ = 0, side_ = 0, layer_ = 0, rod_ = 0, ring_ = 0, module_ = 0, isLower_ = 0;
    bool isInverted_ = false;
    ModuleType moduleType_ = PS;
    ModuleLayerType moduleLayerType_ = Pixel;
    Event* event_ = nullptr;
    std::vector<Hit*> hits_;
    std::vector<MiniDoublet*> mds_;
    std::vector<Segment*> sgs_;
    std::vector<Triplet*> tps_;
    std::vector<Tracklet*> tls_;
};

// Layer.h:24-121: objects listed by layer (barrel 1-6, endcap 1-5)
class Layer {
  public:
    enum BarrelLayers { BarrelLayer0 = 1, BarrelLayer1, BarrelLayer2, BarrelLayer3, BarrelLayer4, BarrelLayer5, nBarrelLayer };
    enum EndcapLayers { EndcapLayer0 = 1, EndcapLayer1, EndcapLayer2, EndcapLayer3, EndcapLayer4, EndcapLayer5, nEndcapLayer };
    enum SubDet { Barrel = 5, Endcap = 4 };

    Layer() = default;
    Layer(int layerIdx, unsigned short subdet) : layer_idx_(layerIdx), subdet_(subdet) {}
    const unsigned short& subdet() const { return subdet_; }
    const int& layerIdx() const { return layer_idx_; }
    inline const std::vector<MiniDoublet*>& getMiniDoubletPtrs() const;
    inline const std::vector<Segment*>& getSegmentPtrs() const;
    inline const std::vector<Triplet*>& getTripletPtrs() const;
    inline const std::vector<Tracklet*>& getTrackletPtrs() const;
    inline const std::vector<TrackCandidate*>& getTrackCandidatePtrs() const;

  private:
    friend class Event;
    int layer_idx_ = 0;
    unsigned short subdet_ = 0;
    Event* event_ = nullptr;
    std::vector<MiniDoublet*> mds_;
    std::vector<Segment*> sgs_;
    std::vector<Triplet*> tps_;
    std::vector<Tracklet*> tls_;
    std::vector<TrackCandidate*> tcs_;
};

// MiniDoublet.h:73-84
class MiniDoublet {
  public:
    Hit* lowerHitPtr() const { return lo_; }
    Hit* upperHitPtr() const { return up_; }
    // MiniDoublet.cc:60-81: the pixel-side hit of a PS module, the lower hit of a 2S module
    Hit* anchorHitPtr() const {
        const Module& m = lo_->getModule();
        if (m.moduleType() == Module::PS) return m.moduleLayerType() == Module::Pixel ? lo_ : up_;
        return lo_;
    }
    const float& getDz() const { return v_[0]; }
    const float& getShiftedDz() const { return v_[1]; }
    const float& getDeltaPhi() const { return v_[2]; }
    const float& getDeltaPhiChange() const { return v_[3]; }
    inline const std::vector<Segment*>& getListOfOutwardSegmentPtrs();
    inline const std::vector<Segment*>& getListOfInwardSegmentPtrs();
    bool isIdxMatched(const MiniDoublet& o) const {  // MiniDoublet.cc:686-693
        return lo_->isIdxMatched(*o.lo_) && up_->isIdxMatched(*o.up_);
    }

  private:
    friend class Event;
    Hit *lo_ = nullptr, *up_ = nullptr;
    float v_[4] = {0, 0, 0, 0};
    Event* event_ = nullptr;
    std::vector<Segment*> out_, in_;
};

// Segment.h:110-127 (the values the segment algorithms keep; the anchor
// hits' rt and z as getRtIn/getRtOut/getZIn/getZOut, Segment.cc:443-458)
class Segment {
  public:
    MiniDoublet* innerMiniDoubletPtr() const { return in_; }
    MiniDoublet* outerMiniDoubletPtr() const { return out_; }
    const float& getRtIn() const { return in_->anchorHitPtr()->rt(); }
    const float& getRtOut() const { return out_->anchorHitPtr()->rt(); }
    const float& getZIn() const { return in_->anchorHitPtr()->z(); }
    const float& getZOut() const { return out_->anchorHitPtr()->z(); }
    const float& getDeltaPhi() const { return v_[0]; }
    const float& getDeltaPhiMin() const { return v_[1]; }
    const float& getDeltaPhiMax() const { return v_[2]; }
    const float& getDeltaPhiChange() const { return v_[3]; }
    const float& getDeltaPhiMinChange() const { return v_[4]; }
    const float& getDeltaPhiMaxChange() const { return v_[5]; }
    inline const std::vector<Tracklet*>& getListOfOutwardTrackletPtrs();
    inline const std::vector<Tracklet*>& getListOfInwardTrackletPtrs();
    bool isIdxMatched(const Segment& o) const {  // Segment.cc:868-875
        return in_->isIdxMatched(*o.in_) && out_->isIdxMatched(*o.out_);
    }

  private:
    friend class Event;
    MiniDoublet *in_ = nullptr, *out_ = nullptr;
    float v_[6] = {0, 0, 0, 0, 0, 0};
    Event* event_ = nullptr;
    std::vector<Tracklet*> tl_out_, tl_in_;
};

// TrackletBase.h:49-50
class TrackletBase {
  public:
    virtual ~TrackletBase() = default;
    Segment* innerSegmentPtr() const { return in_; }
    Segment* outerSegmentPtr() const { return out_; }
    bool isIdxMatched(const TrackletBase& o) const {  // Tracklet.cc:3326-3331
        return in_->isIdxMatched(*o.in_) && out_->isIdxMatched(*o.out_);
    }

  protected:
    friend class Event;
    Segment *in_ = nullptr, *out_ = nullptr;
};

class Triplet : public TrackletBase {};

// the tracklet's final cut variables, as the reference's recovars map
// (Tracklet.cc:1440-1495; -999 for BBEE tracklets, whose algorithm records
// none; sdlg_get_tracklet_vars)
class Tracklet : public TrackletBase {
  public:
    inline const std::map<std::string, float>& getRecoVars() const;
    const float& getRecoVar(const std::string& key) const { return getRecoVars().at(key); }

  private:
    friend class Event;
    Event* event_ = nullptr;
    int64_t row_ = 0;
    mutable std::map<std::string, float> vars_;
};

// TrackCandidate.h:91-96
class TrackCandidate {
  public:
    TrackletBase* innerTrackletBasePtr() const { return in_; }
    TrackletBase* outerTrackletBasePtr() const { return out_; }
    Tracklet* innerTrackletPtr() const { return as<Tracklet>(in_, "innerTracklet"); }
    Tracklet* outerTrackletPtr() const { return as<Tracklet>(out_, "outerTracklet"); }
    Triplet* innerTripletPtr() const { return as<Triplet>(in_, "innerTriplet"); }
    Triplet* outerTripletPtr() const { return as<Triplet>(out_, "outerTriplet"); }

  private:
    friend class Event;
    template <class T>
    static T* as(TrackletBase* p, const char* what) {
        T* q = dynamic_cast<T*>(p);
        if (!q) throw std::logic_error(std::string("TrackCandidate::") + what + "Ptr(): this track candidate has none");
        return q;
    }
    TrackletBase *in_ = nullptr, *out_ = nullptr;
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
        for (int i = Layer::BarrelLayer0; i < Layer::nBarrelLayer; ++i) barrel_[i] = Layer(i, Layer::Barrel);
        for (int i = Layer::EndcapLayer0; i < Layer::nEndcapLayer; ++i) endcap_[i] = Layer(i, Layer::Endcap);
        for (int i = Layer::BarrelLayer0; i < Layer::nBarrelLayer; ++i) layer_ptrs_.push_back(&barrel_[i]);
        for (int i = Layer::EndcapLayer0; i < Layer::nEndcapLayer; ++i) layer_ptrs_.push_back(&endcap_[i]);
        for (Layer* l : layer_ptrs_) l->event_ = this;
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
        invalidate_graph();
    }

    // Event.cc:245-305, 445-522, 611-693, 524-597, 823-872: each runs its own stage
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

    // ---- modules and layers (Event.h:197-204, Event.cc:38-118)
    bool hasModule(unsigned int detId) {
        build_hits();
        return modules_by_id_.count(detId) != 0;
    }
    // creates an empty module for an unknown detId, as the reference's does
    Module& getModule(unsigned int detId) {
        build_hits();
        return module_of(detId);
    }
    // modules in the order of their first hit; lower modules among them
    const std::vector<Module*> getModulePtrs() const {
        const_cast<Event*>(this)->build_hits();
        return module_ptrs_;
    }
    const std::vector<Module*> getLowerModulePtrs() const {
        const_cast<Event*>(this)->build_hits();
        return lower_module_ptrs_;
    }
    Layer& getLayer(int layer, Layer::SubDet subdet) {
        if (layer < 1 || layer > (subdet == Layer::Barrel ? 6 : 5)) throw Error(SDLG_ERR_ARG, "no such layer");
        return subdet == Layer::Barrel ? barrel_[layer] : endcap_[layer];
    }
    const std::vector<Layer*> getLayerPtrs() const { return layer_ptrs_; }

    // Event.h:302-311
    unsigned int getNumberOfHits() const { return (unsigned int)x_.size(); }
    unsigned int getNumberOfMiniDoublets() { return count(SDLG_STAGE_MD); }
    unsigned int getNumberOfSegments() { return count(SDLG_STAGE_SG); }
    unsigned int getNumberOfTracklets() { return count(SDLG_STAGE_TL); }
    unsigned int getNumberOfTriplets() { return count(SDLG_STAGE_TP); }
    unsigned int getNumberOfTrackCandidates() { return count(SDLG_STAGE_TC); }

    // hits by layer, lower and upper modules (Event.h:306-315, Event.cc:1170-1190);
    // the layer is 0-based as in the reference's arrays
    unsigned int getNumberOfHitsByLayerBarrel(unsigned int i) { return hit_count(0, i); }
    unsigned int getNumberOfHitsByLayerEndcap(unsigned int i) { return hit_count(1, i); }
    unsigned int getNumberOfHitsByLayerBarrelUpperModule(unsigned int i) { return hit_count(2, i); }
    unsigned int getNumberOfHitsByLayerEndcapUpperModule(unsigned int i) { return hit_count(3, i); }

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

    // ---- the object graph, built on first use after each create* call
    // (called by the Module / Layer / object accessors)
    void materialize(int stage) {
        if (stage < 0 || stage > 4 || built_[stage]) return;
        build_hits();
        if (stage > 0) materialize(stage - 1);
        built_[stage] = true;
        if (ran_ < stage) return;  // not run: empty lists, as the reference's before the call
        if (mod_detids_.empty()) {
            int64_t n = 0;
            check(sdlg_get_module_detids(ctx_, nullptr, 0, &n), "modules");
            mod_detids_.resize((size_t)n);
            if (n) check(sdlg_get_module_detids(ctx_, mod_detids_.data(), n, &n), "modules");
        }
        int64_t n = 0;
        check(sdlg_get_object_links(ctx_, stage, 0, nullptr, nullptr, nullptr, 0, &n), "links");
        const int nv = stage == 0 ? 4 : stage == 1 ? 6 : 0;
        std::vector<int32_t> lk((size_t)(2 * n)), mod((size_t)n);
        std::vector<float> vals((size_t)(n * nv));
        if (n)
            check(sdlg_get_object_links(ctx_, stage, 0, lk.data(), mod.data(), nv ? vals.data() : nullptr, n, &n),
                  "links");
        const int flags = sg_flags_ | tl_flags_ | tc_flags_;
        switch (stage) {
            case SDLG_STAGE_MD:
                mds_.resize((size_t)n);
                for (int64_t k = 0; k < n; ++k) {
                    MiniDoublet& o = mds_[k];
                    o.event_ = this;
                    o.lo_ = &hits_.at((size_t)lk[2 * k]);
                    o.up_ = &hits_.at((size_t)lk[2 * k + 1]);
                    for (int v = 0; v < 4; ++v) o.v_[v] = vals[k * 4 + v];
                    Module& m = module_at(mod[k]);
                    m.mds_.push_back(&o);
                    layer_of(m).mds_.push_back(&o);
                }
                break;
            case SDLG_STAGE_SG:
                sgs_.resize((size_t)n);
                for (int64_t k = 0; k < n; ++k) {
                    Segment& o = sgs_[k];
                    o.event_ = this;
                    o.in_ = &mds_.at((size_t)lk[2 * k]);
                    o.out_ = &mds_.at((size_t)lk[2 * k + 1]);
                    for (int v = 0; v < 6; ++v) o.v_[v] = vals[k * 6 + v];
                    Module& m = module_at(mod[k]);
                    m.sgs_.push_back(&o);
                    layer_of(m).sgs_.push_back(&o);
                    o.in_->out_.push_back(&o);  // Segment.cc:58-62
                    o.out_->in_.push_back(&o);
                }
                break;
            case SDLG_STAGE_TL:
                tls_.resize((size_t)n);
                for (int64_t k = 0; k < n; ++k) {
                    Tracklet& o = tls_[k];
                    o.event_ = this;
                    o.row_ = k;
                    o.in_ = &sgs_.at((size_t)lk[2 * k]);
                    o.out_ = &sgs_.at((size_t)lk[2 * k + 1]);
                    Module& m = module_at(mod[k]);
                    // the layer-pair variant lists tracklets by layer only (Event.cc:785)
                    if (!(flags & SDLG_FLAG_TL_LAYERS)) m.tls_.push_back(&o);
                    layer_of(m).tls_.push_back(&o);
                    o.in_->tl_out_.push_back(&o);  // Tracklet.cc:35-39
                    o.out_->tl_in_.push_back(&o);
                }
                break;
            case SDLG_STAGE_TP:
                tps_.resize((size_t)n);
                for (int64_t k = 0; k < n; ++k) {
                    Triplet& o = tps_[k];
                    o.in_ = &sgs_.at((size_t)lk[2 * k]);
                    o.out_ = &sgs_.at((size_t)lk[2 * k + 1]);
                    Module& m = module_at(mod[k]);
                    m.tps_.push_back(&o);
                    layer_of(m).tps_.push_back(&o);
                }
                break;
            default:
                tcs_.resize((size_t)n);
                for (int64_t k = 0; k < n; ++k) {
                    TrackCandidate& o = tcs_[k];
                    if (flags & SDLG_FLAG_TC_FROM_TP) {
                        o.in_ = &tps_.at((size_t)lk[2 * k]);
                        o.out_ = &tps_.at((size_t)lk[2 * k + 1]);
                    } else {
                        o.in_ = &tls_.at((size_t)lk[2 * k]);
                        o.out_ = &tls_.at((size_t)lk[2 * k + 1]);
                    }
                    // Event.cc:835 and 967 list them in barrel layer 1; Event.cc:1051-1053 by the inner module's layer
                    if (flags & SDLG_FLAG_TC_FROM_TL) layer_of(module_at(mod[k])).tcs_.push_back(&o);
                    else barrel_[1].tcs_.push_back(&o);
                }
        }
    }
    const std::map<std::string, float>& tracklet_vars(const Tracklet& t) {
        if (t.vars_.empty()) {
            if (tl_vars_.empty() && !tls_.empty()) {
                int64_t n = 0;
                tl_vars_.resize(tls_.size() * 15);
                check(sdlg_get_tracklet_vars(ctx_, 0, tl_vars_.data(), (int64_t)tls_.size(), &n), "tracklet vars");
            }
            static const char* names[15] = {"betaIn", "betaInRHmin", "betaInRHmax", "betaOut", "betaOutRHmin",
                                            "betaOutRHmax", "betaAv", "pt_beta", "dBeta", "dBetaCut2", "dBetaLum2",
                                            "dBetaMuls", "dBetaRes", "dBetaRIn2", "dBetaROut2"};
            for (int v = 0; v < 15; ++v) t.vars_[names[v]] = tl_vars_.at((size_t)(t.row_ * 15 + v));
        }
        return t.vars_;
    }

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
            ran_ = -1;
        }
        // the stages after the last one run continue it; a stage run again
        // (or a first call after new hits) runs from the hits
        const int first = (ran_ >= 0 && stage == ran_ + 1) ? stage : 0;
        check(sdlg_run_stages(ctx_, first, stage, sg_flags_ | tl_flags_ | tc_flags_), "run");
        clear_stages(first);
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
    unsigned int hit_count(int which, unsigned int i) {
        build_hits();
        return i < 6 ? hits_by_layer_[which][i] : 0;
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

    // hits and modules in first-hit order (Event.cc:54-78, 120-139, 1170-1190)
    void build_hits() {
        if (hits_built_) return;
        hits_built_ = true;
        const size_t n = x_.size();
        hits_.assign(n, Hit());
        std::vector<float> rt(n), phi(n), eta(n), r3(n);
        if (n) sdlg_hit_derived((int64_t)n, x_.data(), y_.data(), z_.data(), rt.data(), phi.data(), eta.data(), r3.data());
        for (size_t i = 0; i < n; ++i) {
            Hit& h = hits_[i];
            h.x_ = x_[i];
            h.y_ = y_[i];
            h.z_ = z_[i];
            h.idx_ = idx_[i];
            h.rt_ = rt[i];
            h.phi_ = phi[i];
            h.eta_ = eta[i];
            h.r3_ = r3[i];
            Module& m = module_of(det_[i]);
            h.module_ = &m;
            m.hits_.push_back(&h);
            const int which = (m.isLower() ? 0 : 2) + (m.subdet() == Module::Barrel ? 0 : 1);
            if (m.layer() >= 1 && m.layer() <= 6) ++hits_by_layer_[which][m.layer() - 1];
        }
    }
    Module& module_of(unsigned int detId) {
        auto it = modules_by_id_.find(detId);
        if (it != modules_by_id_.end()) return *it->second;
        modules_.emplace_back(detId);
        Module* m = &modules_.back();
        m->event_ = this;
        modules_by_id_[detId] = m;
        module_ptrs_.push_back(m);
        if (m->isLower()) lower_module_ptrs_.push_back(m);
        return *m;
    }
    Module& module_at(int32_t index) { return module_of(mod_detids_.at((size_t)index)); }
    Layer& layer_of(const Module& m) {
        const int l = m.layer();
        if (m.subdet() == Module::Barrel && l >= 1 && l <= 6) return barrel_[l];
        if (m.subdet() == Module::Endcap && l >= 1 && l <= 5) return endcap_[l];
        throw Error(SDLG_ERR_DETID, "module without a layer");
    }
    // drop the object graph of stages >= first (the hits and modules stay)
    void clear_stages(int first) {
        for (int s = first; s < 5; ++s) built_[s] = false;
        for (Module& m : modules_) {
            if (first <= 0) m.mds_.clear();
            if (first <= 1) m.sgs_.clear();
            if (first <= 2) m.tls_.clear();
            if (first <= 3) m.tps_.clear();
        }
        for (Layer* l : layer_ptrs_) {
            if (first <= 0) l->mds_.clear();
            if (first <= 1) l->sgs_.clear();
            if (first <= 2) l->tls_.clear();
            if (first <= 3) l->tps_.clear();
            l->tcs_.clear();
        }
        if (first <= 0) mds_.clear();
        if (first <= 1) {
            sgs_.clear();
            for (MiniDoublet& o : mds_) o.out_.clear(), o.in_.clear();
        }
        if (first <= 2) {
            tls_.clear();
            tl_vars_.clear();
            for (Segment& o : sgs_) o.tl_out_.clear(), o.tl_in_.clear();
        }
        if (first <= 3) tps_.clear();
        tcs_.clear();
    }
    void invalidate_graph() {
        clear_stages(0);
        hits_built_ = false;
        hits_.clear();
        modules_.clear();
        modules_by_id_.clear();
        module_ptrs_.clear();
        lower_module_ptrs_.clear();
        for (auto& a : hits_by_layer_) a.fill(0);
        ran_ = -1;
    }

    sdlg_ctx* ctx_ = nullptr;
    std::vector<float> x_, y_, z_;
    std::vector<int32_t> idx_;
    std::vector<uint32_t> det_;
    bool dirty_ = false;
    int sg_flags_ = 0, tl_flags_ = 0, tc_flags_ = 0;
    int ran_ = -1;
    int stage_ = -1;
    // object graph
    bool hits_built_ = false;
    bool built_[5] = {false, false, false, false, false};
    std::vector<Hit> hits_;
    std::deque<Module> modules_;
    std::map<unsigned int, Module*> modules_by_id_;
    std::vector<Module*> module_ptrs_, lower_module_ptrs_;
    std::array<Layer, 7> barrel_{}, endcap_{};
    std::vector<Layer*> layer_ptrs_;
    std::array<std::array<unsigned int, 6>, 4> hits_by_layer_{};
    std::vector<uint32_t> mod_detids_;
    std::vector<MiniDoublet> mds_;
    std::vector<Segment> sgs_;
    std::vector<Tracklet> tls_;
    std::vector<Triplet> tps_;
    std::vector<TrackCandidate> tcs_;
    std::vector<float> tl_vars_;
};

// accessors that build a stage's objects on first use
inline const std::vector<MiniDoublet*>& Module::getMiniDoubletPtrs() const {
    if (event_) event_->materialize(SDLG_STAGE_MD);
    return mds_;
}
inline const std::vector<Segment*>& Module::getSegmentPtrs() const {
    if (event_) event_->materialize(SDLG_STAGE_SG);
    return sgs_;
}
inline const std::vector<Triplet*>& Module::getTripletPtrs() const {
    if (event_) event_->materialize(SDLG_STAGE_TP);
    return tps_;
}
inline const std::vector<Tracklet*>& Module::getTrackletPtrs() const {
    if (event_) event_->materialize(SDLG_STAGE_TL);
    return tls_;
}
inline const std::vector<MiniDoublet*>& Layer::getMiniDoubletPtrs() const {
    if (event_) event_->materialize(SDLG_STAGE_MD);
    return mds_;
}
inline const std::vector<Segment*>& Layer::getSegmentPtrs() const {
    if (event_) event_->materialize(SDLG_STAGE_SG);
    return sgs_;
}
inline const std::vector<Triplet*>& Layer::getTripletPtrs() const {
    if (event_) event_->materialize(SDLG_STAGE_TP);
    return tps_;
}
inline const std::vector<Tracklet*>& Layer::getTrackletPtrs() const {
    if (event_) event_->materialize(SDLG_STAGE_TL);
    return tls_;
}
inline const std::vector<TrackCandidate*>& Layer::getTrackCandidatePtrs() const {
    if (event_) event_->materialize(SDLG_STAGE_TC);
    return tcs_;
}
inline const std::vector<Segment*>& MiniDoublet::getListOfOutwardSegmentPtrs() {
    if (event_) event_->materialize(SDLG_STAGE_SG);
    return out_;
}
inline const std::vector<Segment*>& MiniDoublet::getListOfInwardSegmentPtrs() {
    if (event_) event_->materialize(SDLG_STAGE_SG);
    return in_;
}
inline const std::vector<Tracklet*>& Segment::getListOfOutwardTrackletPtrs() {
    if (event_) event_->materialize(SDLG_STAGE_TL);
    return tl_out_;
}
inline const std::vector<Tracklet*>& Segment::getListOfInwardTrackletPtrs() {
    if (event_) event_->materialize(SDLG_STAGE_TL);
    return tl_in_;
}
inline const std::map<std::string, float>& Tracklet::getRecoVars() const { return event_->tracklet_vars(*this); }

}  // namespace SDL
