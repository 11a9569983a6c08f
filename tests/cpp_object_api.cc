// Walks the object graph of include/sdl_event.hpp the way a caller of the
// reference does (Event::getLowerModulePtrs -> Module::get*Ptrs -> the
// objects' pointer accessors; Event::getLayerPtrs -> Layer::get*Ptrs) and
// writes what it finds, plus the time of the five create* calls and of one
// whole chain run on the same event.
//   cpp_object_api <tilted> <endcap> <map> <hits.bin> <out.bin> [map|layer|tctl|tctp]
// out.bin: for MD, SG, TL, TP, TC: int64 n, then n rows of the hit-index
// tuple (2, 4, 8, 8, 16 int32) followed for MD by 4 and for SG by 6 float32
// (getDz, getShiftedDz, getDeltaPhi, getDeltaPhiChange; getDeltaPhi,
// getDeltaPhiMin, getDeltaPhiMax, getDeltaPhiChange, getDeltaPhiMinChange,
// getDeltaPhiMaxChange); then uint32 hits by layer [4][6] (barrel, endcap,
// barrel upper, endcap upper); then uint32 getNumberOf*[5] and the number of
// failed consistency checks; then float64 ms of the five create* calls (a
// second pass on warm buffers) and of one sdlg_run of the whole chain.
#include <chrono>
#include <cstdio>
#include <string>
#include <vector>

#include "sdl_event.hpp"

namespace {
double ms_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}
void put_md(std::vector<int32_t>& v, const SDL::MiniDoublet* md) {
    v.push_back(md->lowerHitPtr()->idx());
    v.push_back(md->upperHitPtr()->idx());
}
void put_sg(std::vector<int32_t>& v, const SDL::Segment* sg) {
    put_md(v, sg->innerMiniDoubletPtr());
    put_md(v, sg->outerMiniDoubletPtr());
}
void put_tb(std::vector<int32_t>& v, const SDL::TrackletBase* t) {
    put_sg(v, t->innerSegmentPtr());
    put_sg(v, t->outerSegmentPtr());
}
struct Table {
    std::vector<int32_t> idx;
    std::vector<float> val;
    int64_t n = 0;
};
void write(std::FILE* f, const Table& t) {
    std::fwrite(&t.n, 8, 1, f);
    const size_t w = t.n ? t.idx.size() / t.n : 0, nv = t.n ? t.val.size() / t.n : 0;
    for (int64_t k = 0; k < t.n; ++k) {
        std::fwrite(t.idx.data() + k * w, 4, w, f);
        if (nv) std::fwrite(t.val.data() + k * nv, 4, nv, f);
    }
}
}  // namespace

int main(int argc, char** argv) {
    if (argc < 6) return 2;
    SDL::tiltedGeometry.load(argv[1]);
    SDL::endcapGeometry.load(argv[2]);
    SDL::moduleConnectionMap.load(argv[3]);
    std::FILE* f = std::fopen(argv[4], "rb");
    if (!f) return 2;
    int64_t n = 0;
    if (std::fread(&n, 8, 1, f) != 1) return 2;
    std::vector<float> x(n), y(n), z(n);
    std::vector<int32_t> idx(n);
    std::vector<uint32_t> det(n);
    size_t ok = std::fread(x.data(), 4, n, f) + std::fread(y.data(), 4, n, f) + std::fread(z.data(), 4, n, f) +
                std::fread(idx.data(), 4, n, f) + std::fread(det.data(), 4, n, f);
    std::fclose(f);
    if (ok != (size_t)(5 * n)) return 2;
    const std::string mode = argc > 6 ? argv[6] : "map";
    try {
        SDL::Event ev;
        for (int64_t i = 0; i < n; ++i) ev.addHitToModule(SDL::Hit(x[i], y[i], z[i], idx[i]), det[i]);
        auto chain = [&]() {
            ev.createMiniDoublets();
            if (mode == "layer") ev.createSegments();
            else ev.createSegmentsWithModuleMap();
            if (mode == "layer") ev.createTracklets();
            else ev.createTrackletsWithModuleMap();
            ev.createTriplets();
            if (mode == "tctl") ev.createTrackCandidatesFromTracklets();
            else if (mode == "tctp") ev.createTrackCandidatesFromTriplets();
            else ev.createTrackCandidates();
        };
        chain();  // first pass: allocates the device buffers
        const auto t0 = std::chrono::steady_clock::now();
        chain();
        const double t_create = ms_since(t0);

        Table md, sg, tl, tp, tc;
        uint32_t bad = 0;
        for (SDL::Module* m : ev.getLowerModulePtrs()) {
            for (SDL::MiniDoublet* o : m->getMiniDoubletPtrs()) {
                put_md(md.idx, o);
                md.val.insert(md.val.end(), {o->getDz(), o->getShiftedDz(), o->getDeltaPhi(), o->getDeltaPhiChange()});
                ++md.n;
                bad += o->lowerHitPtr()->getModule().detId() != m->detId();
                bad += o->upperHitPtr()->getModule().detId() != m->partnerDetId();
            }
            for (SDL::Segment* o : m->getSegmentPtrs()) {
                put_sg(sg.idx, o);
                sg.val.insert(sg.val.end(), {o->getDeltaPhi(), o->getDeltaPhiMin(), o->getDeltaPhiMax(),
                                             o->getDeltaPhiChange(), o->getDeltaPhiMinChange(), o->getDeltaPhiMaxChange()});
                ++sg.n;
                // Segment.cc:58-62: the segment is in its mini-doublets' outward / inward lists
                bool found = false;
                for (SDL::Segment* s : o->innerMiniDoubletPtr()->getListOfOutwardSegmentPtrs()) found |= s == o;
                bad += !found;
                found = false;
                for (SDL::Segment* s : o->outerMiniDoubletPtr()->getListOfInwardSegmentPtrs()) found |= s == o;
                bad += !found;
                bad += o->getRtIn() != o->innerMiniDoubletPtr()->anchorHitPtr()->rt();
            }
            for (SDL::Triplet* o : m->getTripletPtrs()) {
                put_tb(tp.idx, o);
                ++tp.n;
            }
        }
        // tracklets and track candidates through the layers (the layer-pair
        // tracklets are listed in no module)
        for (SDL::Layer* l : ev.getLayerPtrs()) {
            for (SDL::Tracklet* o : l->getTrackletPtrs()) {
                put_tb(tl.idx, o);
                ++tl.n;
            }
            for (SDL::TrackCandidate* o : l->getTrackCandidatePtrs()) {
                if (mode == "tctp") {
                    put_tb(tc.idx, o->innerTripletPtr());
                    put_tb(tc.idx, o->outerTripletPtr());
                    try {
                        (void)o->innerTrackletPtr();
                        ++bad;  // a triplet candidate has no tracklet
                    } catch (const std::logic_error&) {
                    }
                } else {
                    put_tb(tc.idx, o->innerTrackletPtr());
                    put_tb(tc.idx, o->outerTrackletPtr());
                }
                ++tc.n;
            }
        }
        uint32_t hl[24];
        for (unsigned i = 0; i < 6; ++i) {
            hl[i] = ev.getNumberOfHitsByLayerBarrel(i);
            hl[6 + i] = i < 5 ? ev.getNumberOfHitsByLayerEndcap(i) : 0;
            hl[12 + i] = ev.getNumberOfHitsByLayerBarrelUpperModule(i);
            hl[18 + i] = i < 5 ? ev.getNumberOfHitsByLayerEndcapUpperModule(i) : 0;
        }
        const uint32_t cnt[6] = {ev.getNumberOfMiniDoublets(), ev.getNumberOfSegments(), ev.getNumberOfTracklets(),
                                 ev.getNumberOfTriplets(), ev.getNumberOfTrackCandidates(), bad};
        // one run of the whole chain on the same event (graph instantiated by the first)
        const int flags = (mode == "layer" ? SDLG_FLAG_SG_LAYERS | SDLG_FLAG_TL_LAYERS : 0) |
                          (mode == "tctl" ? SDLG_FLAG_TC_FROM_TL : 0) | (mode == "tctp" ? SDLG_FLAG_TC_FROM_TP : 0);
        if (sdlg_run(ev.context(), 4, flags) != SDLG_OK) return 1;
        const auto t1 = std::chrono::steady_clock::now();
        if (sdlg_run(ev.context(), 4, flags) != SDLG_OK) return 1;
        const double t_run = ms_since(t1);

        std::FILE* o = std::fopen(argv[5], "wb");
        if (!o) return 2;
        for (const Table* t : {&md, &sg, &tl, &tp, &tc}) write(o, *t);
        std::fwrite(hl, 4, 24, o);
        std::fwrite(cnt, 4, 6, o);
        const double times[2] = {t_create, t_run};
        std::fwrite(times, 8, 2, o);
        std::fclose(o);
        std::printf("create* %.3f ms, one chain run %.3f ms, inconsistencies %u\n", t_create, t_run, bad);
    } catch (const SDL::Error& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return e.code == SDLG_ERR_NO_DEVICE ? 3 : 1;
    }
    return 0;
}
