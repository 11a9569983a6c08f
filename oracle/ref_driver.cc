// Runs the UNMODIFIED reference chain (compiled from its own sources with the
// namespace renamed to SDLref) on one event and dumps every stage's objects as
// hit-index tuples.  Test infrastructure only: it builds the golden fixtures
// and validates the CPU restatement in this directory; nothing in the product
// links it.
//
// usage: ref_driver <tilted.txt> <endcap.txt> <map.txt> <hits.bin> <out.bin> [map|layer]
//
// Hit file: int64 n, float32 x[n], y[n], z[n], int32 idx[n], uint32 detid[n].
// Output file: for each stage MD, SG, TL, TP, TC: int64 count, int64 width,
// int32 tuples[count*width]; then 5 stages x {candidates, objects} x
// {barrel[6], endcap[5]} uint32 counters; then the per-stage seconds (5 double).
//
// The call sequence is the one a reference user makes (Event.h:210,239-300):
// load the three geometry singletons, add hits, then the create* stages.
#include <chrono>
#include <cstdint>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "Event.h"
#include "EndcapGeometry.h"
#include "ModuleConnectionMap.h"
#include "TiltedGeometry.h"
#include "TrackCandidate.h"

namespace {

void pushMD(std::vector<int32_t>& v, const SDL::MiniDoublet* md) {
    v.push_back(md->lowerHitPtr()->idx());
    v.push_back(md->upperHitPtr()->idx());
}
void pushSG(std::vector<int32_t>& v, const SDL::Segment* sg) {
    pushMD(v, sg->innerMiniDoubletPtr());
    pushMD(v, sg->outerMiniDoubletPtr());
}
void pushTLB(std::vector<int32_t>& v, const SDL::TrackletBase* tl) {
    pushSG(v, tl->innerSegmentPtr());
    pushSG(v, tl->outerSegmentPtr());
}

void writeStage(FILE* f, const std::vector<int32_t>& v, int64_t width) {
    int64_t n = width ? (int64_t)v.size() / width : 0;
    fwrite(&n, 8, 1, f);
    fwrite(&width, 8, 1, f);
    if (!v.empty()) fwrite(v.data(), 4, v.size(), f);
}

double now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 6) {
        std::fprintf(stderr, "usage: %s tilted endcap map hits.bin out.bin [map|layer|nav|tctl|tctp]\n", argv[0]);
        return 2;
    }
    std::string mode = argc > 6 ? argv[6] : "map";
    SDL::tiltedGeometry.load(argv[1]);
    SDL::endcapGeometry.load(argv[2]);
    SDL::moduleConnectionMap.load(argv[3]);

    FILE* fh = std::fopen(argv[4], "rb");
    if (!fh) { std::perror("hits"); return 1; }
    int64_t n = 0;
    if (std::fread(&n, 8, 1, fh) != 1) return 1;
    std::vector<float> x(n), y(n), z(n);
    std::vector<int32_t> idx(n);
    std::vector<uint32_t> det(n);
    if (n > 0) {
        if (std::fread(x.data(), 4, n, fh) != (size_t)n || std::fread(y.data(), 4, n, fh) != (size_t)n ||
            std::fread(z.data(), 4, n, fh) != (size_t)n || std::fread(idx.data(), 4, n, fh) != (size_t)n ||
            std::fread(det.data(), 4, n, fh) != (size_t)n) {
            std::fprintf(stderr, "short hit file\n");
            return 1;
        }
    }
    std::fclose(fh);

    SDL::Event ev;
    for (int64_t i = 0; i < n; ++i) ev.addHitToModule(SDL::Hit(x[i], y[i], z[i], idx[i]), det[i]);

    double t[5];
    double t0 = now();
    ev.createMiniDoublets();
    t[0] = now() - t0; t0 = now();
    // mode tokens: "layer" (createSegments + createTracklets), "nav"
    // (createTrackletsViaNavigation), "tctl" / "tctp" (createTrackCandidatesFrom
    // Tracklets / Triplets); the module-map variants otherwise
    const bool layer = mode.find("layer") != std::string::npos;
    const bool nav = mode.find("nav") != std::string::npos;
    const bool tctl = mode.find("tctl") != std::string::npos;
    const bool tctp = mode.find("tctp") != std::string::npos;
    if (layer) ev.createSegments(); else ev.createSegmentsWithModuleMap();
    t[1] = now() - t0; t0 = now();
    if (layer) ev.createTracklets();
    else if (nav) ev.createTrackletsViaNavigation();
    else ev.createTrackletsWithModuleMap();
    t[2] = now() - t0; t0 = now();
    ev.createTriplets();
    t[3] = now() - t0; t0 = now();
    if (tctp) ev.createTrackCandidatesFromTriplets();
    else if (tctl) ev.createTrackCandidatesFromTracklets();
    else ev.createTrackCandidates();
    t[4] = now() - t0;

    // the tracklets' final recovars (Tracklet.cc:1440-1495) in tracklet order
    static const char* const kVars[15] = {"betaIn", "betaInRHmin", "betaInRHmax", "betaOut", "betaOutRHmin",
                                          "betaOutRHmax", "betaAv", "pt_beta", "dBeta", "dBetaCut2", "dBetaLum2",
                                          "dBetaMuls", "dBetaRes", "dBetaRIn2", "dBetaROut2"};
    std::vector<float> tlvars;
    std::vector<int32_t> md, sg, tl, tp, tc;
    for (SDL::Layer* L : ev.getLayerPtrs()) {
        for (auto* o : L->getMiniDoubletPtrs()) pushMD(md, o);
        for (auto* o : L->getSegmentPtrs()) pushSG(sg, o);
        for (auto* o : L->getTrackletPtrs()) {
            pushTLB(tl, o);
            const auto& rv = o->getRecoVars();
            for (const char* k : kVars) {
                auto it = rv.find(k);
                tlvars.push_back(it == rv.end() ? std::nanf("") : it->second);
            }
        }
        for (auto* o : L->getTripletPtrs()) pushTLB(tp, o);
        for (auto* o : L->getTrackCandidatePtrs()) {
            pushTLB(tc, o->innerTrackletBasePtr());
            pushTLB(tc, o->outerTrackletBasePtr());
        }
    }
    FILE* fo = std::fopen(argv[5], "wb");
    if (!fo) { std::perror("out"); return 1; }
    writeStage(fo, md, 2);
    writeStage(fo, sg, 4);
    writeStage(fo, tl, 8);
    writeStage(fo, tp, 8);
    writeStage(fo, tc, 16);
    std::vector<uint32_t> cnt;
    for (unsigned i = 0; i < 6; ++i) cnt.push_back(ev.getNumberOfMiniDoubletCandidatesByLayerBarrel(i));
    for (unsigned i = 0; i < 5; ++i) cnt.push_back(ev.getNumberOfMiniDoubletCandidatesByLayerEndcap(i));
    for (unsigned i = 0; i < 6; ++i) cnt.push_back(ev.getNumberOfMiniDoubletsByLayerBarrel(i));
    for (unsigned i = 0; i < 5; ++i) cnt.push_back(ev.getNumberOfMiniDoubletsByLayerEndcap(i));
    for (unsigned i = 0; i < 6; ++i) cnt.push_back(ev.getNumberOfSegmentCandidatesByLayerBarrel(i));
    for (unsigned i = 0; i < 5; ++i) cnt.push_back(ev.getNumberOfSegmentCandidatesByLayerEndcap(i));
    for (unsigned i = 0; i < 6; ++i) cnt.push_back(ev.getNumberOfSegmentsByLayerBarrel(i));
    for (unsigned i = 0; i < 5; ++i) cnt.push_back(ev.getNumberOfSegmentsByLayerEndcap(i));
    for (unsigned i = 0; i < 6; ++i) cnt.push_back(ev.getNumberOfTrackletCandidatesByLayerBarrel(i));
    for (unsigned i = 0; i < 5; ++i) cnt.push_back(ev.getNumberOfTrackletCandidatesByLayerEndcap(i));
    for (unsigned i = 0; i < 6; ++i) cnt.push_back(ev.getNumberOfTrackletsByLayerBarrel(i));
    for (unsigned i = 0; i < 5; ++i) cnt.push_back(ev.getNumberOfTrackletsByLayerEndcap(i));
    for (unsigned i = 0; i < 6; ++i) cnt.push_back(ev.getNumberOfTripletCandidatesByLayerBarrel(i));
    for (unsigned i = 0; i < 5; ++i) cnt.push_back(ev.getNumberOfTripletCandidatesByLayerEndcap(i));
    for (unsigned i = 0; i < 6; ++i) cnt.push_back(ev.getNumberOfTripletsByLayerBarrel(i));
    for (unsigned i = 0; i < 5; ++i) cnt.push_back(ev.getNumberOfTripletsByLayerEndcap(i));
    for (unsigned i = 0; i < 6; ++i) cnt.push_back(ev.getNumberOfTrackCandidateCandidatesByLayerBarrel(i));
    for (unsigned i = 0; i < 5; ++i) cnt.push_back(ev.getNumberOfTrackCandidateCandidatesByLayerEndcap(i));
    for (unsigned i = 0; i < 6; ++i) cnt.push_back(ev.getNumberOfTrackCandidatesByLayerBarrel(i));
    for (unsigned i = 0; i < 5; ++i) cnt.push_back(ev.getNumberOfTrackCandidatesByLayerEndcap(i));
    fwrite(cnt.data(), 4, cnt.size(), fo);
    fwrite(t, 8, 5, fo);
    if (argc > 7) {  // optional: the tracklet recovars, 15 floats per tracklet of stage 2
        FILE* fv = std::fopen(argv[7], "wb");
        if (!fv) { std::perror("vars"); return 1; }
        fwrite(tlvars.data(), 4, tlvars.size(), fv);
        std::fclose(fv);
    }
    std::fclose(fo);
    std::fprintf(stderr, "ref: hits %lld MD %zu SG %zu TL %zu TP %zu TC %zu | s: %.3f %.3f %.3f %.3f %.3f\n",
                 (long long)n, md.size() / 2, sg.size() / 4, tl.size() / 8, tp.size() / 8, tc.size() / 16,
                 t[0], t[1], t[2], t[3], t[4]);
    return 0;
}
