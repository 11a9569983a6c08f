// Drives the chain through include/sdl_event.hpp exactly as a caller of the
// reference's SDL::Event would, and prints the object counts per stage.
//   cpp_event_api <tilted> <endcap> <map> <hits.bin> [map|layer|nav|tctl|tctp]
// "layer" selects createSegments / createTracklets (layer pairs) instead of
// the module-map variants, "nav" createTrackletsViaNavigation, "tctl" /
// "tctp" createTrackCandidatesFromTracklets / FromTriplets.
// hits.bin: int64 n, float32 x[n], y[n], z[n], int32 idx[n], uint32 detid[n].
// Exit code 3 when no CUDA device is available.
#include <cstdio>
#include <string>
#include <vector>

#include "sdl_event.hpp"

int main(int argc, char** argv) {
    if (argc < 5) return 2;
    SDL::tiltedGeometry.load(argv[1]);
    SDL::endcapGeometry.load(argv[2]);
    SDL::moduleConnectionMap.load(argv[3]);
    FILE* f = std::fopen(argv[4], "rb");
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
    try {
        SDL::Event ev;
        for (int64_t i = 0; i < n; ++i) ev.addHitToModule(SDL::Hit(x[i], y[i], z[i], idx[i]), det[i]);
        ev.createMiniDoublets();
        const std::string mode = argc > 5 ? argv[5] : "map";
        const bool layer = mode == "layer";
        if (layer) ev.createSegments();
        else ev.createSegmentsWithModuleMap();
        if (layer) ev.createTracklets();
        else if (mode == "nav") ev.createTrackletsViaNavigation();
        else ev.createTrackletsWithModuleMap();
        ev.createTriplets();
        if (mode == "tctl") ev.createTrackCandidatesFromTracklets();
        else if (mode == "tctp") ev.createTrackCandidatesFromTriplets();
        else ev.createTrackCandidates();
        std::printf("%u %u %u %u %u %u\n", ev.getNumberOfHits(), ev.getNumberOfMiniDoublets(), ev.getNumberOfSegments(),
                    ev.getNumberOfTracklets(), ev.getNumberOfTriplets(), ev.getNumberOfTrackCandidates());
        const auto tc = ev.getTrackCandidates();
        std::printf("tc0 %d\n", tc.empty() ? -1 : tc[0][0]);
    } catch (const SDL::Error& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return e.code == SDLG_ERR_NO_DEVICE ? 3 : 1;
    }
    return 0;
}
