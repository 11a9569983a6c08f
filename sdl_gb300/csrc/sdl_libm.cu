// The host libm's float functions on the device.
//
// The reference calls std::asin, std::atan, std::sin, std::cos and std::tan
// on floats (e.g. MiniDoublet.cc:777 and 1017-1071, Segment.cc:446-448 and
// 915, Tracklet.cc:1270 and 3195-3215), which resolve to the host C
// library's float functions (glibc's asinf, atanf, sinf, cosf, tanf).  These
// are not correctly rounded: on glibc 2.39 they return the neighbour of the
// correctly rounded float for 0.4-3 % of the inputs, and a cut decision that
// sits exactly at its threshold then depends on it.  The device evaluates the
// correctly rounded float (sdl_device.cuh) and moves it to the host
// function's value with a table built here, once per process, by calling the
// host's own functions: for every |x| bit pattern of a function's range, a
// 2-bit code (same value, next float up, next float down, or an entry of an
// exception list).  Outside the ranges below the host functions return the
// correctly rounded value (tiny arguments, where f(x) rounds to x or 1, and
// atan of large arguments); sdlg_libm_eval lets a test check the device's
// values against the host's on every float of each function's domain.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>
#include <thread>
#include <utility>
#include <vector>

#include "sdl_kernels.h"

namespace sdlg {
namespace {

// |x| ranges of the tables: [2^-12, hi[fn]] (the arguments the chain passes:
// asin of at most 0.95, tan of an asin of at most 0.95, sin and cos of
// angles in [0, 2 pi] and differences of angles, atan of any float)
const float kLo = 0x1p-12f;
const float kHi[kLmCount] = {0.95f, 0x1p27f, 6.3f, 6.3f, 1.26f};

struct HostTab {
    uint32_t lo = 0, n = 0;
    std::vector<uint32_t> code;
    std::vector<std::pair<uint32_t, float>> exc;
};
HostTab g_host[kLmCount];
std::once_flag g_host_once;

inline uint32_t bits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}
inline float from_bits(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

float host_float(int fn, float x) {
    switch (fn) {
        case kLmAsin: return std::asin(x);
        case kLmAtan: return std::atan(x);
        case kLmSin: return std::sin(x);
        case kLmCos: return std::cos(x);
        default: return std::tan(x);
    }
}
double host_double(int fn, double x) {
    switch (fn) {
        case kLmAsin: return std::asin(x);
        case kLmAtan: return std::atan(x);
        case kLmSin: return std::sin(x);
        case kLmCos: return std::cos(x);
        default: return std::tan(x);
    }
}

// codes of table words [w0, w1) of function fn
void fill_words(int fn, uint64_t w0, uint64_t w1, std::vector<std::pair<uint32_t, float>>& exc) {
    HostTab& t = g_host[fn];
    for (uint64_t w = w0; w < w1; ++w) {
        uint32_t word = 0;
        for (uint32_t j = 0; j < 16; ++j) {
            const uint64_t k = w * 16 + j;
            if (k >= t.n) break;
            const uint32_t u = t.lo + (uint32_t)k;
            const float x = from_bits(u);
            const float g = host_float(fn, x);
            const float r = (float)host_double(fn, (double)x);
            uint32_t c;
            if (g == r) c = 0;
            else if (g == std::nextafter(r, INFINITY)) c = 1;
            else if (g == std::nextafter(r, -INFINITY)) c = 2;
            else {
                c = 3;
                exc.push_back({u, g});
            }
            word |= c << (2 * j);
        }
        t.code[w] = word;
    }
}

void build_host_tables() {
    uint64_t total = 0;
    for (int fn = 0; fn < kLmCount; ++fn) {
        HostTab& t = g_host[fn];
        t.lo = bits(kLo);
        t.n = bits(kHi[fn]) - t.lo + 1;
        t.code.assign((t.n + 15) / 16, 0u);
        total += t.code.size();
    }
    // chunks of 4096 words (65,536 floats) handed out to the host's threads
    const uint64_t kChunk = 4096;
    std::vector<std::pair<int, uint64_t>> chunks;
    for (int fn = 0; fn < kLmCount; ++fn)
        for (uint64_t w = 0; w < g_host[fn].code.size(); w += kChunk) chunks.push_back({fn, w});
    std::atomic<size_t> next(0);
    std::mutex mu;
    auto work = [&]() {
        std::vector<std::pair<uint32_t, float>> exc[kLmCount];
        for (;;) {
            const size_t c = next.fetch_add(1);
            if (c >= chunks.size()) break;
            const int fn = chunks[c].first;
            const uint64_t w0 = chunks[c].second;
            fill_words(fn, w0, std::min<uint64_t>(w0 + kChunk, g_host[fn].code.size()), exc[fn]);
        }
        std::lock_guard<std::mutex> lk(mu);
        for (int fn = 0; fn < kLmCount; ++fn) g_host[fn].exc.insert(g_host[fn].exc.end(), exc[fn].begin(), exc[fn].end());
    };
    const unsigned nt = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (unsigned i = 0; i < nt; ++i) th.emplace_back(work);
    for (auto& x : th) x.join();
    for (int fn = 0; fn < kLmCount; ++fn) std::sort(g_host[fn].exc.begin(), g_host[fn].exc.end());
    (void)total;
}

constexpr int kMaxDevices = 64;
std::mutex g_dev_mu;
bool g_dev_ok[kMaxDevices] = {};
LibmTab g_dev_tab[kMaxDevices][kLmCount];

}  // namespace

int libm_setup(int device, const char** err) {
    if (device < 0 || device >= kMaxDevices) {
        *err = "device ordinal out of range for the libm tables";
        return -1;
    }
    std::call_once(g_host_once, build_host_tables);
    std::lock_guard<std::mutex> lk(g_dev_mu);
    if (!g_dev_ok[device]) {
        for (int fn = 0; fn < kLmCount; ++fn) {
            const HostTab& h = g_host[fn];
            LibmTab& t = g_dev_tab[device][fn];
            t = LibmTab{};
            uint32_t* code = nullptr;
            uint32_t* ex = nullptr;
            float* ev = nullptr;
            const size_t ne = std::max<size_t>(1, h.exc.size());
            std::vector<uint32_t> hx(ne, 0);
            std::vector<float> hv(ne, 0.f);
            for (size_t i = 0; i < h.exc.size(); ++i) {
                hx[i] = h.exc[i].first;
                hv[i] = h.exc[i].second;
            }
            if (cudaMalloc(&code, h.code.size() * sizeof(uint32_t)) != cudaSuccess ||
                cudaMalloc(&ex, ne * sizeof(uint32_t)) != cudaSuccess || cudaMalloc(&ev, ne * sizeof(float)) != cudaSuccess ||
                cudaMemcpy(code, h.code.data(), h.code.size() * sizeof(uint32_t), cudaMemcpyHostToDevice) != cudaSuccess ||
                cudaMemcpy(ex, hx.data(), ne * sizeof(uint32_t), cudaMemcpyHostToDevice) != cudaSuccess ||
                cudaMemcpy(ev, hv.data(), ne * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
                *err = "device memory for the libm tables";
                return -1;
            }
            t.code = code;
            t.exc_x = ex;
            t.exc_v = ev;
            t.lo = h.lo;
            t.n = h.n;
            t.n_exc = (uint32_t)h.exc.size();
        }
        g_dev_ok[device] = true;
    }
    if (set_libm_tables(g_dev_tab[device]) != cudaSuccess) {
        *err = "cudaMemcpyToSymbol of the libm tables";
        return -1;
    }
    return 0;
}

void libm_stats(int fn, uint64_t* out3) {
    std::call_once(g_host_once, build_host_tables);
    const HostTab& t = g_host[fn];
    uint64_t moved = 0;
    for (uint32_t w : t.code)
        for (int j = 0; j < 16; ++j) moved += ((w >> (2 * j)) & 3u) != 0;
    out3[0] = t.n;
    out3[1] = moved;
    out3[2] = t.exc.size();
}

}  // namespace sdlg
