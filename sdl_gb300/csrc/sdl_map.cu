// Straight-line module connection map on the GPU.
//
// The reference reads its module map from a text file
// (ModuleConnectionMap.cc:18-47: "detId n d1 .. dn" per lower module) and
// builds none; the map of the synthetic detector is made by propagating
// straight lines from the luminous region.  For every lower module, lines
// from five vertex positions z0 in [-15, 15] cm through nine points of the
// module (a 3 x 3 grid at 0 and +-98 % of its half extents) are extended to
// the next layer (the next barrel cylinder, or the first disk when they
// leave the barrel; the next disk for endcap modules), widened in phi by the
// bend of a 1 GeV track between the two radii, and the lower module covering
// each crossing is connected.  One thread per (module, point, vertex) makes
// the crossings in double precision; the host sorts and deduplicates the
// pairs into the map's CSR.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/sdl_gpu.h"

namespace {

constexpr double kTwoPi = 2.0 * M_PI;

struct Layout {
    double barrel_r[6];
    int barrel_nphi[6];
    double zmax, mod_dz, flat_zmax_tilted, lum_z, r1gev;
    int n_tilt_rings, has_tilt, has_endcap;
    double disk_z[5];
    int disk_nrings[5];
    double ec_rmin, ec_rmax;
};

// x mod 2 pi in [0, 2 pi) (floored modulo)
__device__ __forceinline__ double mod2pi(double x) {
    double m = fmod(x, kTwoPi);
    if (m != 0.0 && m < 0.0) m += kTwoPi;
    return m;
}
__device__ __forceinline__ int64_t imod(int64_t a, int64_t n) { return ((a % n) + n) % n; }

// lower detId of the barrel module covering (phi, z) in `layer`, 0 if none
__device__ uint32_t barrel_lower(const Layout& L, int layer, double phi, double z) {
    const int nphi = L.barrel_nphi[layer - 1];
    const int64_t k = imod((int64_t)floor(mod2pi(phi) / (kTwoPi / nphi) + 0.5), nphi) + 1;
    const bool use_tilt = L.has_tilt && layer <= 3;
    const double zflat = use_tilt ? L.flat_zmax_tilted : L.zmax;
    const bool flat = fabs(z) < zflat;
    const int64_t nz = (int64_t)llrint(2.0 * zflat / L.mod_dz);
    int64_t iz = (int64_t)floor((z + zflat) / L.mod_dz) + 1;
    iz = iz < 1 ? 1 : (iz > nz ? nz : iz);
    const bool inv = layer <= 3 ? (iz % 2 == 1) : (iz % 2 == 0);
    uint32_t out = 0;
    if (flat)
        out = (5u << 25) | ((uint32_t)layer << 20) | (3u << 18) | ((uint32_t)k << 10) | ((uint32_t)iz << 2) | (inv ? 2u : 1u);
    if (use_tilt) {
        const double zabs = fabs(z);
        int64_t ring = (int64_t)floor((zabs - L.flat_zmax_tilted) / L.mod_dz);
        ring = ring < 0 ? 0 : (ring > L.n_tilt_rings - 1 ? L.n_tilt_rings - 1 : ring);
        const uint32_t side = z > 0 ? 2u : 1u;
        const int64_t rod = side == 2 ? ring + 1 : L.n_tilt_rings - ring;
        const bool tinv = layer <= 2 ? (k % 2 == 1) : (k % 2 == 0);
        if (!flat && zabs <= L.zmax)
            out = (5u << 25) | ((uint32_t)layer << 20) | (side << 18) | ((uint32_t)rod << 10) | ((uint32_t)k << 2) |
                  (tinv ? 2u : 1u);
    }
    return fabs(z) <= L.zmax ? out : 0u;
}

// lower detId of the endcap module covering (rho, phi) on disk `disk`, side `side`, 0 if none
__device__ uint32_t endcap_lower(const Layout& L, int disk, int side, double rho, double phi) {
    const int nr = L.disk_nrings[disk - 1];
    const double dr_ring = (L.ec_rmax - L.ec_rmin) / nr;
    int64_t ring = (int64_t)floor((rho - L.ec_rmin) / dr_ring) + 1;
    const bool ok = rho >= L.ec_rmin && rho < L.ec_rmax;
    ring = ring < 1 ? 1 : (ring > nr ? nr : ring);
    const double rm = L.ec_rmin + dr_ring * ((double)ring - 0.5);
    const int64_t nmod = (int64_t)ceil(2.0 * M_PI * rm / 10.0);
    const int64_t k = imod((int64_t)floor(mod2pi(phi) / (kTwoPi / (double)nmod) + 0.5), nmod) + 1;
    const bool inv = side == 1 ? (k % 2 == 1) : (k % 2 == 0);
    const uint32_t id = (4u << 25) | ((uint32_t)side << 23) | ((uint32_t)disk << 18) | ((uint32_t)ring << 12) |
                        ((uint32_t)k << 2) | (inv ? 2u : 1u);
    return ok ? id : 0u;
}

// |asin(min(rho / 2R, 1)) - asin(min(rhoP / 2R, 1))|: the bend of a 1 GeV track between two radii
__device__ __forceinline__ double bend(const Layout& L, double rho, double rhoP) {
    const double d = 2.0 * L.r1gev;
    return fabs(asin(fmin(rho / d, 1.0)) - asin(fmin(rhoP / d, 1.0)));
}

// geometry of a lower module (16 doubles): center xyz, tangential axis xyz,
// long axis xyz, half width, half length, ring radii r0 r1, centre phi, half
// phi width, tilt angle
__global__ void k_line_map(Layout L, int64_t n, const uint32_t* __restrict__ detid, const int8_t* __restrict__ kind,
                           const double* __restrict__ g, uint32_t* __restrict__ out) {
    const double fr[3] = {-0.98, 0.0, 0.98};
    const double z0s[5] = {-L.lum_z, -L.lum_z / 2, 0.0, L.lum_z / 2, L.lum_z};
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n * 45; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t m = q / 45;
        const int s = (int)((q / 5) % 9), zi = (int)(q % 5);
        uint32_t* o = out + 3 * q;
        o[0] = o[1] = o[2] = 0u;
        const double a = fr[s / 3], b = fr[s % 3], z0 = z0s[zi];
        const double* G = g + 16 * m;
        const int kd = kind[m];
        double P[3];
        if (kd == 2) {  // endcap: a point of the ring sector
            const double rho_e = 0.5 * (G[11] + G[12]) + 0.5 * a * (G[12] - G[11]);
            const double ph_e = G[13] + b * G[14];
            P[0] = rho_e * cos(ph_e);
            P[1] = rho_e * sin(ph_e);
            P[2] = G[2];
        } else {  // barrel: centre + a * half width * t + b * half length * u
            const double hu = kd == 1 ? G[10] / cos(G[15]) : G[10];
            for (int c = 0; c < 3; ++c) P[c] = G[c] + (a * G[9]) * G[3 + c] + (b * hu) * G[6 + c];
        }
        const uint32_t d = detid[m];
        const bool isec = kd == 2;
        const int layer = isec ? (int)((d >> 18) & 7) : (int)((d >> 20) & 7);
        const double rhoP = hypot(P[0], P[1]);
        const double phiP = atan2(P[1], P[0]);
        if (!isec) {
            if (layer < 1 || layer > 5) continue;
            const double rn = L.barrel_r[layer];
            const double zq = z0 + (P[2] - z0) * (rn / rhoP);
            if (fabs(zq) <= L.zmax) {
                const double dphi = bend(L, rn, rhoP);
                for (int k = 0; k < 3; ++k) o[k] = barrel_lower(L, layer + 1, phiP + (k - 1) * dphi, zq);
            } else if (L.has_endcap) {
                const int side = zq > 0 ? 2 : 1;
                const double zd = side == 2 ? L.disk_z[0] : -L.disk_z[0];
                const double lamd = (zd - z0) / (P[2] - z0);
                if (lamd > 1) {
                    const double rho = rhoP * lamd;
                    const double dphi = bend(L, rho, rhoP);
                    for (int k = 0; k < 3; ++k) o[k] = endcap_lower(L, 1, side, rho, phiP + (k - 1) * dphi);
                }
            }
        } else if (L.has_endcap && layer >= 1 && layer <= 4) {
            const int side = (int)((d >> 23) & 3);
            const double zn = side == 2 ? L.disk_z[layer] : -L.disk_z[layer];
            const double lamd = (zn - z0) / (P[2] - z0);
            const double rho = rhoP * lamd;
            const double dphi = bend(L, rho, rhoP);
            for (int k = 0; k < 3; ++k) o[k] = endcap_lower(L, layer + 1, side, rho, phiP + (k - 1) * dphi);
        }
    }
}

}  // namespace

extern "C" int sdlg_build_line_map(int device, const sdlg_line_map_layout* layout, int64_t n, const uint32_t* detid,
                                   const int8_t* kind, const double* geom, int64_t cap_keys, int64_t cap_dst,
                                   uint32_t* keys, int64_t* off, uint32_t* dst, int64_t* n_keys, int64_t* n_dst) {
    if (!layout || n < 0 || !n_keys || !n_dst || (n > 0 && (!detid || !kind || !geom))) return SDLG_ERR_ARG;
    Layout L;
    for (int i = 0; i < 6; ++i) {
        L.barrel_r[i] = layout->barrel_r[i];
        L.barrel_nphi[i] = layout->barrel_nphi[i];
        if (L.barrel_nphi[i] <= 0) return SDLG_ERR_ARG;
    }
    L.zmax = layout->zmax;
    L.mod_dz = layout->module_dz;
    L.flat_zmax_tilted = layout->flat_zmax_tilted;
    L.lum_z = layout->lum_z;
    L.r1gev = layout->radius_1gev;
    L.n_tilt_rings = layout->n_tilt_rings;
    L.has_tilt = layout->has_tilt;
    L.has_endcap = layout->has_endcap;
    for (int i = 0; i < 5; ++i) {
        L.disk_z[i] = layout->disk_z[i];
        L.disk_nrings[i] = layout->disk_nrings[i];
        if (L.has_endcap && L.disk_nrings[i] <= 0) return SDLG_ERR_ARG;
    }
    L.ec_rmin = layout->ec_rmin;
    L.ec_rmax = layout->ec_rmax;
    if (!(L.mod_dz > 0) || !(L.r1gev > 0) || (L.has_tilt && L.n_tilt_rings <= 0)) return SDLG_ERR_ARG;
    int cur = 0;
    if (cudaGetDevice(&cur) != cudaSuccess) return SDLG_ERR_NO_DEVICE;
    if (cudaSetDevice(device) != cudaSuccess) return SDLG_ERR_NO_DEVICE;
    std::vector<uint32_t> pairs;
    int rc = SDLG_OK;
    if (n > 0) {
        uint32_t* d_det = nullptr;
        int8_t* d_kind = nullptr;
        double* d_g = nullptr;
        uint32_t* d_out = nullptr;
        const size_t n_out = (size_t)n * 45 * 3;
        cudaError_t e = cudaMalloc(&d_det, n * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMalloc(&d_kind, n);
        if (e == cudaSuccess) e = cudaMalloc(&d_g, n * 16 * sizeof(double));
        if (e == cudaSuccess) e = cudaMalloc(&d_out, n_out * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMemcpy(d_det, detid, n * sizeof(uint32_t), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(d_kind, kind, n, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(d_g, geom, n * 16 * sizeof(double), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) {
            const int64_t work = n * 45;
            const int grid = (int)std::min<int64_t>((work + 255) / 256, 65535);
            k_line_map<<<grid, 256>>>(L, n, d_det, d_kind, d_g, d_out);
            e = cudaGetLastError();
        }
        std::vector<uint32_t> h(n_out);
        if (e == cudaSuccess) e = cudaMemcpy(h.data(), d_out, n_out * sizeof(uint32_t), cudaMemcpyDeviceToHost);
        cudaFree(d_det);
        cudaFree(d_kind);
        cudaFree(d_g);
        cudaFree(d_out);
        if (e != cudaSuccess) rc = SDLG_ERR_CUDA;
        else {
            // (source, destination) pairs; each thread's three crossings belong to module q / 45
            pairs.reserve(n_out / 4);
            for (size_t q = 0; q < n_out; ++q)
                if (h[q]) {
                    pairs.push_back(detid[q / (45 * 3)]);
                    pairs.push_back(h[q]);
                }
        }
    }
    cudaSetDevice(cur);
    if (rc) return rc;
    std::vector<uint64_t> key(pairs.size() / 2);
    for (size_t i = 0; i < key.size(); ++i) key[i] = ((uint64_t)pairs[2 * i] << 32) | pairs[2 * i + 1];
    std::sort(key.begin(), key.end());
    key.erase(std::unique(key.begin(), key.end()), key.end());
    int64_t nk = 0;
    for (size_t i = 0; i < key.size(); ++i)
        if (i == 0 || (key[i] >> 32) != (key[i - 1] >> 32)) ++nk;
    *n_keys = nk;
    *n_dst = (int64_t)key.size();
    if (!keys && !off && !dst) return SDLG_OK;  // a size query
    if (!keys || !off || !dst || cap_keys < nk || cap_dst < (int64_t)key.size()) return SDLG_ERR_ARG;
    int64_t k = -1;
    for (size_t i = 0; i < key.size(); ++i) {
        const uint32_t src = (uint32_t)(key[i] >> 32);
        if (k < 0 || keys[k] != src) {
            ++k;
            keys[k] = src;
            off[k] = (int64_t)i;
        }
        dst[i] = (uint32_t)(key[i] & 0xffffffffu);
    }
    off[nk] = (int64_t)key.size();
    return SDLG_OK;
}
