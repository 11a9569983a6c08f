// Learned pre-filter for tracklet candidates (no counterpart in the
// reference).  A 12-64-64-1 perceptron with ReLU hidden layers scores each
// (inner segment, outer segment) candidate of the tracklet step before the
// reference's cuts; a candidate whose logit is below the threshold is dropped
// and every other one is judged by the exact cuts as before, so the pruned
// chain's tracklets are a subset of the plain chain's.
//
// Numerics (shared by inference and training): features, W1, b1, W2, b2,
// w3 and the first hidden layer are rounded to BF16; every sum accumulates in
// FP32; b3 and the output layer's sum are FP32.  The bias b1 rides in the
// first MMA as the weight of a constant 13th input, b2 in the second as the
// weight of a constant 65th one (K = 80).  Inference uses the tensor cores
// (tcgen05.mma kind::f16, one 128-candidate tile per MMA, FP32 accumulators
// in tensor memory); training uses CUDA-core kernels.
#pragma once
#include <cstdint>
#include <cstring>

namespace sdlg {

constexpr int kMlpIn = 12;      // features per candidate
constexpr int kMlpK1 = 16;      // first-layer K: 12 features, the constant 1, padding
constexpr int kMlpHid = 64;     // units per hidden layer (the MMAs' N)
constexpr int kMlpK2 = 64;      // second-layer K: the 64 units
constexpr int kMlpTile = 128;   // candidates per tile (the MMAs' M)

// FP32 parameter vector: W1[64][12], b1[64], W2[64][64], b2[64], w3[64], b3
constexpr int kMlpW1 = 0;
constexpr int kMlpB1 = kMlpW1 + kMlpHid * kMlpIn;
constexpr int kMlpW2 = kMlpB1 + kMlpHid;
constexpr int kMlpB2 = kMlpW2 + kMlpHid * kMlpHid;
constexpr int kMlpW3 = kMlpB2 + kMlpHid;
constexpr int kMlpB3 = kMlpW3 + kMlpHid;
constexpr int kMlpParams = kMlpB3 + 1;  // 5057

// Packed inference weights, copied into shared memory by every CTA: [W1 b1]
// (64 x 16) and W2 (64 x 64) in BF16 in the tensor cores' K-major
// core-matrix layout, b2 as a 64 x 16 BF16 tile of the same layout (column 0,
// the weight of the constant input; zeros elsewhere), the BF16-rounded w3 and
// b3 in FP32, then the threshold.
constexpr int kPackW1 = 0;                                  // 64 x 16 bf16
constexpr int kPackW2 = kPackW1 + kMlpHid * kMlpK1 * 2;     // 64 x 64 bf16
constexpr int kPackB2 = kPackW2 + kMlpHid * kMlpK2 * 2;     // 64 x 16 bf16
constexpr int kPackW3 = kPackB2 + kMlpHid * 16 * 2;
constexpr int kPackB3 = kPackW3 + kMlpHid * 4;
constexpr int kPackBytes = kPackB3 + 16;                    // 12560, a multiple of 16

// Byte offset of element (row, k) of a K-major BF16 tile without swizzling:
// 8-row x 16-byte core matrices, `kgroups` of them along K per 8-row group
// (so the byte stride between core matrices along K is 128 and between 8-row
// groups kgroups * 128).
__host__ __device__ constexpr uint32_t cm_offset(int row, int k, int kgroups) {
    return (uint32_t)((row >> 3) * (kgroups * 128) + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// round-to-nearest-even FP32 -> BF16 bits (finite inputs)
__host__ __device__ inline uint16_t bf16_bits(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    u += 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}
__host__ __device__ inline float bf16_round(float f) {
    uint32_t u = (uint32_t)bf16_bits(f) << 16;
    float r;
    memcpy(&r, &u, 4);
    return r;
}

struct MlpStats {
    unsigned long long candidates;  // tracklet candidates
    unsigned long long scored;      // through the float cuts (phase A) and scored
    unsigned long long kept;        // logit >= threshold (phase B load)
    unsigned long long timeouts;    // tensor-core waits that gave up
};

#if defined(__CUDACC__)

// ------------------------------------------------------------------ PTX
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared memory matrix descriptor: start address, byte offset between core
// matrices along K (lbo) and along M/N (sbo), descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

// instruction descriptor, kind::f16: FP32 accumulator (bits 4-5 = 1), BF16 A
// and B (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24
constexpr uint32_t kIdescBf16M128N64 = (1u << 4) | (1u << 7) | (1u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void tc_alloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes -> visible to the tensor cores
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(mbar))
                 : "memory");
}
__device__ __forceinline__ void mbar_init(uint64_t* mbar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mbar)), "r"(1u) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}
// wait for the mbarrier phase of the given parity, at most ~0.25 s or
// max_it polls (0: give up at once, the failure-path self-test)
constexpr uint32_t kMbarPolls = 1u << 24;
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, uint32_t max_it = kMbarPolls) {
    const uint32_t a = smem_addr(mbar);
    uint64_t t0 = 0;
    for (uint32_t it = 0; it < max_it; ++it) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if (it == 0) t0 = global_ns();
        else if ((it & 63u) == 0 && global_ns() - t0 > 250000000ull) return false;
    }
    return false;
}
// two floats rounded to BF16 (to nearest, ties to even) and packed, lo in
// the low half; the .relu form first clamps negative values to zero
__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    uint32_t d;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
    return d;
}
__device__ __forceinline__ uint32_t pack_bf16x2_relu(float lo, float hi) {
    uint32_t d;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
    return d;
}

// packed FP32 pairs (lo in the low word): the sm_100-family fma.f32x2, one
// instruction for two lanes of arithmetic, each rounded to nearest like the
// scalar form
__device__ __forceinline__ uint64_t f2_pack(float lo, float hi) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ float2 f2_unpack(uint64_t v) {
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
    return r;
}
__device__ __forceinline__ uint64_t f2_fma(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
__device__ __forceinline__ uint64_t f2_relu(uint64_t v) {
    const float2 p = f2_unpack(v);
    return f2_pack(fmaxf(p.x, 0.f), fmaxf(p.y, 0.f));
}

// 16 consecutive FP32 columns of this thread's tensor-memory lane
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// ------------------------------------------------------------------ tile
// Shared memory of one CTA running the tensor-core MLP (128 threads, thread
// t owns tile row t).
struct __align__(128) MlpSmem {
    alignas(128) unsigned char w[kPackBytes];
    // A operand of both layers, BF16, 8 k-groups per 8-row group: columns
    // 0-15 hold a candidate's features and the constant 1 for the first MMA,
    // then columns 0-63 its first hidden layer for the second (the features
    // are consumed before the layer overwrites them, and the layer before the
    // next tile's features)
    alignas(128) unsigned char a2[kMlpTile * kMlpK2 * 2];
    // the second layer's constant input, K = 64-79 of its A operand: 1 in
    // column 0 of every row, zeros after it (2 k-groups per 8-row group)
    alignas(128) unsigned char aone[kMlpTile * 16 * 2];
    alignas(8) uint64_t mbar;
    uint32_t tmem;       // base address of 64 tensor-memory columns (both layers' accumulators)
};

// Per-thread state of the tile loop.  `phase` is the parity of the next
// mbarrier phase; `abort` turns true (on every thread at the next barrier)
// once a tensor-core wait gave up, after which no MMA is issued.
struct MlpThread {
    uint32_t phase = 0;
    bool abort = false;
    bool pending = false;       // an MMA whose completion was not seen may still run
    uint32_t polls = kMbarPolls;  // poll limit of the next layer wait (0 once: the failure-path self-test)
};

// copy the packed weights, set up the mbarrier and tensor memory (all 128 threads)
__device__ __forceinline__ void mlp_setup(MlpSmem& sm, const unsigned char* __restrict__ pack) {
    const uint4* src = reinterpret_cast<const uint4*>(pack);
    uint4* dst = reinterpret_cast<uint4*>(sm.w);
    for (int k = threadIdx.x; k < kPackBytes / 16; k += blockDim.x) dst[k] = __ldg(src + k);
    *reinterpret_cast<uint4*>(sm.aone + cm_offset(threadIdx.x, 0, 2)) = make_uint4(0x3f80u, 0u, 0u, 0u);
    *reinterpret_cast<uint4*>(sm.aone + cm_offset(threadIdx.x, 8, 2)) = make_uint4(0u, 0u, 0u, 0u);
    if (threadIdx.x == 0) mbar_init(&sm.mbar);
    if (threadIdx.x < 32) tc_alloc(&sm.tmem, 64);
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
}

// release tensor memory (all 128 threads; after the last tile), after one
// more bounded wait for an MMA whose completion was not seen
__device__ __forceinline__ void mlp_teardown(MlpSmem& sm, MlpThread& st) {
    if (st.pending) (void)mbar_wait(&sm.mbar, st.phase);
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x < 32) {
        tc_fence_after();
        tc_dealloc(sm.tmem, 64);
    }
}

// make this thread's shared-memory tile rows visible, issue the MMAs of one
// layer from thread 0 and wait for them (all threads, uniform control flow).
// Both layers accumulate into the same 64 columns: the barrier orders every
// thread's reads of the previous accumulator before the next MMA.
__device__ __forceinline__ void mlp_layer_sync(MlpSmem& sm, int layer, MlpThread& st) {
    fence_async_smem();
    tc_fence_before();
    if (__syncthreads_or(st.abort ? 1 : 0)) {
        st.abort = true;
        return;
    }
    if (threadIdx.x == 0) {
        tc_fence_after();
        const uint32_t w = smem_addr(sm.w);
        if (layer == 0) {
            tc_mma(sm.tmem, smem_desc(smem_addr(sm.a2), 128, 1024), smem_desc(w + kPackW1, 128, 256), kIdescBf16M128N64, 0);
        } else {
            const uint32_t a2 = smem_addr(sm.a2);
#pragma unroll
            for (int kc = 0; kc < kMlpK2 / 16; ++kc)
                tc_mma(sm.tmem, smem_desc(a2 + 256 * kc, 128, 1024), smem_desc(w + kPackW2 + 256 * kc, 128, 1024),
                       kIdescBf16M128N64, kc > 0 ? 1u : 0u);
            // + b2, the weight of the constant input
            tc_mma(sm.tmem, smem_desc(smem_addr(sm.aone), 128, 256), smem_desc(w + kPackB2, 128, 256), kIdescBf16M128N64, 1u);
        }
        tc_commit(&sm.mbar);
    }
    const uint32_t polls = st.polls;
    st.polls = kMbarPolls;
    if (mbar_wait(&sm.mbar, st.phase, polls)) {
        st.phase ^= 1u;
    } else {
        st.abort = true;
        st.pending = true;
    }
    tc_fence_after();
}

// First half of a tile: thread t writes the features x of its candidate
// (rounded to BF16, with the constant 1) as row t and thread 0 starts the
// first layer's MMA.  Every thread of the 128-thread CTA calls it; the CTA
// may run other work before mlp_tile_end.
__device__ __forceinline__ void mlp_tile_begin(MlpSmem& sm, const float* x, MlpThread& st) {
    const int t = threadIdx.x;
    uint32_t q[8];
#pragma unroll
    for (int j = 0; j < 6; ++j) q[j] = pack_bf16x2(x[2 * j], x[2 * j + 1]);
    q[6] = 0x3f80u;  // the constant 1 (BF16) that carries b1, then zeros
    q[7] = 0u;
    *reinterpret_cast<uint4*>(sm.a2 + cm_offset(t, 0, 8)) = make_uint4(q[0], q[1], q[2], q[3]);
    *reinterpret_cast<uint4*>(sm.a2 + cm_offset(t, 8, 8)) = make_uint4(q[4], q[5], q[6], q[7]);
    fence_async_smem();
    tc_fence_before();
    if (__syncthreads_or(st.abort ? 1 : 0)) {
        st.abort = true;
        return;
    }
    if (t == 0) {
        tc_fence_after();
        tc_mma(sm.tmem, smem_desc(smem_addr(sm.a2), 128, 1024), smem_desc(smem_addr(sm.w) + kPackW1, 128, 256),
               kIdescBf16M128N64, 0);
        tc_commit(&sm.mbar);
    }
}

// Second half: wait for the first layer, run the second and the output
// layer, return the logit (meaningless after an abort).  Every thread calls it.
__device__ __forceinline__ float mlp_tile_end(MlpSmem& sm, MlpThread& st) {
    const int t = threadIdx.x;
    if (!st.abort) {
        const uint32_t polls = st.polls;
        st.polls = kMbarPolls;
        if (mbar_wait(&sm.mbar, st.phase, polls)) {
            st.phase ^= 1u;
        } else {
            st.abort = true;
            st.pending = true;
        }
        tc_fence_after();
    }
    const uint32_t lane_base = sm.tmem + ((uint32_t)(t & ~31) << 16);
    // tensor memory is read only when the accumulator is known complete; the
    // skip is warp-uniform (tcgen05.ld is a warp-wide instruction)
    if (!__any_sync(0xffffffffu, st.abort)) {
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            float v[16];
            tc_ld16(lane_base + 16 * c, v);
            uint32_t q[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) q[j] = pack_bf16x2_relu(v[2 * j], v[2 * j + 1]);
            *reinterpret_cast<uint4*>(sm.a2 + cm_offset(t, 16 * c, 8)) = make_uint4(q[0], q[1], q[2], q[3]);
            *reinterpret_cast<uint4*>(sm.a2 + cm_offset(t, 16 * c + 8, 8)) = make_uint4(q[4], q[5], q[6], q[7]);
        }
    }
    mlp_layer_sync(sm, 1, st);
    const float b3 = *reinterpret_cast<const float*>(sm.w + kPackB3);
    if (__any_sync(0xffffffffu, st.abort)) return b3;  // meaningless after an abort
    // output layer on packed FP32 pairs (units 2j and 2j+1 side by side): two
    // partial sums, over the even and the odd units, then b3 + even + odd
    const ulonglong2* w3 = reinterpret_cast<const ulonglong2*>(sm.w + kPackW3);
    uint64_t zz = 0ull;  // (0.f, 0.f)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        float v[16];
        tc_ld16(lane_base + 16 * c, v);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const ulonglong2 w = w3[4 * c + j];
            zz = f2_fma(w.x, f2_relu(f2_pack(v[4 * j], v[4 * j + 1])), zz);
            zz = f2_fma(w.y, f2_relu(f2_pack(v[4 * j + 2], v[4 * j + 3])), zz);
        }
    }
    const float2 s = f2_unpack(zz);
    return __fadd_rn(__fadd_rn(b3, s.x), s.y);
}

// One tile: thread t scores the features x of its candidate and gets the logit.
__device__ __forceinline__ float mlp_tile(MlpSmem& sm, const float* x, MlpThread& st) {
    mlp_tile_begin(sm, x, st);
    return mlp_tile_end(sm, st);
}

#endif  // __CUDACC__

}  // namespace sdlg
