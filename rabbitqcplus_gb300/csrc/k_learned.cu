// Learned correction classifier: a 32 -> 64 -> 64 -> 1 MLP over per-column
// MSA features, BF16 weights and activations, FP32 accumulation, sigmoid
// output.  It stands where the reference's forest/logistic-regression
// classifier stands in its correction path (include/classification.hpp:51-157,
// include/forest.hpp:217-226, used by correctAnchorClf in
// include/corrector.hpp:1448-1472); the network, its features and its training
// are this project's own.
//
// All three matrix products (forward, the two weight gradients and the hidden
// gradient) run on the tensor cores with mma.sync.m16n8k16 (BF16 operands,
// FP32 accumulators).  A warp owns 16 columns (rows of the product): the
// first layer's accumulators become the second layer's A operand in registers,
// and the transposed operands of the weight gradients are staged in shared
// memory.  Training is deterministic: every warp writes its partial gradients
// to its own slot and one kernel sums the slots in a fixed order before the
// Adam update.

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "care_device.cuh"
#include "care_internal.h"
#include "care_learned.h"

namespace cg {

namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ uint32_t pack_raw(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

// D += A * B, A 16x16 (row), B 16x8 (col), BF16 in, FP32 accumulate
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Weights staged in shared memory (BF16) with the biases (FP32).
struct SmemMlp {
    __nv_bfloat16 w1[kMlpHidden * kMlpFeatures];
    __nv_bfloat16 w2[kMlpHidden * kMlpHidden];
    __nv_bfloat16 w3[kMlpHidden];
    float b1[kMlpHidden], b2[kMlpHidden], b3;
};

__device__ void stage_weights(SmemMlp& s, const unsigned char* model) {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(model);
    uint32_t* dst = reinterpret_cast<uint32_t*>(s.w1);
    // w1, w2, w3 are contiguous in both layouts
    constexpr int words = (kMlpHidden * kMlpFeatures + kMlpHidden * kMlpHidden + kMlpHidden) / 2;
    for (int i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
    const float* bsrc = reinterpret_cast<const float*>(model + kMlpOffB1);
    for (int i = threadIdx.x; i < kMlpHidden; i += blockDim.x) {
        s.b1[i] = bsrc[i];
        s.b2[i] = bsrc[kMlpHidden + i];
    }
    if (threadIdx.x == 0) s.b3 = bsrc[2 * kMlpHidden];
}

// Forward pass of 16 rows held by one warp.  x(r, f) gives feature f of local
// row r (BF16).  On return h1/h2 hold the BF16-rounded post-ReLU activations
// in accumulator layout (tile nt: rows g and g+8, columns nt*8 + 2t, +1) and
// logit[0]/logit[1] the outputs of rows g and g+8 (the same in all four lanes
// of a group).
template <class XF>
__device__ __forceinline__ void mlp_forward(const SmemMlp& s, XF x, float (&h1)[8][4], float (&h2)[8][4],
                                            float (&logit)[2]) {
    const int lane = (int)lane_id();
    const int g = lane >> 2, t = lane & 3;
    uint32_t ax[2][4];
#pragma unroll
    for (int kc = 0; kc < 2; kc++) {
        const int c0 = kc * 16 + 2 * t;
        ax[kc][0] = pack_raw(x(g, c0), x(g, c0 + 1));
        ax[kc][1] = pack_raw(x(g + 8, c0), x(g + 8, c0 + 1));
        ax[kc][2] = pack_raw(x(g, c0 + 8), x(g, c0 + 9));
        ax[kc][3] = pack_raw(x(g + 8, c0 + 8), x(g + 8, c0 + 9));
    }
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        const int n = nt * 8 + 2 * t;
        h1[nt][0] = h1[nt][2] = s.b1[n];
        h1[nt][1] = h1[nt][3] = s.b1[n + 1];
#pragma unroll
        for (int kc = 0; kc < 2; kc++) {
            const __nv_bfloat16* w = s.w1 + (nt * 8 + g) * kMlpFeatures + kc * 16 + 2 * t;
            const uint32_t b[2] = {*reinterpret_cast<const uint32_t*>(w), *reinterpret_cast<const uint32_t*>(w + 8)};
            mma_bf16(h1[nt], ax[kc], b);
        }
#pragma unroll
        for (int i = 0; i < 4; i++) h1[nt][i] = __bfloat162float(__float2bfloat16_rn(fmaxf(h1[nt][i], 0.0f)));
    }
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        const int n = nt * 8 + 2 * t;
        h2[nt][0] = h2[nt][2] = s.b2[n];
        h2[nt][1] = h2[nt][3] = s.b2[n + 1];
    }
#pragma unroll
    for (int kc = 0; kc < 4; kc++) {
        const uint32_t a[4] = {pack_bf16(h1[2 * kc][0], h1[2 * kc][1]), pack_bf16(h1[2 * kc][2], h1[2 * kc][3]),
                               pack_bf16(h1[2 * kc + 1][0], h1[2 * kc + 1][1]),
                               pack_bf16(h1[2 * kc + 1][2], h1[2 * kc + 1][3])};
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
            const __nv_bfloat16* w = s.w2 + (nt * 8 + g) * kMlpHidden + kc * 16 + 2 * t;
            const uint32_t b[2] = {*reinterpret_cast<const uint32_t*>(w), *reinterpret_cast<const uint32_t*>(w + 8)};
            mma_bf16(h2[nt], a, b);
        }
    }
    float z0 = 0.0f, z1 = 0.0f;
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
#pragma unroll
        for (int i = 0; i < 4; i++) h2[nt][i] = __bfloat162float(__float2bfloat16_rn(fmaxf(h2[nt][i], 0.0f)));
        const int n = nt * 8 + 2 * t;
        const float wa = __bfloat162float(s.w3[n]), wb = __bfloat162float(s.w3[n + 1]);
        z0 = __fadd_rn(z0, __fadd_rn(__fmul_rn(h2[nt][0], wa), __fmul_rn(h2[nt][1], wb)));
        z1 = __fadd_rn(z1, __fadd_rn(__fmul_rn(h2[nt][2], wa), __fmul_rn(h2[nt][3], wb)));
    }
    // the four lanes of a group hold disjoint columns of the same rows
    z0 = __fadd_rn(z0, __shfl_xor_sync(kFull, z0, 1));
    z1 = __fadd_rn(z1, __shfl_xor_sync(kFull, z1, 1));
    z0 = __fadd_rn(z0, __shfl_xor_sync(kFull, z0, 2));
    z1 = __fadd_rn(z1, __shfl_xor_sync(kFull, z1, 2));
    logit[0] = __fadd_rn(z0, s.b3);
    logit[1] = __fadd_rn(z1, s.b3);
}

// ---------------------------------------------------------------- inference (tcgen05)
//
// 128 columns (rows of the product, the MMA's M) per tile.  Operands sit in
// shared memory in the canonical K-major layout without swizzle (8-row x
// 16-byte core matrices; the K/8 core matrices of an 8-row group contiguous);
// one thread issues tcgen05.mma (kind::f16, BF16 A and B, FP32 accumulators
// in tensor memory), tcgen05.commit arrives on an mbarrier, and every thread
// reads its row of the accumulators back with tcgen05.ld (thread = TMEM lane).
// Layer 1 accumulates in TMEM columns 0-63, layer 2 in 64-127; the epilogue of
// layer 1 (bias, ReLU, BF16) writes layer 2's A operand back to shared memory.

constexpr int kTcRows = 128;
constexpr uint32_t kTmemCols = 128;
constexpr uint32_t kWaitSpins = 1u << 20;  // mbarrier polls before a wait is declared failed

// Polls of the per-tile MMA waits (the waits whose failure ends a block);
// set from the host by set_classifier_wait_limit.  The wait that drains a
// failed block's MMAs before its tensor memory is released always uses
// kWaitSpins.
__device__ uint32_t g_tileWaitSpins = kWaitSpins;

// byte offset of element (row, k) of a K-major tile with kdim columns
__device__ __forceinline__ uint32_t core_offset(int row, int k, int kdim) {
    return (uint32_t)((((row >> 3) * (kdim >> 3) + (k >> 3)) << 7) + ((row & 7) << 4) + ((k & 7) << 1));
}

__device__ __forceinline__ uint32_t smem_u32(const void* ptr) { return (uint32_t)__cvta_generic_to_shared(ptr); }

// shared-memory matrix descriptor: start address, leading byte offset (next
// core matrix along K), stride byte offset (next 8-row group), version 1, no
// swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3fffu) | ((uint64_t)((lbo >> 4) & 0x3fffu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3fffu) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, M x N
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void tc_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// bounded wait (at most `polls` polls) for the completion of mbarrier phase `parity`
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, uint32_t polls) {
    for (uint32_t i = 0; i < polls; i++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// 32 consecutive FP32 accumulator columns of this thread's TMEM lane
__device__ __forceinline__ void tc_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
                 : "=r"(r[0]),"=r"(r[1]),"=r"(r[2]),"=r"(r[3]),"=r"(r[4]),"=r"(r[5]),"=r"(r[6]),"=r"(r[7]),"=r"(r[8]),"=r"(r[9]),"=r"(r[10]),"=r"(r[11]),"=r"(r[12]),"=r"(r[13]),"=r"(r[14]),"=r"(r[15]),"=r"(r[16]),"=r"(r[17]),"=r"(r[18]),"=r"(r[19]),"=r"(r[20]),"=r"(r[21]),"=r"(r[22]),"=r"(r[23]),"=r"(r[24]),"=r"(r[25]),"=r"(r[26]),"=r"(r[27]),"=r"(r[28]),"=r"(r[29]),"=r"(r[30]),"=r"(r[31])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// Inference over a column buffer, persistent over 128-column tiles.  With
// `logits` set the outputs are written there; otherwise every column whose
// logit reaches `minLogit` (the logit of the confidence threshold) gets the
// consensus base in its output row, and the others keep the fallback decision
// the MSA kernel already wrote.  A wait that does not end counts in
// counters[kCounterTimeouts] and ends the block (after a second bounded wait
// for its MMAs and the release of its tensor memory).
__global__ void __launch_bounds__(kTcRows) mlp_infer_kernel(const unsigned char* __restrict__ model,
                                                            const __nv_bfloat16* __restrict__ feat,
                                                            const uint2* __restrict__ meta,
                                                            const unsigned int* __restrict__ countPtr,
                                                            unsigned int count, unsigned int cap, float minLogit,
                                                            char* out, int outPitch, float* logits,
                                                            unsigned long long* counters) {
    __shared__ __align__(1024) unsigned char a1[kTcRows * kMlpFeatures * 2];
    __shared__ __align__(1024) unsigned char a2[kTcRows * kMlpHidden * 2];
    __shared__ __align__(1024) unsigned char b1[kMlpHidden * kMlpFeatures * 2];
    __shared__ __align__(1024) unsigned char b2[kMlpHidden * kMlpHidden * 2];
    __shared__ float bias1[kMlpHidden], bias2[kMlpHidden], wout[kMlpHidden];
    __shared__ float bias3;
    __shared__ __align__(8) unsigned long long mbar;
    __shared__ uint32_t tmemBase;
    const int tid = (int)threadIdx.x, warp = tid >> 5;
    // weights into the canonical layout (B operands: N x K, K-major = the stored rows)
    const __nv_bfloat16* w1 = reinterpret_cast<const __nv_bfloat16*>(model + kMlpOffW1);
    const __nv_bfloat16* w2 = reinterpret_cast<const __nv_bfloat16*>(model + kMlpOffW2);
    const __nv_bfloat16* w3 = reinterpret_cast<const __nv_bfloat16*>(model + kMlpOffW3);
    for (int i = tid; i < kMlpHidden * kMlpFeatures; i += kTcRows)
        *reinterpret_cast<__nv_bfloat16*>(b1 + core_offset(i / kMlpFeatures, i % kMlpFeatures, kMlpFeatures)) = w1[i];
    for (int i = tid; i < kMlpHidden * kMlpHidden; i += kTcRows)
        *reinterpret_cast<__nv_bfloat16*>(b2 + core_offset(i / kMlpHidden, i % kMlpHidden, kMlpHidden)) = w2[i];
    const float* bsrc = reinterpret_cast<const float*>(model + kMlpOffB1);
    if (tid < kMlpHidden) {
        bias1[tid] = bsrc[tid];
        bias2[tid] = bsrc[kMlpHidden + tid];
        wout[tid] = __bfloat162float(w3[tid]);
    }
    if (tid == 0) {
        bias3 = bsrc[2 * kMlpHidden];
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmemBase)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = tmemBase;
    const uint32_t lane0 = tbase + ((uint32_t)(warp * 32) << 16);  // this warp's 32 TMEM lanes
    const uint32_t mb = smem_u32(&mbar);
    constexpr uint32_t idesc = instr_desc(kTcRows, kMlpHidden);
    unsigned int n = countPtr ? *countPtr : count;
    if (countPtr && blockIdx.x == 0 && tid == 0 && counters) {
        atomicAdd(&counters[kCounterColumns], (unsigned long long)n);
        if (n > cap) atomicAdd(&counters[kCounterColumnOverflow], (unsigned long long)(n - cap));
    }
    if (n > cap) n = cap;
    uint32_t phase = 0;
    unsigned int taken = 0;
    bool failed = false;
    const uint32_t tilePolls = g_tileWaitSpins;
    for (unsigned int t0 = blockIdx.x * kTcRows; t0 < n; t0 += gridDim.x * kTcRows) {
        const unsigned int row = t0 + (unsigned int)tid;
        uint4 f[4];
#pragma unroll
        for (int j = 0; j < 4; j++) f[j] = make_uint4(0, 0, 0, 0);
        if (row < n) {
            const uint4* src = reinterpret_cast<const uint4*>(feat + (uint64_t)row * kMlpFeatures);
#pragma unroll
            for (int j = 0; j < 4; j++) f[j] = src[j];
        }
#pragma unroll
        for (int j = 0; j < 4; j++) *reinterpret_cast<uint4*>(a1 + core_offset(tid, 8 * j, kMlpFeatures)) = f[j];
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // visible to the tensor core
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
#pragma unroll
            for (int k = 0; k < kMlpFeatures / 16; k++)
                tc_mma(tbase, smem_desc(smem_u32(a1) + 256u * k, 128, 512), smem_desc(smem_u32(b1) + 256u * k, 128, 512),
                       idesc, k > 0);
            tc_commit(mb);
        }
        bool ok = mbar_wait(mb, phase, tilePolls);
        phase ^= 1u;
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        tc_fence_after();
        // layer 1 epilogue: this thread's row -> bias, ReLU, BF16 -> layer 2's A operand
#pragma unroll
        for (int half = 0; half < 2; half++) {
            float v[32];
            tc_ld32(lane0 + 32u * half, v);
#pragma unroll
            for (int j = 0; j < 4; j++) {
                uint32_t w[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int c = 32 * half + 8 * j + 2 * q;
                    w[q] = pack_bf16(fmaxf(__fadd_rn(v[8 * j + 2 * q], bias1[c]), 0.0f),
                                     fmaxf(__fadd_rn(v[8 * j + 2 * q + 1], bias1[c + 1]), 0.0f));
                }
                *reinterpret_cast<uint4*>(a2 + core_offset(tid, 32 * half + 8 * j, kMlpHidden)) =
                    make_uint4(w[0], w[1], w[2], w[3]);
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
#pragma unroll
            for (int k = 0; k < kMlpHidden / 16; k++)
                tc_mma(tbase + kMlpHidden, smem_desc(smem_u32(a2) + 256u * k, 128, 1024),
                       smem_desc(smem_u32(b2) + 256u * k, 128, 1024), idesc, k > 0);
            tc_commit(mb);
        }
        ok = mbar_wait(mb, phase, tilePolls);
        phase ^= 1u;
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        tc_fence_after();
        float z = 0.0f;
#pragma unroll
        for (int half = 0; half < 2; half++) {
            float v[32];
            tc_ld32(lane0 + (uint32_t)kMlpHidden + 32u * half, v);
#pragma unroll
            for (int i = 0; i < 32; i++) {
                const int c = 32 * half + i;
                const float h = __bfloat162float(__float2bfloat16_rn(fmaxf(__fadd_rn(v[i], bias2[c]), 0.0f)));
                z = __fadd_rn(z, __fmul_rn(h, wout[c]));
            }
        }
        z = __fadd_rn(z, bias3);
        if (row < n) {
            if (logits) {
                logits[row] = z;
            } else if (z >= minLogit) {
                const uint2 m = meta[row];
                out[(uint64_t)m.x * outPitch + (m.y & 0xffffu)] = (char)((m.y >> 16) & 0xffu);
                taken++;
            }
        }
        tc_fence_before();  // the next tile's MMAs overwrite the accumulators read here
    }
    if (failed) {
        if (tid == 0 && counters) atomicAdd(&counters[kCounterTimeouts], 1ull);
        mbar_wait(mb, phase ^ 1u, kWaitSpins);  // the MMAs in flight, bounded again at the full limit
    }
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(kTmemCols) : "memory");
    if (counters && !logits) {
        taken = __reduce_add_sync(kFull, taken);
        if ((tid & 31) == 0 && taken) atomicAdd(&counters[kCounterLearnedTaken], (unsigned long long)taken);
    }
}

// ---------------------------------------------------------------- training

constexpr int kTrainWarps = 4;

struct TrainSmem {
    SmemMlp w;
    __nv_bfloat16 x[kTrainWarps][16][kMlpFeatures];
    __nv_bfloat16 h1[kTrainWarps][16][kMlpHidden];
    __nv_bfloat16 d2[kTrainWarps][16][kMlpHidden];
    __nv_bfloat16 d1[kTrainWarps][16][kMlpHidden];
};

// softplus(z) - y*z, the binary cross-entropy of sigmoid(z) against y
__device__ __forceinline__ float bce_logit(float z, float y) {
    const float sp = fmaxf(z, 0.0f) + log1pf(expf(-fabsf(z)));
    return sp - y * z;
}

// One warp = 16 rows of the minibatch: forward, loss and all gradients of the
// mean loss over `total` rows; its partial sums go to part[globalWarp][...]
// in the parameter order of the model (w1, w2, w3, b1, b2, b3, loss).
// Rows index the feature matrix through `perm` (or directly when null).
__global__ void __launch_bounds__(kTrainWarps * 32) mlp_grad_kernel(const unsigned char* __restrict__ model,
                                                                    const __nv_bfloat16* __restrict__ feat,
                                                                    const float* __restrict__ label,
                                                                    const uint32_t* __restrict__ perm,
                                                                    const unsigned long long* stepPtr,
                                                                    unsigned int stepsPerEpoch, unsigned int rows,
                                                                    float invTotal, float* __restrict__ part) {
    extern __shared__ __align__(16) unsigned char smraw[];
    TrainSmem& s = *reinterpret_cast<TrainSmem*>(smraw);
    stage_weights(s.w, model);
    const int wi = (int)(threadIdx.x >> 5);
    const int lane = (int)lane_id();
    const int g = lane >> 2, t = lane & 3;
    // first row of this minibatch
    const uint64_t base = stepPtr ? (*stepPtr % stepsPerEpoch) * (uint64_t)rows : 0;
    const unsigned gw = blockIdx.x * kTrainWarps + wi;
    const unsigned r0 = gw * 16;
    // stage this warp's 16 rows (zero past the end)
    for (int i = lane; i < 16 * kMlpFeatures; i += 32) {
        const int r = i / kMlpFeatures, f = i % kMlpFeatures;
        const unsigned row = r0 + (unsigned)r;
        __nv_bfloat16 v = __float2bfloat16_rn(0.0f);
        if (row < rows) {
            const uint64_t src = perm ? perm[base + row] : base + row;
            v = feat[src * kMlpFeatures + f];
        }
        s.x[wi][r][f] = v;
    }
    __syncthreads();
    auto x = [&](int r, int f) -> __nv_bfloat16 { return s.x[wi][r][f]; };
    float h1[8][4], h2[8][4], z[2];
    mlp_forward(s.w, x, h1, h2, z);

    float dz[2] = {0.0f, 0.0f}, loss = 0.0f;
#pragma unroll
    for (int half = 0; half < 2; half++) {
        const unsigned row = r0 + (unsigned)(g + 8 * half);
        if (row < rows) {
            const uint64_t src = perm ? perm[base + row] : base + row;
            const float y = label[src];
            const float p = 1.0f / (1.0f + expf(-z[half]));
            dz[half] = (p - y) * invTotal;
            if (t == 0) loss += bce_logit(z[half], y) * invTotal;
        }
    }
    float* out = part + (uint64_t)gw * kMlpParams;
    // output layer: dW3, db3; hidden 2 gradient dH2 = dz * w3 * relu'(h2)
    float d2[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        const int n = nt * 8 + 2 * t;
        const float wa = __bfloat162float(s.w.w3[n]), wb = __bfloat162float(s.w.w3[n + 1]);
        float ga = __fadd_rn(__fmul_rn(dz[0], h2[nt][0]), __fmul_rn(dz[1], h2[nt][2]));
        float gb = __fadd_rn(__fmul_rn(dz[0], h2[nt][1]), __fmul_rn(dz[1], h2[nt][3]));
        // sum over the 8 groups (lanes with the same t)
#pragma unroll
        for (int o = 4; o < 32; o <<= 1) {
            ga = __fadd_rn(ga, __shfl_xor_sync(kFull, ga, o));
            gb = __fadd_rn(gb, __shfl_xor_sync(kFull, gb, o));
        }
        if (g == 0) {
            out[kMlpOffW3 / 2 + n] = ga;
            out[kMlpOffW3 / 2 + n + 1] = gb;
        }
        d2[nt][0] = h2[nt][0] > 0.0f ? __fmul_rn(dz[0], wa) : 0.0f;
        d2[nt][1] = h2[nt][1] > 0.0f ? __fmul_rn(dz[0], wb) : 0.0f;
        d2[nt][2] = h2[nt][2] > 0.0f ? __fmul_rn(dz[1], wa) : 0.0f;
        d2[nt][3] = h2[nt][3] > 0.0f ? __fmul_rn(dz[1], wb) : 0.0f;
    }
    {
        float db3 = __fadd_rn(dz[0], dz[1]);
        db3 = __fadd_rn(db3, __shfl_xor_sync(kFull, db3, 4));
        db3 = __fadd_rn(db3, __shfl_xor_sync(kFull, db3, 8));
        db3 = __fadd_rn(db3, __shfl_xor_sync(kFull, db3, 16));
        float l = loss;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) l = __fadd_rn(l, __shfl_xor_sync(kFull, l, o));
        if (lane == 0) {
            out[kMlpParamB3] = db3;
            out[kMlpParamLoss] = l;
        }
    }
    // db2 = column sums of dH2 (FP32); stage BF16 dH2 and h1 for the transposed products
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        const int n = nt * 8 + 2 * t;
        float sa = __fadd_rn(d2[nt][0], d2[nt][2]), sb = __fadd_rn(d2[nt][1], d2[nt][3]);
#pragma unroll
        for (int o = 4; o < 32; o <<= 1) {
            sa = __fadd_rn(sa, __shfl_xor_sync(kFull, sa, o));
            sb = __fadd_rn(sb, __shfl_xor_sync(kFull, sb, o));
        }
        if (g == 0) {
            out[kMlpParamB2 + n] = sa;
            out[kMlpParamB2 + n + 1] = sb;
        }
        s.d2[wi][g][n] = __float2bfloat16_rn(d2[nt][0]);
        s.d2[wi][g][n + 1] = __float2bfloat16_rn(d2[nt][1]);
        s.d2[wi][g + 8][n] = __float2bfloat16_rn(d2[nt][2]);
        s.d2[wi][g + 8][n + 1] = __float2bfloat16_rn(d2[nt][3]);
        s.h1[wi][g][n] = __float2bfloat16_rn(h1[nt][0]);
        s.h1[wi][g][n + 1] = __float2bfloat16_rn(h1[nt][1]);
        s.h1[wi][g + 8][n] = __float2bfloat16_rn(h1[nt][2]);
        s.h1[wi][g + 8][n + 1] = __float2bfloat16_rn(h1[nt][3]);
    }
    __syncwarp();
    // dH1 = (dH2 W2) * relu'(h1): A = dH2 (16 x 64), B[k=j][n=i] = W2[j][i]
    float d1[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; nt++) d1[nt][0] = d1[nt][1] = d1[nt][2] = d1[nt][3] = 0.0f;
#pragma unroll
    for (int kc = 0; kc < 4; kc++) {
        const int c0 = kc * 16 + 2 * t;
        const uint32_t a[4] = {pack_raw(s.d2[wi][g][c0], s.d2[wi][g][c0 + 1]),
                               pack_raw(s.d2[wi][g + 8][c0], s.d2[wi][g + 8][c0 + 1]),
                               pack_raw(s.d2[wi][g][c0 + 8], s.d2[wi][g][c0 + 9]),
                               pack_raw(s.d2[wi][g + 8][c0 + 8], s.d2[wi][g + 8][c0 + 9])};
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
            const int col = nt * 8 + g;
            const uint32_t b[2] = {pack_raw(s.w.w2[c0 * kMlpHidden + col], s.w.w2[(c0 + 1) * kMlpHidden + col]),
                                   pack_raw(s.w.w2[(c0 + 8) * kMlpHidden + col], s.w.w2[(c0 + 9) * kMlpHidden + col])};
            mma_bf16(d1[nt], a, b);
        }
    }
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        const int n = nt * 8 + 2 * t;
#pragma unroll
        for (int i = 0; i < 4; i++) d1[nt][i] = h1[nt][i] > 0.0f ? d1[nt][i] : 0.0f;
        float sa = __fadd_rn(d1[nt][0], d1[nt][2]), sb = __fadd_rn(d1[nt][1], d1[nt][3]);
#pragma unroll
        for (int o = 4; o < 32; o <<= 1) {
            sa = __fadd_rn(sa, __shfl_xor_sync(kFull, sa, o));
            sb = __fadd_rn(sb, __shfl_xor_sync(kFull, sb, o));
        }
        if (g == 0) {
            out[kMlpParamB1 + n] = sa;
            out[kMlpParamB1 + n + 1] = sb;
        }
        s.d1[wi][g][n] = __float2bfloat16_rn(d1[nt][0]);
        s.d1[wi][g][n + 1] = __float2bfloat16_rn(d1[nt][1]);
        s.d1[wi][g + 8][n] = __float2bfloat16_rn(d1[nt][2]);
        s.d1[wi][g + 8][n + 1] = __float2bfloat16_rn(d1[nt][3]);
    }
    __syncwarp();
    // dW2[j][i] = sum_r dH2[r][j] h1[r][i]: A[m=j][k=r] = dH2[r][j], B[k=r][n=i] = h1[r][i]
    // dW1[i][f] = sum_r dH1[r][i] x[r][f]:  A[m=i][k=r] = dH1[r][i], B[k=r][n=f] = x[r][f]
#pragma unroll
    for (int mt = 0; mt < 4; mt++) {
        const int m = mt * 16 + g;
        const uint32_t a2[4] = {pack_raw(s.d2[wi][2 * t][m], s.d2[wi][2 * t + 1][m]),
                                pack_raw(s.d2[wi][2 * t][m + 8], s.d2[wi][2 * t + 1][m + 8]),
                                pack_raw(s.d2[wi][2 * t + 8][m], s.d2[wi][2 * t + 9][m]),
                                pack_raw(s.d2[wi][2 * t + 8][m + 8], s.d2[wi][2 * t + 9][m + 8])};
        const uint32_t a1[4] = {pack_raw(s.d1[wi][2 * t][m], s.d1[wi][2 * t + 1][m]),
                                pack_raw(s.d1[wi][2 * t][m + 8], s.d1[wi][2 * t + 1][m + 8]),
                                pack_raw(s.d1[wi][2 * t + 8][m], s.d1[wi][2 * t + 9][m]),
                                pack_raw(s.d1[wi][2 * t + 8][m + 8], s.d1[wi][2 * t + 9][m + 8])};
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
            const int col = nt * 8 + g;
            const uint32_t b[2] = {pack_raw(s.h1[wi][2 * t][col], s.h1[wi][2 * t + 1][col]),
                                   pack_raw(s.h1[wi][2 * t + 8][col], s.h1[wi][2 * t + 9][col])};
            float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            mma_bf16(acc, a2, b);
            const int n = nt * 8 + 2 * t;
            out[kMlpOffW2 / 2 + m * kMlpHidden + n] = acc[0];
            out[kMlpOffW2 / 2 + m * kMlpHidden + n + 1] = acc[1];
            out[kMlpOffW2 / 2 + (m + 8) * kMlpHidden + n] = acc[2];
            out[kMlpOffW2 / 2 + (m + 8) * kMlpHidden + n + 1] = acc[3];
        }
#pragma unroll
        for (int nt = 0; nt < 4; nt++) {
            const int col = nt * 8 + g;
            const uint32_t b[2] = {pack_raw(s.x[wi][2 * t][col], s.x[wi][2 * t + 1][col]),
                                   pack_raw(s.x[wi][2 * t + 8][col], s.x[wi][2 * t + 9][col])};
            float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            mma_bf16(acc, a1, b);
            const int n = nt * 8 + 2 * t;
            out[kMlpOffW1 / 2 + m * kMlpFeatures + n] = acc[0];
            out[kMlpOffW1 / 2 + m * kMlpFeatures + n + 1] = acc[1];
            out[kMlpOffW1 / 2 + (m + 8) * kMlpFeatures + n] = acc[2];
            out[kMlpOffW1 / 2 + (m + 8) * kMlpFeatures + n + 1] = acc[3];
        }
    }
}

// One thread per parameter: the sum of the warps' partials in warp order, then
// (with `state`) an Adam step on the FP32 master copy and the BF16/FP32 model
// the kernels read.  Thread kMlpParamLoss sums the loss into `lossOut`.
__global__ void mlp_reduce_kernel(const float* __restrict__ part, unsigned int warps, float* __restrict__ grad,
                                  float* lossOut, MlpAdam* state, unsigned char* model,
                                  unsigned long long* stepPtr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kMlpParams) return;
    float sum = 0.0f;
    for (unsigned w = 0; w < warps; w++) sum = __fadd_rn(sum, part[(uint64_t)w * kMlpParams + i]);
    if (grad) grad[i] = sum;
    if (i == kMlpParamLoss) {
        if (lossOut) lossOut[stepPtr ? *stepPtr : 0] = sum;
        return;
    }
    if (!state) return;
    MlpAdam& a = *state;
    const float m = a.beta1 * a.m[i] + (1.0f - a.beta1) * sum;
    const float v = a.beta2 * a.v[i] + (1.0f - a.beta2) * sum * sum;
    a.m[i] = m;
    a.v[i] = v;
    const float b1p = a.beta1Pow * a.beta1, b2p = a.beta2Pow * a.beta2;  // powers of this step
    const float mh = m / (1.0f - b1p), vh = v / (1.0f - b2p);
    const float w = a.master[i] - a.lr * mh / (sqrtf(vh) + a.eps);
    a.master[i] = w;
    if (i < kMlpWeightCount) {
        reinterpret_cast<__nv_bfloat16*>(model)[i] = __float2bfloat16_rn(w);
    } else {
        reinterpret_cast<float*>(model + kMlpOffB1)[i - kMlpWeightCount] = w;
    }
}

// advances the step (after every thread of the reduce has read the old powers)
__global__ void mlp_step_kernel(MlpAdam* state, unsigned long long* stepPtr) {
    if (state) {
        state->beta1Pow *= state->beta1;
        state->beta2Pow *= state->beta2;
    }
    *stepPtr += 1;
}

__global__ void to_bf16_kernel(const float* __restrict__ in, uint64_t n, __nv_bfloat16* __restrict__ out) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = __float2bfloat16_rn(in[i]);
}

}  // namespace

size_t mlp_grad_smem_bytes() { return sizeof(TrainSmem); }

cudaError_t launch_mlp_infer(const unsigned char* model, const __nv_bfloat16* feat, const uint2* meta,
                             const unsigned int* countPtr, unsigned int count, unsigned int cap, float minLogit,
                             char* out, int outPitch, float* logits, unsigned long long* counters, int blocks,
                             cudaStream_t s) {
    if (blocks <= 0) blocks = 1;
    mlp_infer_kernel<<<blocks, kTcRows, 0, s>>>(model, feat, meta, countPtr, count, cap, minLogit, out, outPitch,
                                                 logits, counters);
    return cudaGetLastError();
}

cudaError_t set_classifier_wait_limit(uint32_t polls) {
    return cudaMemcpyToSymbol(g_tileWaitSpins, &polls, sizeof(polls));
}

cudaError_t launch_mlp_grad(const unsigned char* model, const __nv_bfloat16* feat, const float* label,
                            const uint32_t* perm, const unsigned long long* stepPtr, unsigned int stepsPerEpoch,
                            unsigned int rows, float invTotal, float* part, cudaStream_t s) {
    const size_t smem = sizeof(TrainSmem);
    cudaError_t e = cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const unsigned warps = (rows + 15) / 16;
    const unsigned blocks = (warps + kTrainWarps - 1) / kTrainWarps;
    mlp_grad_kernel<<<blocks, kTrainWarps * 32, smem, s>>>(model, feat, label, perm, stepPtr,
                                                           stepsPerEpoch ? stepsPerEpoch : 1u, rows, invTotal, part);
    return cudaGetLastError();
}

unsigned int mlp_grad_warps(unsigned int rows) {
    const unsigned warps = (rows + 15) / 16;
    return (warps + kTrainWarps - 1) / kTrainWarps * kTrainWarps;
}

cudaError_t launch_mlp_reduce(const float* part, unsigned int warps, float* grad, float* lossOut, MlpAdam* state,
                              unsigned char* model, unsigned long long* stepPtr, cudaStream_t s) {
    mlp_reduce_kernel<<<(kMlpParams + 255) / 256, 256, 0, s>>>(part, warps, grad, lossOut, state, model, stepPtr);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !stepPtr) return e;
    mlp_step_kernel<<<1, 1, 0, s>>>(state, stepPtr);
    return cudaGetLastError();
}

cudaError_t launch_to_bf16(const float* in, uint64_t n, __nv_bfloat16* out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    to_bf16_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(in, n, out);
    return cudaGetLastError();
}

}  // namespace cg
