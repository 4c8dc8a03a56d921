// Learned correction classifier: a 32 -> 64 -> 64 -> 1 MLP over per-column
// MSA features, BF16 weights and activations, FP32 accumulation, sigmoid
// output.  It stands where the reference's forest/logistic-regression
// classifier stands in its correction path (include/classification.hpp:51-157,
// include/forest.hpp:217-226, used by correctAnchorClf in
// include/corrector.hpp:1448-1472); the network, its features and its training
// are this project's own.
//
// Every matrix product runs on the tcgen05 tensor cores (kind::f16: BF16
// operands in shared memory, FP32 accumulators in tensor memory).  Inference
// scores 128 columns per tile; training takes a 128-row tile of a minibatch
// per block through the forward pass, the hidden gradient and both weight
// gradients (one product over transposed tiles).  Training is deterministic:
// every block writes its partial gradients to its own slot and one kernel sums
// the slots in a fixed order before the Adam update.

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

// ---------------------------------------------------------------- training (tcgen05)
//
// One block of 128 threads per 128-row tile of the minibatch (thread = row =
// TMEM lane): the forward pass and every gradient of the mean loss over the
// tile, as partial sums in part[tile][...] (parameter order of the model: w1,
// w2, w3, b1, b2, b3, loss) that mlp_reduce_kernel adds in tile order.  The
// matrix products run on tcgen05.mma (kind::f16, BF16 operands in shared
// memory in the canonical K-major layout, FP32 accumulators in tensor memory):
//   forward   D1 = X W1^T, D2 = H1 W2^T                (M = 128 rows)
//   backward  dH1 = dH2 W2                              (M = 128 rows)
//             [dW2; dW1] = [dH2^T; dH1^T] [H1^T | X^T]  (one M = 128, N = 96,
//             K = 128 product: rows 0-63 x columns 0-63 are dW2, rows 64-127
//             x columns 64-95 are dW1; the cross terms are not read)
// BF16 rounding at the same points as the oracle (oracle/mlp.py): the
// features, h1 and h2 after ReLU, dH2 before the products, dH1 before dW1;
// FP32 elsewhere.  dW3 and the bias gradients are column sums over the tile's
// rows (warp shuffles, then the four warps in order).

constexpr int kTrainRows = 128;
constexpr uint32_t kTrainTmemCols = 256;  // D1/D2 (0-127, later [dW2 dW1] at 0-95), dH1 (128-191)
constexpr int kTrainOutCols = kMlpHidden + kMlpFeatures;  // N of the weight-gradient product

// shared memory of one block (every operand tile 1024-byte aligned)
struct TrainTc {
    unsigned char xa[kTrainRows * kMlpFeatures * 2];        // A of D1: X [128][32]
    unsigned char w1[kMlpHidden * kMlpFeatures * 2];        // B of D1: W1 [64][32]
    unsigned char h1a[kTrainRows * kMlpHidden * 2];         // A of D2: H1 [128][64]
    unsigned char w2[kMlpHidden * kMlpHidden * 2];          // B of D2: W2 [64 out][64 in]
    unsigned char d2a[kTrainRows * kMlpHidden * 2];         // A of dH1: dH2 [128][64]
    unsigned char w2t[kMlpHidden * kMlpHidden * 2];         // B of dH1: W2^T [64 in][64 out]
    unsigned char gA[kTrainRows * kTrainRows * 2];          // A of [dW2; dW1]: [dH2^T; dH1^T] [128][128 rows]
    unsigned char gB[kTrainOutCols * kTrainRows * 2];       // B of [dW2; dW1]: [H1^T | X^T] [96][128 rows]
    float b1[kMlpHidden], b2[kMlpHidden], w3[kMlpHidden];
    float red[4][3 * kMlpHidden + 2];                       // per-warp column sums: dW3, db2, db1, db3, loss
    float b3;
    unsigned long long mbar;
    uint32_t tmemBase;
};

__global__ void __launch_bounds__(kTrainRows, 1) mlp_grad_kernel(const unsigned char* __restrict__ model,
                                                                 const __nv_bfloat16* __restrict__ feat,
                                                                 const float* __restrict__ label,
                                                                 const uint32_t* __restrict__ perm,
                                                                 const unsigned long long* stepPtr,
                                                                 unsigned int stepsPerEpoch, unsigned int rows,
                                                                 float invTotal, float* __restrict__ part,
                                                                 unsigned long long* failed) {
    extern __shared__ __align__(1024) unsigned char smraw[];
    TrainTc& s = *reinterpret_cast<TrainTc*>(smraw);
    const int tid = (int)threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const __nv_bfloat16* w1g = reinterpret_cast<const __nv_bfloat16*>(model + kMlpOffW1);
    const __nv_bfloat16* w2g = reinterpret_cast<const __nv_bfloat16*>(model + kMlpOffW2);
    const __nv_bfloat16* w3g = reinterpret_cast<const __nv_bfloat16*>(model + kMlpOffW3);
    for (int i = tid; i < kMlpHidden * kMlpFeatures; i += kTrainRows)
        *reinterpret_cast<__nv_bfloat16*>(s.w1 + core_offset(i / kMlpFeatures, i % kMlpFeatures, kMlpFeatures)) =
            w1g[i];
    for (int i = tid; i < kMlpHidden * kMlpHidden; i += kTrainRows) {
        const int o = i / kMlpHidden, in = i % kMlpHidden;
        *reinterpret_cast<__nv_bfloat16*>(s.w2 + core_offset(o, in, kMlpHidden)) = w2g[i];
        *reinterpret_cast<__nv_bfloat16*>(s.w2t + core_offset(in, o, kMlpHidden)) = w2g[i];
    }
    const float* bsrc = reinterpret_cast<const float*>(model + kMlpOffB1);
    if (tid < kMlpHidden) {
        s.b1[tid] = bsrc[tid];
        s.b2[tid] = bsrc[kMlpHidden + tid];
        s.w3[tid] = __bfloat162float(w3g[tid]);
    }
    if (tid == 0) {
        s.b3 = bsrc[2 * kMlpHidden];
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s.mbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s.tmemBase)),
                     "r"(kTrainTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    // this thread's row of the minibatch (zero features past the end)
    const uint64_t base = stepPtr ? (*stepPtr % stepsPerEpoch) * (uint64_t)rows : 0;
    const unsigned row = blockIdx.x * kTrainRows + (unsigned)tid;
    const bool valid = row < rows;
    const uint64_t src = valid ? (perm ? perm[base + row] : base + row) : 0;
    {
        uint4 f[4];
#pragma unroll
        for (int j = 0; j < 4; j++) f[j] = make_uint4(0, 0, 0, 0);
        if (valid) {
            const uint4* x = reinterpret_cast<const uint4*>(feat + src * kMlpFeatures);
#pragma unroll
            for (int j = 0; j < 4; j++) f[j] = x[j];
        }
#pragma unroll
        for (int j = 0; j < 4; j++) *reinterpret_cast<uint4*>(s.xa + core_offset(tid, 8 * j, kMlpFeatures)) = f[j];
        // X^T into rows 64-95 of the weight-gradient B operand (column = this row)
        const __nv_bfloat16* fv = reinterpret_cast<const __nv_bfloat16*>(f);
#pragma unroll
        for (int k = 0; k < kMlpFeatures; k++)
            *reinterpret_cast<__nv_bfloat16*>(s.gB + core_offset(kMlpHidden + k, tid, kTrainRows)) = fv[k];
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = s.tmemBase;
    const uint32_t laneAddr = tbase + ((uint32_t)(warp * 32) << 16);
    const uint32_t mb = smem_u32(&s.mbar);
    uint32_t phase = 0;
    bool ok = true;
    auto wait_mma = [&]() {
        if (!mbar_wait(mb, phase, kWaitSpins)) ok = false;
        phase ^= 1u;
        ok = !__syncthreads_or(!ok);
        tc_fence_after();
    };
    // ---- D1 = X W1^T (TMEM columns 0-63)
    if (tid == 0) {
#pragma unroll
        for (int k = 0; k < kMlpFeatures / 16; k++)
            tc_mma(tbase, smem_desc(smem_u32(s.xa) + 256u * k, 128, 512), smem_desc(smem_u32(s.w1) + 256u * k, 128, 512),
                   instr_desc(kTrainRows, kMlpHidden), k > 0);
        tc_commit(mb);
    }
    wait_mma();
    uint64_t h1pos = 0, h2pos = 0;  // ReLU masks of this row
    if (ok) {
#pragma unroll
        for (int half = 0; half < 2; half++) {
            float v[32];
            tc_ld32(laneAddr + 32u * half, v);
#pragma unroll
            for (int j = 0; j < 4; j++) {
                uint32_t w[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int c = 32 * half + 8 * j + 2 * q;
                    const float a = fmaxf(__fadd_rn(v[8 * j + 2 * q], s.b1[c]), 0.0f);
                    const float b = fmaxf(__fadd_rn(v[8 * j + 2 * q + 1], s.b1[c + 1]), 0.0f);
                    h1pos |= (uint64_t)(a > 0.0f) << c;
                    h1pos |= (uint64_t)(b > 0.0f) << (c + 1);
                    w[q] = pack_bf16(a, b);
                }
                *reinterpret_cast<uint4*>(s.h1a + core_offset(tid, 32 * half + 8 * j, kMlpHidden)) =
                    make_uint4(w[0], w[1], w[2], w[3]);
#pragma unroll
                for (int q = 0; q < 4; q++) {  // H1^T into rows 0-63 of the weight-gradient B operand
                    const int c = 32 * half + 8 * j + 2 * q;
                    *reinterpret_cast<uint16_t*>(s.gB + core_offset(c, tid, kTrainRows)) = (uint16_t)(w[q] & 0xffffu);
                    *reinterpret_cast<uint16_t*>(s.gB + core_offset(c + 1, tid, kTrainRows)) = (uint16_t)(w[q] >> 16);
                }
            }
        }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    // ---- D2 = H1 W2^T (TMEM columns 64-127)
    if (ok && tid == 0) {
#pragma unroll
        for (int k = 0; k < kMlpHidden / 16; k++)
            tc_mma(tbase + kMlpHidden, smem_desc(smem_u32(s.h1a) + 256u * k, 128, 1024),
                   smem_desc(smem_u32(s.w2) + 256u * k, 128, 1024), instr_desc(kTrainRows, kMlpHidden), k > 0);
        tc_commit(mb);
    }
    if (ok) wait_mma();
    // output layer, loss, dH2
    float h2[kMlpHidden];
    float dz = 0.0f, loss = 0.0f;
    if (ok) {
        float z = 0.0f;
#pragma unroll
        for (int half = 0; half < 2; half++) {
            float v[32];
            tc_ld32(laneAddr + (uint32_t)kMlpHidden + 32u * half, v);
#pragma unroll
            for (int i = 0; i < 32; i++) {
                const int c = 32 * half + i;
                const float r = fmaxf(__fadd_rn(v[i], s.b2[c]), 0.0f);
                h2pos |= (uint64_t)(r > 0.0f) << c;
                h2[c] = __bfloat162float(__float2bfloat16_rn(r));
                z = __fadd_rn(z, __fmul_rn(h2[c], s.w3[c]));
            }
        }
        z = __fadd_rn(z, s.b3);
        if (valid) {
            const float y = label[src];
            const float pr = 1.0f / (1.0f + expf(-z));
            dz = (pr - y) * invTotal;
            const float sp = fmaxf(z, 0.0f) + log1pf(expf(-fabsf(z)));
            loss = (sp - y * z) * invTotal;
        }
    }
    // column sums over the block's rows: four warps' shuffle sums, then in warp order
    auto colsum = [&](float v, int slot) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = __fadd_rn(v, __shfl_xor_sync(kFull, v, o));
        if (lane == 0) s.red[warp][slot] = v;
    };
    if (ok) {
#pragma unroll 4
        for (int c = 0; c < kMlpHidden; c++) {
            const float d2 = (h2pos >> c) & 1ull ? __fmul_rn(dz, s.w3[c]) : 0.0f;
            colsum(__fmul_rn(dz, h2[c]), c);           // dW3
            colsum(d2, kMlpHidden + c);                 // db2
            const __nv_bfloat16 b = __float2bfloat16_rn(d2);
            *reinterpret_cast<__nv_bfloat16*>(s.d2a + core_offset(tid, c, kMlpHidden)) = b;
            *reinterpret_cast<__nv_bfloat16*>(s.gA + core_offset(c, tid, kTrainRows)) = b;  // dH2^T, rows 0-63
        }
        colsum(dz, 3 * kMlpHidden);      // db3
        colsum(loss, 3 * kMlpHidden + 1);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    // ---- dH1 = dH2 W2 (TMEM columns 128-191)
    if (ok && tid == 0) {
#pragma unroll
        for (int k = 0; k < kMlpHidden / 16; k++)
            tc_mma(tbase + 2 * kMlpHidden, smem_desc(smem_u32(s.d2a) + 256u * k, 128, 1024),
                   smem_desc(smem_u32(s.w2t) + 256u * k, 128, 1024), instr_desc(kTrainRows, kMlpHidden), k > 0);
        tc_commit(mb);
    }
    if (ok) wait_mma();
    if (ok) {
#pragma unroll
        for (int half = 0; half < 2; half++) {
            float v[32];
            tc_ld32(laneAddr + 2u * kMlpHidden + 32u * half, v);
#pragma unroll 4
            for (int i = 0; i < 32; i++) {
                const int c = 32 * half + i;
                const float d1 = (h1pos >> c) & 1ull ? v[i] : 0.0f;
                colsum(d1, 2 * kMlpHidden + c);  // db1
                *reinterpret_cast<__nv_bfloat16*>(s.gA + core_offset(kMlpHidden + c, tid, kTrainRows)) =
                    __float2bfloat16_rn(d1);  // dH1^T, rows 64-127
            }
        }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    // ---- [dW2; dW1] = [dH2^T; dH1^T] [H1^T | X^T] (TMEM columns 0-95; D1 and D2 were read)
    if (ok && tid == 0) {
#pragma unroll
        for (int k = 0; k < kTrainRows / 16; k++)
            tc_mma(tbase, smem_desc(smem_u32(s.gA) + 256u * k, 128, 2048), smem_desc(smem_u32(s.gB) + 256u * k, 128, 2048),
                   instr_desc(kTrainRows, kTrainOutCols), k > 0);
        tc_commit(mb);
    }
    if (ok) wait_mma();
    float* out = part + (uint64_t)blockIdx.x * kMlpParams;
    if (ok) {
        if (tid < kMlpHidden) {  // row o of dW2: columns 0-63
#pragma unroll
            for (int half = 0; half < 2; half++) {
                float v[32];
                tc_ld32(laneAddr + 32u * half, v);
#pragma unroll
                for (int i = 0; i < 32; i++) out[kMlpOffW2 / 2 + tid * kMlpHidden + 32 * half + i] = v[i];
            }
        } else {  // row i of dW1: columns 64-95
            float v[32];
            tc_ld32(laneAddr + (uint32_t)kMlpHidden, v);
#pragma unroll
            for (int f = 0; f < kMlpFeatures; f++) out[kMlpOffW1 / 2 + (tid - kMlpHidden) * kMlpFeatures + f] = v[f];
        }
    }
    __syncthreads();
    if (ok) {
        for (int i = tid; i < 3 * kMlpHidden + 2; i += kTrainRows) {
            const float v = __fadd_rn(__fadd_rn(__fadd_rn(s.red[0][i], s.red[1][i]), s.red[2][i]), s.red[3][i]);
            int dst;
            if (i < kMlpHidden) dst = kMlpOffW3 / 2 + i;
            else if (i < 2 * kMlpHidden) dst = kMlpParamB2 + (i - kMlpHidden);
            else if (i < 3 * kMlpHidden) dst = kMlpParamB1 + (i - 2 * kMlpHidden);
            else if (i == 3 * kMlpHidden) dst = kMlpParamB3;
            else dst = kMlpParamLoss;
            out[dst] = v;
        }
    } else {
        for (int i = tid; i < kMlpParams; i += kTrainRows) out[i] = 0.0f;
        if (tid == 0 && failed) atomicAdd(failed, 1ull);
        mbar_wait(mb, phase ^ 1u, kWaitSpins);  // the MMAs in flight, bounded again
    }
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(kTrainTmemCols)
                     : "memory");
}

// One thread per parameter: the sum of the tiles' partials in tile order, then
// (with `state`) an Adam step on the FP32 master copy and the BF16/FP32 model
// the kernels read.  Thread kMlpParamLoss sums the loss into `lossOut`.
__global__ void mlp_reduce_kernel(const float* __restrict__ part, unsigned int parts, float* __restrict__ grad,
                                  float* lossOut, MlpAdam* state, unsigned char* model,
                                  unsigned long long* stepPtr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kMlpParams) return;
    float sum = 0.0f;
    for (unsigned w = 0; w < parts; w++) sum = __fadd_rn(sum, part[(uint64_t)w * kMlpParams + i]);
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

size_t mlp_grad_smem_bytes() { return sizeof(TrainTc) + 1024; }

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
                            unsigned int rows, float invTotal, float* part, unsigned long long* failed,
                            cudaStream_t s) {
    const size_t smem = mlp_grad_smem_bytes();
    cudaError_t e = cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    mlp_grad_kernel<<<mlp_grad_parts(rows), kTrainRows, smem, s>>>(model, feat, label, perm, stepPtr,
                                                                   stepsPerEpoch ? stepsPerEpoch : 1u, rows, invTotal,
                                                                   part, failed);
    return cudaGetLastError();
}

unsigned int mlp_grad_parts(unsigned int rows) { return (rows + kTrainRows - 1) / kTrainRows; }

cudaError_t launch_mlp_reduce(const float* part, unsigned int parts, float* grad, float* lossOut, MlpAdam* state,
                              unsigned char* model, unsigned long long* stepPtr, cudaStream_t s) {
    mlp_reduce_kernel<<<(kMlpParams + 255) / 256, 256, 0, s>>>(part, parts, grad, lossOut, state, model, stepPtr);
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
