// Learned correction classifier: model layout, column records and launches.
//
// Model blob (the device copy the kernels read, and the payload of the file
// cg_load_classifier accepts after its header):
//   byte 0      w1  BF16 [64][32]   hidden 1 <- features (row = neuron)
//   byte 4096   w2  BF16 [64][64]   hidden 2 <- hidden 1
//   byte 12288  w3  BF16 [64]       output  <- hidden 2
//   byte 12416  b1  FP32 [64], b2 FP32 [64], b3 FP32
// Parameter index (gradients, optimiser state): the BF16 elements in blob
// order (w1, w2, w3: 6208), then b1, b2, b3; index 6337 carries the loss.
#ifndef CARE_LEARNED_H
#define CARE_LEARNED_H

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "care_internal.h"

namespace cg {

constexpr int kMlpFeatures = kLearnedFeatures;
constexpr int kMlpHidden = 64;
constexpr int kMlpOffW1 = 0;
constexpr int kMlpOffW2 = kMlpOffW1 + kMlpHidden * kMlpFeatures * 2;
constexpr int kMlpOffW3 = kMlpOffW2 + kMlpHidden * kMlpHidden * 2;
constexpr int kMlpOffB1 = kMlpOffW3 + kMlpHidden * 2;
constexpr int kMlpBytes = (kMlpOffB1 + (2 * kMlpHidden + 1) * 4 + 15) / 16 * 16;
constexpr int kMlpWeightCount = kMlpOffB1 / 2;
constexpr int kMlpParamB1 = kMlpWeightCount;
constexpr int kMlpParamB2 = kMlpParamB1 + kMlpHidden;
constexpr int kMlpParamB3 = kMlpParamB2 + kMlpHidden;
constexpr int kMlpParamLoss = kMlpParamB3 + 1;
constexpr int kMlpParams = kMlpParamLoss + 1;
static_assert(kMlpOffB1 % 4 == 0, "bias alignment");

// Adam state in device memory (FP32 master weights in parameter order).
struct MlpAdam {
    float m[kMlpParams], v[kMlpParams], master[kMlpParams];
    float beta1, beta2, beta1Pow, beta2Pow, lr, eps;
};

size_t mlp_grad_smem_bytes();
// partial-gradient slots (128-row tiles) one minibatch of `rows` rows writes
unsigned int mlp_grad_parts(unsigned int rows);

// Inference over `count` (or *countPtr, at most cap) columns: logits to
// `logits`, or the consensus base into out[meta.x][meta.y & 0xffff] for every
// logit >= minLogit (meta.y >> 16 = the consensus base).
cudaError_t launch_mlp_infer(const unsigned char* model, const __nv_bfloat16* feat, const uint2* meta,
                             const unsigned int* countPtr, unsigned int count, unsigned int cap, float minLogit,
                             char* out, int outPitch, float* logits, unsigned long long* counters, int blocks,
                             cudaStream_t s);
// Polls of the inference kernel's per-tile MMA waits on the current device
// (default 1 << 20); a block whose wait runs out counts in
// counters[kCounterTimeouts] and leaves its columns to the fallback decision.
cudaError_t set_classifier_wait_limit(uint32_t polls);
// Partial gradients of the mean binary cross-entropy over `rows` rows of a
// minibatch, one slot per 128-row tile (tcgen05 products): rows
// perm[step * rows + r] of feat/label (perm may be null; step = *stepPtr %
// stepsPerEpoch, or 0 without stepPtr).  A tile whose MMA wait runs out
// writes zeros and counts in *failed.
cudaError_t launch_mlp_grad(const unsigned char* model, const __nv_bfloat16* feat, const float* label,
                            const uint32_t* perm, const unsigned long long* stepPtr, unsigned int stepsPerEpoch,
                            unsigned int rows, float invTotal, float* part, unsigned long long* failed,
                            cudaStream_t s);
// Sum of the partials (-> grad, loss -> lossOut[*stepPtr or 0]); with `state`
// an Adam step that rewrites `model`; with stepPtr the step counter advances.
cudaError_t launch_mlp_reduce(const float* part, unsigned int parts, float* grad, float* lossOut, MlpAdam* state,
                              unsigned char* model, unsigned long long* stepPtr, cudaStream_t s);
cudaError_t launch_to_bf16(const float* in, uint64_t n, __nv_bfloat16* out, cudaStream_t s);

}  // namespace cg

// Checks a serialized classifier (header + blob) and extracts the blob.
bool cg_parse_classifier(const void* data, size_t size, std::vector<unsigned char>* blob);

namespace cg {

}  // namespace cg

#endif
