// C ABI of the learned classifier's training and stand-alone inference
// (include/care_gpu.h: cg_train_classifier, cg_classifier_gradients,
// cg_classifier_logits).  No reference counterpart: the reference ships a
// forest/logistic-regression classifier trained outside the program
// (include/classification.hpp:51-157); this network is trained here, on the
// device, by the kernels of k_learned.cu.
//
// Training: minibatch Adam on the mean binary cross-entropy.  One step is two
// kernels (partial gradients of the minibatch, then the ordered sum and the
// Adam update) captured once into a CUDA graph and replayed for every step of
// every epoch; the step counter and the optimiser state live on the device,
// and the host only uploads a new row permutation per epoch.

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>
#include <random>
#include <vector>

#include "care_gpu.h"
#include "care_internal.h"
#include "care_learned.h"

using namespace cg;

namespace {

constexpr char kMagic[8] = {'C', 'G', 'M', 'L', 'P', '0', '0', '1'};
constexpr size_t kHeader = 32;

struct Header {
    char magic[8];
    uint32_t features, hidden1, hidden2, payload;
    uint32_t reserved[2];
};
static_assert(sizeof(Header) == kHeader, "classifier header");

// A device allocation freed on scope exit.
struct Dev {
    void* p = nullptr;
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, std::max<size_t>(n, 16)); }
    ~Dev() {
        if (p) cudaFree(p);
    }
    template <class T>
    T* as() const {
        return static_cast<T*>(p);
    }
};

int cuda_status(cudaError_t e) {
    if (e == cudaSuccess) return CG_OK;
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? CG_ERR_OUT_OF_MEMORY : CG_ERR_CUDA;
}

#define TRY(call)                                 \
    do {                                          \
        const int rc_ = cuda_status(call);        \
        if (rc_ != CG_OK) return rc_;             \
    } while (0)

float bf16_to_float(uint16_t v) {
    uint32_t u = (uint32_t)v << 16;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

uint16_t float_to_bf16(float f) {  // round to nearest even (finite inputs)
    uint32_t u;
    std::memcpy(&u, &f, 4);
    u += 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

// He-uniform weights, zero biases, from a seeded generator
std::vector<unsigned char> init_blob(uint32_t seed) {
    std::vector<unsigned char> blob(kMlpBytes, 0);
    std::mt19937_64 rng(seed);
    auto fill = [&](int off, int n, int fanIn) {
        std::uniform_real_distribution<float> u(-std::sqrt(6.0f / fanIn), std::sqrt(6.0f / fanIn));
        uint16_t* w = reinterpret_cast<uint16_t*>(blob.data() + off);
        for (int i = 0; i < n; i++) w[i] = float_to_bf16(u(rng));
    };
    fill(kMlpOffW1, kMlpHidden * kMlpFeatures, kMlpFeatures);
    fill(kMlpOffW2, kMlpHidden * kMlpHidden, kMlpHidden);
    fill(kMlpOffW3, kMlpHidden, kMlpHidden);
    return blob;
}

bool parse(const void* data, size_t size, std::vector<unsigned char>* blob) {
    if (!data || size < kHeader) return false;
    Header h;
    std::memcpy(&h, data, kHeader);
    if (std::memcmp(h.magic, kMagic, 8) != 0 || h.features != (uint32_t)kMlpFeatures ||
        h.hidden1 != (uint32_t)kMlpHidden || h.hidden2 != (uint32_t)kMlpHidden || h.payload != (uint32_t)kMlpBytes ||
        size < kHeader + kMlpBytes)
        return false;
    const unsigned char* p = static_cast<const unsigned char*>(data) + kHeader;
    blob->assign(p, p + kMlpBytes);
    return true;
}

void serialize(const std::vector<unsigned char>& blob, void* out) {
    Header h{};
    std::memcpy(h.magic, kMagic, 8);
    h.features = kMlpFeatures;
    h.hidden1 = kMlpHidden;
    h.hidden2 = kMlpHidden;
    h.payload = kMlpBytes;
    std::memcpy(out, &h, kHeader);
    std::memcpy(static_cast<unsigned char*>(out) + kHeader, blob.data(), kMlpBytes);
}

// features (FP32, host) -> BF16 on the device
int upload_features(const float* features, uint64_t n, Dev& f32, Dev& bf, cudaStream_t s) {
    const uint64_t elems = n * kMlpFeatures;
    TRY(f32.alloc(elems * sizeof(float)));
    TRY(bf.alloc(elems * sizeof(__nv_bfloat16)));
    TRY(cudaMemcpyAsync(f32.p, features, elems * sizeof(float), cudaMemcpyHostToDevice, s));
    TRY(launch_to_bf16(f32.as<float>(), elems, bf.as<__nv_bfloat16>(), s));
    return CG_OK;
}

// a stream on `device`, destroyed on scope exit
struct Stream {
    cudaStream_t s = nullptr;
    ~Stream() {
        if (s) cudaStreamDestroy(s);
    }
};

}  // namespace

bool cg_parse_classifier(const void* data, size_t size, std::vector<unsigned char>* blob) {
    return parse(data, size, blob);
}

extern "C" {

size_t cg_classifier_size(void) { return kHeader + kMlpBytes; }

void cg_default_train_options(cg_train_options* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->epochs = 4;
    o->batch_rows = 4096;
    o->learning_rate = 2e-3f;
    o->seed = 1;
}

int cg_train_classifier(const cg_train_options* o, const float* features, const uint8_t* labels, uint64_t n,
                        void* model_out, size_t model_capacity, float* losses, uint64_t loss_capacity,
                        uint64_t* steps_out) {
    if (!o || !features || !labels || !model_out) return CG_ERR_INVALID_ARGUMENT;
    if (model_capacity < kHeader + kMlpBytes) return CG_ERR_INVALID_ARGUMENT;
    if (o->epochs < 1 || o->batch_rows < 16 || o->batch_rows % 16 || !(o->learning_rate > 0.0f))
        return CG_ERR_INVALID_ARGUMENT;
    const uint64_t B = (uint64_t)o->batch_rows;
    if (n < B || n > 0xffffffffull) return CG_ERR_INVALID_ARGUMENT;
    std::vector<unsigned char> blob;
    if (o->init_model) {
        if (!parse(o->init_model, o->init_model_size, &blob)) return CG_ERR_INVALID_ARGUMENT;
    } else {
        blob = init_blob(o->seed);
    }
    const uint32_t stepsPerEpoch = (uint32_t)(n / B);
    const uint64_t totalSteps = (uint64_t)stepsPerEpoch * (uint64_t)o->epochs;
    TRY(cudaSetDevice(o->device));
    Stream st;
    TRY(cudaStreamCreateWithFlags(&st.s, cudaStreamNonBlocking));
    cudaStream_t s = st.s;
    Dev f32, bf, lab, perm, model, part, adam, step, loss, failed;
    int rc = upload_features(features, n, f32, bf, s);
    if (rc != CG_OK) return rc;
    std::vector<float> hl(n);
    for (uint64_t i = 0; i < n; i++) hl[i] = labels[i] ? 1.0f : 0.0f;
    TRY(lab.alloc(n * sizeof(float)));
    TRY(cudaMemcpyAsync(lab.p, hl.data(), n * sizeof(float), cudaMemcpyHostToDevice, s));
    TRY(perm.alloc(n * sizeof(uint32_t)));
    TRY(model.alloc(kMlpBytes));
    TRY(cudaMemcpyAsync(model.p, blob.data(), kMlpBytes, cudaMemcpyHostToDevice, s));
    const unsigned parts = mlp_grad_parts((unsigned)B);
    TRY(part.alloc((size_t)parts * kMlpParams * sizeof(float)));
    TRY(cudaMemsetAsync(part.p, 0, (size_t)parts * kMlpParams * sizeof(float), s));
    TRY(failed.alloc(sizeof(unsigned long long)));
    TRY(cudaMemsetAsync(failed.p, 0, sizeof(unsigned long long), s));
    // optimiser state: master weights from the initial model
    auto hs = std::make_unique<MlpAdam>();
    std::memset(hs.get(), 0, sizeof(MlpAdam));
    const uint16_t* wb = reinterpret_cast<const uint16_t*>(blob.data());
    for (int i = 0; i < kMlpWeightCount; i++) hs->master[i] = bf16_to_float(wb[i]);
    const float* bb = reinterpret_cast<const float*>(blob.data() + kMlpOffB1);
    for (int i = kMlpWeightCount; i < kMlpParamLoss; i++) hs->master[i] = bb[i - kMlpWeightCount];
    hs->beta1 = 0.9f;
    hs->beta2 = 0.999f;
    hs->beta1Pow = 1.0f;
    hs->beta2Pow = 1.0f;
    hs->lr = o->learning_rate;
    hs->eps = 1e-8f;
    TRY(adam.alloc(sizeof(MlpAdam)));
    TRY(cudaMemcpyAsync(adam.p, hs.get(), sizeof(MlpAdam), cudaMemcpyHostToDevice, s));
    TRY(step.alloc(sizeof(unsigned long long)));
    TRY(cudaMemsetAsync(step.p, 0, sizeof(unsigned long long), s));
    TRY(loss.alloc(totalSteps * sizeof(float)));
    // one training step, captured
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = launch_mlp_grad(model.as<unsigned char>(), bf.as<__nv_bfloat16>(), lab.as<float>(),
                                    perm.as<uint32_t>(), step.as<unsigned long long>(), stepsPerEpoch, (unsigned)B,
                                    1.0f / (float)B, part.as<float>(), failed.as<unsigned long long>(), s);
    if (e == cudaSuccess)
        e = launch_mlp_reduce(part.as<float>(), parts, nullptr, loss.as<float>(), adam.as<MlpAdam>(),
                              model.as<unsigned char>(), step.as<unsigned long long>(), s);
    const cudaError_t e2 = cudaStreamEndCapture(s, &graph);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return cuda_status(e != cudaSuccess ? e : e2);
    }
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_status(e);
    std::vector<uint32_t> order(n);
    std::mt19937_64 rng(o->seed * 0x9E3779B97F4A7C15ull + 7);
    rc = CG_OK;
    for (int ep = 0; ep < o->epochs && rc == CG_OK; ep++) {
        std::iota(order.begin(), order.end(), 0u);
        std::shuffle(order.begin(), order.end(), rng);
        // the previous epoch's replays read the old order: wait before overwriting it
        rc = cuda_status(cudaStreamSynchronize(s));
        if (rc == CG_OK)
            rc = cuda_status(cudaMemcpyAsync(perm.p, order.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
        for (uint32_t k = 0; k < stepsPerEpoch && rc == CG_OK; k++) rc = cuda_status(cudaGraphLaunch(exec, s));
    }
    if (rc == CG_OK) rc = cuda_status(cudaStreamSynchronize(s));
    unsigned long long nFailed = 0;
    if (rc == CG_OK) rc = cuda_status(cudaMemcpy(&nFailed, failed.p, sizeof(nFailed), cudaMemcpyDeviceToHost));
    if (rc == CG_OK && nFailed) rc = CG_ERR_TIMEOUT;  // a tile gave up waiting for its tensor-core products
    if (rc == CG_OK) rc = cuda_status(cudaMemcpy(blob.data(), model.p, kMlpBytes, cudaMemcpyDeviceToHost));
    if (rc == CG_OK && losses && loss_capacity) {
        const uint64_t k = std::min<uint64_t>(loss_capacity, totalSteps);
        rc = cuda_status(cudaMemcpy(losses, loss.p, k * sizeof(float), cudaMemcpyDeviceToHost));
    }
    cudaGraphExecDestroy(exec);
    if (rc != CG_OK) return rc;
    serialize(blob, model_out);
    if (steps_out) *steps_out = totalSteps;
    return CG_OK;
}

int cg_classifier_gradients(int device, const void* model_data, size_t model_size, const float* features,
                            const uint8_t* labels, uint32_t n, float* grads, float* loss_out) {
    if (!features || !labels || !grads || n == 0) return CG_ERR_INVALID_ARGUMENT;
    std::vector<unsigned char> blob;
    if (!parse(model_data, model_size, &blob)) return CG_ERR_INVALID_ARGUMENT;
    TRY(cudaSetDevice(device));
    Stream st;
    TRY(cudaStreamCreateWithFlags(&st.s, cudaStreamNonBlocking));
    cudaStream_t s = st.s;
    Dev f32, bf, lab, model, part, grad, failed;
    int rc = upload_features(features, n, f32, bf, s);
    if (rc != CG_OK) return rc;
    std::vector<float> hl(n);
    for (uint32_t i = 0; i < n; i++) hl[i] = labels[i] ? 1.0f : 0.0f;
    TRY(lab.alloc(n * sizeof(float)));
    TRY(cudaMemcpyAsync(lab.p, hl.data(), n * sizeof(float), cudaMemcpyHostToDevice, s));
    TRY(model.alloc(kMlpBytes));
    TRY(cudaMemcpyAsync(model.p, blob.data(), kMlpBytes, cudaMemcpyHostToDevice, s));
    const unsigned parts = mlp_grad_parts(n);
    TRY(part.alloc((size_t)parts * kMlpParams * sizeof(float)));
    TRY(cudaMemsetAsync(part.p, 0, (size_t)parts * kMlpParams * sizeof(float), s));
    TRY(grad.alloc(kMlpParams * sizeof(float)));
    TRY(failed.alloc(sizeof(unsigned long long)));
    TRY(cudaMemsetAsync(failed.p, 0, sizeof(unsigned long long), s));
    TRY(launch_mlp_grad(model.as<unsigned char>(), bf.as<__nv_bfloat16>(), lab.as<float>(), nullptr, nullptr, 1, n,
                        1.0f / (float)n, part.as<float>(), failed.as<unsigned long long>(), s));
    TRY(launch_mlp_reduce(part.as<float>(), parts, grad.as<float>(), nullptr, nullptr, nullptr, nullptr, s));
    std::vector<float> g(kMlpParams);
    unsigned long long nFailed = 0;
    TRY(cudaMemcpyAsync(g.data(), grad.p, kMlpParams * sizeof(float), cudaMemcpyDeviceToHost, s));
    TRY(cudaMemcpyAsync(&nFailed, failed.p, sizeof(nFailed), cudaMemcpyDeviceToHost, s));
    TRY(cudaStreamSynchronize(s));
    if (nFailed) return CG_ERR_TIMEOUT;
    std::memcpy(grads, g.data(), (kMlpParams - 1) * sizeof(float));
    if (loss_out) *loss_out = g[kMlpParamLoss];
    return CG_OK;
}

int cg_classifier_logits(int device, const void* model_data, size_t model_size, const float* features, uint64_t n,
                         float* logits) {
    if (!features || !logits) return CG_ERR_INVALID_ARGUMENT;
    if (n == 0) return CG_OK;
    if (n > 0xffffffffull) return CG_ERR_INVALID_ARGUMENT;
    std::vector<unsigned char> blob;
    if (!parse(model_data, model_size, &blob)) return CG_ERR_INVALID_ARGUMENT;
    TRY(cudaSetDevice(device));
    Stream st;
    TRY(cudaStreamCreateWithFlags(&st.s, cudaStreamNonBlocking));
    cudaStream_t s = st.s;
    Dev f32, bf, model, out, counters;
    int rc = upload_features(features, n, f32, bf, s);
    if (rc != CG_OK) return rc;
    TRY(model.alloc(kMlpBytes));
    TRY(cudaMemcpyAsync(model.p, blob.data(), kMlpBytes, cudaMemcpyHostToDevice, s));
    TRY(out.alloc(n * sizeof(float)));
    TRY(counters.alloc(kNumCounters * sizeof(unsigned long long)));
    TRY(cudaMemsetAsync(counters.p, 0, kNumCounters * sizeof(unsigned long long), s));
    int sms = 1;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) sms = 1;
    const int blocks = (int)std::min<uint64_t>((n + 127) / 128, 2ull * (uint64_t)std::max(sms, 1));
    TRY(launch_mlp_infer(model.as<unsigned char>(), bf.as<__nv_bfloat16>(), nullptr, nullptr, (unsigned)n,
                         (unsigned)n, 0.0f, nullptr, 0, out.as<float>(), counters.as<unsigned long long>(), blocks,
                         s));
    unsigned long long hc[kNumCounters];
    TRY(cudaMemcpyAsync(hc, counters.p, sizeof(hc), cudaMemcpyDeviceToHost, s));
    TRY(cudaMemcpyAsync(logits, out.p, n * sizeof(float), cudaMemcpyDeviceToHost, s));
    TRY(cudaStreamSynchronize(s));
    if (hc[kCounterTimeouts]) return CG_ERR_TIMEOUT;
    return CG_OK;
}

}  // extern "C"
