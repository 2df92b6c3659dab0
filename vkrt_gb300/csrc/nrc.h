// nrc.h — host interface of the neural radiance cache (nrc.cu).
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "nrc.cuh"

namespace vkrt {

// tensor-core path of cache inference: tcgen05 MMAs with tensor-memory accumulators (kNrcInferUmma), or warp-level
// mma.sync (kNrcForward, which training always uses)
enum NrcTensorPath : uint32_t { kNrcTensorTcgen05 = 0, kNrcTensorMmaSync = 1 };

struct NrcSettings {
    float learningRate;
    float beta1, beta2, epsilon;
    uint32_t seed;
};

// Parameters, optimiser state and scratch of one cache. All device memory; methods run asynchronously on `stream`.
class NrcEngine {
public:
    NrcEngine();
    ~NrcEngine();
    NrcEngine(const NrcEngine&) = delete;
    NrcEngine& operator=(const NrcEngine&) = delete;

    // (Re)initialises the parameters (seeded) and the optimiser; `lo`/`hi` bound the scene for the hash grid.
    cudaError_t reset(const NrcSettings& s, float3 lo, float3 hi, cudaStream_t stream);
    bool ready() const { return table_ != nullptr; }
    const NrcGridInfo& grid() const { return grid_; }

    // Radiance predictions (float4 per input, xyz used) for n inputs in device memory.
    cudaError_t infer(const NrcInput* inputs, uint32_t n, float4* out, cudaStream_t stream);
    // Device-side count: infers *count inputs (at most capacity), for graph-captured frames.
    cudaError_t inferCounted(const NrcInput* inputs, const uint32_t* count, uint32_t capacity, float4* out,
                             cudaStream_t stream);
    // One optimiser step on n records (inputs and float4 targets, xyz used) with the relative L2 loss; adds the
    // step's mean loss to *lossOut (device float) when given. applyUpdate = false keeps the parameters (gradients only).
    cudaError_t train(const NrcInput* inputs, const float4* targets, uint32_t n, float* lossOut, bool applyUpdate,
                      cudaStream_t stream);

    // parameter and gradient access for tests: FP16 weights (kNrcWeightCount) and table (kNrcTableParams halves);
    // FP32 gradients of the last step with respect to the same parameters (already divided by the batch size); the
    // table gradient is consumed (cleared) by a step that applies the update
    __half* weights() { return wHalf_; }
    __half* table() { return reinterpret_cast<__half*>(table_); }
    float* weightGrad() { return wGrad_; }
    float* tableGrad() { return tGrad_; }
    // refresh the FP32 master copies from the FP16 parameters (after a test wrote them)
    cudaError_t syncMasters(cudaStream_t stream);
    // allocates the inference scratch for `capacity` rows ahead of a graph capture (no allocation while capturing)
    cudaError_t reserveInference(uint32_t capacity);
    void setTensorPath(uint32_t path) { tensorPath_ = path; }
    // inference reads an exponential moving average of the parameters (per optimiser step: avg = decay avg +
    // (1 - decay) param) when decay > 0; the average restarts from the current parameters
    cudaError_t setAverageDecay(float decay, cudaStream_t stream) {
        averageDecay_ = decay;
        return refreshAverage(0.0f, stream);
    }
    uint32_t tensorPath() const { return tensorPath_; }
    // device error word (bit 0: a tcgen05 completion wait ran out), read synchronously on `stream`
    cudaError_t errorWord(unsigned int* out, cudaStream_t stream);

private:
    cudaError_t ensureScratch(uint32_t n);
    cudaError_t refreshAverage(float decay, cudaStream_t stream);
    NrcSettings s_{};
    NrcGridInfo grid_{};
    uint32_t step_ = 0;
    // parameters: FP16 working copies, FP32 masters, Adam moments, gradients
    __half* wHalf_ = nullptr;
    float *wMaster_ = nullptr, *wM_ = nullptr, *wV_ = nullptr, *wGrad_ = nullptr;
    __half2* table_ = nullptr;
    float *tMaster_ = nullptr, *tM_ = nullptr, *tV_ = nullptr, *tGrad_ = nullptr;
    bool tGradClear_ = false;  // the table gradient is all zeros (the sparse Adam step clears what it consumes)
    // scratch for n rows
    uint32_t cap_ = 0;
    __half *x0_ = nullptr, *acts_ = nullptr, *dz_ = nullptr, *dy_ = nullptr;
    __half* x0Infer_ = nullptr;
    uint32_t capInfer_ = 0;
    float* dx0_ = nullptr;
    uint32_t* masks_ = nullptr;  // ReLU masks of the forward pass, 5 x tiles x 32 words
    float4* out_ = nullptr;
    unsigned int* error_ = nullptr;
    uint32_t tensorPath_ = kNrcTensorTcgen05;
    float averageDecay_ = 0.0f;
    __half* wAvg_ = nullptr;   // parameter averages read by inference
    __half2* tAvg_ = nullptr;
};

}  // namespace vkrt
