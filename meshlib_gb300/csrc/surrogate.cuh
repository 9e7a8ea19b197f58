// Surrogate signed-distance network (mlp_net.cu) and the banded grid that uses it.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "common.cuh"

namespace gbfwn {

constexpr int kSurrogateParams = 74369;

struct NetMeta {
    float center[3] = {0, 0, 0};
    float scale = 1.f;   // u = (p - center) * scale
    float freq[32] = {};
    float clampD = 1.f;  // training target clamp
    // validated bound of |pred| - |d| (how far the prediction may overstate the distance) over the
    // held-out samples with |d| < limit: the only error that can make a brick cull wrong, checked only
    // where a wrong cull can happen
    float margin = 0.f;
    float limit = 0.f;
    float marginAll = 0.f;  // validated bound of |pred - clamp(d)| over all held-out samples
};

struct TrainOptions {
    int64_t samples = 2000000;
    int64_t validation = 1000000;
    int steps = 3000;
    int batch = 16384;
    float lr = 2e-3f;
    float sigma = 0.01f;     // standard deviation of the near-surface offsets
    float beta = 2.f;        // winding-number beta of the exact targets
    float lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};  // sampling box
    float marginScale = 1.25f, marginFloor = 0.f;
    float limit = 0.f;  // |d| below which the one-sided margin is validated (0: everywhere)
    uint64_t seed = 1;
};

struct TrainStats {
    float trainLoss = 0, valMaxErr = 0, margin = 0, sampleSeconds = 0, trainSeconds = 0, valOverestimate = 0, limit = 0;
    int steps = 0;
};

struct BandedStats {
    int bricks = 0, keptBricks = 0;
    float cullMs = 0, exactMs = 0;
};

class SurrogateNet {
public:
    NetMeta meta;
    ~SurrogateNet();
    cudaError_t init(uint64_t seed);
    cudaError_t setParams(const float* hostParams, cudaStream_t s);
    cudaError_t getParams(float* hostParams, cudaStream_t s) const;
    cudaError_t ensureWork(int batchPad);
    cudaError_t train(const QueryTree& t, unsigned* scratch, const TrainOptions& o, TrainStats& st, cudaStream_t s);
    cudaError_t infer(const float* pts, int64_t n, float* out, cudaStream_t s);
    // forward + backward on n rows (padded to nPad, a multiple of 128), gradients left in grads()
    cudaError_t step(const float* pts, const float* targets, const int32_t* idx, int64_t idxMod, int n, int nPad, bool update,
                     int totalSteps, float lr, cudaStream_t s);
    const float* grads() const { return grads_; }
    int workRows() const;
    const float* lossPtr() const { return scalars_; }
    unsigned* statusPtr() const { return reinterpret_cast<unsigned*>(counters_ + 3); }

private:
    struct Work;
    cudaError_t alloc(void** p, size_t bytes);
    cudaError_t pack(cudaStream_t s);
    void release();
    std::vector<void*> mem_;
    float *params_ = nullptr, *grads_ = nullptr, *m_ = nullptr, *v_ = nullptr, *scalars_ = nullptr;
    __nv_bfloat16* img_ = nullptr;  // bf16 shared-memory images of W1..W4 (training and inference)
    int32_t* counters_ = nullptr;  // [0] step, [1] batch offset, [3] status
    Work* work_ = nullptr;
    cudaGraphExec_t graph_ = nullptr;
};

cudaError_t bandedGrid(const QueryTree& t, SurrogateNet* net, const GridRange& g, const Xf& xf, const DistOpts& o, int precise,
                       float* out, unsigned* scratch, BandedStats& st, cudaStream_t s);

}  // namespace gbfwn
