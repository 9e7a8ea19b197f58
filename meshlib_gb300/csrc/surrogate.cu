// C ABI of the surrogate network: training on the GPU from exact samples, parameters in and out,
// inference, gradients (for checking against the CPU oracle), and the banded signed-distance grid
// that culls bricks with the surrogate (or with exact brick-centre distances).
#include <cuda_bf16.h>

#include <cfloat>
#include <cmath>
#include <cstring>

#include "../../include/gbfwn.h"
#include "handle.cuh"
#include "mlp.cuh"
#include "surrogate.cuh"

using namespace gbfwn;

struct gbfwn_surrogate_s {
    int device = 0;
    SurrogateNet net;
    float band = 0.f;
};

namespace {

// centre xyz, scale, 32 frequencies, clampD, margin, band, limit, marginAll, 7 reserved
constexpr int kMetaFloats = 48;

void metaOut(const gbfwn_surrogate_s* s, float* m) {
    std::memset(m, 0, sizeof(float) * kMetaFloats);
    for (int i = 0; i < 3; ++i) m[i] = s->net.meta.center[i];
    m[3] = s->net.meta.scale;
    for (int k = 0; k < 32; ++k) m[4 + k] = s->net.meta.freq[k];
    m[36] = s->net.meta.clampD;
    m[37] = s->net.meta.margin;
    m[38] = s->band;
    m[39] = s->net.meta.limit;
    m[40] = s->net.meta.marginAll;
}

void metaIn(gbfwn_surrogate_s* s, const float* m) {
    for (int i = 0; i < 3; ++i) s->net.meta.center[i] = m[i];
    s->net.meta.scale = m[3];
    for (int k = 0; k < 32; ++k) s->net.meta.freq[k] = m[4 + k];
    s->net.meta.clampD = m[36];
    s->net.meta.margin = m[37];
    s->band = m[38];
    s->net.meta.limit = m[39];
    s->net.meta.marginAll = m[40];
}

bool xfOk(const float* xf, Xf& X) {
    if (!xf) return false;
    for (int i = 0; i < 9; ++i) X.a[i] = xf[i];
    for (int i = 0; i < 3; ++i) X.b[i] = xf[9 + i];
    return true;
}

}  // namespace

extern "C" {

GBFWN_API void gbfwn_surrogate_default_opts(gbfwn_surrogate_opts* o) {
    if (!o) return;
    o->samples = 2000000;
    o->validation = 1000000;
    o->steps = 3000;
    o->batch = 16384;
    o->learningRate = 2e-3f;
    o->band = 0.f;
    o->beta = 2.f;
    o->seed = 1;
}

GBFWN_API int gbfwn_surrogate_train(gbfwn_handle h, const int32_t dims[3], const float xf[12], const gbfwn_surrogate_opts* opts,
                                    gbfwn_surrogate* out, gbfwn_surrogate_stats* stats) {
    Xf X;
    if (!h || !dims || dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0 || !xfOk(xf, X) || !opts || !out || opts->band <= 0.f ||
        opts->steps <= 0 || opts->batch < 128 || opts->samples < opts->batch || opts->validation < 0)
        return fail(GBFWN_INVALID, "gbfwn_surrogate_train: bad arguments");
    *out = nullptr;
    std::lock_guard<std::mutex> lk(h->mu);
    DeviceGuard g(h->device);
    auto* s = new gbfwn_surrogate_s;
    s->device = h->device;
    s->band = opts->band;
    cudaError_t e = s->net.init(opts->seed);
    if (e) {
        delete s;
        return cudaFail(e, "gbfwn_surrogate_train init");
    }
    // sampling box = the grid's box (voxel centres +- half a voxel), bounds of the 8 corners
    TrainOptions t;
    for (int a = 0; a < 3; ++a) {
        t.lo[a] = FLT_MAX;
        t.hi[a] = -FLT_MAX;
    }
    for (int c = 0; c < 8; ++c) {
        const float v[3] = {(c & 1) ? dims[0] - 0.5f : -0.5f, (c & 2) ? dims[1] - 0.5f : -0.5f, (c & 4) ? dims[2] - 0.5f : -0.5f};
        for (int a = 0; a < 3; ++a) {
            const float p = X.a[3 * a] * v[0] + X.a[3 * a + 1] * v[1] + X.a[3 * a + 2] * v[2] + X.b[a];
            t.lo[a] = std::fmin(t.lo[a], p);
            t.hi[a] = std::fmax(t.hi[a], p);
        }
    }
    float ext = 0.f;
    for (int a = 0; a < 3; ++a) {
        s->net.meta.center[a] = 0.5f * (t.lo[a] + t.hi[a]);
        ext = std::fmax(ext, t.hi[a] - t.lo[a]);
    }
    s->net.meta.scale = 2.f / ext;
    s->net.meta.clampD = 6.f * opts->band;
    t.samples = opts->samples;
    t.validation = opts->validation;
    t.steps = opts->steps;
    t.batch = opts->batch;
    t.lr = opts->learningRate;
    t.sigma = opts->band;
    t.beta = opts->beta;
    t.seed = opts->seed;
    t.marginFloor = 1e-3f * opts->band;
    // the one-sided margin is validated out to band + twice the half diagonal of this grid's 8x8x8
    // bricks, which covers the brick centres a banded call on this grid (or a finer one) can keep
    {
        float r = 0.f;
        for (int c = 0; c < 8; ++c) {
            const float d[3] = {(c & 1) ? 3.5f : -3.5f, (c & 2) ? 3.5f : -3.5f, (c & 4) ? 3.5f : -3.5f};
            float r2 = 0.f;
            for (int a = 0; a < 3; ++a) {
                const float w = X.a[3 * a] * d[0] + X.a[3 * a + 1] * d[1] + X.a[3 * a + 2] * d[2];
                r2 += w * w;
            }
            r = std::fmax(r, std::sqrt(r2));
        }
        t.limit = opts->band + 2.f * 1.0001f * r;
    }
    TrainStats st;
    e = s->net.train(h->tree.q, h->scratch, t, st, h->stream);
    if (e) {
        delete s;
        return e == cudaErrorLaunchTimeout ? fail(GBFWN_TIMEOUT, "gbfwn_surrogate_train: a tensor-core wait timed out")
                                           : cudaFail(e, "gbfwn_surrogate_train");
    }
    if (stats) {
        stats->trainLoss = st.trainLoss;
        stats->validationMaxError = st.valMaxErr;
        stats->margin = st.margin;
        stats->sampleSeconds = st.sampleSeconds;
        stats->trainSeconds = st.trainSeconds;
        stats->steps = st.steps;
        stats->validationOverestimate = st.valOverestimate;
        stats->limit = st.limit;
    }
    *out = s;
    return GBFWN_OK;
}

GBFWN_API int gbfwn_surrogate_destroy(gbfwn_surrogate s) {
    if (!s) return GBFWN_OK;
    DeviceGuard g(s->device);
    cudaDeviceSynchronize();
    delete s;  // frees the network's device memory with its device current
    return GBFWN_OK;
}

GBFWN_API int gbfwn_surrogate_get(gbfwn_surrogate s, float* params, float* meta) {
    if (!s) return fail(GBFWN_INVALID, "gbfwn_surrogate_get: null surrogate");
    DeviceGuard g(s->device);
    if (params) {
        const cudaError_t e = s->net.getParams(params, nullptr);
        if (e) return cudaFail(e, "gbfwn_surrogate_get");
    }
    if (meta) metaOut(s, meta);
    return GBFWN_OK;
}

GBFWN_API int gbfwn_surrogate_create(int device, const float* params, const float* meta, gbfwn_surrogate* out) {
    if (!params || !meta || !out) return fail(GBFWN_INVALID, "gbfwn_surrogate_create: bad arguments");
    *out = nullptr;
    DeviceGuard g(device);
    auto* s = new gbfwn_surrogate_s;
    s->device = device;
    cudaError_t e = s->net.init(1);
    if (!e) e = s->net.setParams(params, nullptr);
    if (!e) e = s->net.ensureWork(16384);
    if (!e) e = cudaDeviceSynchronize();
    if (e) {
        delete s;
        return cudaFail(e, "gbfwn_surrogate_create");
    }
    metaIn(s, meta);
    *out = s;
    return GBFWN_OK;
}

GBFWN_API int gbfwn_surrogate_eval_dev(gbfwn_surrogate s, const float* d_pts, int64_t n, float* d_out, void* stream) {
    if (!s || n < 0 || (n > 0 && (!d_pts || !d_out))) return fail(GBFWN_INVALID, "gbfwn_surrogate_eval_dev: bad arguments");
    DeviceGuard g(s->device);
    cudaError_t e = s->net.ensureWork(16384);
    if (!e) e = s->net.infer(d_pts, n, d_out, static_cast<cudaStream_t>(stream));
    return e ? cudaFail(e, "gbfwn_surrogate_eval_dev") : GBFWN_OK;
}

GBFWN_API int gbfwn_surrogate_gradients_dev(gbfwn_surrogate s, const float* d_pts, const float* d_targets, int32_t n,
                                            float* grads, float* loss) {
    if (!s || n <= 0 || n > 16384 || !d_pts || !d_targets || !grads)
        return fail(GBFWN_INVALID, "gbfwn_surrogate_gradients_dev: bad arguments");
    DeviceGuard g(s->device);
    cudaError_t e = s->net.ensureWork(16384);
    const int nPad = (n + 127) / 128 * 128;
    if (!e && nPad > s->net.workRows()) return fail(GBFWN_INVALID, "gbfwn_surrogate_gradients_dev: n exceeds the training batch");
    if (!e) e = s->net.step(d_pts, d_targets, nullptr, n, n, nPad, false, 1, 0.f, nullptr);
    if (!e) e = cudaMemcpy(grads, s->net.grads(), sizeof(float) * kSurrogateParams, cudaMemcpyDeviceToHost);
    if (!e && loss) e = cudaMemcpy(loss, s->net.lossPtr(), sizeof(float), cudaMemcpyDeviceToHost);
    return e ? cudaFail(e, "gbfwn_surrogate_gradients_dev") : GBFWN_OK;
}

GBFWN_API int gbfwn_from_grid_with_distances_banded_dev(gbfwn_handle h, gbfwn_surrogate s, const int32_t dims[3],
                                                        const float xf[12], const gbfwn_dist_opts* opts, float* d_out,
                                                        gbfwn_banded_stats* stats, void* stream) {
    Xf X;
    if (!h || !dims || dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0 || !xfOk(xf, X) || !opts || !d_out ||
        !(opts->maxDistSq > 0.f && opts->maxDistSq < FLT_MAX) || !opts->nullOutsideMinMax)
        return fail(GBFWN_INVALID, "gbfwn_from_grid_with_distances_banded_dev: needs a finite maxDistSq and nullOutsideMinMax");
    if (gridTiles(dims[0], dims[1], dims[2]) > kMaxTilesPerLaunch) return fail(GBFWN_INVALID, "grid too large");
    std::lock_guard<std::mutex> lk(h->mu);
    DeviceGuard g(h->device);
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : h->stream;
    const DistOpts o{opts->minDistSq, opts->maxDistSq, opts->nullOutsideMinMax, opts->windingNumberThreshold, opts->windingNumberBeta};
    const GridRange r{dims[0], dims[1], dims[2], 0, dims[2], 0};
    BandedStats bs;
    cudaError_t e = cudaMemsetAsync(h->scratch, 0, 2 * sizeof(unsigned), st);
    if (!e) e = bandedGrid(h->tree.q, s ? &s->net : nullptr, r, X, o, h->precise, d_out, h->scratch, bs, st);
    if (e) return cudaFail(e, "gbfwn_from_grid_with_distances_banded_dev");
    if (stats) {
        stats->bricks = bs.bricks;
        stats->keptBricks = bs.keptBricks;
        stats->cullMs = bs.cullMs;
        stats->exactMs = bs.exactMs;
    }
    return GBFWN_OK;
}

GBFWN_API int gbfwn_debug_wait_timeout(uint32_t maxPolls, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned* d = nullptr;
    cudaError_t e = devMalloc((void**)&d, sizeof(unsigned));
    if (!e) e = cudaMemsetAsync(d, 0, sizeof(unsigned), s);
    if (!e) e = launchWaitTimeout(maxPolls, d, s);
    unsigned st = 0;
    if (!e) e = cudaMemcpyAsync(&st, d, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    if (!e) e = cudaStreamSynchronize(s);
    if (d) cudaFree(d);
    if (e) return cudaFail(e, "gbfwn_debug_wait_timeout");
    return (st & 2u) ? fail(GBFWN_TIMEOUT, "a bounded device-side wait gave up") : GBFWN_OK;
}

GBFWN_API int gbfwn_debug_gemm_bf16(const void* d_a, const void* d_b, float* d_d, int32_t m, int32_t n, int32_t k,
                                    int32_t split_k, void* stream) {
    if (!d_a || !d_b || !d_d) return GBFWN_INVALID;
    GemmEpilogue ep;
    ep.mode = GemmEpilogue::kStoreF32;
    ep.D = d_d;
    ep.ldd = n;
    const cudaError_t e = launchGemmBf16(static_cast<const __nv_bfloat16*>(d_a), k, static_cast<const __nv_bfloat16*>(d_b), k, m,
                                         n, k, split_k, ep, static_cast<cudaStream_t>(stream));
    if (e == cudaErrorInvalidValue) return GBFWN_INVALID;
    return e ? GBFWN_CUDA_ERROR : GBFWN_OK;
}

}  // extern "C"
