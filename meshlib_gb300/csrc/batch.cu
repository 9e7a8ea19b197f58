// C ABI of the batched signed-distance launch: many meshes, each with its own grid, computed by one
// persistent kernel fed from a single work queue, optionally replayed from a CUDA graph, with the
// tile shape and block size picked by timing every variant on the batch itself.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <vector>

#include "../../include/gbfwn.h"
#include "handle.cuh"

using namespace gbfwn;

struct gbfwn_batch_s {
    int device = 0;
    int precise = 1;
    int nItems = 0;
    int config = 0;
    BatchItem* dItems[kBatchConfigs] = {};
    uint32_t totalTiles[kBatchConfigs] = {};
    unsigned* scratch = nullptr;  // ticket counter + status word of this batch
    bool pairOk = true;           // no item with a lower distance bound: the paired variants apply
    void* fix = nullptr;          // the precise paired walk's list (counter + entries)
    cudaStream_t captureStream = nullptr;
    cudaGraphExec_t graph = nullptr;
    int graphConfig = -1;
    // every distinct mesh of the batch, each holding one reference: gbfwn_destroy refuses a mesh
    // that a live batch still points into
    std::vector<gbfwn_mesh_s*> meshes;
    ~gbfwn_batch_s() {
        for (auto* m : meshes) m->batchRefs.fetch_sub(1);
        DeviceGuard g(device);
        if (graph) cudaGraphExecDestroy(graph);
        if (captureStream) cudaStreamDestroy(captureStream);
        for (auto* p : dItems)
            if (p) cudaFree(p);
        if (scratch) cudaFree(scratch);
        if (fix) cudaFree(fix);
    }
};

extern "C" {

GBFWN_API int gbfwn_batch_create(const gbfwn_batch_item* items, int32_t n, gbfwn_batch* out) {
    if (!items || n <= 0 || !out) return fail(GBFWN_INVALID, "gbfwn_batch_create: bad arguments");
    *out = nullptr;
    const int device = items[0].mesh ? items[0].mesh->device : 0;
    std::vector<int> order(n);
    std::vector<double> cost(n);
    for (int i = 0; i < n; ++i) {
        const gbfwn_batch_item& it = items[i];
        if (!it.mesh || !it.d_out || it.dims[0] <= 0 || it.dims[1] <= 0 || it.dims[2] <= 0 || it.mesh->device != device)
            return fail(GBFWN_INVALID, "gbfwn_batch_create: bad item (null mesh or output, empty grid, other device)");
        const double vox = double(it.dims[0]) * it.dims[1] * it.dims[2];
        cost[i] = vox * (1.0 + std::log2(1.0 + double(it.mesh->tree.nLeaves)));
        order[i] = i;
    }
    // most expensive first: their tiles are dequeued first, the cheap grids fill the tail
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
    auto* b = new gbfwn_batch_s;
    b->device = device;
    b->precise = items[0].mesh->precise;
    b->nItems = n;
    for (int i = 0; i < n; ++i) {
        gbfwn_mesh_s* m = items[i].mesh;
        if (std::find(b->meshes.begin(), b->meshes.end(), m) == b->meshes.end()) {
            m->batchRefs.fetch_add(1);
            b->meshes.push_back(m);
        }
    }
    DeviceGuard g(device);
    cudaError_t e = cudaSuccess;
    for (int c = 0; c < kBatchConfigs && !e; ++c) {
        std::vector<BatchItem> h(n);
        uint64_t base = 0;
        for (int k = 0; k < n; ++k) {
            const gbfwn_batch_item& it = items[order[k]];
            BatchItem& bi = h[k];
            bi.t = it.mesh->tree.q;
            bi.g = GridRange{it.dims[0], it.dims[1], it.dims[2], 0, it.dims[2], 0};
            for (int j = 0; j < 9; ++j) bi.xf.a[j] = it.xf[j];
            for (int j = 0; j < 3; ++j) bi.xf.b[j] = it.xf[9 + j];
            bi.o = DistOpts{it.opts.minDistSq, it.opts.maxDistSq, it.opts.nullOutsideMinMax, it.opts.windingNumberThreshold,
                            it.opts.windingNumberBeta};
            bi.out = it.d_out;
            if (it.opts.minDistSq > 0.f) b->pairOk = false;
            bi.tileBase = uint32_t(base);
            base += batchTiles(c, it.dims[0], it.dims[1], it.dims[2]);
        }
        if (base > kMaxTilesPerLaunch) {
            delete b;
            return fail(GBFWN_INVALID, "gbfwn_batch_create: batch too large for one work queue (2^32-1 tiles)");
        }
        b->totalTiles[c] = uint32_t(base);
        e = devMalloc((void**)&b->dItems[c], sizeof(BatchItem) * size_t(n));
        if (!e) e = cudaMemcpy(b->dItems[c], h.data(), sizeof(BatchItem) * size_t(n), cudaMemcpyHostToDevice);
    }
    if (!e) e = devMalloc((void**)&b->scratch, 64);
    uint32_t maxTiles = 0;
    for (int c = 0; c < kBatchConfigs; ++c) maxTiles = std::max(maxTiles, b->totalTiles[c]);
    if (!e && b->precise && b->pairOk) e = devMalloc(&b->fix, sizeof(uint4) * (size_t(batchFixCap(maxTiles)) + 1));
    if (!e) e = cudaMemset(b->scratch, 0, 64);
    if (!e) e = cudaStreamCreateWithFlags(&b->captureStream, cudaStreamNonBlocking);
    if (e) {
        delete b;
        return cudaFail(e, "gbfwn_batch_create");
    }
    *out = b;
    return GBFWN_OK;
}

GBFWN_API int gbfwn_batch_destroy(gbfwn_batch b) {
    delete b;
    return GBFWN_OK;
}

GBFWN_API int32_t gbfwn_batch_num_configs(void) { return kBatchConfigs; }

GBFWN_API const char* gbfwn_batch_config_name(int32_t config) { return batchConfigName(config); }

GBFWN_API int gbfwn_batch_set_config(gbfwn_batch b, int32_t config) {
    if (!b || config < 0 || config >= kBatchConfigs) return fail(GBFWN_INVALID, "gbfwn_batch_set_config: bad arguments");
    b->config = config;
    return GBFWN_OK;
}

GBFWN_API int gbfwn_batch_run_dev(gbfwn_batch b, void* stream) {
    if (!b) return fail(GBFWN_INVALID, "gbfwn_batch_run_dev: null batch");
    DeviceGuard g(b->device);
    const cudaError_t e = launchBatchSdf(b->dItems[b->config], b->nItems, b->totalTiles[b->config], b->precise, b->config,
                                         b->pairOk, b->fix, b->scratch, static_cast<cudaStream_t>(stream));
    return e ? cudaFail(e, "gbfwn_batch_run_dev") : GBFWN_OK;
}

GBFWN_API int gbfwn_batch_graph_launch(gbfwn_batch b, void* stream) {
    if (!b) return fail(GBFWN_INVALID, "gbfwn_batch_graph_launch: null batch");
    DeviceGuard g(b->device);
    cudaError_t e = cudaSuccess;
    if (!b->graph || b->graphConfig != b->config) {
        if (b->graph) cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
        cudaGraph_t graph = nullptr;
        e = cudaStreamBeginCapture(b->captureStream, cudaStreamCaptureModeThreadLocal);
        if (!e) {
            const cudaError_t le = launchBatchSdf(b->dItems[b->config], b->nItems, b->totalTiles[b->config], b->precise,
                                                  b->config, b->pairOk, b->fix, b->scratch, b->captureStream);
            e = cudaStreamEndCapture(b->captureStream, &graph);
            if (!e) e = le;
        }
        if (!e) e = cudaGraphInstantiate(&b->graph, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (e) return cudaFail(e, "gbfwn_batch_graph_launch capture");
        b->graphConfig = b->config;
    }
    e = cudaGraphLaunch(b->graph, static_cast<cudaStream_t>(stream));
    return e ? cudaFail(e, "gbfwn_batch_graph_launch") : GBFWN_OK;
}

GBFWN_API int gbfwn_batch_autotune(gbfwn_batch b, int32_t* best, float* times_ms) {
    if (!b) return fail(GBFWN_INVALID, "gbfwn_batch_autotune: null batch");
    DeviceGuard g(b->device);
    cudaStream_t s = b->captureStream;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float bestMs = FLT_MAX;
    int bestC = 0;
    cudaError_t e = cudaSuccess;
    for (int c = 0; c < kBatchConfigs && !e; ++c) {
        float ms = FLT_MAX;
        for (int rep = 0; rep < 3 && !e; ++rep) {  // first repetition warms caches and loads the kernel
            cudaEventRecord(e0, s);
            e = launchBatchSdf(b->dItems[c], b->nItems, b->totalTiles[c], b->precise, c, b->pairOk, b->fix, b->scratch, s);
            cudaEventRecord(e1, s);
            if (!e) e = cudaEventSynchronize(e1);
            float t = 0.f;
            cudaEventElapsedTime(&t, e0, e1);
            if (rep > 0) ms = std::min(ms, t);
        }
        if (times_ms) times_ms[c] = ms;
        if (ms < bestMs) {
            bestMs = ms;
            bestC = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e) return cudaFail(e, "gbfwn_batch_autotune");
    b->config = bestC;
    if (best) *best = bestC;
    return GBFWN_OK;
}

}  // extern "C"
