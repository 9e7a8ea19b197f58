// Internal: the mesh handle behind gbfwn_handle, error reporting and device allocation helpers
// shared by the C ABI translation units.
#pragma once

#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gbfwn.h"
#include "common.cuh"

namespace gbfwn {

// Records the message of a failure for gbfwn_last_error() (per calling thread) and returns status.
int fail(int status, const std::string& msg);
// Maps a CUDA error to GBFWN_OUT_OF_MEMORY / GBFWN_CUDA_ERROR with "NVIDIA GPU error: ..." text.
int cudaFail(cudaError_t e, const char* what);
// cudaMalloc honouring the fault-injection hook gbfwn_debug_fail_next_allocs.
cudaError_t devMalloc(void** p, size_t bytes);
// The library's stream-ordered memory pool on a device (freed memory is kept for reuse), an
// allocation from it (honouring the same hook; complete when it returns) and a stream-ordered free.
cudaMemPool_t devicePool(int device);
cudaError_t poolMalloc(void** p, size_t bytes, int device, cudaStream_t s);
void poolFree(void* p, cudaStream_t s);

// Allocations freed together.  With a device set, they come from that device's pool (complete, and
// usable from any stream, when alloc returns) and go back to it on freeAll, stream-ordered on
// `stream`: the caller makes sure nothing still uses them, as cudaFree's synchronisation used to.
struct ListAllocator : Allocator {
    std::vector<void*> ptrs;
    int device = -1;
    cudaStream_t stream = nullptr;
    cudaError_t alloc(void** p, size_t bytes) override {
        cudaError_t e = device >= 0 ? poolMalloc(p, bytes, device, stream) : devMalloc(p, bytes);
        if (e == cudaSuccess) ptrs.push_back(*p);
        return e;
    }
    void freeAll() {
        for (void* p : ptrs) {
            if (device >= 0)
                poolFree(p, stream);
            else
                cudaFree(p);
        }
        ptrs.clear();
    }
};

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

}  // namespace gbfwn

struct gbfwn_mesh_s {
    int device = 0;
    cudaStream_t stream = nullptr, copyStream = nullptr;
    gbfwn::ListAllocator treeMem;
    gbfwn::DeviceTree tree;
    float* dVerts = nullptr;
    int32_t* dTris = nullptr;
    int64_t nv = 0, nt = 0;
    unsigned* scratch = nullptr;  // [0] ticket counter, [1] status bits
    int precise = 1;
    int signReuse = 1;  // signed-distance grids of closed surfaces may take a voxel's sign from the voxel below
    void applySignReuse() { tree.q.closed = (signReuse && tree.closed) ? 1 : 0; }
    // device staging reused across host-API calls
    void* outBuf = nullptr;
    size_t outCap = 0;
    void* inBuf = nullptr;
    size_t inCap = 0;
    void* sortBuf = nullptr;  // Morton order + radix-sort scratch of point queries
    size_t sortCap = 0;
    void* colBuf = nullptr;  // column hand-over words of signed-distance grid launches
    size_t colCap = 0;
    std::vector<cudaEvent_t> events;
    std::mutex mu;  // calls on one handle are serialised (the reference is not re-entrant per object)
    std::atomic<int> batchRefs{0};  // live batches whose work items point into this handle's tree

    // grows a staging buffer; buffers come from the device's pool, so one freed by an earlier handle
    // is reused without mapping new memory
    cudaError_t ensure(void** buf, size_t* cap, size_t bytes) {
        if (*cap >= bytes) return cudaSuccess;
        if (*buf) {
            cudaDeviceSynchronize();  // no call may still use it on another stream (as cudaFree ensured)
            gbfwn::poolFree(*buf, stream);
        }
        *buf = nullptr;
        *cap = 0;
        cudaError_t e = gbfwn::poolMalloc(buf, bytes, device, stream);
        if (e == cudaSuccess) *cap = bytes;
        return e;
    }
    cudaError_t ensureEvents(size_t n) {
        while (events.size() < n) {
            cudaEvent_t ev;
            cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
            if (e) return e;
            events.push_back(ev);
        }
        return cudaSuccess;
    }
    int checkStatus() {
        unsigned st[2] = {0, 0};
        cudaError_t e = cudaMemcpyAsync(st, scratch, sizeof(st), cudaMemcpyDeviceToHost, stream);
        if (!e) e = cudaStreamSynchronize(stream);
        if (e) return gbfwn::cudaFail(e, "status read");
        if (st[1] & gbfwn::kStatusStackOverflow)
            return gbfwn::fail(GBFWN_TRAVERSAL_OVERFLOW, "traversal stack overflow (tree deeper than 32 levels)");
        if (st[1] & gbfwn::kStatusTimeout) return gbfwn::fail(GBFWN_TIMEOUT, "device-side wait timed out");
        return GBFWN_OK;
    }
    cudaError_t resetStatus(cudaStream_t s) { return cudaMemsetAsync(scratch, 0, 2 * sizeof(unsigned), s); }
};
