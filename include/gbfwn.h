/*
 * gbfwn.h -- C ABI of the GB300-native fast-winding-number / signed-distance library.
 *
 * This is the drop-in boundary for MeshLib's `MR::IFastWindingNumber` hot path.  Every entry
 * point is plain C: pointers, sizes and status codes, no C++ or torch types, so that a C++
 * adapter (include/gbfwn.hpp), a ctypes stub or any other FFI can bind it.  Each function cites
 * the reference interface it replaces (paths inside the MeshLib project).
 *
 * Conventions shared by all calls
 *  - Meshes are indexed triangle lists: `verts` = nv x 3 floats, `tris` = nt x 3 int32 vertex
 *    ids.  A triangle with any negative vertex id is an invalid (deleted) face: it is not part
 *    of the tree and is never reported as self-intersecting -- MeshLib's `getValidFaces()`.
 *  - Grids: voxel (x, y, z), x fastest, is written at x + y*dims[0] + z*dims[0]*dims[1]
 *    (MRMesh/MRVolumeIndexer.h:131-139).  The voxel centre is gridToMeshXf applied to the float
 *    vector (x, y, z); `xf` is 12 floats: the 3x3 linear part row by row, then the translation
 *    (MRMesh/MRAffineXf.h:46).
 *  - Calls without a `_dev` suffix take and return HOST memory and are synchronous, like
 *    `MR::Cuda::FastWindingNumber`.  Where the GPU reads and writes pageable host memory itself
 *    (Grace-Blackwell's coherent NVLink-C2C) and the caller's grid buffer is already populated (a
 *    std::vector that was resized, a buffer reused across calls), a whole-grid call without a
 *    progress callback writes the grid straight into that buffer instead of into a device buffer
 *    followed by a copy; the values are the same either way.  `_dev` calls take DEVICE pointers and only enqueue work on
 *    `stream`: NULL = the handle's own stream; any cudaStream_t, including cudaStreamLegacy
 *    (0x1) and cudaStreamPerThread (0x2), is accepted.
 *  - A handle owns one work-queue counter and staging buffers: calls on the same handle must not
 *    overlap on the GPU (keep them on one stream, or serialise them); different handles are
 *    independent.
 *  - Traversal status: the kernels record a traversal-stack overflow (GBFWN_TRAVERSAL_OVERFLOW) in a
 *    device status word.  Host-memory calls read it back before returning; `_dev` calls only enqueue
 *    work and do not.  An overflow cannot happen for the trees this library builds: the median split
 *    of at most 2^30 faces gives a depth of at most 30, and a depth-first walk that pushes at most
 *    two children per step then holds at most 31 entries, below the fixed depth of 32.
 *  - Progress callbacks receive a fraction in [0, 1] and return nonzero to continue, zero to
 *    cancel (MRMesh/MRProgressCallback.h); a cancelled call returns GBFWN_CANCELLED.
 *  - Errors: a nonzero status; `gbfwn_last_error()` gives the message of the last failure on the
 *    calling thread (MeshLib's Expected<void> error string, MRCuda/MRCudaBasic.cpp:109-129).
 */
#ifndef GBFWN_H
#define GBFWN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define GBFWN_API __declspec(dllexport)
#else
#define GBFWN_API __attribute__((visibility("default")))
#endif

enum gbfwn_status {
    GBFWN_OK = 0,
    GBFWN_CANCELLED = 1,      /* progress callback returned 0 (MeshLib: unexpectedOperationCanceled) */
    GBFWN_OUT_OF_MEMORY = 2,  /* a device or pinned allocation failed */
    GBFWN_CUDA_ERROR = 3,     /* any other CUDA runtime error ("NVIDIA GPU error: ...") */
    GBFWN_INVALID = 4,        /* bad argument: null pointer, non-positive dims, vertex id out of range */
    GBFWN_TIMEOUT = 5,        /* a bounded device-side wait gave up */
    GBFWN_TRAVERSAL_OVERFLOW = 6 /* a traversal stack exceeded its fixed depth (tree too deep) */
};

typedef struct gbfwn_mesh_s* gbfwn_handle;

/* MR::DistanceToMeshOptions (MRMesh/MRDistanceToMeshOptions.h:10-33); same field meaning and
 * defaults: minDistSq = 0, maxDistSq = FLT_MAX, nullOutsideMinMax = 1, threshold = 0.5, beta = 2. */
typedef struct gbfwn_dist_opts {
    float minDistSq;
    float maxDistSq;
    int32_t nullOutsideMinMax;
    float windingNumberThreshold;
    float windingNumberBeta;
} gbfwn_dist_opts;

typedef int (*gbfwn_progress_cb)(float progress, void* user);

/* IFastWindingNumberByParts::GridByPartsFunc (MRMesh/MRFastWindingNumber.h:88): receives one
 * z-slab of `dims[2]` whole XY layers starting at layer `zOffset`, in host memory that stays valid
 * only during the call.  Return 0 to continue; any other value aborts the whole call with that
 * status. */
typedef int (*gbfwn_slab_cb)(const float* data, const int32_t dims[3], int32_t zOffset, void* user);

/* Computation knobs.  precise = 1 (default): compensated (Kahan) summation of the winding-number
 * terms and FP64 re-evaluation of solid angles and point-triangle projections for queries within
 * a few ulps of a triangle plane.  precise = 0: the reference's FP32 arithmetic, plain sums. */
GBFWN_API void gbfwn_set_precise(gbfwn_handle h, int precise);

/* Exact signs on closed surfaces (default on).  When the mesh's valid faces form a closed oriented
 * surface (every edge used equally often in both directions; gbfwn_is_closed), the exact winding
 * number is an integer, constant along any segment not meeting the surface, to which the
 * reference's approximated winding number rounds with windingNumberBeta >= 2 and a threshold whose
 * fractional part lies in (0.25, 0.75) (the default 0.5).  Under those conditions:
 *  - a grid whose z axis is vertical (xf's third column (0, 0, +s); any rotation about z) takes the
 *    signs of its voxels from its columns: the signed number of crossings of the column above each
 *    voxel (signed-distance grids and gbfwn_make_signed_by_winding_number_dev);
 *  - other grids, and points, take a voxel's sign from the voxel below it when no surface lies
 *    between them, or from the crossings of one vertical ray;
 * and a voxel or point on the surface (up to rounding) evaluates its approximated winding number.
 * Distances are unaffected.  enable = 0 evaluates every voxel's winding number, as the reference
 * does. */
GBFWN_API void gbfwn_set_sign_reuse(gbfwn_handle h, int enable);

/* 1 if the mesh's valid faces form a closed oriented surface (fingerprint of the directed edges,
 * computed when the handle is created), else 0. */
GBFWN_API int gbfwn_is_closed(gbfwn_handle h);

/* Library version string. */
GBFWN_API const char* gbfwn_version(void);

/* Message of the last failure on this thread ("" if none). */
GBFWN_API const char* gbfwn_last_error(void);

/* Replaces MR::Cuda::FastWindingNumber::FastWindingNumber(const Mesh&) (MRCuda/MRCudaFastWindingNumber.h:21)
 * together with its lazy prepareData_ (MRCuda/MRCudaFastWindingNumber.cpp:46-85): uploads the mesh to
 * `device` and builds the AABB tree and dipoles there.  The tree is the reference's tree
 * (MRMesh/MRAABBTreeMaker.hpp:51-165), node for node. */
GBFWN_API int gbfwn_create(const float* verts, int64_t nv, const int32_t* tris, int64_t nt, int device,
                           gbfwn_handle* out);

/* Same, but the vertex and triangle arrays are already in device memory of `device`. */
GBFWN_API int gbfwn_create_dev(const float* d_verts, int64_t nv, const int32_t* d_tris, int64_t nt, int device,
                               gbfwn_handle* out);

/* Frees the device data of the handle.  A handle that is an item of a live batch (gbfwn_batch_create)
 * is not freed: the call returns GBFWN_INVALID and the handle stays valid until the batch is
 * destroyed. */
GBFWN_API int gbfwn_destroy(gbfwn_handle h);

/* Moved vertices, same triangles: MR::AABBTree::refit (MRMesh/MRAABBTree.cpp:62-94) as
 * MR::Mesh::updateCaches calls it (MRMesh/MRMesh.cpp:571-583), then the dipoles recomputed
 * (updateCaches drops them; MRMesh/MRDipole.cpp:23-71 rebuilds them on the next query).  `verts`
 * holds all nv vertices at their new positions; `changedVerts` (ceil(nv/64) little-endian 64-bit
 * words, MeshLib's VertBitSet blocks; NULL = every vertex) marks the moved ones: the boxes of the
 * faces around them and of every node above those are recomputed, the tree topology is kept (so
 * queries may be slower than after a rebuild, as in the reference) and every query afterwards sees
 * the new positions.  Synchronous; must not overlap with other calls on the handle.  The `_dev`
 * variant takes device pointers (d_verts may be the handle's own vertex array). */
GBFWN_API int gbfwn_refit(gbfwn_handle h, const float* verts, const uint64_t* changedVerts);
GBFWN_API int gbfwn_refit_dev(gbfwn_handle h, const float* d_verts, const uint64_t* d_changedVerts, void* stream);

/* Number of triangles (faces, valid or not) and of tree nodes (2 * valid - 1). */
GBFWN_API int64_t gbfwn_num_faces(gbfwn_handle h);
GBFWN_API int64_t gbfwn_num_nodes(gbfwn_handle h);

/* Copies the tree to host memory in the reference layout (MRMesh/MRAABBTreeNode.h:29-46):
 * per node 8 words = box min xyz, box max xyz (float), l, r (int32; leaf <=> r < 0, then l = face),
 * nodes in the reference's pre-order.  `dipoles` (may be NULL) receives 8 floats per node:
 * pos xyz, area, dirArea xyz, rr (MRMesh/MRDipole.h:10-28). */
GBFWN_API int gbfwn_get_tree(gbfwn_handle h, void* nodes, float* dipoles);

/* IFastWindingNumber::calcFromVector (MRMesh/MRFastWindingNumber.h:26;
 * MRCuda/MRCudaFastWindingNumber.cpp:87-127): winding numbers at n points (3 floats each).
 * skipFace < 0: none. */
GBFWN_API int gbfwn_from_vector(gbfwn_handle h, const float* pts, int64_t n, float beta, int32_t skipFace, float* out,
                                gbfwn_progress_cb cb, void* user);
GBFWN_API int gbfwn_from_vector_dev(gbfwn_handle h, const float* d_pts, int64_t n, float beta, int32_t skipFace,
                                    float* d_out, void* stream);

/* IFastWindingNumber::calcSelfIntersections (MRMesh/MRFastWindingNumber.h:31;
 * MRCuda/MRCudaFastWindingNumber.cpp:129-173): bit f of `bits` (ceil(nt/64) little-endian 64-bit
 * words, MeshLib's FaceBitSet block layout) is set when the winding number at the centroid of valid
 * face f, skipping f itself, is < 0 or > 1.  `wn` (may be NULL) receives those winding numbers
 * (NaN for invalid faces). */
GBFWN_API int gbfwn_self_intersections(gbfwn_handle h, float beta, uint64_t* bits, float* wn, gbfwn_progress_cb cb,
                                       void* user);
GBFWN_API int gbfwn_self_intersections_dev(gbfwn_handle h, float beta, uint64_t* d_bits, float* d_wn, void* stream);

/* IFastWindingNumber::calcFromGrid (MRMesh/MRFastWindingNumber.h:38;
 * MRCuda/MRCudaFastWindingNumber.cpp:175-228): winding number at every voxel centre. */
GBFWN_API int gbfwn_from_grid(gbfwn_handle h, const int32_t dims[3], const float xf[12], float beta, float* out,
                              gbfwn_progress_cb cb, void* user);
GBFWN_API int gbfwn_from_grid_dev(gbfwn_handle h, const int32_t dims[3], const float xf[12], float beta, float* d_out,
                                  void* stream);

/* IFastWindingNumber::calcFromGridWithDistances (MRMesh/MRFastWindingNumber.h:44;
 * MRMesh/MRFastWindingNumber.cpp:69-94; MRCuda/MRCudaFastWindingNumber.cpp:230-283): distance to the
 * mesh with the winding-number sign (negative where the winding number > threshold); NaN where the
 * squared distance is outside [minDistSq, maxDistSq) and nullOutsideMinMax is set. */
GBFWN_API int gbfwn_from_grid_with_distances(gbfwn_handle h, const int32_t dims[3], const float xf[12],
                                             const gbfwn_dist_opts* opts, float* out, gbfwn_progress_cb cb, void* user);
GBFWN_API int gbfwn_from_grid_with_distances_dev(gbfwn_handle h, const int32_t dims[3], const float xf[12],
                                                 const gbfwn_dist_opts* opts, float* d_out, void* stream);

/* One z-slab of a grid: layers [z0, z1) of the dims grid (voxel centres exactly as in the whole-grid
 * call), written to d_out as (z1 - z0) whole XY layers.  The unit a multi-GPU caller shards a grid by
 * (the slab of MRMesh/MRFastWindingNumber.h:96-106 by-parts calls, MRMesh/MRChunkIterator.h:44-47);
 * slabs computed separately and stacked equal the whole grid bit for bit. */
GBFWN_API int gbfwn_from_grid_slab_dev(gbfwn_handle h, const int32_t dims[3], const float xf[12], float beta, int32_t z0,
                                       int32_t z1, float* d_out, void* stream);
GBFWN_API int gbfwn_from_grid_with_distances_slab_dev(gbfwn_handle h, const int32_t dims[3], const float xf[12],
                                                      const gbfwn_dist_opts* opts, int32_t z0, int32_t z1, float* d_out,
                                                      void* stream);

/* No counterpart in the reference.  Allocation-free variant of gbfwn_from_grid_with_distances_dev for
 * callers that may not call cudaMalloc/cudaFree when they need a grid -- a host application that
 * owns the device-memory budget and gives plugins preallocated buffers only, or a latency-bound loop
 * that cannot take cudaFree's implicit device synchronisation.  Create the handle beforehand (that
 * allocates); this call then allocates nothing: the output is the caller's device buffer and the
 * kernel's scratch (work-queue counter + status word) is a fixed 256-byte device array that every
 * GPU loading the library keeps until exit.  Each call looks up that array's device address
 * (cudaGetSymbolAddress, a host-side query); the first call on a device may also load the library's
 * device code there, so make that first call before any stream capture.  Every
 * call shares the array and clears it first, so calls that overlap on the GPU (concurrent streams,
 * threads or handles) race: serialise them.  Limit: at most 2^32-1 warp tiles of 4x4x2 voxels per
 * call (the counter is 32 bits); larger grids are rejected with GBFWN_INVALID.  Enqueues on
 * `stream` (NULL = the handle's stream) and returns without waiting; like the other `_dev` calls it
 * does not read the status word back (see the note on traversal status above). */
GBFWN_API int gbfwn_from_grid_with_distances_noalloc(gbfwn_handle h, const int32_t dims[3], const float xf[12],
                                                     const gbfwn_dist_opts* opts, float* d_out, void* stream);

/* MR::FastWindingNumber::calcWithDistances at arbitrary points (MRMesh/MRFastWindingNumber.h:62; the CPU
 * class has it, the interface does not). */
GBFWN_API int gbfwn_vector_with_distances(gbfwn_handle h, const float* pts, int64_t n, const gbfwn_dist_opts* opts,
                                          float* out, gbfwn_progress_cb cb, void* user);
GBFWN_API int gbfwn_vector_with_distances_dev(gbfwn_handle h, const float* d_pts, int64_t n,
                                              const gbfwn_dist_opts* opts, float* d_out, void* stream);

/* ---------------------------------------------------------------------------------------------
 * Points-to-mesh projection, MR::IPointsToMeshProjector::findProjections
 * (MRMesh/MRPointsToMeshProjector.h:11-30; CPU MRMesh/MRPointsToMeshProjector.cpp:17-32 over
 * MRMesh/MRMeshProject.cpp:13-104; GPU MRCuda/MRCudaPointsToMeshProjector.cpp:53-126).
 * One record per point, the memory layout of MR::MeshProjectionResult (MRMesh/MRMeshProject.h:17-31):
 * the closest point on the mesh, its face (-1 when nothing lies closer than sqrt(upDistLimitSq)),
 * its barycentric coordinates in that face's vertex order (point = (1-a-b) v0 + a v1 + b v2) and
 * the squared distance.  `edge` is always -1: the caller's half-edge topology supplies
 * edgeWithLeft(face), as the reference's GPU class does on the host (.cpp:117-123). */
typedef struct gbfwn_projection {
    int32_t face;
    float point[3];
    int32_t edge;
    float bary[2];
    float distSq;
} gbfwn_projection;

/* Projects n points (3 floats each).  objXf (12 floats, may be NULL) maps the points, refXf (may be
 * NULL) maps the mesh; a rigid refXf is folded into the point map and a non-rigid one is applied to
 * the mesh on the fly (MRMesh/MRMeshProject.cpp:105-121).  The search stops early for a point once a
 * triangle within sqrt(loDistLimitSq) is found. */
GBFWN_API int gbfwn_find_projections(gbfwn_handle h, const float* pts, int64_t n, const float* objXf, const float* refXf,
                                     float upDistLimitSq, float loDistLimitSq, gbfwn_projection* out,
                                     gbfwn_progress_cb cb, void* user);
GBFWN_API int gbfwn_find_projections_dev(gbfwn_handle h, const float* d_pts, int64_t n, const float* objXf,
                                         const float* refXf, float upDistLimitSq, float loDistLimitSq,
                                         gbfwn_projection* d_out, void* stream);
/* IPointsToMeshProjector::projectionsHeapBytes: device bytes a call on n points needs beyond the mesh. */
GBFWN_API size_t gbfwn_projections_heap_bytes(int64_t n);

/* IFastWindingNumberByParts::calcFromGridByParts / calcFromGridWithDistancesByParts
 * (MRMesh/MRFastWindingNumber.h:96-106; MRCuda/MRCudaFastWindingNumber.cpp:285-431): the grid is
 * produced in z-slabs of whole XY layers, consecutive slabs overlapping by `layerOverlap` layers,
 * and handed to `slab` in order while the GPU computes the next slab.  `maxLayersPerSlab` <= 0
 * picks the slab height from free device memory. */
GBFWN_API int gbfwn_from_grid_by_parts(gbfwn_handle h, const int32_t dims[3], const float xf[12], float beta,
                                       int32_t layerOverlap, int32_t maxLayersPerSlab, gbfwn_slab_cb slab,
                                       void* slabUser, gbfwn_progress_cb cb, void* user);
GBFWN_API int gbfwn_from_grid_with_distances_by_parts(gbfwn_handle h, const int32_t dims[3], const float xf[12],
                                                      const gbfwn_dist_opts* opts, int32_t layerOverlap,
                                                      int32_t maxLayersPerSlab, gbfwn_slab_cb slab, void* slabUser,
                                                      gbfwn_progress_cb cb, void* user);

/* GPU memory estimators, MR::CudaAccessor::fastWindingNumberMeshMemory / fromGridMemory /
 * fromVectorMemory / selfIntersectionsMemory (MRViewer/MRCudaAccessor.cpp:162-194). */
GBFWN_API size_t gbfwn_mesh_memory(int64_t nv, int64_t nt);
GBFWN_API size_t gbfwn_from_grid_memory(int64_t nv, int64_t nt, const int32_t dims[3]);
GBFWN_API size_t gbfwn_from_vector_memory(int64_t nv, int64_t nt, int64_t npts);
GBFWN_API size_t gbfwn_self_intersections_memory(int64_t nv, int64_t nt);

/* ---------------------------------------------------------------------------------------------
 * Learned band culling (no counterpart in the reference).  A small per-mesh network predicts the
 * signed distance; bricks of 8x8x8 voxels whose predicted |d|, less a validated error margin and
 * less the brick's half diagonal, is still >= the band are known to be NaN and are skipped; every
 * other voxel goes through the exact traversal, so the result is the reference's banded result
 * (maxDistSq = band^2, nullOutsideMinMax) wherever the margin holds.  The margin bounds how far the
 * prediction overstates |d|, measured on held-out samples with |d| below a limit that covers every
 * brick centre able to hold an in-band voxel (the only error that can make a cull wrong); a banded
 * call whose band plus brick half diagonal exceeds that limit uses the two-sided margin instead.  Network: Fourier features
 * of the point (32 frequencies x 3 axes x sin/cos = 192) -> 4 x 128 SiLU -> 1; BF16 weights and
 * activations on the tcgen05 tensor cores, FP32 accumulation; trained on the GPU on samples whose
 * targets come from the exact traversal (half uniform in the grid box, half near the surface). */
typedef struct gbfwn_surrogate_s* gbfwn_surrogate;

typedef struct gbfwn_surrogate_opts {
    int64_t samples;     /* training samples (2,000,000) */
    int64_t validation;  /* held-out samples that set the error margin (1,000,000) */
    int32_t steps;       /* optimizer steps (3000) */
    int32_t batch;       /* rows per step (16384) */
    float learningRate;  /* peak Adam step size, cosine decay to 1/100 (2e-3) */
    float band;          /* distance band the network serves, world units (required, > 0) */
    float beta;          /* winding-number beta of the exact targets (2) */
    uint64_t seed;
} gbfwn_surrogate_opts;

typedef struct gbfwn_surrogate_stats {
    float trainLoss;           /* last mean squared error (targets clamped to +-6 band) */
    float validationMaxError;  /* max |prediction - clamped target| on the held-out samples */
    float margin;              /* culling margin: 1.25 x validationOverestimate + 0.001 band */
    float sampleSeconds;       /* sample generation + exact targets */
    float trainSeconds;        /* optimizer steps */
    int32_t steps;
    float validationOverestimate; /* max (|prediction| - |d|) over held-out samples with |d| < limit */
    float limit;               /* band + twice the half diagonal of the training grid's 8x8x8 bricks */
} gbfwn_surrogate_stats;

typedef struct gbfwn_banded_stats {
    int32_t bricks, keptBricks;  /* 8x8x8-voxel bricks in the grid / sent to the exact traversal */
    float cullMs, exactMs;       /* time of the culling pass and of the exact pass */
} gbfwn_banded_stats;

GBFWN_API void gbfwn_surrogate_default_opts(gbfwn_surrogate_opts* opts);

/* Trains a network for the grid (dims, xf): its box is the sampling box. */
GBFWN_API int gbfwn_surrogate_train(gbfwn_handle h, const int32_t dims[3], const float xf[12],
                                    const gbfwn_surrogate_opts* opts, gbfwn_surrogate* out, gbfwn_surrogate_stats* stats);
GBFWN_API int gbfwn_surrogate_destroy(gbfwn_surrogate s);

/* Parameters (74,369 floats: W1[128x192] b1 W2[128x128] b2 W3 b3 W4 b4 w5[128] b5) and 48 floats of
 * metadata (input centre xyz, input scale, 32 frequencies, target clamp, culling margin, band, limit,
 * two-sided margin, 7 reserved), so that a trained network can be stored and re-created without
 * retraining. */
GBFWN_API int gbfwn_surrogate_get(gbfwn_surrogate s, float* params, float* meta);
GBFWN_API int gbfwn_surrogate_create(int device, const float* params, const float* meta, gbfwn_surrogate* out);

/* Network prediction at n points (device pointers). */
GBFWN_API int gbfwn_surrogate_eval_dev(gbfwn_surrogate s, const float* d_pts, int64_t n, float* d_out, void* stream);

/* Loss and parameter gradients (host, 74,369 floats, same layout as the parameters) of the mean
 * squared error against clamped targets on n <= 16384 points (device pointers); no update.  For
 * checking the backward kernels against a CPU reference. */
GBFWN_API int gbfwn_surrogate_gradients_dev(gbfwn_surrogate s, const float* d_pts, const float* d_targets, int32_t n,
                                            float* grads, float* loss);

/* Banded calcFromGridWithDistances: opts must have a finite maxDistSq (the band squared) and
 * nullOutsideMinMax set.  s = NULL culls bricks with the exact unsigned distance at brick centres
 * instead of the network (same result, no learned part).  Writes every voxel of d_out. */
GBFWN_API int gbfwn_from_grid_with_distances_banded_dev(gbfwn_handle h, gbfwn_surrogate s, const int32_t dims[3],
                                                        const float xf[12], const gbfwn_dist_opts* opts, float* d_out,
                                                        gbfwn_banded_stats* stats, void* stream);

/* ---------------------------------------------------------------------------------------------
 * Batched signed-distance grids (no counterpart in the reference, which handles one mesh per
 * call): many meshes, each with its own grid, options and device output, computed by ONE
 * persistent kernel fed from a single work queue.  Grids are queued most expensive first (voxels x
 * log2 triangles) so that uneven batches balance.  Twelve kernel variants (voxel-tile shape x block
 * size, each with a one-voxel and a paired walk; the paired ones run as their one-voxel counterparts
 * when an item has minDistSq > 0) can be timed on the batch and the fastest kept; a batch can be
 * replayed from a CUDA graph. */
typedef struct gbfwn_batch_s* gbfwn_batch;

/* A batch keeps device pointers into every item's mesh and output: each item's handle and d_out must
 * stay alive and unmoved until gbfwn_batch_destroy (also for graph replays and autotuning).  The
 * library enforces the handle part -- gbfwn_destroy refuses a handle that a live batch references --
 * while the output buffers are the caller's to keep. */
typedef struct gbfwn_batch_item {
    gbfwn_handle mesh;      /* all meshes of a batch on one device; the first mesh's precise setting applies */
    int32_t dims[3];
    float xf[12];
    gbfwn_dist_opts opts;
    float* d_out;           /* dims[0] * dims[1] * dims[2] floats, device memory */
} gbfwn_batch_item;

GBFWN_API int gbfwn_batch_create(const gbfwn_batch_item* items, int32_t n, gbfwn_batch* out);
GBFWN_API int gbfwn_batch_destroy(gbfwn_batch b);
GBFWN_API int32_t gbfwn_batch_num_configs(void);
GBFWN_API const char* gbfwn_batch_config_name(int32_t config);
GBFWN_API int gbfwn_batch_set_config(gbfwn_batch b, int32_t config);
/* Times every variant on the batch (three runs each, best of the last two) and keeps the fastest;
 * times_ms (may be NULL) receives gbfwn_batch_num_configs() values. */
GBFWN_API int gbfwn_batch_autotune(gbfwn_batch b, int32_t* best, float* times_ms);
/* Enqueues the batch on `stream` (plain launch, or the CUDA graph captured on first use). */
GBFWN_API int gbfwn_batch_run_dev(gbfwn_batch b, void* stream);
GBFWN_API int gbfwn_batch_graph_launch(gbfwn_batch b, void* stream);

/* makeSignedByWindingNumber (MRVoxels/MRVDBConversions.cpp:491-571) on a dense device grid: the
 * winding number of every voxel (centre = xf applied to (x, y, z), as for gbfwn_from_grid) is computed
 * and each value whose voxel's winding number exceeds `threshold` is negated in place (on closed
 * meshes with a vertical grid z axis from the columns' crossings, see gbfwn_set_sign_reuse; the
 * handle's work buffer grows by 72 bytes per grid column for them).  MeshLib's VDB path reaches the
 * same computation through IFastWindingNumberByParts::calcFromGridByParts; this is for grids that
 * already live in device memory.  Enqueued on `stream` (NULL = the handle's). */
GBFWN_API int gbfwn_make_signed_by_winding_number_dev(gbfwn_handle h, const int32_t dims[3], const float xf[12],
                                                      float beta, float threshold, float* d_values, void* stream);

/* ---------------------------------------------------------------------------------------------
 * Marching cubes: the mesher that consumes the signed-distance grid in MeshLib's offsetting
 * (mcOffsetMesh, MRVoxels/MROffset.cpp:185-226).  Output = the reference's TriMesh bit for bit
 * (same points in the same order, same triangles, same faceMap) of
 *   marchingCubes(SimpleVolume, MarchingCubesParams)       MRVoxels/MRMarchingCubes.h:65-67
 *   MarchingCubesByParts::addPart ... finalize()           MRVoxels/MRMarchingCubes.h:96-122
 * for the default linear positioner.  The volume is x-fastest (MRMesh/MRVolumeIndexer.h:131-139).
 * The mesh stays on the device until copied out. */

/* MR::MarchingCubesParams (MRVoxels/MRMarchingCubes.h:18-61): origin, iso, lessInside, maxVertices;
 * wantFaceMap = outVoxelPerFaceMap requested.  voxelSize is the volume's (SimpleVolume::voxelSize).
 * A mesh with more than maxVertices vertices is an error, as in the reference (start from
 * gbfwn_mc_default_params: a zeroed struct allows no vertex).  Defaults: origin 0, voxelSize 1,
 * iso 0, lessInside 0, maxVertices INT32_MAX, wantFaceMap 0. */
typedef struct gbfwn_mc_params {
    float origin[3];
    float voxelSize[3];
    float iso;
    int32_t lessInside;
    int64_t maxVertices;
    int32_t wantFaceMap;
} gbfwn_mc_params;

typedef struct gbfwn_trimesh_s* gbfwn_trimesh;

GBFWN_API void gbfwn_mc_default_params(gbfwn_mc_params* p);

/* marchingCubes(SimpleVolume) with the volume in host memory (synchronous).  partStarts / nParts:
 * optional first layers of the overlapping parts a MarchingCubesByParts call sequence would add
 * (the last layer of a part is the first of the next); they only change the rounding of the z
 * coordinates, as in the reference.  nParts = 0: the whole volume at once.  Errors (the reference's
 * Expected strings): a part with fewer than two layers, parts beyond the volume, more vertices than
 * maxVertices ("Vertices number limit exceeded.").  A volume with a non-positive dimension gives an
 * empty mesh. */
GBFWN_API int gbfwn_marching_cubes(const float* volume, const int32_t dims[3], const gbfwn_mc_params* params,
                                   const int32_t* partStarts, int32_t nParts, int device, gbfwn_trimesh* out,
                                   gbfwn_progress_cb cb, void* user);
/* The same on a device volume; enqueued on `stream` (no handle here: NULL = the legacy default
 * stream), returns once the mesh is built. */
GBFWN_API int gbfwn_marching_cubes_dev(const float* d_volume, const int32_t dims[3], const gbfwn_mc_params* params,
                                       const int32_t* partStarts, int32_t nParts, int device, gbfwn_trimesh* out,
                                       void* stream);
/* Device bytes a mesher call needs (MRCuda/MRCudaAccessor.cpp:162-194 gives such estimators for the
 * reference's GPU calls): work arrays (about 3 bytes per voxel) plus the output and the cell list for
 * `expectedTriangles` triangles; the host-volume call adds 4 bytes per voxel for the volume. */
GBFWN_API size_t gbfwn_marching_cubes_memory(const int32_t dims[3], int64_t expectedTriangles);
/* The mesher keeps its work arrays on the device between calls; this frees them. */
GBFWN_API int gbfwn_mc_release_workspace(int device);
GBFWN_API int gbfwn_trimesh_sizes(gbfwn_trimesh m, int64_t* numPoints, int64_t* numTris);
/* Copies the mesh to host arrays (points: 3 floats per vertex; tris: 3 vertex ids per triangle;
 * faceMap: voxel id of each triangle's cell, only if requested).  Any pointer may be NULL. */
GBFWN_API int gbfwn_trimesh_copy(gbfwn_trimesh m, float* points, int32_t* tris, int32_t* faceMap);
/* Device arrays of the mesh (owned by it). */
GBFWN_API int gbfwn_trimesh_device(gbfwn_trimesh m, const float** d_points, const int32_t** d_tris,
                                   const int32_t** d_faceMap);
GBFWN_API int gbfwn_trimesh_destroy(gbfwn_trimesh m);

/* MR::MarchingCubesByParts (MRVoxels/MRMarchingCubes.h:96-122): parts of whole XY layers added in
 * z order, each starting at nextZ() (the previous part's last layer repeated); finalize() builds the
 * mesh ("Provided parts do not cover whole volume" when the parts stop short).  The parts are
 * gathered into one device volume, so a repeated layer takes the values of the later part. */
typedef struct gbfwn_mc_parts_s* gbfwn_mc_parts;
GBFWN_API int gbfwn_mc_parts_create(const int32_t dims[3], const gbfwn_mc_params* params, int device,
                                    gbfwn_mc_parts* out);
GBFWN_API int32_t gbfwn_mc_parts_next_z(gbfwn_mc_parts p);
/* part: host (or, for _dev, device) volume of partDims[0] x partDims[1] x partDims[2] voxels. */
GBFWN_API int gbfwn_mc_parts_add(gbfwn_mc_parts p, const float* part, const int32_t partDims[3]);
GBFWN_API int gbfwn_mc_parts_add_dev(gbfwn_mc_parts p, const float* d_part, const int32_t partDims[3], void* stream);
GBFWN_API int gbfwn_mc_parts_finalize(gbfwn_mc_parts p, gbfwn_trimesh* out);
GBFWN_API int gbfwn_mc_parts_destroy(gbfwn_mc_parts p);

/* mcOffsetMesh's volume step fused on the device (no counterpart in the reference, which copies
 * the distance grid to the host slab by slab and meshes it there): the signed-distance grid of
 * `dims` voxels with centres at origin + (i + 0.5) * voxelSize (the basis of MROffset.cpp:201) is
 * computed into device memory with `opts` (banded with brick culling when maxDistSq is finite and
 * nullOutsideMinMax is set; s = the optional surrogate), then meshed with `mc` (mcOffsetMesh passes
 * origin, iso = offset, lessInside = 1) and optional partStarts; the grid never leaves the device. */
GBFWN_API int gbfwn_grid_to_mesh(gbfwn_handle h, gbfwn_surrogate s, const int32_t dims[3], const float origin[3],
                                 const float voxelSize[3], const gbfwn_dist_opts* opts, const gbfwn_mc_params* mc,
                                 const int32_t* partStarts, int32_t nParts, gbfwn_trimesh* out, gbfwn_progress_cb cb,
                                 void* user);

/* Diagnostic (no counterpart in the reference): D[m x n] (+)= A[m x k] * B[n x k]^T on the tcgen05 tensor
 * cores, bf16 inputs (row-major, k contiguous), FP32 output (row-major); m % 128 == 0, n in {128, 192},
 * k % 64 == 0; with split_k > 1 the output is accumulated atomically (zero it first).  Device pointers,
 * enqueued on `stream`.  Used by the tests of the surrogate network's GEMM. */
/* No counterpart in the reference: exercises the tensor-core kernels' timeout path -- one warp
 * allocates TMEM, waits at most maxPolls polls on an mbarrier that nothing arrives on, records the
 * timeout and frees its TMEM.  Returns GBFWN_TIMEOUT (the expected outcome) or an error; the device
 * stays usable.  Synchronous on `stream`. */
GBFWN_API int gbfwn_debug_wait_timeout(uint32_t maxPolls, void* stream);
GBFWN_API int gbfwn_debug_gemm_bf16(const void* d_a, const void* d_b, float* d_d, int32_t m, int32_t n, int32_t k,
                                    int32_t split_k, void* stream);

/* The library keeps device memory for reuse: staging buffers of freed handles (so creating a handle
 * per call, as MeshLib does, does not map a grid-sized buffer every time) and the mesher's work
 * arrays.  This returns all of it on `device` to the driver. */
GBFWN_API int gbfwn_release_cached_memory(int device);

/* Test hook: makes the next `count` device allocations of this thread fail with
 * GBFWN_OUT_OF_MEMORY (host-side fault injection; no device fault is involved). */
GBFWN_API void gbfwn_debug_fail_next_allocs(int count);

#ifdef __cplusplus
}
#endif

#endif /* GBFWN_H */
