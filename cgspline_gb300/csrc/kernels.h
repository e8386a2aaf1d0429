// kernels.h -- host-side launchers of the CUDA kernels (one header for all
// translation units of libcgspline_gb300.so).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "device.cuh"

namespace cgs {

// Rays as structure of arrays; tmax null = +inf; group null = group 0.
struct RaysSoA { const float *ox, *oy, *oz, *dx, *dy, *dz, *tmax; const uint32_t* group; };
struct HitsSoA { float *t, *u, *v; int32_t *patch, *object; };

// ---------------------------------------------------------- ray queries --
// spline::doBezierClipping on explicit (ray, patch) pairs, one thread per pair;
// a patch id at or past `patches` (the surface's count) is a miss and raises
// error bit kErrPatchId.
cudaError_t launch_patch_pairs(const DevScene& S, uint32_t surface, uint32_t patches, RaysSoA rays,
                               const uint32_t* patch_ids, uint32_t n, Query q, HitsSoA hits, Counters* counters,
                               cudaStream_t stream);
// rt::normal (src/rt/Primitive.cu:270-275) at (u[k], v[k]) of patch patch_ids[k]:
// the unit normal in the surface's space, written as SoA nx | ny | nz (3 n
// floats); an id past the surface's count gives (0, 0, 0) and kErrPatchId.
cudaError_t launch_patch_normals(const DevScene& S, uint32_t surface, uint32_t patches, const uint32_t* patch_ids,
                                 const float* u, const float* v, uint32_t n, float* normals, Counters* counters,
                                 cudaStream_t stream);

// One thread per ray with the whole search inline (the plain query path);
// `group` applies where rays.group is null.  Any hit writes hits.patch only.
cudaError_t launch_query_plain(const DevScene& S, RaysSoA rays, uint32_t n, uint32_t group, Query q, bool any,
                               HitsSoA hits, Counters* counters, cudaStream_t stream);

// A query request's slice in a batch: rays [base, base + n) of the batch
// come from src[0..6] (ox oy oz dx dy dz tmax; tmax nullable) and their hits
// go to out (any-hit: out.patch only).
struct QueryChunk
{
    const float* src[7];
    uint32_t group, n, base, pad;
    HitsSoA out;
};
// hdr (device) = (chunks, total rays) of the batch; cap = the staging
// capacity (SoA stride, grid size).
cudaError_t launch_gather_rays(const QueryChunk* table, const uint32_t* hdr, uint32_t cap, float* rays,
                               uint32_t* group, cudaStream_t stream);
cudaError_t launch_scatter_hits(const QueryChunk* table, const uint32_t* hdr, uint32_t cap, HitsSoA hits, bool any,
                                cudaStream_t stream);

// The pure-FP64 closest-hit search (precision 2), one thread per ray: n rays
// (or *nDev, with n bounding the grid), FP64 clip tolerance `tol`.
constexpr double kTolFP64 = 1e-9;
cudaError_t launch_query_fp64(const DevScene& S, RaysSoA rays, uint32_t n, const uint32_t* nDev, double tol,
                              HitsSoA hits, Counters* counters, cudaStream_t stream);

// ---------------------------------------------------------- query engine --
// Closest / any hit of n rays (n from the host, or *nDev when nDev != null;
// capacity bounds both) by alternating traversal and clip passes
// (k_engine.cu).  scratch holds engine_words(capacity, passes) words.
size_t engine_words(uint32_t capacity, int passes);
cudaError_t run_query(const DevScene& S, RaysSoA rays, uint32_t n, const uint32_t* nDev, Query q, bool any,
                      HitsSoA hits, int32_t* occluded, uint32_t* scratch, uint32_t capacity, int passes,
                      Counters* counters, cudaStream_t stream, int* launches);
// The first collect pass of run_query alone (no clipping): each ray's
// candidate list of that pass, its length copied to listLengths (device, may
// be null).  For timing and profiling the traversal kernel.
cudaError_t run_traverse(const DevScene& S, RaysSoA rays, uint32_t n, bool any, uint32_t* scratch, uint32_t capacity,
                         Counters* cnt, cudaStream_t stream, uint32_t* listLengths, int* launches);
constexpr int kEnginePasses = 12;

// Runtime settings of the query engine: collect / resolve passes before the
// inline fallback, block sizes (collect 128 or 256, resolve 64 or 128) and
// resident blocks per SM (0 = as many as fit).  Process-wide; a change bumps
// the generation, which keys the captured CUDA graphs.
struct EngineConfig
{
    int passes = 2;
    int collectThreads = 256;
    int resolveThreads = 128;
    int collectOccupancy = 0;
    int resolveOccupancy = 0;
    int backtrackCache = 1;  // 1: backtracks read postponed siblings from a per-lane ring first
    int compressedNodes = 0; // 1: the traversal reads the 32-byte compressed node mirror
    int queueChunk = 64;     // candidate-list entries a ray may fill in the first pass (4..64, multiple of 4);
                             // each later pass doubles it, up to 64
    int packetWidth = 8;     // the traversal refills a warp once this many lanes are idle (1..32)
    int rayOrder = 1;        // primary rays of a render: 0 in scanline order, 1 in 8 x 4 pixel tiles
    int originLast = 0;      // any hit: 1 searches the candidates whose leaf box holds the origin last
    int subdivLevels = 4;    // subdivision searches: bisection levels a lane runs per resolve round (1..64)
};
EngineConfig engine_config();
bool set_engine_config(const EngineConfig& c);
bool valid_engine_config(const EngineConfig& c);
uint64_t engine_config_generation();

// --------------------------------------------------------------- render --
struct CameraSetup
{
    float c2w[16];   // camera to world, column-major
    float pos[3];
    float tl[2];     // top-left corner of the image plane at z = -1
    float half_dx, half_dy;
};

// One render request of a batch: rows [row0, row0 + height) of an image
// whose camera set-up is `cam` (a request may be split into row chunks).  Its
// samples are the global sample indices [sampleBase, sampleBase +
// width*height*spp); its pixels [pixelBase, pixelBase + width*height).  fb and
// linear point at the chunk's first row.
struct DevRequest
{
    CameraSetup cam;
    uint32_t group, width, height, spp;
    int depth;
    uint32_t sampleBase, pixelBase, stride, row0;
    uint32_t* fb;
    float* linear;
};

struct RenderBatch
{
    const DevRequest* req;   // device
    uint32_t nreq;
    uint32_t samples;        // total samples (primary rays)
    uint32_t pixels;         // total output pixels
    int maxDepth;
    float eps;
    Query q;
    int sampling;            // 0: mirror bounce (reference default); 1: Monte-Carlo microfacet bounce
};

// Work buffers of the wavefront schedule (device memory, sized for `capacity` samples).
struct WavefrontBuffers
{
    // ray queues (two, ping-pong): 9 floats per ray SoA (ox oy oz dx dy dz ax ay az)
    float* ray[2];
    uint32_t* sample[2];  // the primary sample each ray belongs to
    uint32_t* group[2];
    uint32_t* depth[2];   // bounces still allowed
    uint32_t* count;      // [0..1] queue sizes, [2] shadow count
    HitsSoA hit[2];       // per ray of the queue of an even / odd bounce level
    int32_t* occluded;    // per shadow ray
    uint32_t* engine;     // query-engine scratch of the closest-hit queries
    uint32_t* engine2;    // ... of the shadow queries, which run beside the next level's closest query
    uint32_t engineCapacity, engine2Capacity;
    cudaStream_t side;    // the shadow queries' stream (null: one stream for everything)
    cudaEvent_t fork, join;
    float* shadow;        // 7 floats per shadow ray SoA: ox oy oz dx dy dz max
    uint32_t* shadowGroup;
    uint32_t* shadowSlot; // (ray index * lightCapacity + light) of each shadow ray
    float* contrib;       // 3 floats per (ray, light) slot
    int32_t* visible;     // per (ray, light) slot: 1 = lit, 0 = not
    float* base;          // 3 floats per ray: the ambient term
    float* accum;         // 3 floats per sample
    uint32_t capacity;    // rays
    uint32_t lightCapacity;
};

// Primary rays (one per pixel centre) of a w x h image, SoA (7, w*h), tmax = inf.
cudaError_t launch_camera_rays(const CameraSetup& cam, uint32_t w, uint32_t h, float* rays, cudaStream_t stream);
cudaError_t launch_render_plain(const DevScene& S, const RenderBatch& b, const DevRequest* hostReq,
                                Counters* counters, cudaStream_t stream, int* launches);
// The wavefront schedule of batch b.  The kernels read the batch from bDev
// (a device copy of b, uploaded by the caller), so that the launch sequence
// depends only on the buffers, b.maxDepth, b.eps and b.q and can be replayed
// from a captured CUDA graph for any batch of that shape.
cudaError_t launch_render_wavefront(const DevScene& S, const RenderBatch& b, const RenderBatch* bDev,
                                    const WavefrontBuffers& wb, Counters* counters, cudaStream_t stream, int* launches);

// ---------------------------------------------------------- perfect hash --
struct HashScratch
{
    uint32_t* bsize;      // [displSize]
    uint32_t* bkeys;      // [4 * displSize]
    uint32_t* rank;       // [displSize]
    uint32_t* dcur;       // [displSize]
    uint32_t* state;      // [displSize]: bit0 active, bit1 feasible
    uint32_t* slots;      // [4 * displSize]
    uint32_t* occ;        // [ceil(Nmax/32)]
    unsigned long long* owner;  // [Nmax]
    uint32_t* blockCounts;      // [2 * rankBlocks] packed class counts
    uint32_t* misc;       // [16]: 0 error bits, 1..4 class counts, 5..8 class remaining, 9 failures
};

// Sizes of the scratch for n keys (in 4-byte words, owner in 8-byte words).
void hash_scratch_words(uint32_t n, size_t& words32, size_t& words64);
void hash_scratch_carve(HashScratch& s, uint32_t n, uint32_t* base32, unsigned long long* base64);

// One BVH's build in a batch (hash_build_blocks): its keys at
// keys[keyOff..keyOff+n), displacements written at disps[dispOff..+mask+1),
// table at tables[tableOff..+tableCap), the 16 trials' coefficients; a
// BVH above kHashBlockMaxKeys keys works in gscratch[scratchOff..+
// hash_block_scratch_words(n)).
struct HashJob
{
    uint32_t keyOff, n, dispOff, tableOff, tableCap, mask, scratchOff, pad;
    uint32_t A[16], B[16];
};
constexpr uint32_t kHashBlockMaxKeys = 8192;          // one CTA, scratch in shared memory
constexpr uint32_t kHashGlobalBlockMaxKeys = 131072;  // one CTA, scratch in global memory
// Dynamic shared memory of the CTA that builds a BVH of maxKeys keys.
size_t hash_block_smem(uint32_t maxKeys);
// Global scratch words of the CTA that builds a BVH of n keys (above kHashBlockMaxKeys).
uint64_t hash_block_scratch_words(uint32_t n);
// Builds every job's table, one CTA each, in one launch (asynchronous):
// all jobs at most kHashBlockMaxKeys keys (shared-memory scratch), or all in
// (kHashBlockMaxKeys, kHashGlobalBlockMaxKeys] with gscratch.  out[8 j ..]:
// status (0 ok, 3 no trial found a table, 4 bucket overflow, 5 duplicate
// slot), A, B, N, mask, trial -- the values hash_build_device returns.
cudaError_t hash_build_blocks(const uint32_t* keys, const HashJob* jobs, uint32_t njobs, uint32_t maxKeys,
                              uint32_t* disps, uint32_t* tables, uint32_t* out, cudaStream_t stream,
                              uint32_t* gscratch = nullptr);

// Deterministic perfect hash of keys[0..n).  A[], B[] are the 16 trials'
// coefficients, drawn on the host.  Writes disp[displSize] and
// table[N] (table[h(key_i)] = i); returns the trial used (0..15) in params,
// or an error code.  Synchronises the stream once per trial.
int hash_build_device(const uint32_t* keys, uint32_t n, const uint32_t A[16], const uint32_t B[16],
                      uint32_t* disp, uint32_t* table, uint32_t tableCapacity, HashScratch& scratch,
                      uint32_t params[5], cudaStream_t stream, int* launches);

}  // namespace cgs
