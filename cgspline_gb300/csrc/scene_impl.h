// scene_impl.h -- host-side structures of libcgspline_gb300.so shared by
// scene.cu (store, BVH build, upload, perfect hash) and api.cu (queries,
// rendering, serving).
#pragma once

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <functional>
#include <initializer_list>
#include <mutex>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "../../include/cgspline.h"
#include "kernels.h"

namespace cgs {

// ------------------------------------------------------------- host BVH --
struct Box
{
    float lo[3] = {INFINITY, INFINITY, INFINITY};
    float hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    void inflate(const float p[3])
    {
        for (int k = 0; k < 3; k++) { lo[k] = std::min(lo[k], p[k]); hi[k] = std::max(hi[k], p[k]); }
    }
    void inflate(const Box& b) { inflate(b.lo); inflate(b.hi); }
};

struct Element { Box bounds; float centroid[3]; uint32_t index; };
struct Node { Box leftBox, rightBox; uint32_t left, right; };

// BVH::build / split / wrap (src/rt/BVH.cpp:9-108), see scene.cu.
struct HostBVH
{
    std::vector<Node> nodes;
    std::vector<uint32_t> keys, indices;
    uint32_t perNode = 1;
    int split_mode = CGS_SPLIT_REFERENCE;
    bool emptyLeaf = false;
    uint32_t wrap(Element* e, size_t count, uint32_t key);
    uint32_t split(Element* e, size_t count, uint32_t key);
    void build(std::vector<Element>& el);
};

struct Surface
{
    std::vector<float> points;   // 4 per point
    std::vector<uint32_t> indices;
    HostBVH bvh;
    uint32_t patchCount() const { return uint32_t(indices.size() / 16); }
};

struct Object
{
    uint32_t surface, group;
    float l2w[16], w2l[16];
    cgs_material material;
    std::vector<uint32_t> patchMaterial;
    std::vector<cgs_material> materials;
};

// A group is one scene of the store: its objects, its object-level BVH, its
// lights and environment (rt::Scene, src/rt/Scene.h:97-159).
struct Group
{
    std::vector<uint32_t> objects;  // global object ids
    std::vector<cgs_light> lights;
    float background[3] = {0.1f, 0.1f, 0.1f};
    float ambient[3] = {0.1f, 0.1f, 0.1f};
    HostBVH top;
    bool touched = false;  // objects, lights or environment were set
};

// Failure injection (cgs_debug_fail_allocation): growths left before the one
// that reports out of memory, 0 when off.
extern std::atomic<uint32_t> g_failAllocation;
inline bool injected_allocation_failure()
{
    uint32_t k = g_failAllocation.load(std::memory_order_relaxed);
    while (k != 0 && !g_failAllocation.compare_exchange_weak(k, k - 1, std::memory_order_relaxed)) {}
    return k == 1;
}

template<class T> struct DBuf
{
    T* p = nullptr;
    size_t n = 0;
    cudaError_t reserve(size_t count)
    {
        if (count <= n) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr; n = 0;
        if (injected_allocation_failure()) return cudaErrorMemoryAllocation;
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess) n = count;
        return e;
    }
    void release() { if (p) cudaFree(p); p = nullptr; n = 0; }
    size_t bytes() const { return n * sizeof(T); }
};

inline int cuda_status(cudaError_t e)
{
    if (e == cudaSuccess) return CGS_OK;
    if (e == cudaErrorMemoryAllocation) return CGS_ERR_OUT_OF_MEMORY;
    return CGS_ERR_CUDA;
}

#define CGS_TRY(expr)                                  \
    do {                                               \
        cudaError_t _e = (expr);                       \
        if (_e != cudaSuccess) return cuda_status(_e); \
    } while (0)

// Executable CUDA graphs of launch sequences, keyed by a hash of everything a
// sequence depends on (buffers, sizes, options).  A key runs eagerly the
// first time (one-time initialisation, occupancy queries), is captured on
// the second and replayed from then on.
struct GraphCache
{
    struct Entry { cudaGraphExec_t exec; int launches; };
    std::unordered_map<uint64_t, Entry> execs;
    std::unordered_set<uint64_t> seen;
    cudaStream_t capture = nullptr;
    bool disabled = false;
    uint64_t replays = 0, captures = 0;
    void release();
};

// FNV-1a over 64-bit words.
inline uint64_t key_of(std::initializer_list<uint64_t> words)
{
    uint64_t h = 1469598103934665603ull;
    for (uint64_t w : words)
        for (int k = 0; k < 8; k++) { h ^= (w >> (8 * k)) & 0xFF; h *= 1099511628211ull; }
    return h;
}
inline uint64_t key_of(const void* p) { return uint64_t(reinterpret_cast<uintptr_t>(p)); }
uint64_t scene_key(const DevScene& S);
uint64_t query_key(const Query& q);

// Runs fn(stream, &launches) -- a launch sequence -- through gc.
cudaError_t run_cached(GraphCache& gc, uint64_t key, cudaStream_t stream, int* launches,
                       const std::function<cudaError_t(cudaStream_t, int*)>& fn);

// Device buffers of one in-flight render batch (wavefront queues, engine
// scratch, request table, counters).  A scene owns one; the server owns one
// per concurrently running batch.
struct RenderSlot
{
    WavefrontBuffers wb {};
    DBuf<RenderBatch> batch;  // device copy of the batch description
    GraphCache graphs;
    DBuf<float> ray0, ray1, shadow, contrib, base, accum, hitF, hitF2;
    DBuf<uint32_t> smp0, smp1, grp0, grp1, dep0, dep1, count, shadowSlot, shadowGroup, engine, engine2;
    DBuf<int32_t> visible, hitI, hitI2, occluded;
    cudaStream_t side = nullptr;  // the shadow queries' stream, forked from and joined to the render's
    cudaEvent_t fork = nullptr, join = nullptr;
    DBuf<DevRequest> req;
    DBuf<Counters> counters;
    uint32_t engineCapacity = 0, engine2Capacity = 0;
    int ensure(uint32_t samples, uint32_t lights, uint32_t nreq);
    int ensure_engine(uint32_t rays);  // query-engine scratch for `rays` rays
    void release();
    uint64_t bytes() const;
    static uint64_t bytes_for(uint32_t samples, uint32_t lights);
};

}  // namespace cgs

struct cgs_scene
{
    int device = 0;
    std::mutex mu;
    std::vector<cgs::Surface> surfaces;
    std::vector<cgs::Object> objects;
    std::vector<cgs::Group> groups;
    uint32_t current = 0;  // group receiving add_object / set_lights / set_environment
    int splitMode = CGS_SPLIT_REFERENCE;
    bool bvhBuilt = false, uploaded = false, hashed = false;

    // device side
    cgs::DBuf<float4> patches, nodes;
    cgs::DBuf<uint4> qnodes;  // the compressed mirror of nodes (32 bytes per node)
    cgs::DBuf<uint32_t> indices, tables, disps, patchBase, patchMaterial, keys, groupTop;
    cgs::DBuf<uint2> groupLights;
    cgs::DBuf<float> groupEnv;
    cgs::DBuf<cgs::DevBVH> bvhs;
    cgs::DBuf<cgs::DevObject> dobjects;
    cgs::DBuf<cgs::DevMaterial> materials;
    cgs::DBuf<cgs::DevLight> dlights;
    std::vector<cgs::DevBVH> hbvh;
    std::vector<uint32_t> tableCap;  // per BVH
    cgs::DBuf<uint32_t> scratch32;
    cgs::DBuf<uint32_t> hashJobs;  // the batched hash build's job table and results
    cgs::DBuf<unsigned long long> scratch64;
    cgs::DBuf<cgs::Counters> counters;

    // query staging and engine scratch
    cgs::DBuf<float> rayStage, hitF;
    cgs::DBuf<int32_t> hitI;
    cgs::DBuf<uint32_t> groupStage, engine;
    uint32_t engineCapacity = 0;

    // rendering
    cgs::RenderSlot slot;
    cgs::DBuf<uint32_t> fbStage;
    cgs::DBuf<float> linStage;
    cudaEvent_t finished = nullptr;
    // queries share the counters and engine scratch: the last query's stream
    // and an event after its work, so that a query on another stream waits
    cudaEvent_t queryDone = nullptr;
    cudaStream_t queryStream = nullptr;
    bool queryIssued = false;
    std::mutex hostMu;  // held through a host-staged call (cgs_intersect_host, cgs_render_host)
    cudaStream_t lastStream = nullptr;
    cgs::Counters* lastCounters = nullptr;
    int launches = 0;

    cgs::DevScene dev() const;
    // bvhs: surfaces 0..S-1, then one object-level BVH per group
    const cgs::HostBVH& bvh(uint32_t which) const
    {
        return which < surfaces.size() ? surfaces[which].bvh : groups[which - surfaces.size()].top;
    }
    uint32_t nbvh() const { return uint32_t(surfaces.size() + groups.size()); }
    uint32_t maxLights() const
    {
        size_t m = 1;
        for (const auto& g : groups) m = std::max(m, g.lights.size());
        return uint32_t(m);
    }
    ~cgs_scene();
};

namespace cgs {

void camera_setup(const cgs_camera& c, uint32_t w, uint32_t h, int flip, CameraSetup& s);
int upload_store(cgs_scene* sc);
uint32_t table_capacity(uint32_t n);
uint32_t displ_size(uint32_t n);
void hash_coefficients(uint32_t n, uint32_t A[16], uint32_t B[16]);
int ensure_engine(cgs_scene* sc, uint32_t capacity);
inline bool valid_query(int method, int precision)
{
    return (method == 0 || method == 1) && precision >= 0 && precision <= 3;
}
// Fill `out` (device request table of `slot`) and the batch description for
// n requests; validates them.  Returns a status.
int prepare_batch(cgs_scene* sc, const cgs_render_request* reqs, uint32_t n, const cgs_render_options* opt,
                  std::vector<DevRequest>& host, RenderBatch& b);
int run_batch(cgs_scene* sc, RenderSlot& slot, const std::vector<DevRequest>& host, RenderBatch& b, int schedule,
              cudaStream_t stream, int* launches);
// The wavefront sequence of batch b (already uploaded to slot.batch, its
// request table to slot.req) through the slot's graph cache.
cudaError_t launch_wavefront_cached(const DevScene& S, RenderSlot& slot, const RenderBatch& b, cudaStream_t stream,
                                    int* launches);

}  // namespace cgs
