// k_query.cu -- ray-query kernels: closest hit, any hit, explicit (ray, patch) pairs.
#include "kernels.h"

namespace cgs {

namespace {

__device__ __forceinline__ void load_ray(const RaysSoA& r, uint32_t i, float3& o, float3& d, float& tmax)
{
    o = f3(__ldg(r.ox + i), __ldg(r.oy + i), __ldg(r.oz + i));
    d = f3(__ldg(r.dx + i), __ldg(r.dy + i), __ldg(r.dz + i));
    tmax = __ldg(r.tmax + i);
}

constexpr int kQueryThreads = 128;

// Persistent: each warp takes the next 32 rays until n; one thread per ray.
template<bool kAny>
__global__ void __launch_bounds__(kQueryThreads) k_query(DevScene S, RaysSoA rays, uint32_t n, Query q, HitsSoA hits,
                                                         int32_t* occluded, uint32_t* next, Counters* cnt)
{
    LocalCounters lc;
    uint32_t nrays = 0;
    for (;;)
    {
        uint32_t base = 0;
        if (lane_id() == 0) base = atomicAdd(next, 32u);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= n) break;
        const uint32_t i = base + lane_id();
        if (i < n)
        {
            float3 o, d; float tmax;
            load_ray(rays, i, o, d, tmax);
            nrays++;
            if (kAny)
                occluded[i] = scene_any(S, o, d, tmax, q, lc) ? 0 : -1;
            else
            {
                HitRecord h {tmax, 0.0f, 0.0f, -1, -1};
                int ob = scene_closest(S, o, d, tmax, q, h, lc);
                hits.t[i] = ob >= 0 ? h.t : tmax;
                hits.u[i] = h.u;
                hits.v[i] = h.v;
                hits.patch[i] = ob >= 0 ? h.patch : -1;
                hits.object[i] = ob;
            }
        }
    }
    flush_counters(cnt, lc, nrays);
}

__global__ void __launch_bounds__(kQueryThreads) k_patch_pairs(DevScene S, uint32_t surface, RaysSoA rays,
                                                               const uint32_t* __restrict__ pids, uint32_t n, Query q,
                                                               HitsSoA hits, Counters* cnt)
{
    LocalCounters lc;
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        float3 o, d; float tmax;
        load_ray(rays, i, o, d, tmax);
        const float4* P = S.patches + 16ull * (__ldg(S.patchBase + surface) + __ldg(pids + i));
        HitSink sink {P, o, d, hits.t[i], make_float2(0.0f, 0.0f)};
        bool b = search_patch(sink, q, lc);
        if (b) { hits.t[i] = sink.dist; hits.u[i] = sink.uv.x; hits.v[i] = sink.uv.y; }
        hits.patch[i] = b ? 1 : 0;
    }
    flush_counters(cnt, lc, i < n ? 1u : 0u);
}

int persistent_blocks(const void* fn, int threads)
{
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, threads, 0);
    return sms * (per > 0 ? per : 1);
}

}  // namespace

cudaError_t launch_closest(const DevScene& S, RaysSoA rays, uint32_t n, Query q, HitsSoA hits, uint32_t* next,
                           Counters* counters, cudaStream_t stream)
{
    static int blocks = 0;
    if (!blocks) blocks = persistent_blocks((const void*)k_query<false>, kQueryThreads);
    cudaMemsetAsync(next, 0, sizeof(uint32_t), stream);
    uint32_t need = (n + 31) / 32 * 32 / kQueryThreads + 1;
    int grid = int(need < uint32_t(blocks) ? need : uint32_t(blocks));
    k_query<false><<<grid, kQueryThreads, 0, stream>>>(S, rays, n, q, hits, nullptr, next, counters);
    return cudaGetLastError();
}

cudaError_t launch_any(const DevScene& S, RaysSoA rays, uint32_t n, Query q, int32_t* occluded, uint32_t* next,
                       Counters* counters, cudaStream_t stream)
{
    static int blocks = 0;
    if (!blocks) blocks = persistent_blocks((const void*)k_query<true>, kQueryThreads);
    cudaMemsetAsync(next, 0, sizeof(uint32_t), stream);
    uint32_t need = (n + 31) / 32 * 32 / kQueryThreads + 1;
    int grid = int(need < uint32_t(blocks) ? need : uint32_t(blocks));
    k_query<true><<<grid, kQueryThreads, 0, stream>>>(S, rays, n, q, HitsSoA {}, occluded, next, counters);
    return cudaGetLastError();
}

cudaError_t launch_patch_pairs(const DevScene& S, uint32_t surface, RaysSoA rays, const uint32_t* patch_ids,
                               uint32_t n, Query q, HitsSoA hits, Counters* counters, cudaStream_t stream)
{
    if (n == 0) return cudaSuccess;
    k_patch_pairs<<<(n + kQueryThreads - 1) / kQueryThreads, kQueryThreads, 0, stream>>>(S, surface, rays, patch_ids,
                                                                                          n, q, hits, counters);
    return cudaGetLastError();
}

}  // namespace cgs
