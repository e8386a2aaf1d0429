// k_query.cu -- per-thread query kernels: spline::doBezierClipping /
// doSubdivision on explicit (ray, patch) pairs (src/Spline.h:488-508), the
// plain one-thread-per-ray scene query, and the gather / scatter of the ray
// arrays of several query requests into one batch.
#include <algorithm>

#include "kernels.h"

namespace cgs {

namespace {

constexpr int kPairThreads = 128;

__global__ void __launch_bounds__(kPairThreads) k_patch_pairs(DevScene S, uint32_t surface, uint32_t patches,
                                                              RaysSoA rays, const uint32_t* __restrict__ pids,
                                                              uint32_t n, Query q, HitsSoA hits, Counters* cnt)
{
    LocalCounters lc;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && __ldg(pids + i) >= patches)
    {
        hits.patch[i] = 0;
        lc.errors |= kErrPatchId;
    }
    else if (i < n)
    {
        const float3 o = f3(__ldg(rays.ox + i), __ldg(rays.oy + i), __ldg(rays.oz + i));
        const float3 d = f3(__ldg(rays.dx + i), __ldg(rays.dy + i), __ldg(rays.dz + i));
        const float4* P = S.patches + 16ull * (__ldg(S.patchBase + surface) + __ldg(pids + i));
        HitSink sink {P, o, d, hits.t[i], make_float2(0.0f, 0.0f)};
        const bool b = search_patch(sink, q, lc);
        if (b) { hits.t[i] = sink.dist; hits.u[i] = sink.uv.x; hits.v[i] = sink.uv.y; }
        hits.patch[i] = b ? 1 : 0;
    }
    flush_counters(cnt, lc, i < n ? 1u : 0u);
}

// One thread per ray, the whole search inline (the reference's per-ray
// kernel shape, src/rt/RayTracer.cu:171-274): the plain query path.
__global__ void __launch_bounds__(128) k_query_plain(DevScene S, RaysSoA rays, uint32_t n, uint32_t group0,
                                                     Query q, bool any, HitsSoA hits, Counters* cnt)
{
    LocalCounters lc;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        const float3 o = f3(rays.ox[i], rays.oy[i], rays.oz[i]);
        const float3 d = f3(rays.dx[i], rays.dy[i], rays.dz[i]);
        const float tmax = rays.tmax ? rays.tmax[i] : INFINITY;
        const uint32_t g = rays.group ? rays.group[i] : group0;
        if (g >= S.ngroups)
        {
            lc.errors |= kErrGroup;
            if (!any) { hits.t[i] = tmax; hits.u[i] = 0.0f; hits.v[i] = 0.0f; hits.object[i] = -1; }
            hits.patch[i] = -1;
        }
        else if (any)
        {
            Query q32 = q;
            q32.precision = 0;  // any-hit searches run at level 0
            hits.patch[i] = scene_any(S, g, o, d, tmax, q32, lc) ? 0 : -1;
        }
        else
        {
            HitRecord h {tmax, 0.0f, 0.0f, -1, -1};
            const int ob = scene_closest(S, g, o, d, tmax, q, h, lc);
            hits.t[i] = ob >= 0 ? h.t : tmax; hits.u[i] = h.u; hits.v[i] = h.v;
            hits.patch[i] = ob >= 0 ? h.patch : -1; hits.object[i] = ob;
        }
    }
    flush_counters(cnt, lc, i < n ? 1u : 0u);
}

__device__ __forceinline__ uint32_t find_chunk(const QueryChunk* tab, uint32_t n, uint32_t k)
{
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1)
    {
        const uint32_t mid = (lo + hi) >> 1;
        if (tab[mid].base <= k) lo = mid; else hi = mid;
    }
    return lo;
}

// hdr = (chunks, total rays) of the batch, on the device.
__global__ void k_gather_rays(const QueryChunk* tab, const uint32_t* hdr, float* rays, uint32_t cap, uint32_t* group)
{
    const uint32_t nchunks = hdr[0], total = hdr[1];
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x)
    {
        const QueryChunk& c = tab[find_chunk(tab, nchunks, k)];
        const uint32_t i = k - c.base;
#pragma unroll
        for (int j = 0; j < 6; j++) rays[size_t(j) * cap + k] = c.src[j][i];
        rays[6ull * cap + k] = c.src[6] ? c.src[6][i] : INFINITY;
        group[k] = c.group;
    }
}

__global__ void k_scatter_hits(const QueryChunk* tab, const uint32_t* hdr, HitsSoA hits, bool any)
{
    const uint32_t nchunks = hdr[0], total = hdr[1];
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x)
    {
        const QueryChunk& c = tab[find_chunk(tab, nchunks, k)];
        const uint32_t i = k - c.base;
        c.out.patch[i] = hits.patch[k];
        if (!any)
        {
            c.out.t[i] = hits.t[k]; c.out.u[i] = hits.u[k]; c.out.v[i] = hits.v[k];
            c.out.object[i] = hits.object[k];
        }
    }
}

}  // namespace

cudaError_t launch_query_plain(const DevScene& S, RaysSoA rays, uint32_t n, uint32_t group, Query q, bool any,
                               HitsSoA hits, Counters* counters, cudaStream_t stream)
{
    if (n == 0) return cudaSuccess;
    k_query_plain<<<(n + 127) / 128, 128, 0, stream>>>(S, rays, n, group, q, any, hits, counters);
    return cudaGetLastError();
}

cudaError_t launch_gather_rays(const QueryChunk* table, const uint32_t* hdr, uint32_t cap, float* rays,
                               uint32_t* group, cudaStream_t stream)
{
    if (cap == 0) return cudaSuccess;
    const uint32_t blocks = std::min<uint32_t>((cap + 255) / 256, 4096u);
    k_gather_rays<<<blocks, 256, 0, stream>>>(table, hdr, rays, cap, group);
    return cudaGetLastError();
}

cudaError_t launch_scatter_hits(const QueryChunk* table, const uint32_t* hdr, uint32_t cap, HitsSoA hits, bool any,
                                cudaStream_t stream)
{
    if (cap == 0) return cudaSuccess;
    const uint32_t blocks = std::min<uint32_t>((cap + 255) / 256, 4096u);
    k_scatter_hits<<<blocks, 256, 0, stream>>>(table, hdr, hits, any);
    return cudaGetLastError();
}

cudaError_t launch_patch_pairs(const DevScene& S, uint32_t surface, uint32_t patches, RaysSoA rays,
                               const uint32_t* patch_ids, uint32_t n, Query q, HitsSoA hits, Counters* counters,
                               cudaStream_t stream)
{
    if (n == 0) return cudaSuccess;
    k_patch_pairs<<<(n + kPairThreads - 1) / kPairThreads, kPairThreads, 0, stream>>>(S, surface, patches, rays,
                                                                                      patch_ids, n, q, hits, counters);
    return cudaGetLastError();
}

__global__ void k_patch_normals(DevScene S, uint32_t surface, uint32_t patches, const uint32_t* __restrict__ pids,
                                const float* __restrict__ u, const float* __restrict__ v, uint32_t n, float* normals,
                                Counters* cnt)
{
    LocalCounters lc;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        const uint32_t p = __ldg(pids + i);
        float3 N = f3(0.0f, 0.0f, 0.0f);
        if (p < patches) N = versor(patch_normal(S.patches + 16ull * (__ldg(S.patchBase + surface) + p),
                                                 __ldg(u + i), __ldg(v + i)));
        else lc.errors |= kErrPatchId;
        normals[i] = N.x; normals[n + i] = N.y; normals[2ull * n + i] = N.z;
    }
    flush_counters(cnt, lc, 0);
}

cudaError_t launch_patch_normals(const DevScene& S, uint32_t surface, uint32_t patches, const uint32_t* patch_ids,
                                 const float* u, const float* v, uint32_t n, float* normals, Counters* counters,
                                 cudaStream_t stream)
{
    if (n == 0) return cudaSuccess;
    k_patch_normals<<<(n + 255) / 256, 256, 0, stream>>>(S, surface, patches, patch_ids, u, v, n, normals, counters);
    return cudaGetLastError();
}

}  // namespace cgs
