// k_query.cu -- spline::doBezierClipping / doSubdivision on explicit
// (ray, patch) pairs (src/Spline.h:488-508), one thread per pair.
#include "kernels.h"

namespace cgs {

namespace {

constexpr int kPairThreads = 128;

__global__ void __launch_bounds__(kPairThreads) k_patch_pairs(DevScene S, uint32_t surface, RaysSoA rays,
                                                              const uint32_t* __restrict__ pids, uint32_t n, Query q,
                                                              HitsSoA hits, Counters* cnt)
{
    LocalCounters lc;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
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

}  // namespace

cudaError_t launch_patch_pairs(const DevScene& S, uint32_t surface, RaysSoA rays, const uint32_t* patch_ids,
                               uint32_t n, Query q, HitsSoA hits, Counters* counters, cudaStream_t stream)
{
    if (n == 0) return cudaSuccess;
    k_patch_pairs<<<(n + kPairThreads - 1) / kPairThreads, kPairThreads, 0, stream>>>(S, surface, rays, patch_ids, n,
                                                                                      q, hits, counters);
    return cudaGetLastError();
}

}  // namespace cgs
