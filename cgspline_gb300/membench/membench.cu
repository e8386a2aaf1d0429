// membench.cu -- load-bandwidth probes for the roofline denominators.
//
// The traversal kernel reads its 64-byte BVH nodes from L1 and L2 (the scenes
// of the frame workloads are L2-resident), so HBM bandwidth does not bound
// it.  These probes measure the two on-chip roofs on the running GPU with
// plain loads and CUDA events, so that a kernel's achieved bytes per second
// can be set against the roof that binds it:
//
//   L1: every CTA reads its own `slice` bytes (a slice fits in L1) `reps`
//       times with 16-byte loads through the non-coherent path; all reads
//       after a CTA's first pass hit in L1.
//   L2: all CTAs stream a `bytes` buffer (larger than the L1s together,
//       smaller than L2) `reps` times with 16-byte loads that bypass L1
//       (ld.global.cg); all reads after the first pass hit in L2.
//
// Each probe returns the bytes loaded per second over the timed launches.
// Loaded values are summed and the sum is stored only when it equals a value
// no input produces, so the loads cannot be removed.
#include <cstdint>
#include <cuda_runtime.h>

namespace {

__device__ __forceinline__ float4 ld_nc(const float4* p)
{
    float4 v;
    asm volatile("ld.global.nc.v4.f32 {%0,%1,%2,%3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p));
    return v;
}

__device__ __forceinline__ float4 ld_cg(const float4* p)
{
    float4 v;
    asm volatile("ld.global.cg.v4.f32 {%0,%1,%2,%3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p));
    return v;
}

// Each CTA loops over its own slice of n4 float4s (slices of consecutive CTAs
// are consecutive).
__global__ void k_l1(const float4* __restrict__ buf, uint32_t n4, uint32_t slices, int reps, float* sink)
{
    const float4* s = buf + size_t(blockIdx.x % slices) * n4;
    float acc = 0.0f;
    for (int r = 0; r < reps; r++)
        for (uint32_t i = threadIdx.x; i < n4; i += blockDim.x)
        {
            const float4 v = ld_nc(s + i);
            acc += (v.x + v.y) + (v.z + v.w);
        }
    if (acc == -1.2345e30f) sink[blockIdx.x] = acc;
}

// All CTAs stream the whole buffer of n4 float4s, grid-strided.
__global__ void k_l2(const float4* __restrict__ buf, uint64_t n4, int reps, float* sink)
{
    float acc = 0.0f;
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (int r = 0; r < reps; r++)
        for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n4; i += stride)
        {
            const float4 v = ld_cg(buf + i);
            acc += (v.x + v.y) + (v.z + v.w);
        }
    if (acc == -1.2345e30f) sink[blockIdx.x] = acc;
}

}  // namespace

extern "C" {

// level 1: L1 probe, `bytes` is the per-CTA slice; level 2: L2 probe, `bytes`
// is the buffer.  `ctas_per_sm` x SMs CTAs of `threads`; `timed` launches after
// one warm-up.  *gbs receives the loaded GB/s of the timed launches.
// Returns 0, or a cudaError_t.
int cgs_membench(int level, uint64_t bytes, int ctas_per_sm, int threads, int reps, int timed, double* gbs)
{
    if (!gbs || bytes < 4096 || threads <= 0 || threads > 1024 || reps <= 0 || timed <= 0 || ctas_per_sm <= 0)
        return int(cudaErrorInvalidValue);
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return int(e);
    const int ctas = sms * ctas_per_sm;
    const uint64_t n4 = bytes / 16;
    // the L1 probe gives every CTA of an SM its own slice, so a buffer of
    // ctas slices; the L2 probe one buffer
    const uint32_t slices = level == 1 ? uint32_t(ctas) : 1u;
    const size_t alloc = size_t(n4) * 16 * slices;
    float4* buf = nullptr;
    float* sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if ((e = cudaMalloc(&buf, alloc)) != cudaSuccess) return int(e);
    if ((e = cudaMalloc(&sink, sizeof(float) * ctas)) != cudaSuccess) { cudaFree(buf); return int(e); }
    cudaMemset(buf, 0, alloc);
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    auto launch = [&]() {
        if (level == 1) k_l1<<<ctas, threads>>>(buf, uint32_t(n4), slices, reps, sink);
        else k_l2<<<ctas, threads>>>(buf, n4, reps, sink);
    };
    launch();
    e = cudaDeviceSynchronize();
    float ms = 0.0f;
    if (e == cudaSuccess)
    {
        cudaEventRecord(e0);
        for (int k = 0; k < timed; k++) launch();
        cudaEventRecord(e1);
        e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    }
    if (e == cudaSuccess)
    {
        const double loaded = level == 1 ? double(n4) * 16.0 * reps * ctas * timed
                                         : double(n4) * 16.0 * reps * timed;
        *gbs = loaded / (double(ms) * 1e-3) / 1e9;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    cudaFree(buf);
    return int(e);
}

}  // extern "C"
