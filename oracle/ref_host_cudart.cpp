// ref_host_cudart.cpp -- TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.
//
// Host-memory definitions of the five CUDA runtime calls that the
// reference's hot-path code makes on the host (managed allocation in
// src/rt/CUDAUtility.h:81-98 and src/rt/CUDAUtility.cpp:39-57, and the error
// queries of its CUDA_CHECK).  oracle/build_ref.py links them into
// oracle/_ref/libcgs_ref.so instead of the CUDA runtime, so the reference's
// host code runs on a machine without a GPU: managed memory becomes ordinary
// host memory, which is what the host side of managed memory is.
#include <cstdlib>
#include <cuda_runtime_api.h>

extern "C" {

cudaError_t cudaMallocManaged(void** p, size_t n, unsigned int)
{
    if (!p) return cudaErrorInvalidValue;
    *p = std::aligned_alloc(256, ((n ? n : 1) + 255) / 256 * 256);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}

cudaError_t cudaFree(void* p)
{
    std::free(p);
    return cudaSuccess;
}

cudaError_t cudaGetLastError(void) { return cudaSuccess; }

const char* cudaGetErrorName(cudaError_t e) { return e == cudaSuccess ? "cudaSuccess" : "cudaError"; }

const char* cudaGetErrorString(cudaError_t e) { return e == cudaSuccess ? "no error" : "error (host stand-in)"; }

} // extern "C"
