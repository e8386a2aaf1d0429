// noalloc.cu -- cgs_perfect_hash_build_noalloc: the deterministic GPU
// perfect-hash build without any device allocation.
//
// cgs_perfect_hash_build takes its working memory from cudaMallocAsync.  Some
// callers cannot allocate at the moment they need a hash table: code running
// while a stream is being captured into a CUDA graph, code inside a
// framework's allocator callback, or services that must not grow the device
// heap after start-up.  This entry point runs the same kernels on a
// fixed-size scratch array that lives in the library itself, so the caller
// supplies only the keys and the output buffers.
//
// The scratch is a file-scope __device__ array sized for at most
// kNoAllocMaxKeys keys (about 6.9 MB).  Every GPU that loads the library holds
// it until the process exits.  All calls on a device share it and it keeps
// the contents of the last call; the build clears what must start from zero
// (bucket sizes, counters, slot owners) at the start of each call, so
// consecutive calls give independent results, but calls whose work overlaps
// on the GPU (on different streams, or from different host threads without
// ordering) race on the array and must be serialised by the caller.
//
// The first call on a device (with that device current) looks the array's
// device address up with cudaGetSymbolAddress and caches it; make that first
// call before any stream capture begins.
#include <mutex>
#include <numeric>
#include <random>

#include "../../include/cgspline.h"
#include "kernels.h"

namespace {

constexpr uint32_t kNoAllocMaxKeys = CGS_NOALLOC_MAX_KEYS;
// hash_scratch_words(kNoAllocMaxKeys): 800,784 32-bit words and 458,797 64-bit words
constexpr size_t kNoAllocWords64 = 458797 + (800784 + 1) / 2;

static __device__ __align__(256) unsigned long long g_noallocScratch[kNoAllocWords64];

constexpr int kMaxDevices = 64;
std::mutex g_noallocMutex;
void* g_noallocAddress[kMaxDevices] = {};

// std::mt19937(42) with std::uniform_int_distribution<uint32_t>(0, n) and
// gcd(n, A) == 1 retries: the 16 trials' coefficients (as the allocating
// entry point draws them).
void draw_coefficients(uint32_t n, uint32_t A[16], uint32_t B[16])
{
    std::mt19937 mt(42);
    std::uniform_int_distribution<uint32_t> d(0, n);
    for (int t = 0; t < 16; t++)
    {
        uint32_t a, b;
        do
        {
            a = d(mt);
            if (a == 0) a = 31;
            b = d(mt);
        } while (std::gcd(n, a) > 1);
        A[t] = a;
        B[t] = b;
    }
}

uint32_t displacement_size(uint32_t n)
{
    int s = int(n - 1) >> 1;
    if (s < 2) s = 2;
    uint32_t r = 1;
    while (r <= uint32_t(s) / 2) r <<= 1;
    return r;
}

}  // namespace

extern "C" int cgs_perfect_hash_build_noalloc(const uint32_t* keys, uint32_t n, uint32_t* disp,
                                              uint32_t displ_capacity, uint32_t* table, uint32_t table_capacity,
                                              uint32_t params[5], void* stream)
{
    if (!keys || !disp || !table || !params || n == 0) return CGS_ERR_INVALID_ARGUMENT;
    if (n > kNoAllocMaxKeys) return CGS_ERR_CAPACITY;
    const uint32_t step = std::max<uint32_t>(4u, uint32_t(0.05f * float(n)));
    if (displ_capacity < displacement_size(n) || table_capacity < n + 15u * step) return CGS_ERR_INVALID_ARGUMENT;
    size_t w32 = 0, w64 = 0;
    cgs::hash_scratch_words(n, w32, w64);
    if (w64 + (w32 + 1) / 2 > kNoAllocWords64) return CGS_ERR_CAPACITY;

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return CGS_ERR_CUDA;
    void* base = nullptr;
    {
        std::lock_guard<std::mutex> g(g_noallocMutex);
        if (!g_noallocAddress[dev])
        {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noallocScratch) != cudaSuccess || !p) return CGS_ERR_CUDA;
            g_noallocAddress[dev] = p;
        }
        base = g_noallocAddress[dev];
    }
    unsigned long long* base64 = static_cast<unsigned long long*>(base);
    uint32_t* base32 = reinterpret_cast<uint32_t*>(base64 + w64);
    cgs::HashScratch hs {};
    cgs::hash_scratch_carve(hs, n, base32, base64);
    uint32_t A[16], B[16];
    draw_coefficients(n, A, B);
    const int r = cgs::hash_build_device(keys, n, A, B, disp, table, table_capacity, hs, params,
                                         static_cast<cudaStream_t>(stream), nullptr);
    if (r == 4) return CGS_ERR_HASH_BUCKET_OVERFLOW;
    if (r < 0) return CGS_ERR_CUDA;
    if (r) return CGS_ERR_HASH_FAILED;
    return CGS_OK;
}
