// noalloc.cu -- cgs_perfect_hash_build_noalloc: the deterministic GPU
// perfect-hash build without any device allocation.
//
// cgs_perfect_hash_build takes its working memory from cudaMallocAsync.  Some
// callers cannot allocate at the moment they need a hash table: code inside a
// framework's allocator callback (allocating there re-enters the allocator),
// or services that reserve their device memory at start-up and must not grow
// the device heap afterwards.  This entry point runs the same kernels on a
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
// In host code the array's name is a host-side stand-in, not a device
// address.  Each call looks the device address up with cudaGetSymbolAddress
// for the current device and checks the result; the lookup is cheap once the
// module is loaded, and it stays correct after cudaDeviceReset, which may
// load the module at another address.
#include "../../include/cgspline.h"
#include "kernels.h"
#include "scene_impl.h"

namespace {

constexpr uint32_t kNoAllocMaxKeys = CGS_NOALLOC_MAX_KEYS;
// hash_scratch_words(kNoAllocMaxKeys): 800,784 32-bit words and 458,797 64-bit words
constexpr size_t kNoAllocWords64 = 458797 + (800784 + 1) / 2;

static __device__ __align__(256) unsigned long long g_noallocScratch[kNoAllocWords64];

}  // namespace

extern "C" int cgs_perfect_hash_build_noalloc(const uint32_t* keys, uint32_t n, uint32_t* disp,
                                              uint32_t displ_capacity, uint32_t* table, uint32_t table_capacity,
                                              uint32_t params[5], void* stream)
{
    if (!keys || !disp || !table || !params || n == 0) return CGS_ERR_INVALID_ARGUMENT;
    if (n > kNoAllocMaxKeys) return CGS_ERR_CAPACITY;
    if (displ_capacity < cgs::displ_size(n) || table_capacity < cgs::table_capacity(n))
        return CGS_ERR_INVALID_ARGUMENT;
    size_t w32 = 0, w64 = 0;
    cgs::hash_scratch_words(n, w32, w64);
    if (w64 + (w32 + 1) / 2 > kNoAllocWords64) return CGS_ERR_CAPACITY;

    void* base = nullptr;
    if (cudaGetSymbolAddress(&base, g_noallocScratch) != cudaSuccess || !base) return CGS_ERR_CUDA;
    unsigned long long* base64 = static_cast<unsigned long long*>(base);
    uint32_t* base32 = reinterpret_cast<uint32_t*>(base64 + w64);
    cgs::HashScratch hs {};
    cgs::hash_scratch_carve(hs, n, base32, base64);
    uint32_t A[16], B[16];
    cgs::hash_coefficients(n, A, B);
    const int r = cgs::hash_build_device(keys, n, A, B, disp, table, table_capacity, hs, params,
                                         static_cast<cudaStream_t>(stream), nullptr);
    if (r == 4) return CGS_ERR_HASH_BUCKET_OVERFLOW;
    if (r < 0) return CGS_ERR_CUDA;
    if (r) return CGS_ERR_HASH_FAILED;
    return CGS_OK;
}
