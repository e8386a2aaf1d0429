// k_hash.cu -- deterministic GPU build of the BVH's perfect hash
// (PerfectHashFunction::build, src/rt/PerfectHashFunction.cu:229-503).
//
// Same sizing and hash family as the reference: displacement table of
// bit_floor(max(2,(n-1)>>1)) buckets (key & mask), bucket capacity 4,
// h(k) = (A k + B + disp[k & mask]) mod N, 32 attempts per bucket with the
// displacement growing by rank+1, up to 16 trials that grow N by
// max(4, 0.05 n).  The reference places the buckets of one size class with
// racing atomicInc/atomicDec (:147-227), so its tables vary run to run.  Here
// a size class resolves in synchronous rounds -- every unplaced bucket whose
// slots are free and pairwise distinct bids for them with a 64-bit
// atomicMin of (round tag, rank); a bucket that owns all of its slots is
// placed, the others add rank+1 to their displacement -- which makes the table
// a pure function of the keys.  Each round is two kernel launches (bid,
// commit); there is no device-wide barrier and no spin-wait.
#include <atomic>
#include <type_traits>
#include <algorithm>

#include "kernels.h"

namespace cgs {

namespace {

constexpr uint32_t kCap = 4;
constexpr int kThreads = 256;
constexpr int kBlockThreads = 1024;  // one CTA per small BVH
constexpr int kRankChunk = 4096;  // buckets per rank block (counts fit 16 bits)

enum : uint32_t { kActive = 1u, kFeasible = 2u };
enum : uint32_t { kErrOverflow = 1u, kErrDuplicate = 2u };

// misc layout
enum { M_ERR = 0, M_CLASS = 1, M_REMAIN = 5, M_FAIL = 9 };

__global__ void k_bucket(const uint32_t* __restrict__ keys, uint32_t n, uint32_t mask, uint32_t* bsize,
                         uint32_t* bkeys, uint32_t* misc)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        uint32_t key = keys[i], j = key & mask;
        uint32_t s = atomicAdd(bsize + j, 1u);
        if (s >= kCap) atomicOr(misc + M_ERR, kErrOverflow);  // reference: __trap()
        else bkeys[kCap * j + s] = key;
    }
}

// Per-chunk counts of buckets of each size 1..4, packed 16 bits per class.
__device__ __forceinline__ unsigned long long class_bits(uint32_t size)
{
    return (size >= 1 && size <= 4) ? (1ull << (16 * (size - 1))) : 0ull;
}

__global__ void __launch_bounds__(kThreads) k_rank_count(const uint32_t* bsize, uint32_t nb, unsigned long long* blockCounts)
{
    __shared__ unsigned long long red[kThreads];
    const uint32_t b0 = blockIdx.x * kRankChunk;
    unsigned long long acc = 0;
    for (uint32_t b = b0 + threadIdx.x; b < min(nb, b0 + kRankChunk); b += kThreads) acc += class_bits(min(bsize[b], 5u));
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = kThreads / 2; s > 0; s >>= 1)
    {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) blockCounts[blockIdx.x] = red[0];
}

// One block: exclusive prefix of the per-chunk counts, per class (64-bit
// totals per class are kept separately to avoid 16-bit overflow).
__global__ void k_rank_scan(unsigned long long* blockCounts, uint32_t nblocks, unsigned long long* prefix, uint32_t* misc)
{
    if (threadIdx.x != 0) return;
    uint32_t tot[4] = {0, 0, 0, 0};
    for (uint32_t k = 0; k < nblocks; k++)
    {
        unsigned long long c = blockCounts[k];
        // store prefix for this block as four 16-bit... counts may exceed 16 bits
        // across blocks, so keep 2 x 64-bit words: classes 1,2 and 3,4 (32 bits each)
        prefix[2 * k] = (unsigned long long)tot[0] | ((unsigned long long)tot[1] << 32);
        prefix[2 * k + 1] = (unsigned long long)tot[2] | ((unsigned long long)tot[3] << 32);
        for (int cl = 0; cl < 4; cl++) tot[cl] += uint32_t((c >> (16 * cl)) & 0xFFFFu);
    }
    for (int cl = 0; cl < 4; cl++) { misc[M_CLASS + cl] = tot[cl]; }
}

// rank[b] = number of buckets b' < b with the same size (ascending bucket id).
__global__ void __launch_bounds__(kThreads) k_rank_apply(const uint32_t* bsize, uint32_t nb,
                                                         const unsigned long long* prefix, uint32_t* rank)
{
    __shared__ unsigned long long scan[kThreads];
    const uint32_t b0 = blockIdx.x * kRankChunk;
    const uint32_t per = kRankChunk / kThreads;  // contiguous buckets per thread
    const uint32_t t0 = b0 + threadIdx.x * per;
    unsigned long long local = 0;
    for (uint32_t k = 0; k < per; k++)
    {
        uint32_t b = t0 + k;
        if (b < nb) local += class_bits(min(bsize[b], 5u));
    }
    scan[threadIdx.x] = local;
    __syncthreads();
    // Hillis-Steele inclusive scan over packed 16-bit counts (chunk <= 4096 < 65536)
    for (int off = 1; off < kThreads; off <<= 1)
    {
        unsigned long long v = threadIdx.x >= off ? scan[threadIdx.x - off] : 0ull;
        __syncthreads();
        scan[threadIdx.x] += v;
        __syncthreads();
    }
    unsigned long long excl = scan[threadIdx.x] - local;
    uint32_t run[4];
    unsigned long long p0 = prefix[2 * blockIdx.x], p1 = prefix[2 * blockIdx.x + 1];
    run[0] = uint32_t(p0) + uint32_t(excl & 0xFFFFu);
    run[1] = uint32_t(p0 >> 32) + uint32_t((excl >> 16) & 0xFFFFu);
    run[2] = uint32_t(p1) + uint32_t((excl >> 32) & 0xFFFFu);
    run[3] = uint32_t(p1 >> 32) + uint32_t((excl >> 48) & 0xFFFFu);
    for (uint32_t k = 0; k < per; k++)
    {
        uint32_t b = t0 + k;
        if (b >= nb) break;
        uint32_t s = min(bsize[b], 5u);
        if (s >= 1 && s <= 4) rank[b] = run[s - 1]++;
        else rank[b] = 0;
    }
}

__global__ void k_trial_init(const uint32_t* bsize, uint32_t nb, uint32_t* dcur, uint32_t* state, uint32_t* disp,
                             uint32_t* misc)
{
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x)
    {
        dcur[b] = 0;
        disp[b] = 0;
        state[b] = (bsize[b] >= 1 && bsize[b] <= kCap) ? kActive : 0u;
    }
    if (blockIdx.x == 0 && threadIdx.x < 4) misc[M_REMAIN + threadIdx.x] = misc[M_CLASS + threadIdx.x];
    if (blockIdx.x == 0 && threadIdx.x == 0) misc[M_FAIL] = 0;
}

__device__ __forceinline__ unsigned long long owner_tag(uint32_t round, uint32_t rank)
{
    return ((unsigned long long)(0xFFFFFFFFu - round) << 32) | rank;
}

__global__ void __launch_bounds__(kThreads) k_bid(const uint32_t* bsize, const uint32_t* bkeys, const uint32_t* rank,
                                                  const uint32_t* dcur, uint32_t* state, uint32_t* slots,
                                                  const uint32_t* occ, unsigned long long* owner, uint32_t nb,
                                                  uint32_t cls, uint32_t A, uint32_t B, uint32_t N, uint32_t round,
                                                  const uint32_t* misc)
{
    if (misc[M_REMAIN + cls - 1] == 0) return;
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x)
    {
        if (bsize[b] != cls) continue;
        uint32_t st = state[b];
        if (!(st & kActive)) continue;
        uint32_t s[kCap];
        bool f = true;
        for (uint32_t k = 0; k < cls; k++)
        {
            uint32_t sl = (A * bkeys[kCap * b + k] + B + dcur[b]) % N;
            s[k] = sl;
            if (occ[sl >> 5] & (1u << (sl & 31))) f = false;
            for (uint32_t m = 0; m < k; m++) if (s[m] == sl) f = false;
        }
        for (uint32_t k = 0; k < cls; k++) slots[kCap * b + k] = s[k];
        state[b] = f ? (st | kFeasible) : (st & ~kFeasible);
        if (f)
        {
            unsigned long long tag = owner_tag(round, rank[b]);
            for (uint32_t k = 0; k < cls; k++) atomicMin(owner + s[k], tag);
        }
    }
}

__global__ void __launch_bounds__(kThreads) k_commit(const uint32_t* bsize, const uint32_t* rank, uint32_t* dcur,
                                                     uint32_t* state, const uint32_t* slots, uint32_t* occ,
                                                     const unsigned long long* owner, uint32_t* disp, uint32_t nb,
                                                     uint32_t cls, uint32_t round, bool last, uint32_t* misc)
{
    if (misc[M_REMAIN + cls - 1] == 0) return;
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x)
    {
        if (bsize[b] != cls) continue;
        uint32_t st = state[b];
        if (!(st & kActive)) continue;
        bool win = (st & kFeasible) != 0;
        if (win)
        {
            unsigned long long tag = owner_tag(round, rank[b]);
            for (uint32_t k = 0; k < cls; k++) if (owner[slots[kCap * b + k]] != tag) win = false;
        }
        if (win)
        {
            for (uint32_t k = 0; k < cls; k++)
            {
                uint32_t sl = slots[kCap * b + k];
                atomicOr(occ + (sl >> 5), 1u << (sl & 31));
            }
            disp[b] = dcur[b];
            state[b] = 0;
            atomicSub(misc + M_REMAIN + cls - 1, 1u);
        }
        else
        {
            dcur[b] += rank[b] + 1;
            if (last) atomicAdd(misc + M_FAIL, 1u);
        }
    }
}

__global__ void k_fill(const uint32_t* __restrict__ keys, uint32_t n, const uint32_t* __restrict__ disp, uint32_t mask,
                       uint32_t A, uint32_t B, uint32_t N, uint32_t* table, uint32_t* misc)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        uint32_t key = keys[i];
        uint32_t h = (A * key + B + disp[key & mask]) % N;
        uint32_t prev = atomicCAS(table + h, EMPTY, i);
        if (prev != EMPTY) atomicOr(misc + M_ERR, kErrDuplicate);
    }
}

uint32_t bit_floor_u32(uint32_t x)
{
    uint32_t r = 1;
    while (r <= x / 2) r <<= 1;
    return x ? r : 0;
}

// SM count of the current device, cached per device ordinal.  The cache
// entries are atomics: concurrent first calls from several host threads
// store the same value.
int device_sms()
{
    constexpr int kMaxDev = 64;
    static std::atomic<int> cache[kMaxDev];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
    int sms = (dev >= 0 && dev < kMaxDev) ? cache[dev].load(std::memory_order_relaxed) : 0;
    if (sms > 0) return sms;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 1;
    if (dev >= 0 && dev < kMaxDev) cache[dev].store(sms, std::memory_order_relaxed);
    return sms;
}

// ------------------------------------------------------- one CTA per BVH --
// The same build for one BVH run entirely by one CTA: the bid and commit
// phases of a round are separated by __syncthreads instead of kernel
// launches, and a whole store's BVHs are built by one launch, one CTA each,
// with no host round trip between trials.  Up to kHashBlockMaxKeys keys the
// buckets, ranks, displacements, slot owners and occupancy bitmap live in
// shared memory (kShared); up to kHashGlobalBlockMaxKeys in a global scratch
// area per BVH (mostly L2-resident).  The rounds, ranks, tie rule (lowest
// rank wins a slot) and displacement steps are those of k_bid / k_commit,
// so the tables are the same.  Slot owners are tags with the round in the
// high half and the rank in the low half: 16 + 16 bits in shared memory
// (rounds < 2^11, ranks < 2^16 there), 32 + 32 bits in global memory.
struct BlockScratchLayout
{
    uint32_t* bkeys;  // [4 nb]
    uint32_t* dcur;   // [nb]
    uint32_t* bsize;  // [nb]
    uint32_t* rank;   // [nb]
    uint32_t* state;  // [nb]: bit 0 active, bit 1 feasible
    uint32_t* occ;    // [ceil(nmax / 32)]
    void* owner;      // [nmax] tags
};

// Words of a global scratch area for a BVH of n keys (owner tags 64-bit).
__host__ __device__ inline uint64_t block_scratch_words(uint32_t nb, uint32_t nmax)
{
    return 8ull * nb + (nmax + 31) / 32 + 1 + 2ull * nmax;  // +1: 8-byte alignment of the tags
}

__device__ __forceinline__ uint4 warp_incl_scan4(uint4 v)
{
    for (int off = 1; off < 32; off <<= 1)
    {
        uint4 u;
        u.x = __shfl_up_sync(0xFFFFFFFFu, v.x, off);
        u.y = __shfl_up_sync(0xFFFFFFFFu, v.y, off);
        u.z = __shfl_up_sync(0xFFFFFFFFu, v.z, off);
        u.w = __shfl_up_sync(0xFFFFFFFFu, v.w, off);
        if ((threadIdx.x & 31) >= uint32_t(off)) { v.x += u.x; v.y += u.y; v.z += u.z; v.w += u.w; }
    }
    return v;
}

template<bool kShared>
__global__ void __launch_bounds__(kBlockThreads) k_hash_block(const uint32_t* __restrict__ keys,
                                                              const HashJob* __restrict__ jobs, uint32_t* disps,
                                                              uint32_t* tables, uint32_t* out, uint32_t nbMax,
                                                              uint32_t nmaxMax, uint32_t* gscratch)
{
    using Tag = typename std::conditional<kShared, uint32_t, unsigned long long>::type;
    extern __shared__ __align__(16) uint32_t sm[];
    __shared__ uint32_t sErr, sFail, sCount[4], sRemain[4];
    __shared__ uint4 sWarp[kBlockThreads / 32];
    const HashJob& J = jobs[blockIdx.x];
    const uint32_t n = J.n, mask = J.mask, nb = mask + 1;
    const uint32_t step = max(4u, uint32_t(0.05f * float(n)));
    BlockScratchLayout L;
    {
        const uint32_t nbs = kShared ? nbMax : nb;
        const uint32_t nms = kShared ? nmaxMax : n + 16u * step;
        uint32_t* p = kShared ? sm : gscratch + J.scratchOff;
        L.bkeys = p; p += 4ull * nbs;
        L.dcur = p; p += nbs;
        L.bsize = p; p += nbs;
        L.rank = p; p += nbs;
        L.state = p; p += nbs;
        L.occ = p; p += (nms + 31) / 32;
        if (!kShared && (reinterpret_cast<uintptr_t>(p) & 7u)) p++;
        L.owner = p;
    }
    uint32_t *bkeys = L.bkeys, *dcur = L.dcur, *bsize = L.bsize, *rank = L.rank, *state = L.state, *occ = L.occ;
    Tag* owner = static_cast<Tag*>(L.owner);
    const uint32_t tid = threadIdx.x, bd = blockDim.x;
    uint32_t* res = out + 8ull * blockIdx.x;

    for (uint32_t b = tid; b < nb; b += bd) bsize[b] = 0;
    if (tid == 0) { sErr = 0; sFail = 0; }
    __syncthreads();
    for (uint32_t i = tid; i < n; i += bd)
    {
        const uint32_t key = keys[J.keyOff + i], j = key & mask;
        const uint32_t s = atomicAdd(bsize + j, 1u);
        if (s >= kCap) atomicOr(&sErr, kErrOverflow);  // reference: __trap()
        else bkeys[kCap * j + s] = key;
    }
    __syncthreads();
    if (sErr)
    {
        // as hash_build_device reports a bucket overflow (found in trial 0)
        if (tid == 0) { res[0] = 4; res[1] = J.A[0]; res[2] = J.B[0]; res[3] = n; res[4] = mask; res[5] = 0; }
        return;
    }

    // rank[b]: buckets b' < b of the same size; contiguous buckets per thread,
    // the four classes' counts scanned block-wide
    const uint32_t per = (nb + bd - 1) / bd, b0 = tid * per;
    uint4 local = make_uint4(0, 0, 0, 0);
    for (uint32_t k = 0; k < per && b0 + k < nb; k++)
    {
        const uint32_t sz = bsize[b0 + k];
        local.x += sz == 1; local.y += sz == 2; local.z += sz == 3; local.w += sz == 4;
    }
    const uint4 incl = warp_incl_scan4(local);
    if ((tid & 31) == 31) sWarp[tid >> 5] = incl;
    __syncthreads();
    if (tid < 32)
    {
        const uint32_t nw = bd >> 5;
        const uint4 w = tid < nw ? sWarp[tid] : make_uint4(0, 0, 0, 0);
        const uint4 wi = warp_incl_scan4(w);
        if (tid < nw) sWarp[tid] = make_uint4(wi.x - w.x, wi.y - w.y, wi.z - w.z, wi.w - w.w);
        if (tid == 31) { sCount[0] = wi.x; sCount[1] = wi.y; sCount[2] = wi.z; sCount[3] = wi.w; }
    }
    __syncthreads();
    {
        const uint4 wb = sWarp[tid >> 5];
        uint32_t run[4] = {wb.x + incl.x - local.x, wb.y + incl.y - local.y, wb.z + incl.z - local.z,
                           wb.w + incl.w - local.w};
        for (uint32_t k = 0; k < per && b0 + k < nb; k++)
        {
            const uint32_t b = b0 + k, sz = bsize[b];
            rank[b] = (sz >= 1 && sz <= kCap) ? run[sz - 1]++ : 0u;
        }
    }

    uint32_t N = n, trial = 0, A = 0, B = 0;
    bool ok = false;
    for (trial = 0; trial < 16; trial++)
    {
        A = J.A[trial];
        B = J.B[trial];
        for (uint32_t w = tid; w < (N + 31) / 32; w += bd) occ[w] = 0;
        for (uint32_t w = tid; w < N; w += bd) owner[w] = Tag(~Tag(0));
        for (uint32_t b = tid; b < nb; b += bd)
        {
            dcur[b] = 0;
            state[b] = (bsize[b] >= 1 && bsize[b] <= kCap) ? kActive : 0u;
        }
        if (tid == 0)
        {
            sFail = 0;
            for (int c = 0; c < 4; c++) sRemain[c] = sCount[c];
        }
        __syncthreads();
        for (uint32_t cls = kCap; cls >= 1; cls--)
        {
            if (sCount[cls - 1] == 0) continue;
            for (uint32_t r = 0; r < 32; r++)
            {
                const uint32_t round = trial * 128u + (kCap - cls) * 32u + r;
                const Tag tagHi = kShared ? Tag(0xFFFFu - round) << 16 : Tag(0xFFFFFFFFu - round) << 32;
                for (uint32_t b = tid; b < nb; b += bd)
                {
                    if (bsize[b] != cls || !(state[b] & kActive)) continue;
                    uint32_t sl[kCap];
                    bool f = true;
                    for (uint32_t k = 0; k < cls; k++)
                    {
                        sl[k] = (A * bkeys[kCap * b + k] + B + dcur[b]) % N;
                        if (occ[sl[k] >> 5] & (1u << (sl[k] & 31))) f = false;
                        for (uint32_t m = 0; m < k; m++) if (sl[m] == sl[k]) f = false;
                    }
                    state[b] = f ? (kActive | kFeasible) : kActive;
                    if (f)
                        for (uint32_t k = 0; k < cls; k++) atomicMin(owner + sl[k], tagHi | Tag(rank[b]));
                }
                __syncthreads();
                for (uint32_t b = tid; b < nb; b += bd)
                {
                    if (bsize[b] != cls || !(state[b] & kActive)) continue;
                    bool win = (state[b] & kFeasible) != 0;
                    uint32_t sl[kCap];
                    for (uint32_t k = 0; k < cls; k++)
                    {
                        sl[k] = (A * bkeys[kCap * b + k] + B + dcur[b]) % N;
                        if (win && owner[sl[k]] != (tagHi | Tag(rank[b]))) win = false;
                    }
                    if (win)
                    {
                        for (uint32_t k = 0; k < cls; k++) atomicOr(occ + (sl[k] >> 5), 1u << (sl[k] & 31));
                        state[b] = 0;
                        atomicSub(sRemain + cls - 1, 1u);
                    }
                    else
                    {
                        dcur[b] += rank[b] + 1;
                        if (r == 31) atomicAdd(&sFail, 1u);
                    }
                }
                __syncthreads();
                if (sRemain[cls - 1] == 0) break;
            }
        }
        __syncthreads();
        if (sFail == 0) { ok = true; break; }
        N += step;
        __syncthreads();
    }
    if (!ok)
    {
        // as hash_build_device reports a failed build: the last trial's
        // coefficients and the table size grown past it
        if (tid == 0)
        {
            res[0] = 3; res[1] = J.A[15]; res[2] = J.B[15]; res[3] = N; res[4] = mask; res[5] = 16;
        }
        return;
    }
    uint32_t* table = tables + J.tableOff;
    for (uint32_t b = tid; b < nb; b += bd) disps[J.dispOff + b] = dcur[b];
    for (uint32_t w = tid; w < N; w += bd) table[w] = EMPTY;
    __syncthreads();
    for (uint32_t i = tid; i < n; i += bd)
    {
        const uint32_t key = keys[J.keyOff + i];
        const uint32_t h = (A * key + B + dcur[key & mask]) % N;
        if (atomicCAS(table + h, EMPTY, i) != EMPTY) atomicOr(&sErr, kErrDuplicate);
    }
    __syncthreads();
    if (tid == 0)
    {
        res[0] = sErr ? 5u : 0u; res[1] = A; res[2] = B; res[3] = N; res[4] = mask; res[5] = trial;
    }
}

int grid_for(uint64_t items, int threads)
{
    const int sms = device_sms();
    uint64_t g = (items + threads - 1) / threads;
    uint64_t cap = uint64_t(sms) * 8;
    return int(std::max<uint64_t>(1, std::min(g, cap)));
}

}  // namespace

void hash_scratch_words(uint32_t n, size_t& words32, size_t& words64)
{
    int s = int(n - 1) >> 1;
    if (s < 2) s = 2;
    const uint32_t nb = bit_floor_u32(uint32_t(s));
    const uint32_t step = std::max<uint32_t>(4u, uint32_t(0.05f * float(n)));
    const uint64_t nmax = uint64_t(n) + 15ull * step;
    const uint32_t rblocks = (nb + kRankChunk - 1) / kRankChunk;
    words32 = size_t(nb) * (1 + kCap + 1 + 1 + 1 + kCap) + (nmax + 31) / 32 + 16;
    words64 = nmax + 3ull * rblocks;
}

void hash_scratch_carve(HashScratch& s, uint32_t n, uint32_t* base32, unsigned long long* base64)
{
    int sh = int(n - 1) >> 1;
    if (sh < 2) sh = 2;
    const uint32_t nb = bit_floor_u32(uint32_t(sh));
    const uint32_t step = std::max<uint32_t>(4u, uint32_t(0.05f * float(n)));
    const uint64_t nmax = uint64_t(n) + 15ull * step;
    uint32_t* p = base32;
    s.bsize = p; p += nb;
    s.bkeys = p; p += size_t(kCap) * nb;
    s.rank = p; p += nb;
    s.dcur = p; p += nb;
    s.state = p; p += nb;
    s.slots = p; p += size_t(kCap) * nb;
    s.occ = p; p += (nmax + 31) / 32;
    s.misc = p; p += 16;
    s.owner = base64;
    s.blockCounts = reinterpret_cast<uint32_t*>(base64 + nmax);
}

int hash_build_device(const uint32_t* keys, uint32_t n, const uint32_t A[16], const uint32_t B[16], uint32_t* disp,
                      uint32_t* table, uint32_t tableCapacity, HashScratch& sc, uint32_t params[5], cudaStream_t stream,
                      int* launches)
{
    if (n == 0) return 1;
    int sh = int(n - 1) >> 1;
    if (sh < 2) sh = 2;
    const uint32_t nb = bit_floor_u32(uint32_t(sh));
    const uint32_t mask = nb - 1;
    const uint32_t step = std::max<uint32_t>(4u, uint32_t(0.05f * float(n)));
    const uint64_t nmax = uint64_t(n) + 15ull * step;
    if (tableCapacity < nmax) return 2;
    const uint32_t rblocks = (nb + kRankChunk - 1) / kRankChunk;
    unsigned long long* blockCounts = reinterpret_cast<unsigned long long*>(sc.blockCounts);
    unsigned long long* prefix = blockCounts + rblocks;
    int nl = 0;
    cudaMemsetAsync(sc.bsize, 0, sizeof(uint32_t) * nb, stream);
    cudaMemsetAsync(sc.misc, 0, sizeof(uint32_t) * 16, stream);
    cudaMemsetAsync(sc.owner, 0xFF, sizeof(unsigned long long) * nmax, stream);
    k_bucket<<<grid_for(n, kThreads), kThreads, 0, stream>>>(keys, n, mask, sc.bsize, sc.bkeys, sc.misc);
    k_rank_count<<<rblocks, kThreads, 0, stream>>>(sc.bsize, nb, blockCounts);
    k_rank_scan<<<1, 32, 0, stream>>>(blockCounts, rblocks, prefix, sc.misc);
    k_rank_apply<<<rblocks, kThreads, 0, stream>>>(sc.bsize, nb, prefix, sc.rank);
    nl += 4;
    uint32_t host[16];
    int result = 3;  // no trial succeeded
    uint32_t N = n, trial = 0;
    uint32_t round = 0;
    const int gb = grid_for(nb, kThreads);
    for (trial = 0; trial < 16; trial++)
    {
        cudaMemsetAsync(sc.occ, 0, sizeof(uint32_t) * ((N + 31) / 32), stream);
        k_trial_init<<<gb, kThreads, 0, stream>>>(sc.bsize, nb, sc.dcur, sc.state, disp, sc.misc);
        nl++;
        for (uint32_t cls = kCap; cls >= 1; cls--)
            for (uint32_t r = 0; r < 32; r++, round++)
            {
                k_bid<<<gb, kThreads, 0, stream>>>(sc.bsize, sc.bkeys, sc.rank, sc.dcur, sc.state, sc.slots, sc.occ,
                                                   sc.owner, nb, cls, A[trial], B[trial], N, round, sc.misc);
                k_commit<<<gb, kThreads, 0, stream>>>(sc.bsize, sc.rank, sc.dcur, sc.state, sc.slots, sc.occ, sc.owner,
                                                      disp, nb, cls, round, r == 31, sc.misc);
                nl += 2;
            }
        if (cudaMemcpyAsync(host, sc.misc, sizeof host, cudaMemcpyDeviceToHost, stream) != cudaSuccess) return -1;
        if (cudaStreamSynchronize(stream) != cudaSuccess) return -1;
        if (host[M_ERR] & kErrOverflow) { result = 4; break; }
        if (host[M_FAIL] == 0) { result = 0; break; }
        N = N + step;
    }
    if (launches) *launches += nl;
    params[0] = A[trial < 16 ? trial : 15]; params[1] = B[trial < 16 ? trial : 15];
    params[2] = N; params[3] = mask; params[4] = trial;
    if (result) return result;
    cudaMemsetAsync(table, 0xFF, sizeof(uint32_t) * N, stream);
    k_fill<<<grid_for(n, kThreads), kThreads, 0, stream>>>(keys, n, disp, mask, A[trial], B[trial], N, table, sc.misc);
    if (launches) *launches += 1;
    if (cudaMemcpyAsync(host, sc.misc, sizeof host, cudaMemcpyDeviceToHost, stream) != cudaSuccess) return -1;
    if (cudaStreamSynchronize(stream) != cudaSuccess) return -1;
    if (host[M_ERR] & kErrDuplicate) return 5;
    return 0;
}


namespace {

void block_sizes(uint32_t n, uint32_t& nb, uint32_t& nmax)
{
    n = std::max<uint32_t>(n, 1u);
    int sh = int(n - 1) >> 1;
    if (sh < 2) sh = 2;
    nb = bit_floor_u32(uint32_t(sh));
    const uint32_t step = std::max<uint32_t>(4u, uint32_t(0.05f * float(n)));
    nmax = n + 16u * step;
}

}  // namespace

size_t hash_block_smem(uint32_t maxKeys)
{
    uint32_t nb = 0, nmax = 0;
    block_sizes(maxKeys, nb, nmax);
    return sizeof(uint32_t) * (8ull * nb + nmax + (nmax + 31) / 32);
}

uint64_t hash_block_scratch_words(uint32_t n)
{
    uint32_t nb = 0, nmax = 0;
    block_sizes(n, nb, nmax);
    return block_scratch_words(nb, nmax);
}

cudaError_t hash_build_blocks(const uint32_t* keys, const HashJob* jobs, uint32_t njobs, uint32_t maxKeys,
                              uint32_t* disps, uint32_t* tables, uint32_t* out, cudaStream_t stream,
                              uint32_t* gscratch)
{
    if (njobs == 0) return cudaSuccess;
    if (maxKeys > kHashGlobalBlockMaxKeys || (maxKeys > kHashBlockMaxKeys && !gscratch)) return cudaErrorInvalidValue;
    if (maxKeys > kHashBlockMaxKeys)
    {
        k_hash_block<false><<<njobs, kBlockThreads, 0, stream>>>(keys, jobs, disps, tables, out, 0, 0, gscratch);
        return cudaGetLastError();
    }
    uint32_t nb = 0, nmax = 0;
    block_sizes(maxKeys, nb, nmax);
    const size_t smem = hash_block_smem(maxKeys);
    cudaError_t e = cudaFuncSetAttribute(k_hash_block<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    k_hash_block<true><<<njobs, kBlockThreads, smem, stream>>>(keys, jobs, disps, tables, out, nb, nmax, nullptr);
    return cudaGetLastError();
}

}  // namespace cgs
