// k_engine.cu -- the query engine: closest / any hit over the two-level
// hashed stackless BVH with Bezier clipping.
//
// A query runs a few passes of two persistent kernels:
//
// k_collect walks the reference's traversal (BVH::hashIntersect,
// src/rt/BVH.h:178-350, nested through the object level as in
// Context::intersect, src/rt/RayTracer.cu:295-383) -- same stackless key /
// postponed-bit state, same perfect-hash backtracking, same nearer-child-first
// order -- and appends what it meets to the ray's chunk: each patch of a
// leaf with the entry distance of the leaf's box, and markers where it enters
// or leaves an object.  It culls with the ray's best t as known at the start
// of the pass (the ray's extent in the first pass).  When the chunk is full
// the ray parks: its key, postponed bits and node are saved and the next
// pass resumes it.
//
// k_resolve replays the reference's leaf callbacks over the chunk in order: a
// patch whose leaf box starts at or beyond the object's current best t is
// skipped (the reference's `L0 < hit.t` test), any other runs the
// Bezier-clipping search with the current best as hit.distance
// (doBezierClipping, src/Spline_BezierClipping.cu:46-114) and keeps a
// strictly closer hit; leaving an object keeps its hit if it beats the world
// best.  A subtree the reference culls lies behind its box entry, at or
// beyond the best t of that moment, so none of its patches can give a
// strictly closer hit; collecting it anyway changes nothing except for hits
// within the search tolerance of the current best (near-ties).  Any-hit
// queries stop at the first patch that reports a hit; at the end of an
// any-hit launch, lanes without rays share the pending intervals of the long
// searches left in their warp.
//
// Both kernels refill lanes one ray (k_collect) or one clip iteration
// (k_resolve) at a time, so heavy-tailed per-ray work does not idle the other
// lanes of a warp, and take rays in id order so a warp's rays stay coherent.
// Rays still unfinished after the configured number of passes are completed
// by k_rest, the inline version of the same search.  Block sizes, grid
// occupancy and the pass count are runtime settings (EngineConfig), chosen by
// the autotuner (cgs_autotune) or set by the caller.
#include <algorithm>
#include <mutex>

#include "kernels.h"

namespace cgs {

namespace {

constexpr int kCollectThreads = 256;   // launch bound; runtime block size 128 or 256
constexpr int kResolveThreads = 128;   // launch bound; runtime block size 64 or 128
constexpr uint32_t kChunk = 64;        // list entries per ray and pass (the most; EngineConfig::queueChunk is the first pass's)
// One collect step appends at most two entries: a leaf's first patch and,
// when that patch ends the leaf and nothing is postponed inside the object,
// the marker that leaves the object.
constexpr uint32_t kMaxAppendsPerStep = 2;
// Backtrack cache: the node indices of the last kRing postponed siblings of
// each lane's ray, in a ring in shared memory.
constexpr uint32_t kRing = 8;
constexpr int kMaxPasses = 8;

// list entry word 0: a patch index, or one of these markers (word 1 = object)
constexpr uint32_t kLeave = 0xFFFFFFFFu, kEnter = 0xFFFFFFFEu, kCont = 0xFFFFFFFDu;
// ray status
enum : uint32_t { kPending = 0, kTraversed = 1, kFinished = 2 };

struct Eng  // per-ray engine state, SoA over the query's capacity
{
    uint32_t *status, *count;
    uint2* list;  // [cap * kChunk]
    uint32_t *node, *key, *post, *leaf, *tnode, *tkey, *tpost, *tleaf, *jumped;
    int32_t *obj, *lpatch;
    float *leafEntry, *limit, *lt, *lu, *lv;
    // the rays to walk in pass p >= 1 (those that parked in pass p - 1) are
    // queue[p & 1][0 .. ctl[4p + 2]); the rays still parked after the last
    // pass P, for the inline fallback, are queue[P & 1][0 .. ctl[4P + 2]).
    // k_pending builds each in ray order, 256 rays at a time.
    uint32_t* queue[2];
    uint32_t* ctl;  // per pass: collect fetch, resolve fetch, length of the pass's queue
    uint32_t chunk;        // list entries a ray may fill in the first pass; each later pass doubles it (<= kChunk)
    uint32_t packetWidth;  // idle lanes a warp gathers before the traversal refills it
    uint32_t originLast;   // any hit: search candidates whose leaf box holds the ray's origin last
    uint32_t subdivLevels; // subdivision searches: bisection levels a lane runs per resolve round
};

constexpr size_t kWordsPerRay = 2 + 2 * kChunk + 18;

Eng carve(uint32_t* base, uint32_t cap)
{
    Eng e;
    uint32_t* p = base;
    auto take = [&](size_t words) { uint32_t* r = p; p += words; return r; };
    e.status = take(cap); e.count = take(cap);
    e.list = reinterpret_cast<uint2*>(take(2ull * cap * kChunk));
    e.node = take(cap); e.key = take(cap); e.post = take(cap); e.leaf = take(cap); e.tnode = take(cap);
    e.tkey = take(cap); e.tpost = take(cap); e.tleaf = take(cap); e.jumped = take(cap);
    e.obj = reinterpret_cast<int32_t*>(take(cap)); e.lpatch = reinterpret_cast<int32_t*>(take(cap));
    e.leafEntry = reinterpret_cast<float*>(take(cap)); e.limit = reinterpret_cast<float*>(take(cap));
    e.lt = reinterpret_cast<float*>(take(cap)); e.lu = reinterpret_cast<float*>(take(cap));
    e.lv = reinterpret_cast<float*>(take(cap));
    e.queue[0] = take(cap); e.queue[1] = take(cap);
    e.ctl = take(4 * (kMaxPasses + 1));
    return e;
}

// The BVH a lane walks: its index in the scene's BVH table and the two bases
// every step uses.
struct BvhRef { uint32_t idx, nodeBase, indexBase; bool compressed; };

__device__ __forceinline__ BvhRef bvh_ref(const DevScene& S, uint32_t idx)
{
    return BvhRef {idx, __ldg(&S.bvhs[idx].nodeBase), __ldg(&S.bvhs[idx].indexBase),
                   __ldg(&S.bvhs[idx].compressed) != 0};
}

// Warp-wide refill: every lane in `need` gets the next index from *fetch.
// width > 1: the warp waits until at least `width` of its lanes need one (or
// none is busy) and then refills them together: rays enter the warp in
// packets, which keeps its lanes at similar depths of similar walks.
__device__ __forceinline__ uint32_t warp_fetch(uint32_t* fetch, bool need, uint32_t width = 1, bool busy = false)
{
    unsigned m = __ballot_sync(0xFFFFFFFFu, need);
    if (!m) return EMPTY;
    if (width > 1 && uint32_t(__popc(m)) < width && __ballot_sync(0xFFFFFFFFu, busy)) return EMPTY;
    int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if ((int)lane_id() == leader) base = atomicAdd(fetch, (uint32_t)__popc(m));
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    unsigned lt = (1u << lane_id()) - 1u;
    return need ? base + __popc(m & lt) : EMPTY;
}

__device__ __forceinline__ void load_ray(const RaysSoA& r, uint32_t i, float3& o, float3& d, float& tmax)
{
    o = f3(r.ox[i], r.oy[i], r.oz[i]);
    d = f3(r.dx[i], r.dy[i], r.dz[i]);
    tmax = r.tmax ? r.tmax[i] : INFINITY;
}

// ------------------------------------------------------------ collect --
//
// A backtrack goes to the sibling postponed deepest on the current path: the
// one postponed last.  With the backtrack cache on, a step that postpones a
// sibling also pushes its node index on the lane's ring, and a backtrack pops
// it from there while it is still in the ring; otherwise (the ring held more
// than kRing postponed siblings, or the ray was parked since) it looks the
// sibling's key up in the perfect hash as BVH::hashIntersect does.  Both give
// the same node.  `rvalid` counts the entries at the top of the ring that are
// still intact; an object's traversal nests inside the object level's on the
// same ring, since it leaves the object only with nothing postponed.
//
// kQ: read the 32-byte compressed node mirror (one 256-bit load; child boxes
// on an 8-bit grid, widened outward) instead of the exact 64-byte records.
// The decoded boxes contain the exact ones, so the walk meets every leaf the
// exact walk meets (and a few more), with leaf entries no later: the list
// holds the same patches plus some the resolve step then clips or culls.
template<bool kAny, bool kQ>
__global__ void __launch_bounds__(kCollectThreads, 4) k_collect(DevScene S, RaysSoA rays, uint32_t n0,
                                                                const uint32_t* nDev, Eng E, int pass, int cache,
                                                                Counters* cnt)
{
    // entry s of this lane's ring at ring[s * blockDim.x + threadIdx.x]; the
    // ring's state packs its top slot (bits 0-2) with `rvalid` (bits 3-6)
    __shared__ uint32_t ring[kRing * kCollectThreads];
    uint32_t rstate = 0;
    const uint32_t n = nDev ? *nDev : n0;
    LocalCounters lc;
    bool active = false, exhausted = false, jumped = false;
    uint32_t rid = 0, ncand = 0;
    // o, inv, limit: the world ray and its culling bound; co, ci, clim: those
    // of the level walked now (the world's, or the object's local ray and
    // best t), switched where the ray enters or leaves an object
    float3 o = f3(0, 0, 0), inv = f3(0, 0, 0), co = f3(0, 0, 0), ci = f3(0, 0, 0);
    float tmax = 0, limit = 0, clim = 0;
    uint32_t node = 0, key = 1, post = 0, leaf = EMPTY, tnode = 0, tkey = 1, tpost = 0, tleaf = EMPTY;
    float leafEntry = -INFINITY;
    int32_t obj = -1;
    uint32_t topIdx = 0;  // the ray's object-level BVH (its group's)
    BvhRef B {};  // the BVH walked now; its hash parameters are read at a table lookup
    uint32_t nrays = 0;
    uint2* list = nullptr;
    // pass 0 walks every ray; a later pass only the queue of rays that parked
    const uint32_t m = pass == 0 ? n : E.ctl[4 * pass + 2];
    const uint32_t* queue = E.queue[pass & 1];
    for (;;)
    {
        const bool need = !active && !exhausted;
        // a lane the packet rule holds back gets EMPTY (ray counts stay below 2^31)
        const uint32_t idx = warp_fetch(E.ctl + 4 * pass, need, E.packetWidth, active);
        if (need && idx != EMPTY)
        {
            const uint32_t r = idx < m ? (pass == 0 ? idx : queue[idx]) : 0u;
            if (idx >= m)
                exhausted = true;
            else if (pass == 0 && rays.group && __ldg(rays.group + r) >= S.ngroups)
            {
                // a group outside the store: the ray stays a miss and raises an error bit
                lc.errors |= kErrGroup;
                E.count[r] = 0;
                E.status[r] = kTraversed;
            }
            else if (pass == 0 || E.status[r] == kPending)
            {
                rid = r;
                const uint32_t g = rays.group ? __ldg(rays.group + rid) : 0u;
                active = true;
                float3 d;
                load_ray(rays, rid, o, d, tmax);
                inv = f3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
                list = E.list + size_t(rid) * kChunk;
                ncand = 0;
                rstate = 0;
                topIdx = __ldg(S.groupTop + g);
                if (pass == 0)
                {
                    node = 0; key = 1; post = 0; leaf = EMPTY; obj = -1; jumped = false;
                    leafEntry = -INFINITY; limit = tmax;
                    co = o; ci = inv; clim = limit;
                    B = bvh_ref(S, topIdx);
                    nrays++;
                }
                else
                {
                    node = E.node[rid]; key = E.key[rid]; post = E.post[rid]; leaf = E.leaf[rid];
                    jumped = E.jumped[rid] != 0; leafEntry = E.leafEntry[rid]; obj = E.obj[rid];
                    limit = kAny ? tmax : E.limit[rid];
                    co = o; ci = inv; clim = limit;
                    B = bvh_ref(S, topIdx);
                    if (obj >= 0)
                    {
                        tnode = E.tnode[rid]; tkey = E.tkey[rid]; tpost = E.tpost[rid]; tleaf = E.tleaf[rid];
                        const DevObject& O = S.objects[obj];
                        float3 ld; float sinv, lmax;
                        to_local(O, o, d, tmax, co, ld, lmax, sinv);
                        ci = f3(1.0f / ld.x, 1.0f / ld.y, 1.0f / ld.z);
                        clim = kAny ? lmax : E.lt[rid];
                        B = bvh_ref(S, O.surface);
                        list[ncand++] = make_uint2(kCont, uint32_t(obj));
                    }
                }
            }
        }
        if (__ballot_sync(0xFFFFFFFFu, active || !exhausted) == 0) break;
        if (!active) continue;

        if (ncand + kMaxAppendsPerStep > min(kChunk, E.chunk << pass))
        {
            // no room for what one step may append: park before this step
            E.node[rid] = node; E.key[rid] = key; E.post[rid] = post; E.leaf[rid] = leaf;
            E.jumped[rid] = jumped; E.leafEntry[rid] = leafEntry; E.obj[rid] = obj;
            E.tnode[rid] = tnode; E.tkey[rid] = tkey; E.tpost[rid] = tpost; E.tleaf[rid] = tleaf;
            E.count[rid] = ncand;
            E.status[rid] = kPending;
            active = false;
            continue;
        }

        bool ascend = false, done = false;
        if (leaf != EMPTY)
        {
            const uint32_t e = __ldg(S.indices + B.indexBase + leaf);
            if (e != EMPTY)
            {
                leaf++;
                if (obj < 0)
                {
                    // descend into object e (Context::intersect's callback)
                    tnode = node; tkey = key; tpost = post; tleaf = leaf;
                    obj = int32_t(e);
                    const DevObject& O = S.objects[e];
                    const float3 d = f3(rays.dx[rid], rays.dy[rid], rays.dz[rid]);
                    float3 ld; float sinv;
                    to_local(O, o, d, tmax, co, ld, clim, sinv);
                    ci = f3(1.0f / ld.x, 1.0f / ld.y, 1.0f / ld.z);
                    B = bvh_ref(S, O.surface);
                    node = 0; key = 1; post = 0; leaf = EMPTY; jumped = false;
                    leafEntry = -INFINITY;
                    list[ncand++] = make_uint2(kEnter, e);
                }
                else
                    list[ncand++] = make_uint2(e, __float_as_uint(leafEntry));
            }
            else
            {
                leaf = EMPTY;
                ascend = true;
            }
        }
        else
        {
            // the node: its compressed record (one 256-bit load) where the BVH
            // has them, else the exact 64-byte record (two); the box tests of
            // an inner node's children, or of a leaf's own box when the leaf
            // was reached through a backtrack
            const float3 ro = co, ri = ci;
            uint32_t left, right;
            float L0 = 0.0f, R0 = 0.0f;
            bool mL = false, mR = false;
            if (kQ && B.compressed)
            {
                uint4 qa, qb;
                ldg256u(S.qnodes + 2ull * (B.nodeBase + node), qa, qb);
                const bool isLeaf = ((qa.w >> 24) & kQNodeLeaf) != 0;
                left = isLeaf ? EMPTY : node + 1;
                right = qb.w;
                if (!isLeaf || jumped) qslab2(qa, qb, ro, ri, L0, mL, R0, mR);
            }
            else
            {
                const float4* q = S.nodes + 4ull * (B.nodeBase + node);
                float4 q0, q1, q2, q3;
                ldg256(q, q0, q1);
                ldg256(q + 2, q2, q3);
                left = __float_as_uint(q3.x);
                right = __float_as_uint(q3.y);
                if (left != EMPTY || jumped) mL = slab(L0, f3(q0.x, q0.y, q0.z), f3(q0.w, q1.x, q1.y), ro, ri);
                if (left != EMPTY) mR = slab(R0, f3(q1.z, q1.w, q2.x), f3(q2.y, q2.z, q2.w), ro, ri);
            }
            if (left == EMPTY)
            {
                // reached through a backtrack: its entry is the slab test of its own box
                if (jumped) leafEntry = L0;
                jumped = false;
                // the leaf's first element and the one after it in the same step: a
                // one-element leaf (the build's element count per leaf) is done here
                const uint32_t e0 = __ldg(S.indices + B.indexBase + right);
                const uint32_t e1 = __ldg(S.indices + B.indexBase + right + 1);
                leaf = right + 1;
                if (e0 == EMPTY)
                {
                    leaf = EMPTY;
                    ascend = true;
                }
                else if (obj < 0)
                {
                    // descend into object e0 (Context::intersect's callback)
                    tnode = node; tkey = key; tpost = post; tleaf = leaf;
                    obj = int32_t(e0);
                    const DevObject& O = S.objects[e0];
                    const float3 d = f3(rays.dx[rid], rays.dy[rid], rays.dz[rid]);
                    float3 ld; float sinv;
                    to_local(O, o, d, tmax, co, ld, clim, sinv);
                    ci = f3(1.0f / ld.x, 1.0f / ld.y, 1.0f / ld.z);
                    B = bvh_ref(S, O.surface);
                    node = 0; key = 1; post = 0; leaf = EMPTY; jumped = false;
                    leafEntry = -INFINITY;
                    list[ncand++] = make_uint2(kEnter, e0);
                }
                else
                {
                    list[ncand++] = make_uint2(e0, __float_as_uint(leafEntry));
                    if (e1 == EMPTY)
                    {
                        leaf = EMPTY;
                        ascend = true;
                    }
                }
            }
            else
            {
                lc.nodes++;
                jumped = false;
                const float lim = clim;
                const bool iL = mL && L0 < lim;
                const bool iR = mR && R0 < lim;
                if (iL || iR) post <<= 1;
                if (iL && iR)
                {
                    post |= 1u;
                    uint32_t other;
                    if (L0 < R0) { key = key << 1; node = left; leafEntry = L0; other = right; }
                    else { key = (key << 1) ^ 1u; node = right; leafEntry = R0; other = left; }
                    if (cache)
                    {
                        const uint32_t top = (rstate + 1u) & (kRing - 1u);
                        ring[top * blockDim.x + threadIdx.x] = other;
                        rstate = top | (min((rstate >> 3) + 1u, kRing) << 3);
                    }
                }
                else if (iL) { key = key << 1; node = left; leafEntry = L0; }
                else if (iR) { key = (key << 1) ^ 1u; node = right; leafEntry = R0; }
                else ascend = true;
            }
        }
        if (ascend)
        {
            if (post == 0)
            {
                if (obj < 0)
                    done = true;
                else
                {
                    list[ncand++] = make_uint2(kLeave, uint32_t(obj));
                    obj = -1;
                    co = o; ci = inv; clim = limit;
                    B = bvh_ref(S, topIdx);
                    node = tnode; key = tkey; post = tpost; leaf = tleaf;
                    leafEntry = -INFINITY;
                }
            }
            else
            {
                const int levels = __ffs(post) - 1;
                post >>= levels;
                key = (key >> levels) ^ 1u;
                post ^= 1u;
                lc.hashLookups++;
                if (rstate >= kRing)
                {
                    const uint32_t top = rstate & (kRing - 1u);
                    node = ring[top * blockDim.x + threadIdx.x];
                    rstate = ((top - 1u) & (kRing - 1u)) | (rstate - kRing) >> 3 << 3;
                }
                else
                {
                    lc.tableReads++;
                    const DevBVH H = S.bvhs[B.idx];
                    node = __ldg(S.tables + H.tableBase + hash_slot(S, H, key));
                }
                jumped = true;
            }
        }
        if (done)
        {
            E.count[rid] = ncand;
            E.status[rid] = kTraversed;
            active = false;
        }
    }
    flush_counters(cnt, lc, nrays);
}

// ------------------------------------------------------------ resolve --
// kG64: the search may take the FP64 grazing path (precision levels 3 and 5);
// the other levels run an instance without that code.  kSub: the searches
// are the subdivision method's (a separate instance, so that the clipping
// instances' loop holds no subdivision code; at the grazing levels the kG64
// instance runs subdivision searches whole instead).  The FP32 clipping
// instances are held to 128 registers, four 128-thread blocks per SM.
template<bool kAny, bool kG64, bool kSub = false>
__global__ void __launch_bounds__(kResolveThreads, (!kG64 && !kSub) ? 4 : 3) k_resolve(DevScene S, RaysSoA rays, uint32_t n0,
                                                             const uint32_t* nDev, Eng E, int pass, Query q,
                                                             HitsSoA hits, int32_t* occluded, Counters* cnt)
{
    const uint32_t n = nDev ? *nDev : n0;
    LocalCounters lc;
    float4 stack[kClipStack];
    volatile double ray64[6];  // kG64: a near-grazing search's ray in double
    ClipState c;
    HitSink sink {nullptr, f3(0, 0, 0), f3(0, 0, 1), 0.0f, make_float2(0, 0)};
    bool active = false, exhausted = false, clipping = false;
    bool thief = false;  // any hit: the lane searches an interval taken from another lane's search
    // any hit with E.originLast: sweep 0 searches the candidates whose leaf box
    // holds the ray's origin (entry <= 0) not, sweep 1 only those
    bool sweep = false;
    uint32_t rid = 0, k = 0, count = 0, patch = 0;
    int32_t obj = -1, lpatch = -1;
    float3 o = f3(0, 0, 0), d = f3(0, 0, 1);
    float tmax = 0, lmax = 0, sinv = 1, lt = 0, lu = 0, lv = 0, limit = 0;
    const uint2* list = nullptr;
    // pass 0 resolves every ray; a later pass the rays its traversal walked
    const uint32_t m = pass == 0 ? n : E.ctl[4 * pass + 2];
    const uint32_t* queue = E.queue[pass & 1];
    for (;;)
    {
        const bool need = !active && !exhausted;
        const uint32_t idx = warp_fetch(E.ctl + 4 * pass + 1, need);
        if (need)
        {
            if (idx >= m)
                exhausted = true;
            else
            {
                const uint32_t r = pass == 0 ? idx : queue[idx];
                const uint32_t st = E.status[r];
                count = E.count[r];
                if (count > 0 && st != kFinished)
                {
                    rid = r;
                    active = true;
                    k = 0;
                    obj = -1;
                    clipping = false;
                    sweep = false;
                    load_ray(rays, rid, o, d, tmax);
                    limit = kAny ? tmax : (pass == 0 ? tmax : E.limit[rid]);
                    list = E.list + size_t(rid) * kChunk;
                }
            }
        }
        if (__ballot_sync(0xFFFFFFFFu, active || !exhausted) == 0) break;
        if constexpr (kAny && !kSub && !kG64)
        {
            // The tail of an any-hit launch is a few long searches.  A lane
            // left without rays takes the bottom (largest) pending interval of
            // a search in its warp that holds one or more, and searches it as
            // that search would after popping it: the same sub-net, derived
            // from the projected net, and the same cut side.  The searched
            // intervals are the same, so the roots found are; an any-hit
            // answer needs one of them, and whichever lane finds it marks
            // the ray occluded (writes of "occluded" never clear it).
            const unsigned idleM = __ballot_sync(0xFFFFFFFFu, exhausted && !active);
            const unsigned richM = __ballot_sync(0xFFFFFFFFu, clipping && !c.fresh && c.sl >= 1 && c.sl <= 30);
            if (idleM && richM)
            {
                const unsigned lane = lane_id(), below = (1u << lane) - 1u;
                const int pairs = min(__popc(idleM), __popc(richM));
                const int idleRank = __popc(idleM & below), richRank = __popc(richM & below);
                const bool isThief = ((idleM >> lane) & 1u) && idleRank < pairs;
                const bool isVictim = ((richM >> lane) & 1u) && richRank < pairs;
                const int src = isThief ? int(__fns(richM, 0, idleRank + 1)) : int(lane);
                float4 e = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                int bit = 0;
                if (isVictim)
                {
                    // entry i's cut side is bit (sl - i) of the bit stack; the
                    // bits above the bottom entry's are clear
                    e = stack[0];
                    bit = (c.cutsideStack >> c.sl) & 1;
                    c.cutsideStack &= ~(1 << c.sl);
                    for (int i = 1; i < c.sl; i++) stack[i - 1] = stack[i];
                    c.sl--;
                }
                const float4 se = make_float4(__shfl_sync(0xFFFFFFFFu, e.x, src), __shfl_sync(0xFFFFFFFFu, e.y, src),
                                              __shfl_sync(0xFFFFFFFFu, e.z, src), __shfl_sync(0xFFFFFFFFu, e.w, src));
                const int sbit = __shfl_sync(0xFFFFFFFFu, bit, src);
                const uint32_t srid = __shfl_sync(0xFFFFFFFFu, rid, src);
                const unsigned long long sp =
                    __shfl_sync(0xFFFFFFFFu, (unsigned long long)reinterpret_cast<uintptr_t>(sink.P), src);
                const float3 so = f3(__shfl_sync(0xFFFFFFFFu, sink.o.x, src), __shfl_sync(0xFFFFFFFFu, sink.o.y, src),
                                     __shfl_sync(0xFFFFFFFFu, sink.o.z, src));
                const float3 sd = f3(__shfl_sync(0xFFFFFFFFu, sink.d.x, src), __shfl_sync(0xFFFFFFFFu, sink.d.y, src),
                                     __shfl_sync(0xFFFFFFFFu, sink.d.z, src));
                const float sdist = __shfl_sync(0xFFFFFFFFu, sink.dist, src);
                const float stol = __shfl_sync(0xFFFFFFFFu, c.tol, src);
                if (isThief)
                {
                    rid = srid;
                    sink.P = reinterpret_cast<const float4*>(uintptr_t(sp));
                    sink.o = so; sink.d = sd; sink.dist = sdist; sink.uv = make_float2(0.0f, 0.0f);
                    c.emin = make_float2(se.x, se.y);
                    c.emax = make_float2(se.z, se.w);
                    c.cutsideStack = sbit; c.sl = 0; c.it = 0; c.tol = stol;
                    c.found = false; c.b64 = false; c.fresh = false; c.tposed = false;
                    project_net(c.buf, sink.P, sink.o, sink.d);
                    subpatchU(c.buf, se.x, se.z);
                    subpatchV(c.buf, se.y, se.w);
                    active = true; clipping = true; thief = true;
                }
            }
        }
        if (!active) continue;

        bool finished = false;
        // A lane without a search in progress walks its list -- object
        // markers, patches culled by their leaf entry -- until it starts the
        // next search or its chunk ends, so that the clip steps below run with
        // as many lanes as possible.
        while (!clipping && !finished)
        {
            if (kAny && k >= count && E.originLast && !sweep)
            {
                sweep = true;  // the candidates whose leaf box holds the origin, last
                k = 0;
                obj = -1;
                continue;
            }
            if (k >= count)
            {
                // end of this pass's chunk: keep what the next pass needs
                if (!kAny)
                {
                    E.limit[rid] = limit;
                    if (obj >= 0) { E.lt[rid] = lt; E.lu[rid] = lu; E.lv[rid] = lv; E.lpatch[rid] = lpatch; }
                }
                finished = true;
                break;
            }
            const uint2 e = list[k++];
            if (e.x == kEnter || e.x == kCont)
            {
                obj = int32_t(e.y);
                float3 ld;
                to_local(S.objects[obj], o, d, tmax, sink.o, ld, lmax, sinv);
                sink.d = ld;
                if (e.x == kEnter || kAny) { lt = lmax; lpatch = -1; lu = 0.0f; lv = 0.0f; }
                else { lt = E.lt[rid]; lu = E.lu[rid]; lv = E.lv[rid]; lpatch = E.lpatch[rid]; }
            }
            else if (e.x == kLeave)
            {
                if (!kAny && lpatch >= 0)
                {
                    const float t = lt * sinv;
                    if (t < limit)
                    {
                        limit = t;
                        hits.t[rid] = t; hits.u[rid] = lu; hits.v[rid] = lv;
                        hits.patch[rid] = lpatch; hits.object[rid] = obj;
                    }
                }
                obj = -1;
            }
            else
            {
                patch = e.x;
                const float entry = __uint_as_float(e.y);
                const bool turn = !kAny || !E.originLast || ((entry <= 0.0f) == sweep);
                if (turn && entry < (kAny ? lmax : lt))
                {
                    const uint32_t surface = S.objects[obj].surface;
                    sink.P = S.patches + 16ull * (__ldg(S.patchBase + surface) + patch);
                    sink.dist = kAny ? lmax : lt;
                    sink.uv = kAny ? make_float2(0.0f, 0.0f) : make_float2(lu, lv);
                    lc.candidates++;
                    if (kSub) subdiv_begin(c, sink, q.tol);
                    else if (!(kG64 && q.method != 0))
                        clip_begin<kG64>(c, sink, q.tol, graze_sin(q.precision), ray64, &S.objects[obj], o, d);
                    clipping = true;
                }
            }
        }
        if (clipping)
        {
            bool found = false, more = false;
            if (kG64 && q.method != 0)
            {
                // the precision form's subdivision searches run whole, one call each
                found = subdiv_patch(sink, q.tol, lc);
            }
            else if (!kSub)
            {
                more = clip_step<kG64>(c, stack, sink, lc, ray64);
                found = c.found;
                if (kAny && found) more = false;  // an any-hit search ends at its first root
            }
            else
            {
                more = subdiv_step(c, sink, lc, int(E.subdivLevels));
                found = c.found;
                if (kAny && found) more = false;
            }
            if (!more)
            {
                clipping = false;
                if (kAny)
                {
                    if (found) { occluded[rid] = 0; E.status[rid] = kFinished; finished = true; }
                }
                else if (found)
                {
                    lt = sink.dist; lu = sink.uv.x; lv = sink.uv.y; lpatch = int32_t(patch);
                }
            }
        }
        if (finished)
        {
            active = false;
            E.count[rid] = 0;
        }
        if (kAny && thief && !clipping)
        {
            thief = false;
            active = false;
        }
    }
    flush_counters(cnt, lc, 0);
}

// Rays unfinished after the last pass: the inline search from the start.
template<bool kAny>
__global__ void __launch_bounds__(128) k_rest(DevScene S, RaysSoA rays, Eng E, int passes, Query q, HitsSoA hits,
                                              int32_t* occluded, Counters* cnt)
{
    // the rays still parked after the last pass
    const uint32_t m = E.ctl[4 * passes + 2];
    const uint32_t* queue = E.queue[passes & 1];
    LocalCounters lc;
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
    for (uint32_t i = tid; i < m; i += nt)
    {
        const uint32_t rid = queue[i];
        if (E.status[rid] != kPending) continue;
        float3 o, d; float tmax;
        load_ray(rays, rid, o, d, tmax);
        Query q32 = q;
        q32.precision = search_only(q.precision);  // the polish kernel runs afterwards
        const uint32_t g = rays.group ? rays.group[rid] : 0u;
        if (g >= S.ngroups) continue;
        if (kAny)
            occluded[rid] = scene_any(S, g, o, d, tmax, q32, lc) ? 0 : -1;
        else
        {
            HitRecord h {tmax, 0.0f, 0.0f, -1, -1};
            int ob = scene_closest(S, g, o, d, tmax, q32, h, lc);
            hits.t[rid] = ob >= 0 ? h.t : tmax; hits.u[rid] = h.u; hits.v[rid] = h.v;
            hits.patch[rid] = ob >= 0 ? h.patch : -1; hits.object[rid] = ob;
        }
    }
    flush_counters(cnt, lc, 0);
}

// The queue of parked rays for the next pass, in ray order within each tile
// of 256 rays (the tiles' slices land in the order their blocks claim them),
// so that a packet of consecutive queue positions holds neighbouring rays.
constexpr int kPendingThreads = 256;
__global__ void __launch_bounds__(kPendingThreads) k_pending(const uint32_t* __restrict__ status, uint32_t n0,
                                                             const uint32_t* nDev, uint32_t* queue, uint32_t* len)
{
    const uint32_t n = nDev ? *nDev : n0;
    __shared__ uint32_t offset[kPendingThreads / 32];
    __shared__ uint32_t base;
    const uint32_t w = threadIdx.x / 32, lane = threadIdx.x % 32;
    for (uint32_t t0 = blockIdx.x * kPendingThreads; t0 < n; t0 += gridDim.x * kPendingThreads)
    {
        const uint32_t i = t0 + threadIdx.x;
        const bool p = i < n && status[i] == kPending;
        const unsigned m = __ballot_sync(0xFFFFFFFFu, p);
        if (lane == 0) offset[w] = __popc(m);
        __syncthreads();
        if (threadIdx.x == 0)
        {
            uint32_t sum = 0;
            for (uint32_t k = 0; k < kPendingThreads / 32; k++)
            {
                const uint32_t c = offset[k];
                offset[k] = sum;
                sum += c;
            }
            base = sum ? atomicAdd(len, sum) : 0u;
        }
        __syncthreads();
        if (p) queue[base + offset[w] + __popc(m & ((1u << lane) - 1u))] = i;
        __syncthreads();
    }
}

__global__ void k_init(RaysSoA rays, uint32_t n0, const uint32_t* nDev, HitsSoA hits, int32_t* occluded, Eng E)
{
    const uint32_t n = nDev ? *nDev : n0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        E.count[i] = 0;
        if (occluded) { occluded[i] = -1; continue; }
        hits.t[i] = rays.tmax ? rays.tmax[i] : INFINITY;
        hits.u[i] = 0.0f; hits.v[i] = 0.0f; hits.patch[i] = -1; hits.object[i] = -1;
    }
}

// One polish per hit.  A warp gathers the hits of the rays it sweeps into a
// shared-memory list and polishes them 32 at a time, so that its FP64
// instructions run with full lanes where misses are scattered among hits
// (the FP64 pipe takes a warp instruction whatever its active lanes).
constexpr int kPolishThreads = 128;
__device__ __forceinline__ void polish_ray(const DevScene& S, const RaysSoA& rays, HitsSoA& hits, uint32_t i)
{
    HitRecord h {hits.t[i], hits.u[i], hits.v[i], hits.patch[i], hits.object[i]};
    polish_hit(S, f3(rays.ox[i], rays.oy[i], rays.oz[i]), f3(rays.dx[i], rays.dy[i], rays.dz[i]), h);
    hits.t[i] = h.t; hits.u[i] = h.u; hits.v[i] = h.v;
}
__global__ void __launch_bounds__(kPolishThreads) k_polish(DevScene S, RaysSoA rays, uint32_t n0,
                                                           const uint32_t* nDev, HitsSoA hits)
{
    const uint32_t n = nDev ? *nDev : n0;
    __shared__ uint32_t pend[kPolishThreads / 32][64];
    uint32_t* my = pend[threadIdx.x / 32];
    const uint32_t lane = threadIdx.x % 32;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) / 32, nwarps = gridDim.x * blockDim.x / 32;
    uint32_t cnt = 0;  // warp-uniform
    for (uint32_t base = warp * 32; base < n; base += nwarps * 32)
    {
        const uint32_t i = base + lane;
        const bool hit = i < n && hits.object[i] >= 0;
        const unsigned m = __ballot_sync(0xFFFFFFFFu, hit);
        if (hit) my[cnt + __popc(m & ((1u << lane) - 1u))] = i;
        cnt += __popc(m);
        __syncwarp();
        if (cnt >= 32)
        {
            polish_ray(S, rays, hits, my[lane]);
            cnt -= 32;
            const uint32_t rest = lane < cnt ? my[32 + lane] : 0u;
            __syncwarp();
            if (lane < cnt) my[lane] = rest;
            __syncwarp();
        }
    }
    if (lane < cnt) polish_ray(S, rays, hits, my[lane]);
}

int sms()
{
    static const int v = [] {
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        return n > 0 ? n : 1;
    }();
    return v;
}

int resident(const void* fn, int threads)
{
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, threads, 0);
    return sms() * (per > 0 ? per : 1);
}

// Resident blocks per SM of kernel fn at `threads` per block (cached: the
// values depend only on the kernel and the block size).
template<bool kAny, bool kG64, bool kSub = false> int per_sm(bool collect, int threads, bool compressed = true)
{
    static const int v[3][2] = {
        {resident((const void*)k_collect<kAny, false>, 128) / sms(),
         resident((const void*)k_collect<kAny, false>, 256) / sms()},
        {resident((const void*)k_resolve<kAny, kG64, kSub>, 64) / sms(),
         resident((const void*)k_resolve<kAny, kG64, kSub>, 128) / sms()},
        {resident((const void*)k_collect<kAny, true>, 128) / sms(),
         resident((const void*)k_collect<kAny, true>, 256) / sms()}};
    return collect ? v[compressed ? 2 : 0][threads == 256] : v[1][threads == 128];
}

template<bool kAny>
void launch_collect(int grid, int threads, cudaStream_t stream, const DevScene& S, RaysSoA rays, uint32_t n,
                    const uint32_t* nDev, Eng E, int pass, const EngineConfig& c, Counters* cnt)
{
    if (c.compressedNodes)
        k_collect<kAny, true><<<grid, threads, 0, stream>>>(S, rays, n, nDev, E, pass, c.backtrackCache, cnt);
    else
        k_collect<kAny, false><<<grid, threads, 0, stream>>>(S, rays, n, nDev, E, pass, c.backtrackCache, cnt);
}

template<bool kAny, bool kG64, bool kSub = false>
void launch(const DevScene& S, RaysSoA rays, uint32_t n, const uint32_t* nDev, Query q, HitsSoA hits,
            int32_t* occluded, Eng E, Counters* cnt, cudaStream_t stream, int& nl)
{
    const EngineConfig c = engine_config();
    const int ct = c.collectThreads, rt = c.resolveThreads;
    const int pc = per_sm<kAny, kG64, kSub>(true, ct, c.compressedNodes != 0);
    const int pr = per_sm<kAny, kG64, kSub>(false, rt);
    const int cb = sms() * std::max(1, c.collectOccupancy ? std::min(c.collectOccupancy, pc) : pc);
    const int rb = sms() * std::max(1, c.resolveOccupancy ? std::min(c.resolveOccupancy, pr) : pr);
    const uint32_t warps = (n + 31) / 32;
    const int gc = int(std::min<uint32_t>(uint32_t(cb), warps / (ct / 32) + 1));
    const int gr = int(std::min<uint32_t>(uint32_t(rb), warps / (rt / 32) + 1));
    const int gp = int(std::min<uint32_t>(uint32_t(sms() * 8), (n + kPendingThreads - 1) / kPendingThreads));
    for (int p = 0; p < c.passes; p++)
    {
        if (p > 0)
        {
            k_pending<<<gp, kPendingThreads, 0, stream>>>(E.status, n, nDev, E.queue[p & 1], E.ctl + 4 * p + 2);
            nl++;
        }
        launch_collect<kAny>(gc, ct, stream, S, rays, n, nDev, E, p, c, cnt);
        k_resolve<kAny, kG64, kSub><<<gr, rt, 0, stream>>>(S, rays, n, nDev, E, p, q, hits, occluded, cnt);
        nl += 2;
    }
    k_pending<<<gp, kPendingThreads, 0, stream>>>(E.status, n, nDev, E.queue[c.passes & 1], E.ctl + 4 * c.passes + 2);
    k_rest<kAny><<<sms() * 4, 128, 0, stream>>>(S, rays, E, c.passes, q, hits, occluded, cnt);
    nl += 2;
}

}  // namespace

namespace {
std::mutex gConfigMu;
EngineConfig gConfig;
uint64_t gConfigGen = 1;
}  // namespace

EngineConfig engine_config()
{
    std::lock_guard<std::mutex> g(gConfigMu);
    return gConfig;
}

uint64_t engine_config_generation()
{
    std::lock_guard<std::mutex> g(gConfigMu);
    return gConfigGen;
}

bool valid_engine_config(const EngineConfig& c)
{
    return c.passes >= 1 && c.passes <= kMaxPasses && (c.collectThreads == 128 || c.collectThreads == 256) &&
           (c.resolveThreads == 64 || c.resolveThreads == 128) && c.collectOccupancy >= 0 && c.collectOccupancy <= 32 &&
           c.resolveOccupancy >= 0 && c.resolveOccupancy <= 32 && (c.backtrackCache == 0 || c.backtrackCache == 1) &&
           (c.compressedNodes == 0 || c.compressedNodes == 1) && c.queueChunk >= 4 &&
           c.queueChunk <= int(kChunk) && c.queueChunk % 4 == 0 && c.packetWidth >= 1 && c.packetWidth <= 32 &&
           (c.rayOrder == 0 || c.rayOrder == 1) && (c.originLast == 0 || c.originLast == 1) &&
           c.subdivLevels >= 1 && c.subdivLevels <= 64;
}

bool set_engine_config(const EngineConfig& c)
{
    if (!valid_engine_config(c)) return false;
    std::lock_guard<std::mutex> g(gConfigMu);
    gConfig = c;
    gConfigGen++;
    return true;
}

size_t engine_words(uint32_t capacity, int)
{
    return size_t(capacity) * kWordsPerRay + 4 * (kMaxPasses + 1) + 64;
}

cudaError_t run_query(const DevScene& S, RaysSoA rays, uint32_t n, const uint32_t* nDev, Query q, bool any,
                      HitsSoA hits, int32_t* occluded, uint32_t* scratch, uint32_t capacity, int, Counters* cnt,
                      cudaStream_t stream, int* launches)
{
    if (nDev) n = capacity;  // grid sizing only; kernels read *nDev
    if (n == 0) return cudaSuccess;
    if (n > capacity) return cudaErrorInvalidValue;
    if (any) q.precision = 0;  // any-hit searches run at level 0
    if (!any && q.precision == 2)
    {
        // the pure-FP64 search has no traversal / clip split
        if (launches) *launches += 1;
        return launch_query_fp64(S, rays, n, nDev, kTolFP64, hits, cnt, stream);
    }
    Eng E = carve(scratch, capacity);
    {
        const EngineConfig ec = engine_config();
        E.chunk = uint32_t(ec.queueChunk);
        E.packetWidth = uint32_t(ec.packetWidth);
        E.originLast = uint32_t(ec.originLast);
        E.subdivLevels = uint32_t(ec.subdivLevels);
    }
    cudaMemsetAsync(E.ctl, 0, sizeof(uint32_t) * 4 * (kMaxPasses + 1), stream);
    const int flat = sms() * 4;
    k_init<<<flat, 256, 0, stream>>>(rays, n, nDev, hits, any ? occluded : nullptr, E);
    int nl = 1;
    // the FP64 grazing instance serves both methods at its level (its
    // subdivision searches run whole); measured, it also runs the grazing
    // clip 35% faster with that one-call search compiled in (6.35 against
    // 4.72 Mrays/s on 2^20 grazing rays), a code-generation effect
    if (any) q.method != 0 ? launch<true, false, true>(S, rays, n, nDev, q, hits, occluded, E, cnt, stream, nl)
                           : launch<true, false>(S, rays, n, nDev, q, hits, occluded, E, cnt, stream, nl);
    else if (graze_sin(q.precision) > 0.0f) launch<false, true>(S, rays, n, nDev, q, hits, occluded, E, cnt, stream, nl);
    else if (q.method != 0) launch<false, false, true>(S, rays, n, nDev, q, hits, occluded, E, cnt, stream, nl);
    else launch<false, false>(S, rays, n, nDev, q, hits, occluded, E, cnt, stream, nl);
    if (!any && polishes(q.precision))
    {
        k_polish<<<flat * 2, kPolishThreads, 0, stream>>>(S, rays, n, nDev, hits);
        nl++;
    }
    if (launches) *launches += nl;
    return cudaGetLastError();
}

cudaError_t run_traverse(const DevScene& S, RaysSoA rays, uint32_t n, bool any, uint32_t* scratch, uint32_t capacity,
                         Counters* cnt, cudaStream_t stream, uint32_t* listLengths, int* launches)
{
    if (n == 0) return cudaSuccess;
    if (n > capacity) return cudaErrorInvalidValue;
    Eng E = carve(scratch, capacity);
    {
        const EngineConfig ec = engine_config();
        E.chunk = uint32_t(ec.queueChunk);
        E.packetWidth = uint32_t(ec.packetWidth);
        E.originLast = uint32_t(ec.originLast);
        E.subdivLevels = uint32_t(ec.subdivLevels);
    }
    cudaMemsetAsync(E.ctl, 0, sizeof(uint32_t) * 4 * (kMaxPasses + 1), stream);
    const EngineConfig c = engine_config();
    const int ct = c.collectThreads;
    const bool cq = c.compressedNodes != 0;
    const int pc = any ? per_sm<true, false>(true, ct, cq) : per_sm<false, false>(true, ct, cq);
    const int cb = sms() * std::max(1, c.collectOccupancy ? std::min(c.collectOccupancy, pc) : pc);
    const int gc = int(std::min<uint32_t>(uint32_t(cb), (n + 31) / 32 / (ct / 32) + 1));
    if (any) launch_collect<true>(gc, ct, stream, S, rays, n, nullptr, E, 0, c, cnt);
    else launch_collect<false>(gc, ct, stream, S, rays, n, nullptr, E, 0, c, cnt);
    if (launches) *launches += 1;
    if (listLengths) cudaMemcpyAsync(listLengths, E.count, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, stream);
    return cudaGetLastError();
}

}  // namespace cgs
