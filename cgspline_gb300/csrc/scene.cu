// scene.cu -- the scene store of libcgspline_gb300.so: surfaces, objects and
// groups, the host BVH build, device upload, the perfect-hash build of every
// BVH, and the C ABI entry points that build and inspect a store.
#include <atomic>
#include <bit>
#include <thread>
#include <cmath>
#include <numeric>
#include <random>

#include "scene_impl.h"

using namespace cgs;

namespace cgs {

// BVH::build / split / wrap (src/rt/BVH.cpp:9-108): top-down median split,
// heap keys (root 1, children 2k and 2k+1), nodes in pre-order, leaves keep
// their box in leftBox and an EMPTY-terminated element list.  The split axis
// comes from the size of a box that is never inflated (src/rt/BVH.cpp:46-52),
// i.e. an empty box whose three extents compare equal, which selects y; the
// partition is std::nth_element with the same comparator, so the topology
// matches the reference built with the same standard library.  With
// CGS_SPLIT_LONGEST the box is the elements' centroid box (the evident intent
// of that code): same rule, same partition, the longest axis.
uint32_t HostBVH::wrap(Element* e, size_t count, uint32_t key)
{
    if (count == 0) emptyLeaf = true;
    Box box;
    size_t idx = indices.size();
    indices.resize(idx + count + 1);
    for (size_t i = 0; i < count; i++) { indices[idx + i] = e[i].index; box.inflate(e[i].bounds); }
    indices[idx + count] = EMPTY;
    keys.push_back(key);
    nodes.push_back({box, Box {}, EMPTY, uint32_t(idx)});
    return uint32_t(nodes.size() - 1);
}

uint32_t HostBVH::split(Element* e, size_t count, uint32_t key)
{
    if (count <= perNode || (key & (1u << 31))) return wrap(e, count, key);
    Box box;
    if (split_mode == CGS_SPLIT_LONGEST)
        for (size_t i = 0; i < count; i++) box.inflate(e[i].centroid);
    float v[3] = {box.hi[0] - box.lo[0], box.hi[1] - box.lo[1], box.hi[2] - box.lo[2]};
    const int dim = v[2] > v[1] ? (v[0] > v[2] ? 0 : 2) : (v[0] > v[1] ? 0 : 1);
    size_t middle = count / 2;
    std::nth_element(e, e + middle, e + count,
                     [=](const Element& a, const Element& b) { return a.centroid[dim] < b.centroid[dim]; });
    keys.push_back(key);
    size_t idx = nodes.size();
    nodes.push_back({});
    uint32_t l = split(e, middle, key << 1);
    uint32_t r = split(e + middle, count - middle, (key << 1) ^ 1u);
    Node& node = nodes[idx];
    node.left = l;
    node.right = r;
    node.leftBox = nodes[l].leftBox;
    node.rightBox = nodes[r].leftBox;
    if (nodes[l].left != EMPTY) node.leftBox.inflate(nodes[l].rightBox);
    if (nodes[r].left != EMPTY) node.rightBox.inflate(nodes[r].rightBox);
    return uint32_t(idx);
}

void HostBVH::build(std::vector<Element>& el)
{
    nodes.clear(); keys.clear(); indices.clear(); emptyLeaf = false;
    nodes.reserve(2 * el.size()); keys.reserve(2 * el.size()); indices.reserve(2 * el.size());
    split(el.data(), el.size(), 1u);
}

// std::mt19937(42) with std::uniform_int_distribution<uint32_t>(0, n) and
// gcd(n, A) == 1 retries (src/rt/PerfectHashFunction.cu:379-400): the 16
// trials' coefficients.
void hash_coefficients(uint32_t n, uint32_t A[16], uint32_t B[16])
{
    std::mt19937 mt(42);
    std::uniform_int_distribution<uint32_t> d(0, n);
    for (int t = 0; t < 16; t++)
    {
        uint32_t a, b, cof;
        do
        {
            a = d(mt);
            if (a == 0) a = 31;
            b = d(mt);
            cof = std::gcd(n, a);
        } while (cof > 1);
        A[t] = a; B[t] = b;
    }
}

// Table capacity: n plus 15 growth steps of max(4, 5% of n)
// (src/rt/PerfectHashFunction.cu:249-251, 481).
uint32_t table_capacity(uint32_t n)
{
    uint32_t step = std::max<uint32_t>(4u, uint32_t(0.05f * float(n)));
    return n + 15u * step;
}

// Displacement table size: the power of two at or below max(2, (n-1)/2)
// (src/rt/PerfectHashFunction.cu:233-248).
uint32_t displ_size(uint32_t n)
{
    int s = int(n - 1) >> 1;
    if (s < 2) s = 2;
    return std::bit_floor(uint32_t(s));
}

}  // namespace cgs

namespace {

DevMaterial to_dev(const cgs_material& m)
{
    DevMaterial d;
    std::memcpy(&d, &m, sizeof d);
    return d;
}

// BezierSurface::buildBVH (src/rt/Primitive.cu:199-220): per-patch bounds of
// the 16 projected points and their mean as the centroid; `out` takes the
// tree (its split_mode set by the caller).
void build_surface_bvh(const Surface& s, HostBVH& out)
{
    std::vector<Element> el(s.patchCount());
    for (uint32_t i = 0; i < el.size(); i++)
    {
        Element& e = el[i];
        e.bounds = Box {};
        e.centroid[0] = e.centroid[1] = e.centroid[2] = 0.0f;
        e.index = i;
        const float inv = 1.0f / 16.0f;
        for (int j = 0; j < 16; j++)
        {
            const float* w = &s.points[4ull * s.indices[16ull * i + j]];
            float p[3] = {w[0] / w[3], w[1] / w[3], w[2] / w[3]};
            e.bounds.inflate(p);
            for (int k = 0; k < 3; k++) e.centroid[k] = e.centroid[k] + inv * p[k];
        }
    }
    out.build(el);
}

// Scene::buildBVH (src/rt/Scene.cu:218-232) for one group: object bounds of
// the transformed points (BezierSurface::bounds(M), src/rt/Primitive.cu:172-179),
// centroid = box centre, element index = the global object id.
void build_group_bvh(const cgs_scene* sc, const Group& g, HostBVH& out)
{
    std::vector<Element> el(g.objects.size());
    for (uint32_t i = 0; i < el.size(); i++)
    {
        const Object& ob = sc->objects[g.objects[i]];
        const Surface& s = sc->surfaces[ob.surface];
        const float* M = ob.l2w;
        Box b;
        for (uint32_t idx : s.indices)
        {
            const float* w = &s.points[4ull * idx];
            float x = ((w[0] * M[0] + w[1] * M[4]) + w[2] * M[8]) + w[3] * M[12];
            float y = ((w[0] * M[1] + w[1] * M[5]) + w[2] * M[9]) + w[3] * M[13];
            float z = ((w[0] * M[2] + w[1] * M[6]) + w[2] * M[10]) + w[3] * M[14];
            float ww = ((w[0] * M[3] + w[1] * M[7]) + w[2] * M[11]) + w[3] * M[15];
            float p[3] = {x / ww, y / ww, z / ww};
            b.inflate(p);
        }
        el[i].index = g.objects[i];
        el[i].bounds = b;
        for (int k = 0; k < 3; k++) el[i].centroid[k] = 0.5f * (b.lo[k] + b.hi[k]);
    }
    out.build(el);
}

void pack_nodes(const HostBVH& b, std::vector<float4>& out)
{
    for (const Node& n : b.nodes)
    {
        const Box &L = n.leftBox, &R = n.rightBox;
        float4 q0 = make_float4(L.lo[0], L.lo[1], L.lo[2], L.hi[0]);
        float4 q1 = make_float4(L.hi[1], L.hi[2], R.lo[0], R.lo[1]);
        float4 q2 = make_float4(R.lo[2], R.hi[0], R.hi[1], R.hi[2]);
        float4 q3;
        uint32_t l = n.left, r = n.right;
        std::memcpy(&q3.x, &l, 4);
        std::memcpy(&q3.y, &r, 4);
        q3.z = 0.0f; q3.w = 0.0f;
        out.push_back(q0); out.push_back(q1); out.push_back(q2); out.push_back(q3);
    }
}

// ------------------------------------------------- compressed node mirror --
// A device-only copy of every BVH node in 32 bytes (one 256-bit load, one
// 32-byte sector) next to the exact 64-byte record, for the traversal
// kernel.  The child boxes are stored as 8-bit offsets on a per-axis grid
// (the compressed-wide-BVH encoding of Ylitie, Karras and Laine, HPG 2017,
// for binary nodes):
//
//   words 0-2  origin P (float) per axis
//   word  3    bytes 0-2: e per axis (grid step s = 2^(e-127)); byte 3: flags
//              (bit 0: leaf)
//   words 4-6  per axis the bytes (left lo, left hi, right lo, right hi); a
//              leaf keeps its own box in the left bytes
//   word  7    right child (inner node; the left child is the next node in
//              pre-order) or the leaf's first element index
//
// A byte q stands for the coordinate P + q s.  Every child box is widened on
// the grid by at least one step beyond its exact bounds (lo' <= lo - s,
// hi' >= hi + s), which covers the half-step rounding of the traversal's
// decode, so the decoded boxes contain the exact ones: a ray meets every box
// the exact test meets, at an entry distance no larger than the exact one.
// The traversal then visits the same leaves (and a few more) and finds the
// same hits.  A BVH with a node that has no such record (a non-finite box
// coordinate, an extent no grid of 2^-126..2^127 covers, or a left child
// that does not follow its parent, as a loaded blob may have) is read from
// the exact records only.
namespace {

constexpr uint32_t kQLeaf = 1u;

float round_down_float(double x)
{
    float f = float(x);
    if (double(f) > x) f = std::nextafter(f, -INFINITY);
    return f;
}

// Grid of one axis of a node covering [lo, hi] with a two-step margin below
// lo and at least two steps above hi inside 255 steps.  False if none.
bool axis_grid(double lo, double hi, float& P, int& e)
{
    if (!std::isfinite(lo) || !std::isfinite(hi) || hi < lo) return false;
    // the smallest e with 250 s >= extent, from the binary exponent of
    // extent / 250 (then checked upward)
    const double extent = hi - lo;
    int e0 = extent > 0.0 ? std::max(1, std::ilogb(extent / 250.0) + 127) : 1;
    while (e0 < 254 && std::ldexp(250.0, e0 - 127) < extent) e0++;
    for (e = e0; e <= 254; e++)
    {
        const double s = std::ldexp(1.0, e - 127);
        P = round_down_float(lo - 2.0 * s);
        if (!std::isfinite(P)) return false;
        if ((hi - double(P)) / s <= 253.0) return true;
    }
    return false;
}

}  // namespace

// Appends the BVH's compressed records (two uint4 per node); false, with
// zero records written for the failing node on, if a node has none.
bool pack_qnodes(const HostBVH& b, std::vector<uint4>& out)
{
    bool all = true;
    for (size_t i = 0; i < b.nodes.size(); i++)
    {
        const Node& n = b.nodes[i];
        const bool leaf = n.left == EMPTY;
        uint32_t w[8] = {};
        // the compressed record names only the right child: the left one must follow
        bool ok = leaf || n.left == i + 1;
        uint32_t bytes[3] = {}, ex[3] = {};
        for (int a = 0; a < 3 && ok; a++)
        {
            const Box& L = n.leftBox;
            const Box& R = n.rightBox;
            const double lo = leaf ? double(L.lo[a]) : std::min(double(L.lo[a]), double(R.lo[a]));
            const double hi = leaf ? double(L.hi[a]) : std::max(double(L.hi[a]), double(R.hi[a]));
            float P = 0;
            int e = 0;
            if (!axis_grid(lo, hi, P, e)) { ok = false; break; }
            const double s = std::ldexp(1.0, e - 127);
            auto qlo = [&](double c) { return std::ceil((c - double(P)) / s) - 2.0; };
            auto qhi = [&](double c) { return std::floor((c - double(P)) / s) + 2.0; };
            const double q[4] = {qlo(L.lo[a]), qhi(L.hi[a]), leaf ? 0.0 : qlo(R.lo[a]), leaf ? 0.0 : qhi(R.hi[a])};
            for (double v : q) if (!(v >= 0.0 && v <= 255.0)) ok = false;
            if (!ok) break;
            std::memcpy(&w[a], &P, 4);
            ex[a] = uint32_t(e);
            bytes[a] = uint32_t(q[0]) | (uint32_t(q[1]) << 8) | (uint32_t(q[2]) << 16) | (uint32_t(q[3]) << 24);
        }
        if (!ok)
        {
            all = false;
            w[0] = w[1] = w[2] = 0;
            ex[0] = ex[1] = ex[2] = 127;
            bytes[0] = bytes[1] = bytes[2] = 0;
        }
        w[3] = ex[0] | (ex[1] << 8) | (ex[2] << 16) | ((leaf ? kQLeaf : 0u) << 24);
        w[4] = bytes[0]; w[5] = bytes[1]; w[6] = bytes[2];
        w[7] = n.right;
        out.push_back(make_uint4(w[0], w[1], w[2], w[3]));
        out.push_back(make_uint4(w[4], w[5], w[6], w[7]));
    }
    return all;
}

// Lights of all groups, concatenated; groupLights[g] = (first, count);
// groupEnv[g] = background rgb, ambient rgb.
int upload_lights(cgs_scene* sc)
{
    std::vector<DevLight> hl;
    std::vector<uint2> gl;
    std::vector<float> env;
    for (const Group& g : sc->groups)
    {
        gl.push_back(make_uint2(uint32_t(hl.size()), uint32_t(g.lights.size())));
        for (const auto& l : g.lights) { DevLight d; std::memcpy(&d, &l, sizeof d); hl.push_back(d); }
        for (int k = 0; k < 3; k++) env.push_back(g.background[k]);
        for (int k = 0; k < 3; k++) env.push_back(g.ambient[k]);
    }
    CGS_TRY(sc->dlights.reserve(std::max<size_t>(hl.size(), 1)));
    CGS_TRY(sc->groupLights.reserve(gl.size()));
    CGS_TRY(sc->groupEnv.reserve(env.size()));
    if (!hl.empty()) CGS_TRY(cudaMemcpy(sc->dlights.p, hl.data(), hl.size() * sizeof(DevLight), cudaMemcpyHostToDevice));
    CGS_TRY(cudaMemcpy(sc->groupLights.p, gl.data(), gl.size() * sizeof(uint2), cudaMemcpyHostToDevice));
    CGS_TRY(cudaMemcpy(sc->groupEnv.p, env.data(), env.size() * sizeof(float), cudaMemcpyHostToDevice));
    return CGS_OK;
}

}  // namespace

// Device copy of the store's host state (everything but the hash tables).
int cgs::upload_store(cgs_scene* sc)
{
    const uint32_t nb = sc->nbvh();
    std::vector<float4> hp, hn;
    std::vector<uint4> hq;
    std::vector<uint32_t> hi, pbase, pmat, gtop;
    std::vector<DevMaterial> hm;
    std::vector<DevObject> ho;
    sc->hbvh.assign(nb, DevBVH {});
    sc->tableCap.assign(nb, 0);
    uint32_t patchCursor = 0, tableCursor = 0, dispCursor = 0;
    for (uint32_t k = 0; k < nb; k++)
    {
        const HostBVH& b = sc->bvh(k);
        DevBVH& d = sc->hbvh[k];
        d.nodeBase = uint32_t(hn.size() / 4);
        d.indexBase = uint32_t(hi.size());
        pack_nodes(b, hn);
        d.compressed = pack_qnodes(b, hq) ? 1u : 0u;
        hi.insert(hi.end(), b.indices.begin(), b.indices.end());
        uint32_t n = uint32_t(b.keys.size());
        d.tableBase = tableCursor;
        d.dispBase = dispCursor;
        sc->tableCap[k] = table_capacity(n);
        tableCursor += sc->tableCap[k];
        dispCursor += displ_size(n);
        d.mask = displ_size(n) - 1;
        d.N = n; d.A = 31; d.B = 19;
        d.Nmagic = fastmod_magic(std::max<uint32_t>(n, 1));
    }
    for (uint32_t g = 0; g < sc->groups.size(); g++) gtop.push_back(uint32_t(sc->surfaces.size()) + g);
    for (const Surface& s : sc->surfaces)
    {
        pbase.push_back(patchCursor);
        for (uint32_t p = 0; p < s.patchCount(); p++)
            for (int j = 0; j < 16; j++)
            {
                const float* w = &s.points[4ull * s.indices[16ull * p + j]];
                hp.push_back(make_float4(w[0], w[1], w[2], w[3]));
            }
        patchCursor += s.patchCount();
    }
    for (const Object& ob : sc->objects)
    {
        DevObject d {};
        std::memcpy(d.w2l, ob.w2l, sizeof d.w2l);
        d.surface = ob.surface;
        d.material = uint32_t(hm.size());
        hm.push_back(to_dev(ob.material));
        if (!ob.patchMaterial.empty())
        {
            d.patchMaterialBase = int32_t(pmat.size());
            uint32_t mbase = uint32_t(hm.size());
            for (const auto& m : ob.materials) hm.push_back(to_dev(m));
            for (uint32_t pm : ob.patchMaterial) pmat.push_back(mbase + pm);
        }
        else
            d.patchMaterialBase = -1;
        ho.push_back(d);
    }
    CGS_TRY(sc->patches.reserve(hp.size()));
    CGS_TRY(sc->nodes.reserve(hn.size()));
    CGS_TRY(sc->qnodes.reserve(hq.size()));
    CGS_TRY(sc->indices.reserve(hi.size()));
    CGS_TRY(sc->tables.reserve(tableCursor));
    CGS_TRY(sc->disps.reserve(dispCursor));
    CGS_TRY(sc->patchBase.reserve(pbase.size()));
    CGS_TRY(sc->patchMaterial.reserve(std::max<size_t>(pmat.size(), 1)));
    CGS_TRY(sc->bvhs.reserve(nb));
    CGS_TRY(sc->groupTop.reserve(gtop.size()));
    CGS_TRY(sc->dobjects.reserve(ho.size()));
    CGS_TRY(sc->materials.reserve(hm.size()));
    CGS_TRY(sc->counters.reserve(1));
    CGS_TRY(cudaMemcpy(sc->patches.p, hp.data(), hp.size() * sizeof(float4), cudaMemcpyHostToDevice));
    CGS_TRY(cudaMemcpy(sc->nodes.p, hn.data(), hn.size() * sizeof(float4), cudaMemcpyHostToDevice));
    CGS_TRY(cudaMemcpy(sc->qnodes.p, hq.data(), hq.size() * sizeof(uint4), cudaMemcpyHostToDevice));
    CGS_TRY(cudaMemcpy(sc->indices.p, hi.data(), hi.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    CGS_TRY(cudaMemcpy(sc->patchBase.p, pbase.data(), pbase.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    if (!pmat.empty())
        CGS_TRY(cudaMemcpy(sc->patchMaterial.p, pmat.data(), pmat.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    CGS_TRY(cudaMemcpy(sc->dobjects.p, ho.data(), ho.size() * sizeof(DevObject), cudaMemcpyHostToDevice));
    CGS_TRY(cudaMemcpy(sc->materials.p, hm.data(), hm.size() * sizeof(DevMaterial), cudaMemcpyHostToDevice));
    CGS_TRY(cudaMemcpy(sc->groupTop.p, gtop.data(), gtop.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    CGS_TRY(cudaMemcpy(sc->bvhs.p, sc->hbvh.data(), nb * sizeof(DevBVH), cudaMemcpyHostToDevice));
    int r = upload_lights(sc);
    if (r) return r;
    sc->uploaded = true;
    return CGS_OK;
}

namespace {

int upload(cgs_scene* sc) { return upload_store(sc); }

// BVH::buildHashTable (src/rt/BVH.cpp:24-39) for every BVH of the store.
// BVHs of at most kHashBlockMaxKeys keys (most: one per surface) are built
// together, one CTA each with its scratch in shared memory, in one launch;
// those of at most kHashGlobalBlockMaxKeys likewise with a global scratch
// area each, in a second launch; one host round trip reads both launches'
// results.  Larger BVHs run the multi-launch build one at a time.
int hash_all(cgs_scene* sc, cudaStream_t stream)
{
    const uint32_t nb = sc->nbvh();
    std::vector<uint32_t> small, mid, large;
    uint32_t maxSmall = 1, maxMid = 1, maxLarge = 1;
    size_t blockKeys = 0;
    uint64_t midScratch = 0;
    for (uint32_t k = 0; k < nb; k++)
    {
        const uint32_t n = uint32_t(sc->bvh(k).keys.size());
        if (n <= kHashBlockMaxKeys) { small.push_back(k); maxSmall = std::max(maxSmall, n); blockKeys += n; }
        else if (n <= kHashGlobalBlockMaxKeys)
        {
            mid.push_back(k);
            maxMid = std::max(maxMid, n);
            blockKeys += n;
            midScratch += hash_block_scratch_words(n) + 1;
        }
        else { large.push_back(k); maxLarge = std::max(maxLarge, n); }
    }
    CGS_TRY(sc->keys.reserve(std::max<size_t>({blockKeys, size_t(maxLarge), 1})));
    if (!small.empty() || !mid.empty())
    {
        std::vector<uint32_t> hk;
        hk.reserve(blockKeys);
        std::vector<HashJob> jobs(small.size() + mid.size());
        uint64_t scratchCursor = 0;
        for (size_t j = 0; j < jobs.size(); j++)
        {
            const uint32_t k = j < small.size() ? small[j] : mid[j - small.size()];
            const HostBVH& b = sc->bvh(k);
            const uint32_t n = uint32_t(b.keys.size());
            HashJob& J = jobs[j];
            J.keyOff = uint32_t(hk.size());
            J.n = n;
            J.dispOff = sc->hbvh[k].dispBase;
            J.tableOff = sc->hbvh[k].tableBase;
            J.tableCap = sc->tableCap[k];
            J.mask = displ_size(n) - 1;
            J.scratchOff = 0;
            J.pad = 0;
            if (j >= small.size())
            {
                if (scratchCursor > 0xFFFFFFFFull) return CGS_ERR_OUT_OF_MEMORY;
                J.scratchOff = uint32_t(scratchCursor);
                scratchCursor += (hash_block_scratch_words(n) + 2) & ~1ull;  // keep 8-byte alignment
            }
            hash_coefficients(n, J.A, J.B);
            hk.insert(hk.end(), b.keys.begin(), b.keys.end());
        }
        const size_t jobWords = (jobs.size() * sizeof(HashJob) + 3) / 4;
        CGS_TRY(sc->hashJobs.reserve(jobWords + 8 * jobs.size()));
        if (!mid.empty()) CGS_TRY(sc->scratch32.reserve(std::max<uint64_t>(scratchCursor, 1)));
        uint32_t* dJobs = sc->hashJobs.p;
        uint32_t* dOut = sc->hashJobs.p + jobWords;
        CGS_TRY(cudaMemcpyAsync(sc->keys.p, hk.data(), hk.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, stream));
        CGS_TRY(cudaMemcpyAsync(dJobs, jobs.data(), jobs.size() * sizeof(HashJob), cudaMemcpyHostToDevice, stream));
        const HashJob* dj = reinterpret_cast<const HashJob*>(dJobs);
        if (!small.empty())
        {
            CGS_TRY(hash_build_blocks(sc->keys.p, dj, uint32_t(small.size()), maxSmall, sc->disps.p, sc->tables.p,
                                      dOut, stream));
            sc->launches += 1;
        }
        if (!mid.empty())
        {
            CGS_TRY(hash_build_blocks(sc->keys.p, dj + small.size(), uint32_t(mid.size()), maxMid, sc->disps.p,
                                      sc->tables.p, dOut + 8 * small.size(), stream, sc->scratch32.p));
            sc->launches += 1;
        }
        std::vector<uint32_t> res(8 * jobs.size());
        CGS_TRY(cudaMemcpyAsync(res.data(), dOut, res.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
        CGS_TRY(cudaStreamSynchronize(stream));
        for (size_t j = 0; j < jobs.size(); j++)
        {
            const uint32_t* r = &res[8 * j];
            if (r[0] == 4) return CGS_ERR_HASH_BUCKET_OVERFLOW;
            if (r[0]) return CGS_ERR_HASH_FAILED;
            DevBVH& d = sc->hbvh[j < small.size() ? small[j] : mid[j - small.size()]];
            d.A = r[1]; d.B = r[2]; d.N = r[3]; d.mask = r[4];
            d.Nmagic = fastmod_magic(d.N);
        }
    }
    if (!large.empty())
    {
        size_t w32 = 0, w64 = 0;
        hash_scratch_words(maxLarge, w32, w64);
        CGS_TRY(sc->scratch32.reserve(w32));
        CGS_TRY(sc->scratch64.reserve(w64));
        for (uint32_t k : large)
        {
            const HostBVH& b = sc->bvh(k);
            const uint32_t n = uint32_t(b.keys.size());
            HashScratch hs {};
            hash_scratch_carve(hs, n, sc->scratch32.p, sc->scratch64.p);
            CGS_TRY(cudaMemcpyAsync(sc->keys.p, b.keys.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice, stream));
            uint32_t A[16], B[16], params[5];
            hash_coefficients(n, A, B);
            DevBVH& d = sc->hbvh[k];
            int r = hash_build_device(sc->keys.p, n, A, B, sc->disps.p + d.dispBase, sc->tables.p + d.tableBase,
                                      sc->tableCap[k], hs, params, stream, &sc->launches);
            if (r == 4) return CGS_ERR_HASH_BUCKET_OVERFLOW;
            if (r < 0) return CGS_ERR_CUDA;
            if (r) return CGS_ERR_HASH_FAILED;
            d.A = params[0]; d.B = params[1]; d.N = params[2]; d.mask = params[3];
            d.Nmagic = fastmod_magic(d.N);
        }
    }
    CGS_TRY(cudaMemcpyAsync(sc->bvhs.p, sc->hbvh.data(), nb * sizeof(DevBVH), cudaMemcpyHostToDevice, stream));
    CGS_TRY(cudaStreamSynchronize(stream));
    sc->hashed = true;
    return CGS_OK;
}

Group& current_group(cgs_scene* s) { return s->groups[s->current]; }

// The exported form of BVH k of a mirrored store (CGS_SPLIT_MIRROR): the
// reference-topology tree, built again on the host, and, once the store is
// hashed, its perfect-hash table from the same device build as the store's
// (cgs_perfect_hash_build) into temporary buffers.  params = A, B, N, mask.
int mirror_export(const cgs_scene* s, uint32_t k, HostBVH& ref, std::vector<uint32_t>& table,
                  std::vector<uint32_t>& disp, uint32_t params[4])
{
    const size_t ns = s->surfaces.size();
    ref.split_mode = CGS_SPLIT_REFERENCE;
    if (k < ns) build_surface_bvh(s->surfaces[k], ref);
    else build_group_bvh(s, s->groups[k - ns], ref);
    if (ref.emptyLeaf) return CGS_ERR_EMPTY_LEAF;
    params[0] = params[1] = params[2] = params[3] = 0;
    table.clear();
    disp.clear();
    if (!s->hashed) return CGS_OK;
    CGS_TRY(cudaSetDevice(s->device));
    const uint32_t n = uint32_t(ref.keys.size());
    const uint32_t dcap = displ_size(n), tcap = table_capacity(n);
    struct Temp
    {
        DBuf<uint32_t> keys, disp, table;
        ~Temp() { keys.release(); disp.release(); table.release(); }
    } d;
    CGS_TRY(d.keys.reserve(n));
    CGS_TRY(d.disp.reserve(dcap));
    CGS_TRY(d.table.reserve(tcap));
    uint32_t p5[5] = {};
    CGS_TRY(cudaMemcpy(d.keys.p, ref.keys.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice));
    if (int r = cgs_perfect_hash_build(d.keys.p, n, d.disp.p, dcap, d.table.p, tcap, p5, nullptr)) return r;
    if (p5[2] > tcap || size_t(p5[3]) + 1 > dcap) return CGS_ERR_HASH_FAILED;
    table.resize(p5[2]);
    disp.resize(size_t(p5[3]) + 1);
    CGS_TRY(cudaMemcpy(disp.data(), d.disp.p, disp.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    CGS_TRY(cudaMemcpy(table.data(), d.table.p, table.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    for (int j = 0; j < 4; j++) params[j] = p5[j];
    return CGS_OK;
}

bool bvh_index(const cgs_scene* s, int32_t which, uint32_t& k)
{
    if (which >= 0)
    {
        if (uint32_t(which) >= s->surfaces.size()) return false;
        k = uint32_t(which);
        return true;
    }
    uint32_t g = uint32_t(-1 - int64_t(which));
    if (g >= s->groups.size()) return false;
    k = uint32_t(s->surfaces.size()) + g;
    return true;
}

}  // namespace

cgs::DevScene cgs_scene::dev() const
{
    DevScene S {};
    S.patches = patches.p; S.nodes = nodes.p; S.qnodes = qnodes.p; S.indices = indices.p; S.tables = tables.p; S.disps = disps.p;
    S.bvhs = bvhs.p; S.patchBase = patchBase.p; S.objects = dobjects.p; S.materials = materials.p;
    S.patchMaterial = patchMaterial.p; S.lights = dlights.p;
    S.groupTop = groupTop.p; S.groupLights = groupLights.p; S.groupEnv = groupEnv.p;
    S.nobjects = uint32_t(objects.size()); S.nsurfaces = uint32_t(surfaces.size());
    S.ngroups = uint32_t(groups.size());
    return S;
}

cgs_scene::~cgs_scene()
{
    cudaSetDevice(device);
    patches.release(); nodes.release(); qnodes.release();
    for (auto* b : {&indices, &tables, &disps, &patchBase, &patchMaterial, &keys, &groupTop, &scratch32, &groupStage,
                    &hashJobs,
                    &engine, &fbStage})
        b->release();
    rayStage.release(); hitF.release(); linStage.release(); groupEnv.release();
    groupLights.release(); bvhs.release(); dobjects.release(); materials.release(); dlights.release();
    scratch64.release(); counters.release(); hitI.release();
    slot.release();
    if (finished) cudaEventDestroy(finished);
    if (queryDone) cudaEventDestroy(queryDone);
}

// =========================================================== C ABI ====
extern "C" {

const char* cgs_status_string(int s)
{
    switch (s)
    {
    case CGS_OK: return "ok";
    case CGS_ERR_INVALID_ARGUMENT: return "invalid argument";
    case CGS_ERR_CUDA: return "CUDA error";
    case CGS_ERR_OUT_OF_MEMORY: return "out of device memory";
    case CGS_ERR_NOT_BUILT: return "scene not built";
    case CGS_ERR_HASH_BUCKET_OVERFLOW: return "perfect hash: more than 4 keys in a displacement bucket";
    case CGS_ERR_HASH_FAILED: return "perfect hash: no injective table in 16 trials";
    case CGS_ERR_EMPTY_LEAF: return "BVH: empty leaf";
    case CGS_ERR_BUSY: return "render still in flight";
    case CGS_ERR_DEVICE_LIMIT: return "a kernel hit a stack or iteration limit";
    case CGS_ERR_ADMISSION: return "request exceeds the device-memory budget";
    case CGS_ERR_NOT_FOUND: return "not found";
    case CGS_ERR_CAPACITY: return "input exceeds the fixed capacity of this entry point";
    default: return "unknown status";
    }
}

int cgs_version(void) { return 2; }

int cgs_scene_create(cgs_scene** out, int device)
{
    if (!out) return CGS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return CGS_ERR_CUDA;
    CGS_TRY(cudaSetDevice(device));
    auto* s = new (std::nothrow) cgs_scene();
    if (!s) return CGS_ERR_OUT_OF_MEMORY;
    s->device = device;
    s->groups.emplace_back();
    if (cudaEventCreateWithFlags(&s->finished, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->queryDone, cudaEventDisableTiming) != cudaSuccess)
    {
        delete s;
        return CGS_ERR_CUDA;
    }
    *out = s;
    return CGS_OK;
}

int cgs_scene_destroy(cgs_scene* s)
{
    if (!s) return CGS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->device);
    cudaDeviceSynchronize();
    delete s;
    return CGS_OK;
}

int cgs_scene_add_surface(cgs_scene* s, const float* pts, uint32_t npoints, const uint32_t* idx, uint32_t nidx,
                          uint32_t* sid)
{
    if (!s || !pts || !idx || nidx == 0 || nidx % 16 || npoints == 0) return CGS_ERR_INVALID_ARGUMENT;
    for (uint32_t i = 0; i < nidx; i++) if (idx[i] >= npoints) return CGS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    Surface sf;
    sf.points.assign(pts, pts + 4ull * npoints);
    sf.indices.assign(idx, idx + nidx);
    s->surfaces.push_back(std::move(sf));
    s->bvhBuilt = s->uploaded = s->hashed = false;
    if (sid) *sid = uint32_t(s->surfaces.size() - 1);
    return CGS_OK;
}

int cgs_scene_add_group(cgs_scene* s, uint32_t* gid)
{
    if (!s) return CGS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    if (current_group(s).touched)
    {
        s->groups.emplace_back();
        s->current = uint32_t(s->groups.size() - 1);
        s->bvhBuilt = s->uploaded = s->hashed = false;
    }
    if (gid) *gid = s->current;
    return CGS_OK;
}

int cgs_scene_add_object(cgs_scene* s, uint32_t surface, const float l2w[16], const float w2l[16],
                         const cgs_material* material, const uint32_t* pm, const cgs_material* mats, uint32_t nm,
                         uint32_t* oid)
{
    if (!s || !l2w || !w2l || !material) return CGS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    if (surface >= s->surfaces.size()) return CGS_ERR_INVALID_ARGUMENT;
    Object ob;
    ob.surface = surface;
    ob.group = s->current;
    std::memcpy(ob.l2w, l2w, sizeof ob.l2w);
    std::memcpy(ob.w2l, w2l, sizeof ob.w2l);
    ob.material = *material;
    if (pm)
    {
        if (!mats || nm == 0) return CGS_ERR_INVALID_ARGUMENT;
        uint32_t P = s->surfaces[surface].patchCount();
        ob.patchMaterial.assign(pm, pm + P);
        for (uint32_t v : ob.patchMaterial) if (v >= nm) return CGS_ERR_INVALID_ARGUMENT;
        ob.materials.assign(mats, mats + nm);
    }
    s->objects.push_back(std::move(ob));
    current_group(s).objects.push_back(uint32_t(s->objects.size() - 1));
    current_group(s).touched = true;
    s->bvhBuilt = s->uploaded = s->hashed = false;
    if (oid) *oid = uint32_t(s->objects.size() - 1);
    return CGS_OK;
}

int cgs_scene_set_lights(cgs_scene* s, const cgs_light* lights, uint32_t n)
{
    if (!s || (n && !lights)) return CGS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    current_group(s).lights.assign(lights, lights + n);
    current_group(s).touched = true;
    if (!s->uploaded) return CGS_OK;
    CGS_TRY(cudaSetDevice(s->device));
    return upload_lights(s);
}

int cgs_scene_set_environment(cgs_scene* s, const float bg[3], const float amb[3])
{
    if (!s || !bg || !amb) return CGS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    Group& gr = current_group(s);
    for (int k = 0; k < 3; k++) { gr.background[k] = bg[k]; gr.ambient[k] = amb[k]; }
    gr.touched = true;
    if (!s->uploaded) return CGS_OK;
    CGS_TRY(cudaSetDevice(s->device));
    return upload_lights(s);
}

int cgs_scene_set_bvh_split(cgs_scene* s, int mode)
{
    if (!s || (mode != CGS_SPLIT_REFERENCE && mode != CGS_SPLIT_LONGEST && mode != CGS_SPLIT_MIRROR))
        return CGS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    if (s->splitMode != mode) s->bvhBuilt = s->uploaded = s->hashed = false;
    s->splitMode = mode;
    return CGS_OK;
}

int cgs_bvh_build(cgs_scene* s)
{
    if (!s) return CGS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    if (s->objects.empty()) return CGS_ERR_INVALID_ARGUMENT;
    for (const Group& gr : s->groups)
        if (gr.objects.empty()) return CGS_ERR_EMPTY_LEAF;
    // the surfaces' and groups' BVHs are independent: built on all host
    // cores, largest first, each by one thread (the same result as in order)
    const size_t ns = s->surfaces.size(), ng = s->groups.size();
    std::vector<std::pair<uint64_t, size_t>> work;
    for (size_t i = 0; i < ns; i++) work.push_back({s->surfaces[i].patchCount(), i});
    for (size_t g = 0; g < ng; g++)
    {
        uint64_t cost = 0;
        for (uint32_t o : s->groups[g].objects) cost += s->surfaces[s->objects[o].surface].indices.size() / 16;
        work.push_back({cost, ns + g});
    }
    std::sort(work.begin(), work.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
    std::atomic<size_t> next {0};
    auto worker = [&]() {
        for (size_t w; (w = next.fetch_add(1)) < work.size();)
        {
            const size_t i = work[w].second;
            // a mirrored store traverses the longest-axis build
            const int mode = s->splitMode == CGS_SPLIT_MIRROR ? CGS_SPLIT_LONGEST : s->splitMode;
            if (i < ns)
            {
                s->surfaces[i].bvh.split_mode = mode;
                build_surface_bvh(s->surfaces[i], s->surfaces[i].bvh);
            }
            else
            {
                s->groups[i - ns].top.split_mode = mode;
                build_group_bvh(s, s->groups[i - ns], s->groups[i - ns].top);
            }
        }
    };
    const size_t nt = std::min<size_t>(work.size(), std::max(1u, std::min(64u, std::thread::hardware_concurrency())));
    std::vector<std::thread> pool;
    for (size_t t = 1; t < nt; t++) pool.emplace_back(worker);
    worker();
    for (auto& th : pool) th.join();
    for (auto& sf : s->surfaces)
        if (sf.bvh.emptyLeaf) return CGS_ERR_EMPTY_LEAF;
    for (auto& gr : s->groups)
        if (gr.top.emptyLeaf) return CGS_ERR_EMPTY_LEAF;
    s->bvhBuilt = true;
    s->uploaded = s->hashed = false;
    return CGS_OK;
}

int cgs_hash_build(cgs_scene* s, void* stream)
{
    if (!s) return CGS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    if (!s->bvhBuilt) return CGS_ERR_NOT_BUILT;
    CGS_TRY(cudaSetDevice(s->device));
    if (!s->uploaded)
    {
        int r = upload(s);
        if (r) return r;
    }
    return hash_all(s, (cudaStream_t)stream);
}

int cgs_scene_build(cgs_scene* s, void* stream)
{
    int r = cgs_bvh_build(s);
    if (r) return r;
    return cgs_hash_build(s, stream);
}

int cgs_scene_footprint(const cgs_scene* s, uint64_t* bytes)
{
    if (!s || !bytes) return CGS_ERR_INVALID_ARGUMENT;
    uint64_t b = 0;
    b += s->patches.bytes() + s->nodes.bytes() + s->qnodes.bytes() + s->indices.bytes() + s->tables.bytes() + s->disps.bytes();
    b += s->patchBase.bytes() + s->patchMaterial.bytes() + s->bvhs.bytes() + s->dobjects.bytes();
    b += s->materials.bytes() + s->dlights.bytes() + s->groupTop.bytes() + s->groupLights.bytes();
    b += s->groupEnv.bytes();
    *bytes = b;
    return CGS_OK;
}

int cgs_bvh_sizes(const cgs_scene* s, int32_t which, uint32_t sizes[5])
{
    if (!s || !sizes) return CGS_ERR_INVALID_ARGUMENT;
    if (!s->bvhBuilt) return CGS_ERR_NOT_BUILT;
    uint32_t k;
    if (!bvh_index(s, which, k)) return CGS_ERR_INVALID_ARGUMENT;
    if (s->splitMode == CGS_SPLIT_MIRROR)
    {
        HostBVH ref;
        std::vector<uint32_t> table, disp;
        uint32_t params[4];
        if (int r = mirror_export(s, k, ref, table, disp, params)) return r;
        sizes[0] = uint32_t(ref.nodes.size());
        sizes[1] = uint32_t(ref.indices.size());
        sizes[2] = params[2];
        sizes[3] = displ_size(uint32_t(ref.keys.size()));
        sizes[4] = uint32_t(ref.keys.size());
        return CGS_OK;
    }
    const HostBVH& b = s->bvh(k);
    sizes[0] = uint32_t(b.nodes.size());
    sizes[1] = uint32_t(b.indices.size());
    sizes[2] = s->hashed ? s->hbvh[k].N : 0;
    sizes[3] = displ_size(uint32_t(b.keys.size()));
    sizes[4] = uint32_t(b.keys.size());
    return CGS_OK;
}

int cgs_bvh_export(const cgs_scene* s, int32_t which, uint32_t* nodes, uint32_t* keys, uint32_t* indices,
                   uint32_t* table, uint32_t* disp, uint32_t params[4])
{
    if (!s) return CGS_ERR_INVALID_ARGUMENT;
    if (!s->bvhBuilt) return CGS_ERR_NOT_BUILT;
    uint32_t k;
    if (!bvh_index(s, which, k)) return CGS_ERR_INVALID_ARGUMENT;
    HostBVH ref;
    std::vector<uint32_t> mtable, mdisp;
    uint32_t mparams[4] = {};
    const bool mirror = s->splitMode == CGS_SPLIT_MIRROR;
    if (mirror)
        if (int r = mirror_export(s, k, ref, mtable, mdisp, mparams)) return r;
    const HostBVH& b = mirror ? ref : s->bvh(k);
    if (nodes)
        for (size_t i = 0; i < b.nodes.size(); i++)
        {
            const Node& n = b.nodes[i];
            float f[12] = {n.leftBox.lo[0], n.leftBox.lo[1], n.leftBox.lo[2], n.leftBox.hi[0], n.leftBox.hi[1],
                           n.leftBox.hi[2], n.rightBox.lo[0], n.rightBox.lo[1], n.rightBox.lo[2], n.rightBox.hi[0],
                           n.rightBox.hi[1], n.rightBox.hi[2]};
            std::memcpy(nodes + 14 * i, f, sizeof f);
            nodes[14 * i + 12] = n.left;
            nodes[14 * i + 13] = n.right;
        }
    if (keys) std::copy(b.keys.begin(), b.keys.end(), keys);
    if (indices) std::copy(b.indices.begin(), b.indices.end(), indices);
    if (mirror)
    {
        if (s->hashed && table) std::copy(mtable.begin(), mtable.end(), table);
        if (s->hashed && disp) std::copy(mdisp.begin(), mdisp.end(), disp);
        if (params) std::copy(mparams, mparams + 4, params);
    }
    else if (s->hashed)
    {
        CGS_TRY(cudaSetDevice(s->device));
        const DevBVH& d = s->hbvh[k];
        if (table) CGS_TRY(cudaMemcpy(table, s->tables.p + d.tableBase, d.N * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        if (disp) CGS_TRY(cudaMemcpy(disp, s->disps.p + d.dispBase, (d.mask + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        if (params) { params[0] = d.A; params[1] = d.B; params[2] = d.N; params[3] = d.mask; }
    }
    else if (params)
        params[0] = params[1] = params[2] = params[3] = 0;
    return CGS_OK;
}

int cgs_scene_counters(cgs_scene* s, cgs_counters* out)
{
    if (!s || !out) return CGS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    std::memset(out, 0, sizeof *out);
    if (!s->lastCounters) return CGS_OK;
    CGS_TRY(cudaSetDevice(s->device));
    CGS_TRY(cudaStreamSynchronize(s->lastStream));
    Counters c;
    CGS_TRY(cudaMemcpy(&c, s->lastCounters, sizeof c, cudaMemcpyDeviceToHost));
    out->rays = c.rays; out->nodes = c.nodes; out->hash_lookups = c.hashLookups; out->candidates = c.candidates;
    out->iterations = c.iterations; out->device_errors = c.errors; out->kernel_launches = uint64_t(s->launches);
    out->hash_table_reads = c.tableReads;
    return CGS_OK;
}

}  // extern "C"
