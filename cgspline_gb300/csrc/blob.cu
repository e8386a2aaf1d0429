// blob.cu -- scene blobs: a built store (surfaces, objects, groups, BVHs and
// their perfect-hash tables) written to a file and read back without the BVH
// and hash builds, for fast reload of resident scenes by a server.
#include <cstdio>
#include <memory>

#include "scene_impl.h"

using namespace cgs;

namespace {

constexpr uint32_t kMagic = 0x42534743u;  // "CGSB"
constexpr uint32_t kVersion = 1;

struct Writer
{
    FILE* f;
    bool ok = true;
    void raw(const void* p, size_t n) { if (ok && n && std::fwrite(p, 1, n, f) != n) ok = false; }
    void u32(uint32_t v) { raw(&v, 4); }
    template<class T> void vec(const std::vector<T>& v)
    {
        u32(uint32_t(v.size()));
        raw(v.data(), v.size() * sizeof(T));
    }
};

struct Reader
{
    FILE* f;
    bool ok = true;
    uint64_t left;  // bytes left in the file: no count may ask for more
    void raw(void* p, size_t n)
    {
        if (!ok || n > left || (n && std::fread(p, 1, n, f) != n)) { ok = false; return; }
        left -= n;
    }
    uint32_t u32() { uint32_t v = 0; raw(&v, 4); return v; }
    template<class T> void vec(std::vector<T>& v)
    {
        const uint64_t n = u32();
        if (!ok || n * sizeof(T) > left) { ok = false; return; }
        v.resize(n);
        raw(v.data(), n * sizeof(T));
    }
};

void put_bvh(Writer& w, const HostBVH& b)
{
    w.vec(b.nodes); w.vec(b.keys); w.vec(b.indices);
    w.u32(b.emptyLeaf ? 1u : 0u);
}

void get_bvh(Reader& r, HostBVH& b)
{
    r.vec(b.nodes); r.vec(b.keys); r.vec(b.indices);
    b.emptyLeaf = r.u32() != 0;
}

// the structure of a BVH read from a file: node links and leaf lists in range
// Besides the bounds of every index: the layout the traversal relies on to end.
// Children come after their parent (pre-order), so a descent always moves to a
// higher node; children carry the heap keys 2k and 2k+1 of their parent and
// the root key 1, so a backtrack's key names the sibling of an ancestor (the
// hash check below then maps it to that node).
bool bvh_sane(const HostBVH& b, uint32_t elements)
{
    if (b.nodes.empty() || b.keys.size() != b.nodes.size() || b.keys[0] != 1u) return false;
    for (size_t i = 0; i < b.nodes.size(); i++)
    {
        const Node& n = b.nodes[i];
        if (n.left != EMPTY && (n.left <= i || n.right <= i || n.left >= b.nodes.size() ||
                                n.right >= b.nodes.size() || b.keys[n.left] != 2u * b.keys[i] ||
                                b.keys[n.right] != 2u * b.keys[i] + 1u))
            return false;
        if (n.left == EMPTY)
        {
            // a leaf lists at least one element (the build refuses empty leaves)
            if (n.right + 1 >= b.indices.size() || b.indices[n.right] == EMPTY) return false;
            for (size_t j = n.right; ; j++)
            {
                if (j >= b.indices.size()) return false;
                if (b.indices[j] == EMPTY) break;
                if (b.indices[j] >= elements) return false;
            }
        }
    }
    return true;
}

}  // namespace

extern "C" {

int cgs_scene_save(cgs_scene* s, const char* path)
{
    if (!s || !path) return CGS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    if (!s->hashed) return CGS_ERR_NOT_BUILT;
    CGS_TRY(cudaSetDevice(s->device));
    FILE* f = std::fopen(path, "wb");
    if (!f) return CGS_ERR_INVALID_ARGUMENT;
    Writer w {f};
    w.u32(kMagic); w.u32(kVersion);
    w.u32(uint32_t(s->surfaces.size())); w.u32(uint32_t(s->objects.size())); w.u32(uint32_t(s->groups.size()));
    w.u32(uint32_t(s->splitMode));
    for (const Surface& sf : s->surfaces)
    {
        w.vec(sf.points); w.vec(sf.indices);
        put_bvh(w, sf.bvh);
    }
    for (const Object& ob : s->objects)
    {
        w.u32(ob.surface); w.u32(ob.group);
        w.raw(ob.l2w, sizeof ob.l2w); w.raw(ob.w2l, sizeof ob.w2l);
        w.raw(&ob.material, sizeof ob.material);
        w.vec(ob.patchMaterial); w.vec(ob.materials);
    }
    for (const Group& gr : s->groups)
    {
        w.vec(gr.objects); w.vec(gr.lights);
        w.raw(gr.background, sizeof gr.background); w.raw(gr.ambient, sizeof gr.ambient);
        w.u32(gr.touched ? 1u : 0u);
        put_bvh(w, gr.top);
    }
    // the perfect hash of every BVH: parameters, table, displacements
    int status = CGS_OK;
    for (uint32_t k = 0; k < s->nbvh() && status == CGS_OK && w.ok; k++)
    {
        const DevBVH& d = s->hbvh[k];
        w.u32(d.A); w.u32(d.B); w.u32(d.N); w.u32(d.mask);
        std::vector<uint32_t> table(d.N), disp(d.mask + 1);
        if (cudaMemcpy(table.data(), s->tables.p + d.tableBase, d.N * 4ull, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(disp.data(), s->disps.p + d.dispBase, (d.mask + 1) * 4ull, cudaMemcpyDeviceToHost) != cudaSuccess)
            status = CGS_ERR_CUDA;
        w.raw(table.data(), table.size() * 4);
        w.raw(disp.data(), disp.size() * 4);
    }
    const bool ok = w.ok && std::fclose(f) == 0;
    if (status) return status;
    return ok ? CGS_OK : CGS_ERR_INVALID_ARGUMENT;
}

int cgs_scene_load(cgs_scene** out, const char* path, int device)
{
    if (!out || !path) return CGS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    FILE* f = std::fopen(path, "rb");
    if (!f) return CGS_ERR_NOT_FOUND;
    std::fseek(f, 0, SEEK_END);
    const long size = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    Reader r {f, true, uint64_t(size > 0 ? size : 0)};
    cgs_scene* s = nullptr;
    int st = cgs_scene_create(&s, device);
    if (st) { std::fclose(f); return st; }
    std::unique_ptr<cgs_scene, int (*)(cgs_scene*)> guard(s, cgs_scene_destroy);
    const uint32_t magic = r.u32(), version = r.u32();
    const uint32_t ns = r.u32(), no = r.u32(), ng = r.u32(), split = r.u32();
    if (!r.ok || magic != kMagic || version != kVersion || ng == 0 || no == 0 ||
        (split != CGS_SPLIT_REFERENCE && split != CGS_SPLIT_LONGEST && split != CGS_SPLIT_MIRROR) || uint64_t(ns + no + ng) * 8 > r.left)
    {
        std::fclose(f);
        return CGS_ERR_INVALID_ARGUMENT;
    }
    s->splitMode = int(split);
    s->surfaces.resize(ns);
    s->objects.resize(no);
    s->groups.assign(ng, Group {});
    bool sane = true;
    for (Surface& sf : s->surfaces)
    {
        r.vec(sf.points); r.vec(sf.indices);
        get_bvh(r, sf.bvh);
        sane = sane && r.ok && sf.indices.size() % 16 == 0 && !sf.indices.empty() && sf.points.size() % 4 == 0;
        if (sane)
            for (uint32_t v : sf.indices) if (4ull * v >= sf.points.size()) { sane = false; break; }
        sane = sane && bvh_sane(sf.bvh, sf.patchCount());
        if (!sane) break;
    }
    for (uint32_t i = 0; sane && i < no; i++)
    {
        Object& ob = s->objects[i];
        ob.surface = r.u32(); ob.group = r.u32();
        r.raw(ob.l2w, sizeof ob.l2w); r.raw(ob.w2l, sizeof ob.w2l);
        r.raw(&ob.material, sizeof ob.material);
        r.vec(ob.patchMaterial); r.vec(ob.materials);
        sane = r.ok && ob.surface < ns && ob.group < ng &&
               (ob.patchMaterial.empty() || ob.patchMaterial.size() == s->surfaces[ob.surface].patchCount());
        for (uint32_t v : ob.patchMaterial) if (v >= ob.materials.size()) sane = false;
    }
    for (uint32_t gi = 0; sane && gi < ng; gi++)
    {
        Group& gr = s->groups[gi];
        r.vec(gr.objects); r.vec(gr.lights);
        r.raw(gr.background, sizeof gr.background); r.raw(gr.ambient, sizeof gr.ambient);
        gr.touched = r.u32() != 0;
        get_bvh(r, gr.top);
        sane = r.ok && !gr.objects.empty() && bvh_sane(gr.top, no);
        for (uint32_t o : gr.objects) if (o >= no || s->objects[o].group != gi) sane = false;
    }
    if (!sane)
    {
        std::fclose(f);
        return CGS_ERR_INVALID_ARGUMENT;
    }
    s->current = ng - 1;
    s->bvhBuilt = true;
    if (cudaSetDevice(s->device) != cudaSuccess || (st = upload_store(s)) != CGS_OK)
    {
        std::fclose(f);
        return st ? st : CGS_ERR_CUDA;
    }
    // the hash of every BVH, checked against its keys before it reaches the device
    for (uint32_t k = 0; k < s->nbvh() && sane; k++)
    {
        const HostBVH& b = s->bvh(k);
        DevBVH& d = s->hbvh[k];
        const uint32_t A = r.u32(), B = r.u32(), N = r.u32(), mask = r.u32();
        const uint32_t n = uint32_t(b.keys.size());
        if (!r.ok || N < n || N > s->tableCap[k] || mask + 1 != displ_size(n)) { sane = false; break; }
        std::vector<uint32_t> table(N), disp(mask + 1);
        r.raw(table.data(), table.size() * 4);
        r.raw(disp.data(), disp.size() * 4);
        if (!r.ok) { sane = false; break; }
        for (uint32_t i = 0; i < n && sane; i++)
        {
            const uint32_t key = b.keys[i];
            const uint32_t slot = uint32_t((uint64_t(uint32_t(A * key + B + disp[key & mask]))) % N);
            sane = table[slot] == i;
        }
        for (uint32_t v : table) if (v != EMPTY && v >= n) sane = false;
        if (!sane) break;
        if (cudaMemcpy(s->tables.p + d.tableBase, table.data(), N * 4ull, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(s->disps.p + d.dispBase, disp.data(), (mask + 1) * 4ull, cudaMemcpyHostToDevice) != cudaSuccess)
        {
            std::fclose(f);
            return CGS_ERR_CUDA;
        }
        d.A = A; d.B = B; d.N = N; d.mask = mask;
        d.Nmagic = fastmod_magic(N);
    }
    std::fclose(f);
    if (!sane) return CGS_ERR_INVALID_ARGUMENT;
    CGS_TRY(cudaMemcpy(s->bvhs.p, s->hbvh.data(), s->nbvh() * sizeof(DevBVH), cudaMemcpyHostToDevice));
    s->hashed = true;
    *out = guard.release();
    return CGS_OK;
}

}  // extern "C"
