// scene.cu -- host side of libcgspline_gb300.so: scene objects, BVH build,
// device upload, perfect-hash build orchestration and the C ABI of
// include/cgspline.h.
#include <algorithm>
#include <bit>
#include <cmath>
#include <cstring>
#include <mutex>
#include <numeric>
#include <random>
#include <stdexcept>
#include <vector>

#include "../../include/cgspline.h"
#include "kernels.h"

using namespace cgs;

namespace {

// ------------------------------------------------------------- host BVH --
struct Box
{
    float lo[3] = {INFINITY, INFINITY, INFINITY};
    float hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    void inflate(const float p[3])
    {
        for (int k = 0; k < 3; k++) { lo[k] = std::min(lo[k], p[k]); hi[k] = std::max(hi[k], p[k]); }
    }
    void inflate(const Box& b) { inflate(b.lo); inflate(b.hi); }
};

struct Element { Box bounds; float centroid[3]; uint32_t index; };
struct Node { Box leftBox, rightBox; uint32_t left, right; };

// BVH::build / split / wrap (src/rt/BVH.cpp:9-108): top-down median split,
// heap keys (root 1, children 2k and 2k+1), nodes in pre-order, leaves keep
// their box in leftBox and an EMPTY-terminated element list.  The split axis
// comes from the size of a box that is never inflated (src/rt/BVH.cpp:46-52),
// i.e. an empty box whose three extents compare equal, which selects y; the
// partition is std::nth_element with the same comparator, so the topology
// matches the reference built with the same standard library.
struct HostBVH
{
    std::vector<Node> nodes;
    std::vector<uint32_t> keys, indices;
    uint32_t perNode = 1;
    bool emptyLeaf = false;

    uint32_t wrap(Element* e, size_t count, uint32_t key)
    {
        if (count == 0) { emptyLeaf = true; count = 0; }
        Box box;
        size_t idx = indices.size();
        indices.resize(idx + count + 1);
        for (size_t i = 0; i < count; i++) { indices[idx + i] = e[i].index; box.inflate(e[i].bounds); }
        indices[idx + count] = EMPTY;
        keys.push_back(key);
        nodes.push_back({box, Box {}, EMPTY, uint32_t(idx)});
        return uint32_t(nodes.size() - 1);
    }
    uint32_t split(Element* e, size_t count, uint32_t key)
    {
        if (count <= perNode || (key & (1u << 31))) return wrap(e, count, key);
        Box empty;
        float v[3] = {empty.hi[0] - empty.lo[0], empty.hi[1] - empty.lo[1], empty.hi[2] - empty.lo[2]};
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
    void build(std::vector<Element>& el)
    {
        nodes.clear(); keys.clear(); indices.clear(); emptyLeaf = false;
        nodes.reserve(2 * el.size()); keys.reserve(2 * el.size()); indices.reserve(2 * el.size());
        split(el.data(), el.size(), 1u);
    }
};

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

struct Surface
{
    std::vector<float> points;   // 4 per point
    std::vector<uint32_t> indices;
    HostBVH bvh;
    uint32_t patchCount() const { return uint32_t(indices.size() / 16); }
};

struct Object
{
    uint32_t surface;
    float l2w[16], w2l[16];
    cgs_material material;
    std::vector<uint32_t> patchMaterial;
    std::vector<cgs_material> materials;
};

template<class T> struct DBuf
{
    T* p = nullptr;
    size_t n = 0;
    cudaError_t reserve(size_t count)
    {
        if (count <= n) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr; n = 0;
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess) n = count;
        return e;
    }
    void release() { if (p) cudaFree(p); p = nullptr; n = 0; }
};

int cuda_status(cudaError_t e)
{
    if (e == cudaSuccess) return CGS_OK;
    if (e == cudaErrorMemoryAllocation) return CGS_ERR_OUT_OF_MEMORY;
    return CGS_ERR_CUDA;
}

#define CGS_TRY(expr)                          \
    do {                                       \
        cudaError_t _e = (expr);               \
        if (_e != cudaSuccess) return cuda_status(_e); \
    } while (0)

}  // namespace

struct cgs_scene
{
    int device = 0;
    std::mutex mu;
    std::vector<Surface> surfaces;
    std::vector<Object> objects;
    std::vector<cgs_light> lights;
    float background[3] = {0.1f, 0.1f, 0.1f}, ambient[3] = {0.1f, 0.1f, 0.1f};
    HostBVH top;
    bool bvhBuilt = false, uploaded = false, hashed = false;

    // device side
    DBuf<float4> patches, nodes;
    DBuf<uint32_t> indices, tables, disps, patchBase, patchMaterial, keys;
    DBuf<DevBVH> bvhs;
    DBuf<DevObject> dobjects;
    DBuf<DevMaterial> materials;
    DBuf<DevLight> dlights;
    std::vector<DevBVH> hbvh;
    std::vector<uint32_t> tableCap;  // per BVH
    DBuf<uint32_t> scratch32;
    DBuf<unsigned long long> scratch64;
    DBuf<Counters> counters;
    DBuf<uint32_t> work;

    // query staging
    DBuf<float> rayStage;
    DBuf<float> hitF;
    DBuf<int32_t> hitI;

    // wavefront buffers
    WavefrontBuffers wb {};
    DBuf<float> wfRay0, wfRay1, wfShadow, wfContrib, wfBase, wfAccum, wfHitF;
    DBuf<uint32_t> wfPix0, wfPix1, wfCount, wfShadowSlot;
    DBuf<int32_t> wfVisible, wfHitI, wfOccluded;
    DBuf<uint32_t> engine;
    uint32_t engineCapacity = 0;
    DBuf<uint32_t> fbStage;
    DBuf<float> linStage;

    cudaEvent_t finished = nullptr;
    cudaStream_t lastStream = nullptr;
    int launches = 0;
    uint64_t primaryRays = 0, bounceRays = 0, shadowRays = 0;

    DevScene dev() const
    {
        DevScene S {};
        S.patches = patches.p; S.nodes = nodes.p; S.indices = indices.p; S.tables = tables.p; S.disps = disps.p;
        S.bvhs = bvhs.p; S.patchBase = patchBase.p; S.objects = dobjects.p; S.materials = materials.p;
        S.patchMaterial = patchMaterial.p; S.lights = dlights.p;
        S.nobjects = uint32_t(objects.size()); S.nlights = uint32_t(lights.size());
        S.nsurfaces = uint32_t(surfaces.size()); S.topBVH = uint32_t(surfaces.size());
        for (int k = 0; k < 3; k++) { S.background[k] = background[k]; S.ambient[k] = ambient[k]; }
        return S;
    }
    const HostBVH& bvh(uint32_t which) const { return which < surfaces.size() ? surfaces[which].bvh : top; }
    ~cgs_scene()
    {
        cudaSetDevice(device);
        for (auto* b : {&patches, &nodes}) b->release();
        for (auto* b : {&indices, &tables, &disps, &patchBase, &patchMaterial, &keys, &scratch32, &work, &wfPix0,
                        &wfPix1, &wfCount, &wfShadowSlot, &fbStage})
            b->release();
        for (auto* b : {&rayStage, &hitF, &wfRay0, &wfRay1, &wfShadow, &wfContrib, &wfBase, &wfAccum, &linStage,
                        &wfHitF})
            b->release();
        bvhs.release(); dobjects.release(); materials.release(); dlights.release(); scratch64.release();
        counters.release(); hitI.release(); wfHitF.release(); wfHitI.release(); wfOccluded.release();
        wfVisible.release(); engine.release();
        if (finished) cudaEventDestroy(finished);
    }
};

namespace {

DevMaterial to_dev(const cgs_material& m)
{
    DevMaterial d;
    std::memcpy(&d, &m, sizeof d);
    return d;
}

// BezierSurface::buildBVH (src/rt/Primitive.cu:199-220): per-patch bounds of
// the 16 projected points and their mean as the centroid.
void build_surface_bvh(Surface& s)
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
    s.bvh.build(el);
}

// Scene::buildBVH (src/rt/Scene.cu:218-232): object bounds of the transformed
// points (BezierSurface::bounds(M), src/rt/Primitive.cu:172-179), centroid =
// box centre.
void build_top_bvh(cgs_scene* sc)
{
    std::vector<Element> el(sc->objects.size());
    for (uint32_t i = 0; i < el.size(); i++)
    {
        const Object& ob = sc->objects[i];
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
        el[i].index = i;
        el[i].bounds = b;
        for (int k = 0; k < 3; k++) el[i].centroid[k] = 0.5f * (b.lo[k] + b.hi[k]);
    }
    sc->top.build(el);
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

uint32_t table_capacity(uint32_t n)
{
    uint32_t step = std::max<uint32_t>(4u, uint32_t(0.05f * float(n)));
    return n + 15u * step;
}

uint32_t displ_size(uint32_t n)
{
    int s = int(n - 1) >> 1;
    if (s < 2) s = 2;
    return std::bit_floor(uint32_t(s));
}

int upload(cgs_scene* sc)
{
    const uint32_t nb = uint32_t(sc->surfaces.size()) + 1;
    std::vector<float4> hp, hn;
    std::vector<uint32_t> hi, pbase, pmat;
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
    std::vector<DevLight> hl;
    for (const auto& l : sc->lights) { DevLight d; std::memcpy(&d, &l, sizeof d); hl.push_back(d); }
    CGS_TRY(sc->patches.reserve(hp.size()));
    CGS_TRY(sc->nodes.reserve(hn.size()));
    CGS_TRY(sc->indices.reserve(hi.size()));
    CGS_TRY(sc->tables.reserve(tableCursor));
    CGS_TRY(sc->disps.reserve(dispCursor));
    CGS_TRY(sc->patchBase.reserve(pbase.size()));
    CGS_TRY(sc->patchMaterial.reserve(std::max<size_t>(pmat.size(), 1)));
    CGS_TRY(sc->bvhs.reserve(nb));
    CGS_TRY(sc->dobjects.reserve(ho.size()));
    CGS_TRY(sc->materials.reserve(hm.size()));
    CGS_TRY(sc->dlights.reserve(std::max<size_t>(hl.size(), 1)));
    CGS_TRY(sc->counters.reserve(1));
    CGS_TRY(sc->work.reserve(8));
    CGS_TRY(cudaMemcpy(sc->patches.p, hp.data(), hp.size() * sizeof(float4), cudaMemcpyHostToDevice));
    CGS_TRY(cudaMemcpy(sc->nodes.p, hn.data(), hn.size() * sizeof(float4), cudaMemcpyHostToDevice));
    CGS_TRY(cudaMemcpy(sc->indices.p, hi.data(), hi.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    CGS_TRY(cudaMemcpy(sc->patchBase.p, pbase.data(), pbase.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    if (!pmat.empty())
        CGS_TRY(cudaMemcpy(sc->patchMaterial.p, pmat.data(), pmat.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    CGS_TRY(cudaMemcpy(sc->dobjects.p, ho.data(), ho.size() * sizeof(DevObject), cudaMemcpyHostToDevice));
    CGS_TRY(cudaMemcpy(sc->materials.p, hm.data(), hm.size() * sizeof(DevMaterial), cudaMemcpyHostToDevice));
    if (!hl.empty()) CGS_TRY(cudaMemcpy(sc->dlights.p, hl.data(), hl.size() * sizeof(DevLight), cudaMemcpyHostToDevice));
    CGS_TRY(cudaMemcpy(sc->bvhs.p, sc->hbvh.data(), nb * sizeof(DevBVH), cudaMemcpyHostToDevice));
    sc->uploaded = true;
    return CGS_OK;
}

int hash_all(cgs_scene* sc, cudaStream_t stream)
{
    const uint32_t nb = uint32_t(sc->surfaces.size()) + 1;
    uint32_t maxn = 1;
    for (uint32_t k = 0; k < nb; k++) maxn = std::max<uint32_t>(maxn, uint32_t(sc->bvh(k).keys.size()));
    size_t w32 = 0, w64 = 0;
    hash_scratch_words(maxn, w32, w64);
    CGS_TRY(sc->scratch32.reserve(w32));
    CGS_TRY(sc->scratch64.reserve(w64));
    CGS_TRY(sc->keys.reserve(maxn));
    for (uint32_t k = 0; k < nb; k++)
    {
        const HostBVH& b = sc->bvh(k);
        uint32_t n = uint32_t(b.keys.size());
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
    CGS_TRY(cudaMemcpyAsync(sc->bvhs.p, sc->hbvh.data(), nb * sizeof(DevBVH), cudaMemcpyHostToDevice, stream));
    CGS_TRY(cudaStreamSynchronize(stream));
    sc->hashed = true;
    return CGS_OK;
}

void camera_setup(const cgs_camera& c, uint32_t w, uint32_t h, int flip, CameraSetup& s)
{
    // Transform::matrix() = T R S with the quaternion rotation of src/AlignedTypes.h:99-115
    float i = c.rotation[0], j = c.rotation[1], k = c.rotation[2], r = c.rotation[3];
    float ii = 2 * i * i, ij = 2 * i * j, ik = 2 * i * k, jj = 2 * j * j, jk = 2 * j * k, kk = 2 * k * k,
          ri = 2 * r * i, rj = 2 * r * j, rk = 2 * r * k;
    float c0[3] = {1 - jj - kk, ij + rk, ik - rj}, c1[3] = {ij - rk, 1 - ii - kk, jk + ri},
          c2[3] = {ik + rj, jk - ri, 1 - ii - jj};
    for (int q = 0; q < 3; q++)
    {
        s.c2w[q] = c0[q] * c.scale[0];
        s.c2w[4 + q] = c1[q] * c.scale[1];
        s.c2w[8 + q] = c2[q] * c.scale[2];
        s.c2w[12 + q] = c.position[q];
        s.pos[q] = c.position[q];
    }
    s.c2w[3] = s.c2w[7] = s.c2w[11] = 0.0f;
    s.c2w[15] = 1.0f;
    // src/rt/RayTracer.cu:152-163
    float halfHeight = std::tan(0.5f * c.fovy);
    s.half_dy = halfHeight / float(h);
    s.half_dx = s.half_dy;
    s.tl[0] = -s.half_dx * float(w - 1);
    s.tl[1] = halfHeight - s.half_dy;
    if (flip) { s.tl[1] = -s.tl[1]; s.half_dy = -s.half_dy; }
}

int ensure_engine(cgs_scene* sc, uint32_t capacity)
{
    if (sc->engineCapacity >= capacity) return CGS_OK;
    CGS_TRY(sc->engine.reserve(engine_words(capacity, kEnginePasses)));
    sc->engineCapacity = capacity;
    return CGS_OK;
}

int ensure_wavefront(cgs_scene* sc, uint32_t nrays)
{
    uint32_t nl = std::max<uint32_t>(1, uint32_t(sc->lights.size()));
    if (sc->wb.capacity >= nrays && sc->wb.lightCapacity >= nl && sc->wb.engine == sc->engine.p) return CGS_OK;
    size_t cap = nrays, sc_ = size_t(nrays) * nl;
    CGS_TRY(sc->wfRay0.reserve(9 * cap));
    CGS_TRY(sc->wfRay1.reserve(9 * cap));
    CGS_TRY(sc->wfPix0.reserve(cap));
    CGS_TRY(sc->wfPix1.reserve(cap));
    CGS_TRY(sc->wfCount.reserve(8));
    CGS_TRY(sc->wfHitF.reserve(3 * cap));
    CGS_TRY(sc->wfHitI.reserve(2 * cap));
    CGS_TRY(sc->wfOccluded.reserve(sc_));
    {
        int r = ensure_engine(sc, uint32_t(std::max<size_t>(cap, sc_)));
        if (r) return r;
    }
    CGS_TRY(sc->wfShadow.reserve(7 * sc_));
    CGS_TRY(sc->wfShadowSlot.reserve(sc_));
    CGS_TRY(sc->wfContrib.reserve(3 * sc_));
    CGS_TRY(sc->wfVisible.reserve(sc_));
    CGS_TRY(sc->wfBase.reserve(3 * cap));
    CGS_TRY(sc->wfAccum.reserve(3 * cap));
    WavefrontBuffers& wb = sc->wb;
    wb.ray[0] = sc->wfRay0.p; wb.ray[1] = sc->wfRay1.p;
    wb.pixel[0] = sc->wfPix0.p; wb.pixel[1] = sc->wfPix1.p;
    wb.count = sc->wfCount.p; wb.shadow = sc->wfShadow.p; wb.shadowSlot = sc->wfShadowSlot.p;
    wb.hit = HitsSoA {sc->wfHitF.p, sc->wfHitF.p + cap, sc->wfHitF.p + 2 * cap, sc->wfHitI.p, sc->wfHitI.p + cap};
    wb.occluded = sc->wfOccluded.p;
    wb.engine = sc->engine.p;
    wb.engineCapacity = sc->engineCapacity;
    wb.contrib = sc->wfContrib.p; wb.visible = sc->wfVisible.p; wb.base = sc->wfBase.p; wb.accum = sc->wfAccum.p;
    wb.capacity = nrays;
    wb.lightCapacity = nl;
    return CGS_OK;
}

bool valid_query(int method, int precision) { return (method == 0 || method == 1) && precision >= 0 && precision <= 2; }

}  // namespace

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

int cgs_version(void) { return 1; }

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
    if (cudaEventCreateWithFlags(&s->finished, cudaEventDisableTiming) != cudaSuccess) { delete s; return CGS_ERR_CUDA; }
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

int cgs_scene_add_object(cgs_scene* s, uint32_t surface, const float l2w[16], const float w2l[16],
                         const cgs_material* material, const uint32_t* pm, const cgs_material* mats, uint32_t nm,
                         uint32_t* oid)
{
    if (!s || !l2w || !w2l || !material) return CGS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    if (surface >= s->surfaces.size()) return CGS_ERR_INVALID_ARGUMENT;
    Object ob;
    ob.surface = surface;
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
    s->bvhBuilt = s->uploaded = s->hashed = false;
    if (oid) *oid = uint32_t(s->objects.size() - 1);
    return CGS_OK;
}

int cgs_scene_set_lights(cgs_scene* s, const cgs_light* lights, uint32_t n)
{
    if (!s || (n && !lights)) return CGS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    s->lights.assign(lights, lights + n);
    if (s->uploaded)
    {
        cudaSetDevice(s->device);
        CGS_TRY(s->dlights.reserve(std::max<uint32_t>(n, 1)));
        if (n) CGS_TRY(cudaMemcpy(s->dlights.p, lights, n * sizeof(cgs_light), cudaMemcpyHostToDevice));
    }
    return CGS_OK;
}

int cgs_scene_set_environment(cgs_scene* s, const float bg[3], const float amb[3])
{
    if (!s || !bg || !amb) return CGS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    for (int k = 0; k < 3; k++) { s->background[k] = bg[k]; s->ambient[k] = amb[k]; }
    return CGS_OK;
}

int cgs_bvh_build(cgs_scene* s)
{
    if (!s) return CGS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    if (s->objects.empty()) return CGS_ERR_INVALID_ARGUMENT;
    for (auto& sf : s->surfaces)
    {
        build_surface_bvh(sf);
        if (sf.bvh.emptyLeaf) return CGS_ERR_EMPTY_LEAF;
    }
    build_top_bvh(s);
    if (s->top.emptyLeaf) return CGS_ERR_EMPTY_LEAF;
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
    b += s->patches.n * sizeof(float4) + s->nodes.n * sizeof(float4);
    b += (s->indices.n + s->tables.n + s->disps.n + s->patchBase.n + s->patchMaterial.n) * sizeof(uint32_t);
    b += s->bvhs.n * sizeof(DevBVH) + s->dobjects.n * sizeof(DevObject) + s->materials.n * sizeof(DevMaterial);
    b += s->dlights.n * sizeof(DevLight);
    *bytes = b;
    return CGS_OK;
}

int cgs_bvh_sizes(const cgs_scene* s, int32_t which, uint32_t sizes[5])
{
    if (!s || !sizes) return CGS_ERR_INVALID_ARGUMENT;
    if (!s->bvhBuilt) return CGS_ERR_NOT_BUILT;
    uint32_t k = which < 0 ? uint32_t(s->surfaces.size()) : uint32_t(which);
    if (k > s->surfaces.size()) return CGS_ERR_INVALID_ARGUMENT;
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
    uint32_t k = which < 0 ? uint32_t(s->surfaces.size()) : uint32_t(which);
    if (k > s->surfaces.size()) return CGS_ERR_INVALID_ARGUMENT;
    const HostBVH& b = s->bvh(k);
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
    if (s->hashed)
    {
        cudaSetDevice(s->device);
        const DevBVH& d = s->hbvh[k];
        if (table) CGS_TRY(cudaMemcpy(table, s->tables.p + d.tableBase, d.N * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        if (disp) CGS_TRY(cudaMemcpy(disp, s->disps.p + d.dispBase, (d.mask + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        if (params) { params[0] = d.A; params[1] = d.B; params[2] = d.N; params[3] = d.mask; }
    }
    else if (params)
        params[0] = params[1] = params[2] = params[3] = 0;
    return CGS_OK;
}

int cgs_intersect(cgs_scene* s, const cgs_rays* rays, uint32_t n, int method, int precision, float tol, int any_hit,
                  const cgs_hits* hits, void* stream)
{
    if (!s || !rays || !hits || !valid_query(method, precision) || !(tol > 0.0f)) return CGS_ERR_INVALID_ARGUMENT;
    if (!hits->patch || (!any_hit && (!hits->t || !hits->u || !hits->v || !hits->object)))
        return CGS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    if (!s->hashed) return CGS_ERR_NOT_BUILT;
    CGS_TRY(cudaSetDevice(s->device));
    cudaStream_t st = (cudaStream_t)stream;
    CGS_TRY(cudaMemsetAsync(s->counters.p, 0, sizeof(Counters), st));
    RaysSoA r {rays->ox, rays->oy, rays->oz, rays->dx, rays->dy, rays->dz, rays->tmax};
    Query q {method, precision, tol};
    s->launches = 0;
    s->primaryRays = n; s->bounceRays = 0; s->shadowRays = 0;
    {
        int er = ensure_engine(s, n);
        if (er) return er;
    }
    cudaError_t e = run_query(s->dev(), r, n, nullptr, q, any_hit != 0,
                              HitsSoA {hits->t, hits->u, hits->v, hits->patch, hits->object}, hits->patch,
                              s->engine.p, s->engineCapacity, kEnginePasses, s->counters.p, st, &s->launches);
    s->lastStream = st;
    return cuda_status(e);
}

int cgs_intersect_host(cgs_scene* s, const cgs_rays* rays, uint32_t n, int method, int precision, float tol,
                       int any_hit, const cgs_hits* hits, void* stream)
{
    if (!s || !rays || !hits) return CGS_ERR_INVALID_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    {
        std::lock_guard<std::mutex> g(s->mu);
        CGS_TRY(cudaSetDevice(s->device));
        CGS_TRY(s->rayStage.reserve(7ull * std::max<uint32_t>(n, 1)));
        CGS_TRY(s->hitF.reserve(3ull * std::max<uint32_t>(n, 1)));
        CGS_TRY(s->hitI.reserve(2ull * std::max<uint32_t>(n, 1)));
        const float* src[7] = {rays->ox, rays->oy, rays->oz, rays->dx, rays->dy, rays->dz, rays->tmax};
        for (int k = 0; k < 7; k++)
        {
            if (!src[k]) return CGS_ERR_INVALID_ARGUMENT;
            CGS_TRY(cudaMemcpyAsync(s->rayStage.p + size_t(k) * n, src[k], n * sizeof(float), cudaMemcpyHostToDevice, st));
        }
    }
    float* R = s->rayStage.p;
    cgs_rays dr {R, R + n, R + 2ull * n, R + 3ull * n, R + 4ull * n, R + 5ull * n, R + 6ull * n};
    cgs_hits dh {s->hitF.p, s->hitF.p + n, s->hitF.p + 2ull * n, s->hitI.p, s->hitI.p + n};
    int r = cgs_intersect(s, &dr, n, method, precision, tol, any_hit, &dh, stream);
    if (r) return r;
    if (hits->patch) CGS_TRY(cudaMemcpyAsync(hits->patch, dh.patch, n * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    if (!any_hit)
    {
        if (hits->t) CGS_TRY(cudaMemcpyAsync(hits->t, dh.t, n * sizeof(float), cudaMemcpyDeviceToHost, st));
        if (hits->u) CGS_TRY(cudaMemcpyAsync(hits->u, dh.u, n * sizeof(float), cudaMemcpyDeviceToHost, st));
        if (hits->v) CGS_TRY(cudaMemcpyAsync(hits->v, dh.v, n * sizeof(float), cudaMemcpyDeviceToHost, st));
        if (hits->object) CGS_TRY(cudaMemcpyAsync(hits->object, dh.object, n * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    }
    CGS_TRY(cudaStreamSynchronize(st));
    return CGS_OK;
}

int cgs_patch_intersect(cgs_scene* s, uint32_t surface, const cgs_rays* rays, const uint32_t* pids, uint32_t n,
                        int method, float tol, const cgs_hits* hits, void* stream)
{
    if (!s || !rays || !pids || !hits || !hits->t || !hits->u || !hits->v || !hits->patch) return CGS_ERR_INVALID_ARGUMENT;
    if (!valid_query(method, 0) || !(tol > 0.0f)) return CGS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    if (!s->uploaded) return CGS_ERR_NOT_BUILT;
    if (surface >= s->surfaces.size()) return CGS_ERR_INVALID_ARGUMENT;
    CGS_TRY(cudaSetDevice(s->device));
    cudaStream_t st = (cudaStream_t)stream;
    CGS_TRY(cudaMemsetAsync(s->counters.p, 0, sizeof(Counters), st));
    RaysSoA r {rays->ox, rays->oy, rays->oz, rays->dx, rays->dy, rays->dz, rays->tmax};
    Query q {method, 0, tol};
    s->launches = 1;
    s->lastStream = st;
    return cuda_status(launch_patch_pairs(s->dev(), surface, r, pids, n, q,
                                          HitsSoA {hits->t, hits->u, hits->v, hits->patch, hits->object}, s->counters.p,
                                          st));
}

int cgs_render(cgs_scene* s, const cgs_camera* cam, uint32_t w, uint32_t h, const cgs_render_options* opt,
               uint32_t* fb, uint32_t stride, float* linear, void* stream)
{
    if (!s || !cam || !opt || w == 0 || h == 0 || (!fb && !linear) || (fb && stride < w)) return CGS_ERR_INVALID_ARGUMENT;
    if (!valid_query(opt->method, opt->precision) || opt->recursion_depth < 0 || opt->recursion_depth > 64 ||
        !(opt->tol > 0.0f) || (opt->schedule != 0 && opt->schedule != 1))
        return CGS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    if (!s->hashed) return CGS_ERR_NOT_BUILT;
    CGS_TRY(cudaSetDevice(s->device));
    cudaError_t q = cudaEventQuery(s->finished);
    if (q == cudaErrorNotReady) return CGS_ERR_BUSY;
    cudaStream_t st = (cudaStream_t)stream;
    RenderParams p {};
    camera_setup(*cam, w, h, opt->flip_y, p.cam);
    p.width = w; p.height = h; p.stride = fb ? stride : w;
    p.depth = opt->recursion_depth; p.eps = opt->eps;
    p.q = Query {opt->method, opt->precision, opt->tol};
    CGS_TRY(cudaMemsetAsync(s->counters.p, 0, sizeof(Counters), st));
    s->launches = 0;
    cudaError_t e;
    if (opt->schedule == CGS_SCHED_PLAIN)
    {
        e = launch_render_plain(s->dev(), p, fb, linear, s->counters.p, st);
        s->launches = 1;
    }
    else
    {
        int r = ensure_wavefront(s, w * h);
        if (r) return r;
        e = launch_render_wavefront(s->dev(), p, s->wb, fb, linear, s->counters.p, st, &s->launches);
    }
    if (e != cudaSuccess) return cuda_status(e);
    CGS_TRY(cudaEventRecord(s->finished, st));
    s->lastStream = st;
    return CGS_OK;
}

int cgs_render_host(cgs_scene* s, const cgs_camera* cam, uint32_t w, uint32_t h, const cgs_render_options* opt,
                    uint32_t* fb, float* linear, void* stream)
{
    if (!s || (!fb && !linear)) return CGS_ERR_INVALID_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    {
        std::lock_guard<std::mutex> g(s->mu);
        CGS_TRY(cudaSetDevice(s->device));
        if (fb) CGS_TRY(s->fbStage.reserve(size_t(w) * h));
        if (linear) CGS_TRY(s->linStage.reserve(3ull * w * h));
    }
    int r = cgs_render(s, cam, w, h, opt, fb ? s->fbStage.p : nullptr, w, linear ? s->linStage.p : nullptr, stream);
    if (r) return r;
    if (fb) CGS_TRY(cudaMemcpyAsync(fb, s->fbStage.p, size_t(w) * h * 4, cudaMemcpyDeviceToHost, st));
    if (linear) CGS_TRY(cudaMemcpyAsync(linear, s->linStage.p, 12ull * w * h, cudaMemcpyDeviceToHost, st));
    CGS_TRY(cudaStreamSynchronize(st));
    return CGS_OK;
}

int cgs_render_running(cgs_scene* s)
{
    if (!s) return 0;
    return cudaEventQuery(s->finished) == cudaErrorNotReady ? 1 : 0;
}

int cgs_scene_counters(cgs_scene* s, cgs_counters* out)
{
    if (!s || !out) return CGS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    CGS_TRY(cudaSetDevice(s->device));
    if (!s->counters.p) { std::memset(out, 0, sizeof *out); return CGS_OK; }
    CGS_TRY(cudaStreamSynchronize(s->lastStream));
    Counters c;
    CGS_TRY(cudaMemcpy(&c, s->counters.p, sizeof c, cudaMemcpyDeviceToHost));
    std::memset(out, 0, sizeof *out);
    out->rays = c.rays; out->nodes = c.nodes; out->hash_lookups = c.hashLookups; out->candidates = c.candidates;
    out->iterations = c.iterations; out->device_errors = c.errors; out->kernel_launches = uint64_t(s->launches);
    return CGS_OK;
}

int cgs_perfect_hash_build(const uint32_t* keys, uint32_t n, uint32_t* disp, uint32_t dcap, uint32_t* table,
                           uint32_t tcap, uint32_t params[5], void* stream)
{
    if (!keys || !disp || !table || !params || n == 0) return CGS_ERR_INVALID_ARGUMENT;
    if (dcap < displ_size(n) || tcap < table_capacity(n)) return CGS_ERR_INVALID_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    size_t w32 = 0, w64 = 0;
    hash_scratch_words(n, w32, w64);
    uint32_t* s32 = nullptr;
    unsigned long long* s64 = nullptr;
    CGS_TRY(cudaMallocAsync(&s32, w32 * sizeof(uint32_t), st));
    if (cudaMallocAsync(&s64, w64 * sizeof(unsigned long long), st) != cudaSuccess)
    {
        cudaFreeAsync(s32, st);
        return CGS_ERR_OUT_OF_MEMORY;
    }
    HashScratch hs {};
    hash_scratch_carve(hs, n, s32, s64);
    uint32_t A[16], B[16];
    hash_coefficients(n, A, B);
    int r = hash_build_device(keys, n, A, B, disp, table, tcap, hs, params, st, nullptr);
    cudaFreeAsync(s32, st);
    cudaFreeAsync(s64, st);
    cudaStreamSynchronize(st);
    if (r == 4) return CGS_ERR_HASH_BUCKET_OVERFLOW;
    if (r < 0) return CGS_ERR_CUDA;
    if (r) return CGS_ERR_HASH_FAILED;
    return CGS_OK;
}

}  // extern "C"
