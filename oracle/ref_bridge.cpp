// ref_bridge.cpp -- TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.
//
// A C ABI over the reference program's own hot-path code, compiled unchanged
// from the reference's sources by oracle/build_ref.py into
// oracle/_ref/libcgs_ref.so (host only, g++, against the from-scratch Ds
// stand-in in oracle/ds_compat).  The tests use it to check the oracle's
// restatement (oracle/cgs_oracle.cpp) against the reference itself:
//
//   * surface BVHs built by BezierSurface::buildBVH and BVH::build
//     (src/rt/Primitive.cu:199-220, src/rt/BVH.cpp:9-124), the object-level
//     BVH by Scene::buildBVH (src/rt/Scene.cu:39-53);
//   * closest and any hits through CPURayTracer::intersect
//     (src/rt/CPURayTracer.cpp:221-279) -- the two-level traversal,
//     BVH::hashIntersect (src/rt/BVH.h:179-350), rt::intersect
//     (src/rt/Primitive.cu:222-268) and spline::doBezierClipping's host path
//     (src/Spline_BezierClipping.cu:47-445);
//   * frames through CPURayTracer::render (src/rt/CPURayTracer.cpp:55-197),
//     and linear colours through its trace / closestHit and PBR;
//   * single (ray, patch) pairs through spline::doBezierClipping and
//     spline::doSubdivision (host paths, src/Spline_Subdivision.cu:168-302).
//
// Two things are not the reference's code:
//   * PerfectHashFunction::build (src/rt/PerfectHashFunction.cu:229-505)
//     launches CUDA kernels and places buckets with racing atomics, so its
//     tables differ run to run; it cannot run on a host without a GPU.  Its
//     definition below takes the displacement table and coefficients from the
//     oracle's deterministic restatement (ora_hash_build).  The reference's
//     BVH::buildHashTable then fills its table with the reference's own
//     PerfectHashFunction::hash, and the traversal looks nodes up through it.
//   * The CUDA runtime calls of that code (managed allocation) are served by
//     oracle/ref_host_cudart.cpp from host memory.
//
// The tracer's private trace / intersect members and its private scene
// pointer are reached through member pointers formed in explicit template
// instantiations, where C++ waives access checks; the reference's headers
// are included as they are.
#include <algorithm>
#include <cstring>
#include <memory_resource>
#include <thread>
#include <vector>

#include <graphics/Color.h>

#include "rt/CPURayTracer.h"
#include "rt/Primitive.h"
#include "rt/Scene.h"
#include "Spline.h"

extern "C" int ora_hash_build(const uint32_t* keys, uint32_t n, uint32_t* out_params, uint32_t* disp,
                              uint32_t disp_cap, uint32_t* table, uint32_t table_cap);

namespace cg::rt
{

int PerfectHashFunction::build(span<const uint32_t> keys, cudaStream_t)
{
    const uint32_t n = uint32_t(keys.size());
    if (n == 0) return 1;
    const uint32_t step = std::max<uint32_t>(4u, uint32_t(0.05f * float(n)));
    std::vector<uint32_t> disp(std::max<uint32_t>(2u, n)), table(n + 16u * step + 16u);
    uint32_t par[5] = {};
    const int e = ora_hash_build(keys.data(), n, par, disp.data(), uint32_t(disp.size()), table.data(),
                                 uint32_t(table.size()));
    if (e) return e;
    _A = par[0];
    _B = par[1];
    _tableSize = par[2];
    _displMask = par[3];
    _displacement.resize(size_t(par[3]) + 1);
    std::copy_n(disp.data(), size_t(par[3]) + 1, _displacement.data());
    return 0;
}

} // namespace cg::rt

namespace {

using namespace cg;
using rt::CPURayTracer;

// Member pointers to private members, formed where access is not checked.
template<typename Tag, typename Tag::type M>
struct Expose
{
    friend typename Tag::type member(Tag) { return M; }
};

struct TraceTag
{
    using type = rt::vec3 (CPURayTracer::*)(const rt::Ray&, rt::vec3, int) const;
    friend type member(TraceTag);
};
struct ClosestTag
{
    using type = int (CPURayTracer::*)(rt::Intersection&, const rt::Ray&) const;
    friend type member(ClosestTag);
};
struct AnyTag
{
    using type = bool (CPURayTracer::*)(const rt::Ray&) const;
    friend type member(AnyTag);
};
struct SceneTag
{
    using type = const rt::Scene* CPURayTracer::*;
    friend type member(SceneTag);
};
struct PixelTag
{
    using type = rt::vec3 (CPURayTracer::*)(float, float) const;
    friend type member(PixelTag);
};
struct CamPosTag
{
    using type = rt::vec3 CPURayTracer::*;
    friend type member(CamPosTag);
};

template struct Expose<TraceTag, &CPURayTracer::trace>;
template struct Expose<ClosestTag, &CPURayTracer::intersect>;
template struct Expose<AnyTag, &CPURayTracer::intersect>;
template struct Expose<SceneTag, &CPURayTracer::_scene>;
template struct Expose<PixelTag, &CPURayTracer::pixelRayDirection>;
template struct Expose<CamPosTag, &CPURayTracer::_cameraPosition>;

struct SurfaceIn
{
    std::vector<float> points;     // 4 per point
    std::vector<uint32_t> indices; // 16 per patch
};

struct ObjectIn
{
    int surface;
    float l2w[16], w2l[16];
    float material[8];
};

// A scene as the reference's application builds it (src/MainWindow.cpp:363-492),
// in host memory.
struct RefScene
{
    std::vector<SurfaceIn> surfaces;
    std::vector<ObjectIn> objects;
    std::vector<float> lights;  // 12 per light, in rt::Light field order
    float background[3] = {0.1f, 0.1f, 0.1f};
    float ambient[3] = {0.1f, 0.1f, 0.1f};
    std::unique_ptr<rt::Scene> scene;
    bool built = false;
};

rt::mat4 load_mat4(const float* m)
{
    return rt::mat4(rt::vec4(m[0], m[1], m[2], m[3]), rt::vec4(m[4], m[5], m[6], m[7]),
                    rt::vec4(m[8], m[9], m[10], m[11]), rt::vec4(m[12], m[13], m[14], m[15]));
}

template<typename F>
void parallel_ranges(uint64_t n, int threads, F&& fn)
{
    threads = std::max(1, std::min<int>(threads, int(std::min<uint64_t>(n, 256))));
    if (threads <= 1 || n < 64)
    {
        fn(0, n);
        return;
    }
    std::vector<std::thread> pool;
    const uint64_t chunk = (n + threads - 1) / threads;
    for (int t = 0; t < threads; t++)
    {
        const uint64_t a = t * chunk, b = std::min(n, a + chunk);
        if (a < b) pool.emplace_back([&, a, b] { fn(a, b); });
    }
    for (auto& th : pool) th.join();
}

rt::Camera make_camera(const float* c11)
{
    rt::Camera cam {};
    cam.transform.rotation = rt::quat(c11[0], c11[1], c11[2], c11[3]);
    cam.transform.position = rt::vec3(c11[4], c11[5], c11[6]);
    cam.transform.scale = rt::vec3(c11[7], c11[8], c11[9]);
    cam.fieldOfView = c11[10];
    cam.aspectRatio = 1.0f;
    cam.height = 1.0f;
    cam.projection = rt::Camera::Perspective;
    return cam;
}

} // namespace

extern "C" {

void* ref_scene_new() { return new RefScene; }
void ref_scene_free(void* s) { delete static_cast<RefScene*>(s); }

int ref_scene_add_surface(void* s_, const float* points4, uint32_t npoints, const uint32_t* indices,
                          uint32_t nindices)
{
    auto* s = static_cast<RefScene*>(s_);
    if (s->built || nindices == 0 || nindices % 16) return -1;
    SurfaceIn in;
    in.points.assign(points4, points4 + 4 * size_t(npoints));
    in.indices.assign(indices, indices + nindices);
    for (uint32_t i : in.indices)
        if (i >= npoints) return -1;
    s->surfaces.push_back(std::move(in));
    return int(s->surfaces.size()) - 1;
}

// material8 = diffuse[3], specular[3], metalness, roughness (rt::Material)
int ref_scene_add_object(void* s_, int surface, const float* l2w, const float* w2l, const float* material8)
{
    auto* s = static_cast<RefScene*>(s_);
    if (s->built || surface < 0 || surface >= int(s->surfaces.size())) return -1;
    ObjectIn ob;
    ob.surface = surface;
    std::memcpy(ob.l2w, l2w, sizeof ob.l2w);
    std::memcpy(ob.w2l, w2l, sizeof ob.w2l);
    std::memcpy(ob.material, material8, sizeof ob.material);
    s->objects.push_back(ob);
    return int(s->objects.size()) - 1;
}

// lights12 = color[3], strength, position[3], range, direction[3], angle (rt::Light)
int ref_scene_set_lights(void* s_, const float* lights12, uint32_t n)
{
    auto* s = static_cast<RefScene*>(s_);
    if (s->built) return -1;
    s->lights.assign(lights12, lights12 + 12 * size_t(n));
    return 0;
}

void ref_scene_set_env(void* s_, const float* bg3, const float* amb3)
{
    auto* s = static_cast<RefScene*>(s_);
    std::memcpy(s->background, bg3, sizeof s->background);
    std::memcpy(s->ambient, amb3, sizeof s->ambient);
}

// Builds the rt::Scene: control points and indices in scene buffers, one
// BezierSurface and BVH per surface (BezierSurface::buildBVH, then
// BVH::buildHashTable), the objects' matrices and materials, the lights and
// the object-level BVH (Scene::buildBVH, then its hash table).  Returns 0, or
// 1 when a build throws (an empty leaf or a failed hash), 2 without objects.
int ref_scene_build(void* s_)
{
    auto* s = static_cast<RefScene*>(s_);
    if (s->built) return 0;
    if (s->objects.empty()) return 2;
    auto* mr = std::pmr::new_delete_resource();
    try
    {
        s->scene = std::make_unique<rt::Scene>(uint32_t(s->objects.size()), mr);
        rt::Scene& sc = *s->scene;
        sc.surfaces.reserve(s->surfaces.size());
        sc.bvhs.reserve(s->surfaces.size());
        for (const SurfaceIn& in : s->surfaces)
        {
            const uint32_t np = uint32_t(in.points.size() / 4);
            rt::vec4* pts = sc.createBuffer<rt::vec4>(np);
            for (uint32_t i = 0; i < np; i++)
                pts[i] = rt::vec4(in.points[4 * i], in.points[4 * i + 1], in.points[4 * i + 2], in.points[4 * i + 3]);
            uint32_t* idx = sc.createBuffer<uint32_t>(uint32_t(in.indices.size()));
            std::copy(in.indices.begin(), in.indices.end(), idx);
            auto& surf = sc.surfaces.emplace_back();
            surf.vertices = pts;
            surf.indices = idx;
            surf.indexCount = uint32_t(in.indices.size());
            auto& bvh = sc.bvhs.emplace_back(mr);
            surf.buildBVH(bvh);
            bvh.buildHashTable();
        }
        for (const ObjectIn& ob : s->objects)
        {
            rt::Material m {};
            m.diffuse = rt::vec3(ob.material[0], ob.material[1], ob.material[2]);
            m.specular = rt::vec3(ob.material[3], ob.material[4], ob.material[5]);
            m.metalness = ob.material[6];
            m.roughness = ob.material[7];
            // as the reference's application fills the object arrays
            // (src/MainWindow.cpp:425-482)
            using Key = rt::Scene::Key;
            const auto last = sc.objects.size();
            sc.objects.emplace_back();
            sc.objects.get<Key::eLocal2WorldMatrix>(last) = load_mat4(ob.l2w);
            sc.objects.get<Key::eWorld2LocalMatrix>(last) = load_mat4(ob.w2l);
            sc.objects.get<Key::eMaterial>(last) = m;
            sc.objects.get<Key::ePrimitive>(last) = &sc.surfaces[ob.surface];
            sc.objects.get<Key::ePrimitiveType>(last) = rt::PrimitiveType::eBezierSurface;
        }
        for (size_t i = 0; i + 12 <= s->lights.size(); i += 12)
        {
            const float* l = s->lights.data() + i;
            rt::Light L {};
            L.color = rt::vec3(l[0], l[1], l[2]);
            L.strength = l[3];
            L.position = rt::vec3(l[4], l[5], l[6]);
            L.range = l[7];
            L.direction = rt::vec3(l[8], l[9], l[10]);
            L.angle = l[11];
            sc.lights.push_back(L);
        }
        sc.backgroundColor = rt::vec3(s->background[0], s->background[1], s->background[2]);
        sc.ambientLight = rt::vec3(s->ambient[0], s->ambient[1], s->ambient[2]);
        sc.buildBVH();
        sc.topLevelBVH.buildHashTable();
    }
    catch (const std::exception&)
    {
        s->scene.reset();
        return 1;
    }
    s->built = true;
    return 0;
}

// Sizes of BVH `which` (surface index, or -1 for the object-level BVH):
// out3 = nodes, keys, indices.
int ref_bvh_sizes(void* s_, int which, uint32_t* out3)
{
    auto* s = static_cast<RefScene*>(s_);
    if (!s->built) return -1;
    const rt::BVH* b = which < 0 ? &s->scene->topLevelBVH
                                 : (which < int(s->scene->bvhs.size()) ? &s->scene->bvhs[which] : nullptr);
    if (!b) return -1;
    out3[0] = uint32_t(b->nodes().size());
    out3[1] = uint32_t(b->keys().size());
    out3[2] = uint32_t(b->indices().size());
    return 0;
}

// Nodes as 14 words each: leftBox min, max; rightBox min, max (floats), left,
// right/first (u32); then keys and the EMPTY-terminated leaf lists.
int ref_bvh_export(void* s_, int which, uint32_t* nodes14, uint32_t* keys, uint32_t* indices)
{
    auto* s = static_cast<RefScene*>(s_);
    if (!s->built) return -1;
    const rt::BVH* b = which < 0 ? &s->scene->topLevelBVH
                                 : (which < int(s->scene->bvhs.size()) ? &s->scene->bvhs[which] : nullptr);
    if (!b) return -1;
    const auto nodes = b->nodes();
    for (size_t i = 0; i < nodes.size(); i++)
    {
        const auto& n = nodes[i];
        const float f[12] = {n.leftBox.min().x, n.leftBox.min().y, n.leftBox.min().z,
                             n.leftBox.max().x, n.leftBox.max().y, n.leftBox.max().z,
                             n.rightBox.min().x, n.rightBox.min().y, n.rightBox.min().z,
                             n.rightBox.max().x, n.rightBox.max().y, n.rightBox.max().z};
        std::memcpy(nodes14 + 14 * i, f, sizeof f);
        nodes14[14 * i + 12] = n.left;
        nodes14[14 * i + 13] = n.right;
    }
    std::copy(b->keys().begin(), b->keys().end(), keys);
    std::copy(b->indices().begin(), b->indices().end(), indices);
    return 0;
}

// Rays as 7 x n floats (origin, unit direction, max).  Closest hits: out_f =
// 3 x n (t, u, v), out_i = 2 x n (patch, object; -1 for a miss).  Any hit:
// out_i[0][r] = 1 when something blocks ray r before its max, else 0.
int ref_intersect(void* s_, const float* rays, uint64_t n, int any_hit, float* out_f, int32_t* out_i, int nthreads)
{
    auto* s = static_cast<RefScene*>(s_);
    if (!s->built) return -1;
    CPURayTracer tracer;
    tracer.*member(SceneTag {}) = s->scene.get();
    const auto closest = member(ClosestTag {});
    const auto any = member(AnyTag {});
    parallel_ranges(n, nthreads, [&](uint64_t a, uint64_t b) {
        for (uint64_t r = a; r < b; r++)
        {
            rt::Ray ray {};
            ray.origin = rt::vec3(rays[r], rays[n + r], rays[2 * n + r]);
            ray.direction = rt::vec3(rays[3 * n + r], rays[4 * n + r], rays[5 * n + r]);
            ray.max = rays[6 * n + r];
            if (any_hit)
            {
                out_i[r] = (tracer.*any)(ray) ? 1 : 0;
                out_i[n + r] = -1;
                continue;
            }
            rt::Intersection hit {};
            hit.object = nullptr;
            hit.t = ray.max;
            const int ob = (tracer.*closest)(hit, ray);
            out_f[r] = ob >= 0 ? hit.t : ray.max;
            out_f[n + r] = ob >= 0 ? hit.coordinates.x : 0.0f;
            out_f[2 * n + r] = ob >= 0 ? hit.coordinates.y : 0.0f;
            out_i[r] = ob >= 0 ? int32_t(hit.index) : -1;
            out_i[n + r] = ob;
        }
    });
    return 0;
}

// One frame through CPURayTracer::render (32x32 tiles on `nthreads`
// workers, clamp, pack_sRGB) into out_packed (h x w), then, when out_rgb is
// given, every pixel's linear colour again through CPURayTracer::trace,
// clamped to [0, 1] as the tile loop does (h x w x 3).
int ref_render(void* s_, const float* camera11, uint32_t w, uint32_t h, int depth, float eps, int nthreads,
               uint32_t* out_packed, float* out_rgb)
{
    auto* s = static_cast<RefScene*>(s_);
    if (!s->built || w == 0 || h == 0) return -1;
    const rt::Camera cam = make_camera(camera11);
    rt::Frame frame(w, h, std::pmr::new_delete_resource());
    CPURayTracer tracer;
    tracer.options.recursionDepth = depth;
    tracer.options.eps = eps;
    tracer.options.threads = std::max(1, nthreads);
    tracer.options.tileSize = 32;
    tracer.render(&frame, &cam, s->scene.get());
    for (const auto& f : tracer.workers()) f.wait();
    if (out_packed)
        for (uint32_t j = 0; j < h; j++)
            for (uint32_t i = 0; i < w; i++) out_packed[size_t(j) * w + i] = frame.at(i, j);
    if (out_rgb)
    {
        tracer.*member(SceneTag {}) = s->scene.get();
        const auto trace = member(TraceTag {});
        const auto pixel = member(PixelTag {});
        const rt::vec3 origin = tracer.*member(CamPosTag {});
        parallel_ranges(uint64_t(w) * h, nthreads, [&](uint64_t a, uint64_t b) {
            for (uint64_t px = a; px < b; px++)
            {
                const uint32_t i = uint32_t(px % w), j = uint32_t(px / w);
                rt::Ray ray {};
                ray.origin = origin;
                ray.direction = (tracer.*pixel)(float(i), float(j));
                ray.max = std::numeric_limits<float>::infinity();
                rt::vec3 c = (tracer.*trace)(ray, rt::vec3(1), depth);
                out_rgb[3 * px] = std::clamp(c.x, 0.0f, 1.0f);
                out_rgb[3 * px + 1] = std::clamp(c.y, 0.0f, 1.0f);
                out_rgb[3 * px + 2] = std::clamp(c.z, 0.0f, 1.0f);
            }
        });
    }
    return 0;
}

// One (ray, patch) pair: method 0 = spline::doBezierClipping, 1 =
// spline::doSubdivision (both host paths).  ray9 = origin, unit direction,
// tMin, tMax, and the current best distance (in: the cull; out: the hit's t).
// uv receives the hit's (u, v).  Returns 1 on a closer hit, else 0.
int ref_patch_intersect(const float* points4, uint32_t npoints, const uint32_t* idx16, const float* ray9, float tol,
                        int method, float* t_inout, float* uv)
{
    std::vector<spline::vec4> pts(npoints);
    for (uint32_t i = 0; i < npoints; i++)
        pts[i] = spline::vec4(points4[4 * i], points4[4 * i + 1], points4[4 * i + 2], points4[4 * i + 3]);
    for (int i = 0; i < 16; i++)
        if (idx16[i] >= npoints) return -1;
    cg::Ray3f ray {vec3f(ray9[0], ray9[1], ray9[2]), vec3f(ray9[3], ray9[4], ray9[5])};
    ray.tMin = ray9[6];
    ray.tMax = ray9[7];
    cg::Intersection hit {};
    hit.distance = *t_inout;
    const bool found = method == 1 ? spline::doSubdivision(hit, ray, pts.data(), idx16, tol)
                                   : spline::doBezierClipping(hit, ray, pts.data(), idx16, tol);
    if (found)
    {
        *t_inout = hit.distance;
        uv[0] = hit.p.x;
        uv[1] = hit.p.y;
    }
    return found ? 1 : 0;
}

// rt::normal(const BezierSurface&, const Intersection&): the unit normal of
// patch `patch` at (u, v), for n queries.
int ref_patch_normal(const float* points4, uint32_t npoints, const uint32_t* indices, uint32_t npatches,
                     const uint32_t* patch, const float* u, const float* v, uint32_t n, float* out3)
{
    std::vector<rt::vec4> pts(npoints);
    for (uint32_t i = 0; i < npoints; i++)
        pts[i] = rt::vec4(points4[4 * i], points4[4 * i + 1], points4[4 * i + 2], points4[4 * i + 3]);
    rt::BezierSurface surf {};
    surf.vertices = pts.data();
    surf.indices = const_cast<uint32_t*>(indices);
    surf.indexCount = 16 * npatches;
    for (uint32_t q = 0; q < n; q++)
    {
        if (patch[q] >= npatches) return -1;
        rt::Intersection hit {};
        hit.index = patch[q];
        hit.coordinates = rt::vec3(u[q], v[q], 0.0f);
        const rt::vec3 nn = rt::normal(surf, hit);
        out3[3 * q] = nn.x;
        out3[3 * q + 1] = nn.y;
        out3[3 * q + 2] = nn.z;
    }
    return 0;
}

// pack_sRGB of the Ds stand-in, for n colours (3 floats each).
void ref_pack_srgb(const float* rgb, uint64_t n, uint32_t* out)
{
    for (uint64_t i = 0; i < n; i++) out[i] = cg::pack_sRGB(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]);
}

} // extern "C"
