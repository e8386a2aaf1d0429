// k_render.cu -- rendering: camera rays, PBR shading with shadow rays and
// mirror bounces, sRGB packing.  Two schedules:
//   plain     -- one thread per pixel runs the whole bounce chain, 8x8 blocks
//                (the reference's launch shape, src/rt/RayTracer.cu:171-274);
//   wavefront -- a closest-hit pass, a shading pass that queues shadow and
//                bounce rays, an any-hit pass over the shadow queue and a
//                resolve pass, per bounce level; persistent grid-stride kernels
//                read queue sizes from device memory, so a frame needs no
//                host round trip.
#include "kernels.h"

namespace cgs {

namespace {

constexpr float kMinRadiance = 0x1p-8f;  // src/rt/RayTracer.h:16

__device__ __forceinline__ float3 pixel_dir(const CameraSetup& c, float x, float y)  // src/rt/RayTracer.cu:59-71
{
    float3 P = f3(c.tl[0] + c.half_dx * (2.0f * x), c.tl[1] - c.half_dy * (2.0f * y), -1.0f);
    float4 W = m4_point(c.c2w, P);
    return versor(project(W) - f3(c.pos[0], c.pos[1], c.pos[2]));
}

// Shading frame of a hit (Context::closestHit, src/rt/RayTracer.cu:397-437).
struct Frame
{
    float3 P, N, V, diffuse;
    float dotNV;
    DevMaterial m;
};

__device__ __forceinline__ Frame shade_frame(const DevScene& S, float3 o, float3 d, const HitRecord& hit)
{
    Frame f;
    const DevObject& ob = S.objects[hit.object];
    f.m = hit_material(S, ob, uint32_t(hit.patch));
    f.diffuse = (1.0f - f.m.metalness) * (f3(f.m.diffuse[0], f.m.diffuse[1], f.m.diffuse[2]) * kInvPi);
    f.V = -d;
    const float4* P16 = S.patches + 16ull * (__ldg(S.patchBase + ob.surface) + uint32_t(hit.patch));
    float3 N = versor(patch_normal(P16, hit.u, hit.v));  // rt::normal, src/rt/Primitive.cu:270-275
    N = versor(m3T_vec(ob.w2l, N));
    float dotNV = dot(N, f.V);
    if (dotNV < 0.0f) { N = -N; dotNV = -dotNV; }
    f.N = N;
    f.dotNV = dotNV;
    f.P = o + hit.t * d;
    return f;
}

// One light's unshadowed contribution (src/rt/RayTracer.cu:440-466); false
// when the light does not reach the point.
__device__ __forceinline__ bool light_term(const Frame& f, const DevLight& l, float3& contrib, float3& L, float& dist)
{
    if (!lightVector(dist, L, f.P, l)) return false;
    const float dotNL = dot(f.N, L);
    if (dotNL < 1e-14f) return false;
    float3 H = versor(L + f.V);
    float dotHN = dot(H, f.N), dotHL = dot(H, L);
    float3 I = lightColor(dist, l);
    float3 f0 = f3(f.m.specular[0], f.m.specular[1], f.m.specular[2]);
    contrib = (I * dotNL) * (f.diffuse + f.m.metalness * BRDF_specular(dotHL, dotHN, f.dotNV, dotNL, f.m.roughness, f0));
    return true;
}

// Mirror bounce of the non Monte-Carlo path (src/rt/RayTracer.cu:523-542).
__device__ __forceinline__ bool bounce(const Frame& f, float3 att, float3& R, float3& a)
{
    float3 f0 = f3(f.m.specular[0], f.m.specular[1], f.m.specular[2]);
    float3 reflectance = schlick(f0, f.dotNV);
    R = (-f.V) - (2.0f * (-f.dotNV)) * f.N;
    float g = Gsmith(f.dotNV, f.dotNV, f.m.roughness);
    float r1 = 1.0f - f.m.roughness;
    float3 brdf = (f.dotNV * (f.diffuse + f.m.metalness * (reflectance * g))) * (r1 * r1);
    a = att * brdf;
    return vmax3(a) > kMinRadiance;
}

__device__ __forceinline__ void store_pixel(const RenderParams& p, uint32_t px, float3 c, uint32_t* fb, float* linear)
{
    c = f3(__saturatef(c.x), __saturatef(c.y), __saturatef(c.z));
    uint32_t i = px % p.width, j = px / p.width;
    if (fb) fb[size_t(j) * p.stride + i] = pack_srgb(c);
    if (linear) { linear[3ull * px] = c.x; linear[3ull * px + 1] = c.y; linear[3ull * px + 2] = c.z; }
}

// ------------------------------------------------------------- plain --
__global__ void __launch_bounds__(64) k_render_plain(DevScene S, RenderParams p, uint32_t* fb, float* linear,
                                                     Counters* cnt)
{
    const uint32_t i = blockIdx.x * 8 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
    LocalCounters lc;
    uint32_t nrays = 0;
    if (i < p.width && j < p.height)
    {
        float3 o = f3(p.cam.pos[0], p.cam.pos[1], p.cam.pos[2]);
        float3 d = pixel_dir(p.cam, float(i), float(j));
        float3 color = f3(0.0f, 0.0f, 0.0f), att = f3(1.0f, 1.0f, 1.0f);
        int depth = p.depth;
        for (int level = 0; level <= p.depth; level++)
        {
            nrays++;
            HitRecord hit {INFINITY, 0.0f, 0.0f, -1, -1};
            int ob = scene_closest(S, o, d, INFINITY, p.q, hit, lc);
            if (ob < 0) { color = color + f3(S.background[0], S.background[1], S.background[2]) * att; break; }
            Frame f = shade_frame(S, o, d, hit);
            float3 c = f3(S.ambient[0], S.ambient[1], S.ambient[2]) * f.diffuse;
            for (uint32_t l = 0; l < S.nlights; l++)
            {
                float3 contrib, L; float dist;
                if (!light_term(f, S.lights[l], contrib, L, dist)) continue;
                nrays++;
                if (scene_any(S, f.P + p.eps * L, L, dist, p.q, lc)) continue;
                c = c + contrib;
            }
            color = color + (c * kPi) * att;
            if (depth <= 0) break;
            float3 R, a;
            if (!bounce(f, att, R, a)) break;
            o = f.P + p.eps * R;
            d = R;
            att = a;
            depth--;
        }
        store_pixel(p, j * p.width + i, color, fb, linear);
    }
    flush_counters(cnt, lc, nrays);
}

// --------------------------------------------------------- wavefront --
constexpr int kWfThreads = 128;

// queue layout: 9 floats per ray (SoA with stride = capacity)
struct Q
{
    float* r; uint32_t* px; uint32_t cap;
    __device__ __forceinline__ void put(uint32_t k, float3 o, float3 d, float3 a, uint32_t pixel) const
    {
        r[k] = o.x; r[cap + k] = o.y; r[2ull * cap + k] = o.z;
        r[3ull * cap + k] = d.x; r[4ull * cap + k] = d.y; r[5ull * cap + k] = d.z;
        r[6ull * cap + k] = a.x; r[7ull * cap + k] = a.y; r[8ull * cap + k] = a.z;
        px[k] = pixel;
    }
    __device__ __forceinline__ void get(uint32_t k, float3& o, float3& d) const
    {
        o = f3(r[k], r[cap + k], r[2ull * cap + k]);
        d = f3(r[3ull * cap + k], r[4ull * cap + k], r[5ull * cap + k]);
    }
    __device__ __forceinline__ float3 att(uint32_t k) const
    {
        return f3(r[6ull * cap + k], r[7ull * cap + k], r[8ull * cap + k]);
    }
};

__global__ void k_wf_camera(RenderParams p, Q q, float* accum, uint32_t* count)
{
    const uint32_t n = p.width * p.height;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    {
        uint32_t i = k % p.width, j = k / p.width;
        float3 o = f3(p.cam.pos[0], p.cam.pos[1], p.cam.pos[2]);
        q.put(k, o, pixel_dir(p.cam, float(i), float(j)), f3(1.0f, 1.0f, 1.0f), k);
        accum[3ull * k] = 0.0f; accum[3ull * k + 1] = 0.0f; accum[3ull * k + 2] = 0.0f;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) { count[0] = n; count[1] = 0; count[2] = 0; }
}

__global__ void __launch_bounds__(kWfThreads) k_wf_shade(DevScene S, RenderParams p, Q q, Q qn, const uint32_t* count,
                                                         uint32_t* nextCount, uint32_t* shadowCount, HitsSoA hits,
                                                         float* shadow, uint32_t* shadowSlot, uint32_t shadowCap,
                                                         float* contrib, int32_t* visible, float* base, float* accum,
                                                         int depthLeft)
{
    const uint32_t n = *count;
    const uint32_t nl = S.nlights;
    for (uint32_t k0 = blockIdx.x * blockDim.x; k0 < n; k0 += gridDim.x * blockDim.x)
    {
        const uint32_t k = k0 + threadIdx.x;
        const bool live = k < n;
        HitRecord h {INFINITY, 0.0f, 0.0f, -1, -1};
        float3 o = f3(0, 0, 0), d = f3(0, 0, 1), att = f3(0, 0, 0);
        uint32_t pixel = 0;
        if (live)
        {
            h = HitRecord {hits.t[k], hits.u[k], hits.v[k], hits.patch[k], hits.object[k]};
            q.get(k, o, d); att = q.att(k); pixel = q.px[k];
        }
        const bool isHit = live && h.object >= 0;
        if (live && !isHit)
        {
            float3 bg = f3(S.background[0], S.background[1], S.background[2]) * att;
            accum[3ull * pixel] += bg.x; accum[3ull * pixel + 1] += bg.y; accum[3ull * pixel + 2] += bg.z;
        }
        Frame f;
        if (isHit)
        {
            f = shade_frame(S, o, d, h);
            float3 c0 = f3(S.ambient[0], S.ambient[1], S.ambient[2]) * f.diffuse;
            base[3ull * k] = c0.x; base[3ull * k + 1] = c0.y; base[3ull * k + 2] = c0.z;
        }
        for (uint32_t l = 0; l < nl; l++)
        {
            float3 c, L; float dist = 0.0f;
            bool want = isHit && light_term(f, S.lights[l], c, L, dist);
            uint32_t slot = k * nl + l;
            if (isHit)
            {
                visible[slot] = 0;
                if (want) { contrib[3ull * slot] = c.x; contrib[3ull * slot + 1] = c.y; contrib[3ull * slot + 2] = c.z; }
            }
            uint32_t sk = warp_push(shadowCount, want);
            if (want && sk < shadowCap)
            {
                float3 so = f.P + p.eps * L;
                shadow[sk] = so.x; shadow[shadowCap + sk] = so.y; shadow[2ull * shadowCap + sk] = so.z;
                shadow[3ull * shadowCap + sk] = L.x; shadow[4ull * shadowCap + sk] = L.y;
                shadow[5ull * shadowCap + sk] = L.z; shadow[6ull * shadowCap + sk] = dist;
                shadowSlot[sk] = slot;
            }
        }
        float3 R = f3(0, 0, 0), a = f3(0, 0, 0);
        bool more = isHit && depthLeft > 0 && bounce(f, att, R, a);
        uint32_t nk = warp_push(nextCount, more);
        if (more) qn.put(nk, f.P + p.eps * R, R, a, pixel);
    }
}

__global__ void k_wf_visibility(const int32_t* occluded, const uint32_t* shadowSlot, const uint32_t* count, uint32_t cap,
                                int32_t* visible)
{
    const uint32_t n = min(*count, cap);
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        if (occluded[k] < 0) visible[shadowSlot[k]] = 1;
}

__global__ void k_wf_resolve(DevScene S, Q q, const uint32_t* count, HitsSoA hits, const float* contrib,
                             const int32_t* visible, const float* base, float* accum)
{
    const uint32_t n = *count, nl = S.nlights;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    {
        if (hits.object[k] < 0) continue;
        float3 c = f3(base[3ull * k], base[3ull * k + 1], base[3ull * k + 2]);
        for (uint32_t l = 0; l < nl; l++)
        {
            uint32_t slot = k * nl + l;
            if (visible[slot]) c = c + f3(contrib[3ull * slot], contrib[3ull * slot + 1], contrib[3ull * slot + 2]);
        }
        float3 a = q.att(k);
        uint32_t px = q.px[k];
        float3 add = (c * kPi) * a;
        accum[3ull * px] += add.x; accum[3ull * px + 1] += add.y; accum[3ull * px + 2] += add.z;
    }
}

__global__ void k_wf_finish(RenderParams p, const float* accum, uint32_t* fb, float* linear)
{
    const uint32_t n = p.width * p.height;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        store_pixel(p, k, f3(accum[3ull * k], accum[3ull * k + 1], accum[3ull * k + 2]), fb, linear);
}

int sm_count()
{
    static int sms = 0;
    if (!sms)
    {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    }
    return sms;
}

int blocks_for(const void* fn, int threads)
{
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, threads, 0);
    return sm_count() * (per > 0 ? per : 1);
}

}  // namespace

cudaError_t launch_render_plain(const DevScene& S, const RenderParams& p, uint32_t* framebuffer, float* linear,
                                Counters* counters, cudaStream_t stream)
{
    dim3 block(8, 8);
    dim3 grid((p.width + 7) / 8, (p.height + 7) / 8);
    k_render_plain<<<grid, block, 0, stream>>>(S, p, framebuffer, linear, counters);
    return cudaGetLastError();
}

cudaError_t launch_render_wavefront(const DevScene& S, const RenderParams& p, const WavefrontBuffers& wb,
                                    uint32_t* framebuffer, float* linear, Counters* counters, cudaStream_t stream,
                                    int* launches)
{
    static int gShade = 0;
    if (!gShade) gShade = blocks_for((const void*)k_wf_shade, kWfThreads);
    const int gFlat = sm_count() * 8;
    int nl = 0;
    const uint32_t cap = wb.capacity;
    const uint32_t scap = wb.capacity * (wb.lightCapacity ? wb.lightCapacity : 1);
    Q q[2] = {{wb.ray[0], wb.pixel[0], cap}, {wb.ray[1], wb.pixel[1], cap}};
    k_wf_camera<<<gFlat, 256, 0, stream>>>(p, q[0], wb.accum, wb.count);
    nl++;
    Query qa = p.q;
    qa.precision = 0;
    const float* sh = wb.shadow;
    RaysSoA shadowRays {sh, sh + scap, sh + 2ull * scap, sh + 3ull * scap, sh + 4ull * scap, sh + 5ull * scap,
                        sh + 6ull * scap};
    for (int level = 0, cur = 0; level <= p.depth; level++, cur ^= 1)
    {
        cudaMemsetAsync(wb.count + (cur ^ 1), 0, sizeof(uint32_t), stream);
        cudaMemsetAsync(wb.count + 2, 0, sizeof(uint32_t), stream);
        const float* r = wb.ray[cur];
        RaysSoA rays {r, r + cap, r + 2ull * cap, r + 3ull * cap, r + 4ull * cap, r + 5ull * cap, nullptr};
        cudaError_t e = run_query(S, rays, 0, wb.count + cur, p.q, false, wb.hit, nullptr, wb.engine, wb.engineCapacity,
                                  kEnginePasses, counters, stream, &nl);
        if (e != cudaSuccess) return e;
        k_wf_shade<<<gShade, kWfThreads, 0, stream>>>(S, p, q[cur], q[cur ^ 1], wb.count + cur, wb.count + (cur ^ 1),
                                                      wb.count + 2, wb.hit, wb.shadow, wb.shadowSlot, scap, wb.contrib,
                                                      wb.visible, wb.base, wb.accum, p.depth - level);
        e = run_query(S, shadowRays, 0, wb.count + 2, qa, true, HitsSoA {}, wb.occluded, wb.engine, wb.engineCapacity,
                      kEnginePasses, counters, stream, &nl);
        if (e != cudaSuccess) return e;
        k_wf_visibility<<<gFlat, 256, 0, stream>>>(wb.occluded, wb.shadowSlot, wb.count + 2, scap, wb.visible);
        k_wf_resolve<<<gFlat, 256, 0, stream>>>(S, q[cur], wb.count + cur, wb.hit, wb.contrib, wb.visible, wb.base,
                                               wb.accum);
        nl += 3;
    }
    k_wf_finish<<<gFlat, 256, 0, stream>>>(p, wb.accum, framebuffer, linear);
    nl++;
    if (launches) *launches += nl;
    return cudaGetLastError();
}

}  // namespace cgs
