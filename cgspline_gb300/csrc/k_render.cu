// k_render.cu -- rendering a batch of requests: camera rays, PBR shading with
// shadow rays and mirror bounces, sRGB packing (RayTracer::render and
// Context::closestHit, src/rt/RayTracer.cu:107-544, non Monte-Carlo path).
// A request is (group, camera, width, height, spp, depth); with spp > 1 the
// primary rays of sample s are jittered by (s/spp, vdc(s)) as the reference's
// sampled path does (src/rt/RayTracer.cu:226-236) and the samples are
// averaged.  Two schedules:
//   plain     -- one thread per pixel runs all of its samples and the whole
//                bounce chain, 8x8 blocks, one launch per request (the
//                reference's launch shape, src/rt/RayTracer.cu:171-274);
//   wavefront -- all requests' samples together: a closest-hit query, a
//                shading pass that queues shadow and bounce rays, an any-hit
//                query over the shadow queue and a resolve pass per bounce
//                level; queue sizes stay on the device.
#include <algorithm>

#include "kernels.h"

namespace cgs {

namespace {

constexpr float kMinRadiance = 0x1p-8f;  // src/rt/RayTracer.h:16

__device__ __forceinline__ float vdc(uint32_t i)  // Van der Corput, src/rt/PBR.h:143-157
{
    return 0x1p-32f * float(__brev(i));
}

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

// Philox4x32-10 (Salmon, Moraes, Dror & Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC 2011): a counter-based generator, so a ray's random
// numbers are a function of (image sample, bounce) and do not depend on the
// batch it runs in.
__device__ __forceinline__ uint4 philox(uint4 c, uint2 k)
{
#pragma unroll
    for (int r = 0; r < 10; r++)
    {
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}
// 24 random bits to a float in (0, 1)
__device__ __forceinline__ float u01(uint32_t x) { return float(x >> 8) * 0x1p-24f + 0x1p-25f; }

// Monte-Carlo bounce of the sampled path (src/rt/RayTracer.cu:473-521,
// microfacet src/rt/PBR.h:165-176): a GGX microfacet normal from two uniform
// numbers, the reflection about it, and the attenuation
// mix(diffuse/pi, F * G * (M.V) / ((N.V)(M.N)), metalness).  The numbers
// come from Philox with counter (image sample, remaining depth, 0, 0) and
// key (42, 0), in place of the reference's curand state.
__device__ __forceinline__ bool bounce_mc(const Frame& f, float3 att, uint32_t imageSample, uint32_t dep, float3& R,
                                          float3& a)
{
    const uint4 rnd = philox(make_uint4(imageSample, dep, 0u, 0u), make_uint2(42u, 0u));
    const float x = u01(rnd.x), y = u01(rnd.y);
    const float alpha = f.m.roughness * f.m.roughness;
    const float theta = atan2f(alpha * sqrtf(x), sqrtf(1.0f - x)), phi = 2.0f * kPi * y;
    const float3 ts = versor(cross(f.N, f.V)), tp = versor(cross(f.N, ts));
    const float st = sinf(theta), ct = cosf(theta), sp = sinf(phi), cp = cosf(phi);
    const float3 M = versor((st * cp) * ts + (st * sp) * tp + ct * f.N);
    const float dotMV = dot(M, f.V);
    const float3 reflectance = schlick(f3(f.m.specular[0], f.m.specular[1], f.m.specular[2]), dotMV);
    R = (-f.V) - (2.0f * (-dotMV)) * M;
    const float dotMN = dot(M, f.N), dotNR = dot(f.N, R);
    if (dotNR < 1e-14f) return false;
    const float g = Gsmith(dotNR, f.dotNV, f.m.roughness) * dotMV / (f.dotNV * dotMN);
    const float3 kd = f3(f.m.diffuse[0], f.m.diffuse[1], f.m.diffuse[2]) * kInvPi;
    const float3 ks = reflectance * g;
    const float mt = f.m.metalness;
    a = att * (kd * (1.0f - mt) + ks * mt);
    return vmax3(a) > kMinRadiance;
}

__device__ __forceinline__ void store_pixel(const DevRequest& r, uint32_t px, float3 c)
{
    c = f3(__saturatef(c.x), __saturatef(c.y), __saturatef(c.z));
    const uint32_t i = px % r.width, j = px / r.width;
    if (r.fb) r.fb[size_t(j) * r.stride + i] = pack_srgb(c);
    if (r.linear) { r.linear[3ull * px] = c.x; r.linear[3ull * px + 1] = c.y; r.linear[3ull * px + 2] = c.z; }
}

__device__ __forceinline__ float2 sample_xy(const DevRequest& r, uint32_t pixel, uint32_t s)
{
    const float x = float(pixel % r.width), y = float(pixel / r.width + r.row0);
    if (r.spp <= 1) return make_float2(x, y);
    return make_float2(x + float(s) * (1.0f / float(r.spp)), y + vdc(s));
}

// Request owning global index k, by binary search over the bases (field 0: samples, 1: pixels).
__device__ __forceinline__ uint32_t find_request(const DevRequest* req, uint32_t n, uint32_t k, bool pixels)
{
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1)
    {
        const uint32_t mid = (lo + hi) >> 1;
        const uint32_t b = pixels ? req[mid].pixelBase : req[mid].sampleBase;
        if (b <= k) lo = mid; else hi = mid;
    }
    return lo;
}

// ------------------------------------------------------------- plain --
__global__ void __launch_bounds__(64) k_render_plain(DevScene S, DevRequest r, float eps, Query q, int sampling,
                                                     Counters* cnt)
{
    const uint32_t i = blockIdx.x * 8 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
    LocalCounters lc;
    uint32_t nrays = 0;
    if (i < r.width && j < r.height)
    {
        const uint32_t g = r.group;
        const uint2 lights = S.groupLights[g];
        float3 pixel = f3(0.0f, 0.0f, 0.0f);
        for (uint32_t s = 0; s < r.spp; s++)
        {
            const float2 xy = sample_xy(r, j * r.width + i, s);
            float3 o = f3(r.cam.pos[0], r.cam.pos[1], r.cam.pos[2]);
            float3 d = pixel_dir(r.cam, xy.x, xy.y);
            float3 color = f3(0.0f, 0.0f, 0.0f), att = f3(1.0f, 1.0f, 1.0f);
            int depth = r.depth;
            for (int level = 0; level <= r.depth; level++)
            {
                nrays++;
                HitRecord hit {INFINITY, 0.0f, 0.0f, -1, -1};
                int ob = scene_closest(S, g, o, d, INFINITY, q, hit, lc);
                if (ob < 0) { color = color + group_background(S, g) * att; break; }
                Frame f = shade_frame(S, o, d, hit);
                float3 c = group_ambient(S, g) * f.diffuse;
                for (uint32_t l = 0; l < lights.y; l++)
                {
                    float3 contrib, L; float dist;
                    if (!light_term(f, S.lights[lights.x + l], contrib, L, dist)) continue;
                    nrays++;
                    if (scene_any(S, g, f.P + eps * L, L, dist, q, lc)) continue;
                    c = c + contrib;
                }
                color = color + (c * kPi) * att;
                if (depth <= 0) break;
                float3 R, a;
                const uint32_t imageSample = ((j + r.row0) * r.width + i) * r.spp + s;
                if (!(sampling ? bounce_mc(f, att, imageSample, uint32_t(depth), R, a) : bounce(f, att, R, a))) break;
                o = f.P + eps * R;
                d = R;
                att = a;
                depth--;
            }
            pixel = pixel + color;
        }
        if (r.spp > 1) pixel = pixel * (1.0f / float(r.spp));
        store_pixel(r, j * r.width + i, pixel);
    }
    flush_counters(cnt, lc, nrays);
}

// --------------------------------------------------------- wavefront --
constexpr int kWfThreads = 128;

struct Q  // a ray queue: 9 floats per ray (SoA with stride = capacity) + sample, group, depth
{
    float* r; uint32_t* sample; uint32_t* group; uint32_t* depth; uint32_t cap;
    __device__ __forceinline__ void put(uint32_t k, float3 o, float3 d, float3 a, uint32_t smp, uint32_t g,
                                        uint32_t dep) const
    {
        r[k] = o.x; r[cap + k] = o.y; r[2ull * cap + k] = o.z;
        r[3ull * cap + k] = d.x; r[4ull * cap + k] = d.y; r[5ull * cap + k] = d.z;
        r[6ull * cap + k] = a.x; r[7ull * cap + k] = a.y; r[8ull * cap + k] = a.z;
        sample[k] = smp; group[k] = g; depth[k] = dep;
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
    RaysSoA rays() const
    {
        return RaysSoA {r, r + cap, r + 2ull * cap, r + 3ull * cap, r + 4ull * cap, r + 5ull * cap, nullptr, group};
    }
};

// The pixel that queue position p of a w x h image takes in tile order: the
// image is cut into bands of 4 rows and each band into chunks 8 columns wide
// (narrower at the right edge, lower in the last band), taken chunk by chunk,
// row by row inside a chunk, so that a warp's 32 rays cover an 8 x 4 tile.
// A bijection of [0, w*h).
__device__ __forceinline__ uint32_t tiled_pixel(uint32_t p, uint32_t w, uint32_t h)
{
    const uint32_t band = p / (4 * w);
    const uint32_t m = p - band * 4 * w;
    const uint32_t hb = min(4u, h - 4 * band);
    const uint32_t c = m / (8 * hb);
    const uint32_t q = m - c * 8 * hb;
    const uint32_t cw = min(8u, w - 8 * c);
    return (4 * band + q / cw) * w + 8 * c + q % cw;
}

// Primary rays of every sample.  Queue position k holds sample k (scanline
// order), or with `tiled` the sample of its request's tile-order pixel; the
// ray carries its sample index, which keys the accumulation and the
// Monte-Carlo stream, so the order changes no result.
__global__ void k_wf_camera(const RenderBatch* __restrict__ bp, Q q, float* accum, uint32_t* count, int tiled)
{
    const RenderBatch b = *bp;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < b.samples; k += gridDim.x * blockDim.x)
    {
        const DevRequest& r = b.req[find_request(b.req, b.nreq, k, false)];
        const uint32_t local = k - r.sampleBase, s = local % r.spp;
        const uint32_t pixel = tiled ? tiled_pixel(local / r.spp, r.width, r.height) : local / r.spp;
        const uint32_t smp = r.sampleBase + pixel * r.spp + s;
        const float2 xy = sample_xy(r, pixel, s);
        const float3 o = f3(r.cam.pos[0], r.cam.pos[1], r.cam.pos[2]);
        q.put(k, o, pixel_dir(r.cam, xy.x, xy.y), f3(1.0f, 1.0f, 1.0f), smp, r.group, uint32_t(r.depth));
        accum[3ull * smp] = 0.0f; accum[3ull * smp + 1] = 0.0f; accum[3ull * smp + 2] = 0.0f;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) { count[0] = b.samples; count[1] = 0; count[2] = 0; }
}

__global__ void __launch_bounds__(kWfThreads) k_wf_shade(DevScene S, const RenderBatch* __restrict__ bp, float eps,
                                                         int sampling, Q q, Q qn, const uint32_t* count,
                                                         uint32_t* nextCount, uint32_t* shadowCount, HitsSoA hits,
                                                         float* shadow, uint32_t* shadowGroup, uint32_t* shadowSlot,
                                                         uint32_t shadowCap, uint32_t lcap, float* contrib,
                                                         int32_t* visible, float* base, float* accum)
{
    const uint32_t n = *count;
    for (uint32_t k0 = blockIdx.x * blockDim.x; k0 < n; k0 += gridDim.x * blockDim.x)
    {
        const uint32_t k = k0 + threadIdx.x;
        const bool live = k < n;
        HitRecord h {INFINITY, 0.0f, 0.0f, -1, -1};
        float3 o = f3(0, 0, 0), d = f3(0, 0, 1), att = f3(0, 0, 0);
        uint32_t smp = 0, g = 0, dep = 0;
        if (live)
        {
            h = HitRecord {hits.t[k], hits.u[k], hits.v[k], hits.patch[k], hits.object[k]};
            q.get(k, o, d);
            att = q.att(k);
            smp = q.sample[k]; g = q.group[k]; dep = q.depth[k];
        }
        const bool isHit = live && h.object >= 0;
        if (live && !isHit)
        {
            const float3 bg = group_background(S, g) * att;
            accum[3ull * smp] += bg.x; accum[3ull * smp + 1] += bg.y; accum[3ull * smp + 2] += bg.z;
        }
        Frame f;
        uint2 lights = make_uint2(0, 0);
        if (isHit)
        {
            f = shade_frame(S, o, d, h);
            const float3 c0 = group_ambient(S, g) * f.diffuse;
            base[3ull * k] = c0.x; base[3ull * k + 1] = c0.y; base[3ull * k + 2] = c0.z;
            lights = S.groupLights[g];
        }
        // the warp walks the largest light count among its lanes (pushes are warp-wide)
        uint32_t nl = lights.y;
        for (int off = 16; off > 0; off >>= 1) nl = max(nl, __shfl_xor_sync(0xFFFFFFFFu, nl, off));
        for (uint32_t l = 0; l < nl; l++)
        {
            float3 c, L; float dist = 0.0f;
            const bool mine = isHit && l < lights.y;
            const bool want = mine && light_term(f, S.lights[lights.x + l], c, L, dist);
            const uint32_t slot = k * lcap + l;
            if (mine)
            {
                visible[slot] = 0;
                if (want) { contrib[3ull * slot] = c.x; contrib[3ull * slot + 1] = c.y; contrib[3ull * slot + 2] = c.z; }
            }
            const uint32_t sk = warp_push(shadowCount, want);
            if (want && sk < shadowCap)
            {
                const float3 so = f.P + eps * L;
                shadow[sk] = so.x; shadow[shadowCap + sk] = so.y; shadow[2ull * shadowCap + sk] = so.z;
                shadow[3ull * shadowCap + sk] = L.x; shadow[4ull * shadowCap + sk] = L.y;
                shadow[5ull * shadowCap + sk] = L.z; shadow[6ull * shadowCap + sk] = dist;
                shadowGroup[sk] = g;
                shadowSlot[sk] = slot;
            }
        }
        float3 R = f3(0, 0, 0), a = f3(0, 0, 0);
        bool more = false;
        if (isHit && dep > 0)
        {
            if (sampling)
            {
                // the sample's index within its image: request-local sample + rows above the chunk
                const RenderBatch* b = bp;
                const DevRequest& r = b->req[find_request(b->req, b->nreq, smp, false)];
                const uint32_t imageSample = (smp - r.sampleBase) + r.row0 * r.width * r.spp;
                more = bounce_mc(f, att, imageSample, dep, R, a);
            }
            else
                more = bounce(f, att, R, a);
        }
        const uint32_t nk = warp_push(nextCount, more);
        if (more) qn.put(nk, f.P + eps * R, R, a, smp, g, dep - 1);
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
                             const int32_t* visible, const float* base, uint32_t lcap, float* accum)
{
    const uint32_t n = *count;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    {
        if (hits.object[k] < 0) continue;
        const uint2 lights = S.groupLights[q.group[k]];
        float3 c = f3(base[3ull * k], base[3ull * k + 1], base[3ull * k + 2]);
        for (uint32_t l = 0; l < lights.y; l++)
        {
            const uint32_t slot = k * lcap + l;
            if (visible[slot]) c = c + f3(contrib[3ull * slot], contrib[3ull * slot + 1], contrib[3ull * slot + 2]);
        }
        const float3 add = (c * kPi) * q.att(k);
        const uint32_t smp = q.sample[k];
        accum[3ull * smp] += add.x; accum[3ull * smp + 1] += add.y; accum[3ull * smp + 2] += add.z;
    }
}

__global__ void k_wf_finish(const RenderBatch* __restrict__ bp, const float* accum)
{
    const RenderBatch b = *bp;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < b.pixels; p += gridDim.x * blockDim.x)
    {
        const DevRequest& r = b.req[find_request(b.req, b.nreq, p, true)];
        const uint32_t local = p - r.pixelBase;
        const size_t s0 = size_t(r.sampleBase) + size_t(local) * r.spp;
        float3 c = f3(0.0f, 0.0f, 0.0f);
        for (uint32_t s = 0; s < r.spp; s++)
            c = c + f3(accum[3 * (s0 + s)], accum[3 * (s0 + s) + 1], accum[3 * (s0 + s) + 2]);
        if (r.spp > 1) c = c * (1.0f / float(r.spp));
        store_pixel(r, local, c);
    }
}

// Primary rays of a w x h image, one per pixel centre, SoA (7, w*h).
__global__ void k_camera_rays(CameraSetup cam, uint32_t w, uint32_t h, float* rays)
{
    const size_t n = size_t(w) * h;
    for (size_t k = blockIdx.x * size_t(blockDim.x) + threadIdx.x; k < n; k += size_t(gridDim.x) * blockDim.x)
    {
        const float3 d = pixel_dir(cam, float(k % w), float(k / w));
        rays[k] = cam.pos[0]; rays[n + k] = cam.pos[1]; rays[2 * n + k] = cam.pos[2];
        rays[3 * n + k] = d.x; rays[4 * n + k] = d.y; rays[5 * n + k] = d.z; rays[6 * n + k] = INFINITY;
    }
}

int sm_count()
{
    static const int sms = [] {
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        return n > 0 ? n : 1;
    }();
    return sms;
}

int blocks_for(const void* fn, int threads)
{
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, threads, 0);
    return sm_count() * (per > 0 ? per : 1);
}

}  // namespace

cudaError_t launch_render_plain(const DevScene& S, const RenderBatch& b, const DevRequest* hostReq,
                                Counters* counters, cudaStream_t stream, int* launches)
{
    for (uint32_t k = 0; k < b.nreq; k++)
    {
        const DevRequest& r = hostReq[k];
        dim3 block(8, 8);
        dim3 grid((r.width + 7) / 8, (r.height + 7) / 8);
        k_render_plain<<<grid, block, 0, stream>>>(S, r, b.eps, b.q, b.sampling, counters);
    }
    if (launches) *launches += int(b.nreq);
    return cudaGetLastError();
}

cudaError_t launch_camera_rays(const CameraSetup& cam, uint32_t w, uint32_t h, float* rays, cudaStream_t stream)
{
    const size_t n = size_t(w) * h;
    if (n == 0) return cudaSuccess;
    const int blocks = int(std::min<size_t>((n + 255) / 256, size_t(sm_count()) * 8));
    k_camera_rays<<<blocks, 256, 0, stream>>>(cam, w, h, rays);
    return cudaGetLastError();
}

cudaError_t launch_render_wavefront(const DevScene& S, const RenderBatch& b, const RenderBatch* bDev,
                                    const WavefrontBuffers& wb, Counters* counters, cudaStream_t stream, int* launches)
{
    static const int gShade = blocks_for((const void*)k_wf_shade, kWfThreads);  // thread-safe one-time init
    const int gFlat = sm_count() * 8;
    int nl = 0;
    const uint32_t cap = wb.capacity;
    const uint32_t lcap = wb.lightCapacity ? wb.lightCapacity : 1;
    const uint32_t scap = cap * lcap;
    Q q[2] = {{wb.ray[0], wb.sample[0], wb.group[0], wb.depth[0], cap},
              {wb.ray[1], wb.sample[1], wb.group[1], wb.depth[1], cap}};
    k_wf_camera<<<gFlat, 256, 0, stream>>>(bDev, q[0], wb.accum, wb.count, engine_config().rayOrder);
    nl++;
    Query qa = b.q;
    qa.precision = 0;  // shadow rays: any hit at level 0
    const float* sh = wb.shadow;
    const RaysSoA shadowRays {sh, sh + scap, sh + 2ull * scap, sh + 3ull * scap, sh + 4ull * scap, sh + 5ull * scap,
                              sh + 6ull * scap, wb.shadowGroup};
    // Level L's shadow query, visibility and resolve run on the side stream
    // beside level L+1's closest-hit query (they share no buffer: hits and
    // engine scratch alternate, and the queue counts are reset only after the
    // join); level L+1's shading waits for them, so every sample accumulates
    // in the same order as on one stream.
    const bool two = wb.side != nullptr;
    cudaStream_t side = two ? wb.side : stream;
    for (int level = 0, cur = 0; level <= b.maxDepth; level++, cur ^= 1)
    {
        const HitsSoA hit = wb.hit[level & 1];
        cudaError_t e = run_query(S, q[cur].rays(), 0, wb.count + cur, b.q, false, hit, nullptr, wb.engine,
                                  wb.engineCapacity, kEnginePasses, counters, stream, &nl);
        if (e != cudaSuccess) return e;
        if (two && level > 0) cudaStreamWaitEvent(stream, wb.join, 0);
        cudaMemsetAsync(wb.count + (cur ^ 1), 0, sizeof(uint32_t), stream);
        cudaMemsetAsync(wb.count + 2, 0, sizeof(uint32_t), stream);
        k_wf_shade<<<gShade, kWfThreads, 0, stream>>>(S, bDev, b.eps, b.sampling, q[cur], q[cur ^ 1], wb.count + cur,
                                                      wb.count + (cur ^ 1), wb.count + 2, hit, wb.shadow,
                                                      wb.shadowGroup, wb.shadowSlot, scap, lcap, wb.contrib,
                                                      wb.visible, wb.base, wb.accum);
        if (two)
        {
            cudaEventRecord(wb.fork, stream);
            cudaStreamWaitEvent(side, wb.fork, 0);
        }
        e = run_query(S, shadowRays, 0, wb.count + 2, qa, true, HitsSoA {}, wb.occluded,
                      two ? wb.engine2 : wb.engine, two ? wb.engine2Capacity : wb.engineCapacity, kEnginePasses,
                      counters, side, &nl);
        if (e != cudaSuccess) return e;
        k_wf_visibility<<<gFlat, 256, 0, side>>>(wb.occluded, wb.shadowSlot, wb.count + 2, scap, wb.visible);
        k_wf_resolve<<<gFlat, 256, 0, side>>>(S, q[cur], wb.count + cur, hit, wb.contrib, wb.visible, wb.base, lcap,
                                            wb.accum);
        nl += 3;
        if (two) cudaEventRecord(wb.join, side);
    }
    if (two) cudaStreamWaitEvent(stream, wb.join, 0);
    k_wf_finish<<<gFlat, 256, 0, stream>>>(bDev, wb.accum);
    nl++;
    if (launches) *launches += nl;
    return cudaGetLastError();
}

}  // namespace cgs
