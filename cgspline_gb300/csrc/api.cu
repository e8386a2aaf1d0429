// api.cu -- queries and rendering entry points of libcgspline_gb300.so:
// closest / any-hit ray queries, (ray, patch) pair clipping, single and
// batched frame renders, and the standalone perfect-hash build.
#include "scene_impl.h"

#include <map>

using namespace cgs;

namespace cgs {

std::atomic<uint32_t> g_failAllocation {0};

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

// A failed reserve frees the old buffer: each capacity below is cleared
// before its buffer grows, so that it never outlives the memory it describes.
int ensure_engine(cgs_scene* sc, uint32_t capacity)
{
    if (sc->engineCapacity >= capacity && sc->engine.p) return CGS_OK;
    sc->engineCapacity = 0;
    CGS_TRY(sc->engine.reserve(engine_words(capacity, kEnginePasses)));
    sc->engineCapacity = capacity;
    return CGS_OK;
}

void GraphCache::release()
{
    for (auto& kv : execs) cudaGraphExecDestroy(kv.second.exec);
    execs.clear();
    seen.clear();
    if (capture) cudaStreamDestroy(capture);
    capture = nullptr;
}

uint64_t scene_key(const DevScene& S)
{
    return key_of({key_of(S.patches), key_of(S.nodes), key_of(S.indices), key_of(S.tables), key_of(S.disps),
                   key_of(S.bvhs), key_of(S.patchBase), key_of(S.objects), key_of(S.materials),
                   key_of(S.patchMaterial), key_of(S.lights), key_of(S.groupTop), key_of(S.groupLights),
                   key_of(S.groupEnv), S.nobjects, S.nsurfaces, S.ngroups});
}

uint64_t query_key(const Query& q)
{
    uint32_t tol;
    std::memcpy(&tol, &q.tol, 4);
    return key_of({uint64_t(q.method), uint64_t(q.precision), tol});
}

cudaError_t run_cached(GraphCache& gc, uint64_t key, cudaStream_t stream, int* launches,
                       const std::function<cudaError_t(cudaStream_t, int*)>& fn)
{
    auto it = gc.execs.find(key);
    if (it != gc.execs.end())
    {
        if (launches) *launches += it->second.launches;
        gc.replays++;
        return cudaGraphLaunch(it->second.exec, stream);
    }
    if (gc.disabled || gc.seen.insert(key).second) return fn(stream, launches);
    cudaError_t e = cudaSuccess;
    if (!gc.capture) e = cudaStreamCreateWithFlags(&gc.capture, cudaStreamNonBlocking);
    if (e != cudaSuccess) { gc.disabled = true; return fn(stream, launches); }
    // the captured sequence must follow the work already queued on `stream`
    // only when it runs, which the graph launch on `stream` provides
    int nl = 0;
    cudaGraph_t graph = nullptr;
    e = cudaStreamBeginCapture(gc.capture, cudaStreamCaptureModeThreadLocal);
    cudaError_t e1 = e == cudaSuccess ? fn(gc.capture, &nl) : e;
    cudaError_t e2 = e == cudaSuccess ? cudaStreamEndCapture(gc.capture, &graph) : e;
    cudaGraphExec_t exec = nullptr;
    cudaError_t e3 = (e1 == cudaSuccess && e2 == cudaSuccess) ? cudaGraphInstantiate(&exec, graph, 0) : e2;
    if (graph) cudaGraphDestroy(graph);
    if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess)
    {
        // capture is not available here: run eagerly from now on
        cudaGetLastError();
        gc.disabled = true;
        return fn(stream, launches);
    }
    if (gc.execs.size() >= 32)
    {
        for (auto& kv : gc.execs) cudaGraphExecDestroy(kv.second.exec);
        gc.execs.clear();
    }
    gc.execs[key] = GraphCache::Entry {exec, nl};
    gc.captures++;
    if (launches) *launches += nl;
    return cudaGraphLaunch(exec, stream);
}

// Device bytes of a render slot for `samples` primary rays and `lights`
// lights per group (the sizes RenderSlot::ensure reserves).
uint64_t RenderSlot::bytes_for(uint32_t samples, uint32_t lights)
{
    const uint64_t c = samples, l = std::max<uint32_t>(lights, 1), s = c * l;
    uint64_t b = 0;
    b += 2 * 9 * c * 4;          // ray queues
    b += 6 * c * 4;              // sample, group, depth of both queues
    b += 2 * 5 * c * 4;          // hits of even and odd levels
    b += 6 * c * 4;              // base, accum
    b += s * 4 * (1 + 7 + 2 + 3 + 1);  // occluded, shadow rays, slot+group, contrib, visible
    // engine scratch: the closest-hit queries' (samples) and the shadow queries' (samples x lights)
    b += (engine_words(uint32_t(c), kEnginePasses) + engine_words(uint32_t(s), kEnginePasses)) * 4;
    return b;
}

int RenderSlot::ensure(uint32_t samples, uint32_t lights, uint32_t nreq)
{
    const uint32_t nl = std::max<uint32_t>(lights, 1);
    CGS_TRY(req.reserve(std::max<uint32_t>(nreq, 1)));
    CGS_TRY(counters.reserve(1));
    if (!side)
    {
        // the shadow queries run on a stream of their own beside the next
        // level's closest query; without it everything runs on one stream
        if (cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&join, cudaEventDisableTiming) != cudaSuccess)
        {
            cudaGetLastError();
            if (side) cudaStreamDestroy(side);
            if (fork) cudaEventDestroy(fork);
            side = nullptr; fork = nullptr; join = nullptr;
        }
        wb.side = side; wb.fork = fork; wb.join = join;
    }
    if (wb.capacity >= samples && wb.lightCapacity >= nl && wb.engine) return CGS_OK;
    const size_t cap = std::max<uint32_t>(samples, wb.capacity);
    const uint32_t lc = std::max<uint32_t>(nl, wb.lightCapacity);
    // the buffers below may be freed by a reserve that fails: the view is
    // cleared first and set again only once all of them are in place
    wb.capacity = 0; wb.lightCapacity = 0; wb.engine = nullptr; wb.engine2 = nullptr;
    const size_t sc = cap * lc;
    if (sc >= (1ull << 31)) return CGS_ERR_INVALID_ARGUMENT;
    CGS_TRY(ray0.reserve(9 * cap));
    CGS_TRY(ray1.reserve(9 * cap));
    CGS_TRY(smp0.reserve(cap)); CGS_TRY(smp1.reserve(cap));
    CGS_TRY(grp0.reserve(cap)); CGS_TRY(grp1.reserve(cap));
    CGS_TRY(dep0.reserve(cap)); CGS_TRY(dep1.reserve(cap));
    CGS_TRY(count.reserve(8));
    CGS_TRY(hitF.reserve(3 * cap));
    CGS_TRY(hitI.reserve(2 * cap));
    CGS_TRY(hitF2.reserve(3 * cap));
    CGS_TRY(hitI2.reserve(2 * cap));
    CGS_TRY(occluded.reserve(sc));
    // the closest-hit queries hold `cap` rays, the shadow queries `sc`; with no
    // side stream both run on the first scratch
    const uint32_t ecap = uint32_t(side ? cap : std::max(cap, sc)), ecap2 = uint32_t(side ? sc : 0);
    if (engineCapacity < ecap || !engine.p)
    {
        engineCapacity = 0;
        CGS_TRY(engine.reserve(engine_words(ecap, kEnginePasses)));
        engineCapacity = ecap;
    }
    if (ecap2 && (engine2Capacity < ecap2 || !engine2.p))
    {
        engine2Capacity = 0;
        CGS_TRY(engine2.reserve(engine_words(ecap2, kEnginePasses)));
        engine2Capacity = ecap2;
    }
    CGS_TRY(shadow.reserve(7 * sc));
    CGS_TRY(shadowSlot.reserve(sc));
    CGS_TRY(shadowGroup.reserve(sc));
    CGS_TRY(contrib.reserve(3 * sc));
    CGS_TRY(visible.reserve(sc));
    CGS_TRY(base.reserve(3 * cap));
    CGS_TRY(accum.reserve(3 * cap));
    wb.ray[0] = ray0.p; wb.ray[1] = ray1.p;
    wb.sample[0] = smp0.p; wb.sample[1] = smp1.p;
    wb.group[0] = grp0.p; wb.group[1] = grp1.p;
    wb.depth[0] = dep0.p; wb.depth[1] = dep1.p;
    wb.count = count.p;
    wb.hit[0] = HitsSoA {hitF.p, hitF.p + cap, hitF.p + 2 * cap, hitI.p, hitI.p + cap};
    wb.hit[1] = HitsSoA {hitF2.p, hitF2.p + cap, hitF2.p + 2 * cap, hitI2.p, hitI2.p + cap};
    wb.occluded = occluded.p;
    wb.engine = engine.p;
    wb.engine2 = engine2.p;
    wb.engineCapacity = engineCapacity;
    wb.engine2Capacity = engine2Capacity;
    wb.shadow = shadow.p; wb.shadowGroup = shadowGroup.p; wb.shadowSlot = shadowSlot.p;
    wb.contrib = contrib.p; wb.visible = visible.p; wb.base = base.p; wb.accum = accum.p;
    wb.capacity = uint32_t(cap);
    wb.lightCapacity = lc;
    return CGS_OK;
}

int RenderSlot::ensure_engine(uint32_t rays)
{
    if (engineCapacity >= rays && engine.p) return CGS_OK;
    engineCapacity = 0;
    wb.engine = nullptr;
    wb.engineCapacity = 0;
    CGS_TRY(engine.reserve(engine_words(rays, kEnginePasses)));
    engineCapacity = rays;
    wb.engine = engine.p;
    wb.engineCapacity = engineCapacity;
    return CGS_OK;
}

uint64_t RenderSlot::bytes() const
{
    uint64_t b = ray0.bytes() + ray1.bytes() + shadow.bytes() + contrib.bytes() + base.bytes() + accum.bytes();
    b += hitF.bytes() + smp0.bytes() + smp1.bytes() + grp0.bytes() + grp1.bytes() + dep0.bytes() + dep1.bytes();
    b += count.bytes() + shadowSlot.bytes() + shadowGroup.bytes() + engine.bytes() + visible.bytes() + hitI.bytes();
    b += hitF2.bytes() + hitI2.bytes() + engine2.bytes();
    b += occluded.bytes() + req.bytes() + counters.bytes() + batch.bytes();
    return b;
}

void RenderSlot::release()
{
    ray0.release(); ray1.release(); shadow.release(); contrib.release(); base.release(); accum.release();
    hitF.release(); hitF2.release();
    for (auto* b : {&smp0, &smp1, &grp0, &grp1, &dep0, &dep1, &count, &shadowSlot, &shadowGroup, &engine, &engine2})
        b->release();
    visible.release(); hitI.release(); hitI2.release(); occluded.release(); req.release(); counters.release();
    batch.release();
    graphs.release();
    if (side) { cudaStreamSynchronize(side); cudaStreamDestroy(side); }
    if (fork) cudaEventDestroy(fork);
    if (join) cudaEventDestroy(join);
    side = nullptr; fork = nullptr; join = nullptr;
    wb = WavefrontBuffers {};
    engineCapacity = 0;
    engine2Capacity = 0;
}

cudaError_t launch_wavefront_cached(const DevScene& S, RenderSlot& slot, const RenderBatch& b, cudaStream_t stream,
                                    int* launches)
{
    const WavefrontBuffers& w = slot.wb;
    uint32_t eps;
    std::memcpy(&eps, &b.eps, 4);
    const uint64_t key = key_of({scene_key(S), query_key(b.q), uint64_t(b.maxDepth), uint64_t(b.sampling), eps,
                                 engine_config_generation(),
                                 key_of(slot.batch.p),
                                 key_of(slot.counters.p), key_of(w.ray[0]), key_of(w.ray[1]), key_of(w.engine),
                                 key_of(w.shadow), key_of(w.accum), key_of(w.hit[0].t), key_of(w.occluded),
                                 key_of(w.contrib), key_of(w.visible), key_of(w.base), key_of(w.count),
                                 key_of(w.sample[0]), key_of(w.group[0]), key_of(w.depth[0]), w.capacity,
                                 w.lightCapacity, w.engineCapacity, key_of(w.hit[1].t), key_of(w.engine2),
                                 w.engine2Capacity, key_of(w.side)});
    RenderSlot* sp = &slot;
    return run_cached(slot.graphs, key, stream, launches, [&](cudaStream_t st, int* nl) {
        return launch_render_wavefront(S, b, sp->batch.p, sp->wb, sp->counters.p, st, nl);
    });
}

int prepare_batch(cgs_scene* sc, const cgs_render_request* reqs, uint32_t n, const cgs_render_options* opt,
                  std::vector<DevRequest>& host, RenderBatch& b)
{
    if (!reqs || n == 0 || !opt) return CGS_ERR_INVALID_ARGUMENT;
    if (!valid_query(opt->method, opt->precision) || !(opt->tol > 0.0f) ||
        (opt->schedule != CGS_SCHED_PLAIN && opt->schedule != CGS_SCHED_WAVEFRONT) ||
        (opt->sampling != CGS_SAMPLING_MIRROR && opt->sampling != CGS_SAMPLING_MONTE_CARLO))
        return CGS_ERR_INVALID_ARGUMENT;
    host.resize(n);
    uint64_t samples = 0, pixels = 0;
    int maxDepth = 0;
    for (uint32_t k = 0; k < n; k++)
    {
        const cgs_render_request& r = reqs[k];
        if (r.width == 0 || r.height == 0 || r.spp == 0 || r.spp > 4096 || (!r.framebuffer && !r.linear_rgb))
            return CGS_ERR_INVALID_ARGUMENT;
        if (r.group >= sc->groups.size()) return CGS_ERR_INVALID_ARGUMENT;
        const int depth = r.recursion_depth < 0 ? opt->recursion_depth : r.recursion_depth;
        if (depth < 0 || depth > 64) return CGS_ERR_INVALID_ARGUMENT;
        DevRequest& d = host[k];
        camera_setup(r.camera, r.width, r.height, opt->flip_y, d.cam);
        d.group = r.group; d.width = r.width; d.height = r.height; d.spp = r.spp; d.depth = depth;
        d.sampleBase = uint32_t(samples); d.pixelBase = uint32_t(pixels); d.stride = r.width; d.row0 = 0;
        d.fb = r.framebuffer; d.linear = r.linear_rgb;
        samples += uint64_t(r.width) * r.height * r.spp;
        pixels += uint64_t(r.width) * r.height;
        if (samples >= (1ull << 31)) return CGS_ERR_INVALID_ARGUMENT;
        maxDepth = std::max(maxDepth, depth);
    }
    b = RenderBatch {};
    b.nreq = n; b.samples = uint32_t(samples); b.pixels = uint32_t(pixels);
    b.maxDepth = maxDepth; b.eps = opt->eps;
    b.q = Query {opt->method, opt->precision, opt->tol};
    b.sampling = opt->sampling;
    return CGS_OK;
}

int run_batch(cgs_scene* sc, RenderSlot& slot, const std::vector<DevRequest>& host, RenderBatch& b, int schedule,
              cudaStream_t stream, int* launches)
{
    CGS_TRY(slot.counters.reserve(1));
    CGS_TRY(cudaMemsetAsync(slot.counters.p, 0, sizeof(Counters), stream));
    cudaError_t e;
    if (schedule == CGS_SCHED_PLAIN)
        e = launch_render_plain(sc->dev(), b, host.data(), slot.counters.p, stream, launches);
    else
    {
        int r = slot.ensure(b.samples, sc->maxLights(), b.nreq);
        if (r) return r;
        CGS_TRY(slot.batch.reserve(1));
        CGS_TRY(cudaMemcpyAsync(slot.req.p, host.data(), host.size() * sizeof(DevRequest), cudaMemcpyHostToDevice,
                                stream));
        b.req = slot.req.p;
        CGS_TRY(cudaMemcpyAsync(slot.batch.p, &b, sizeof b, cudaMemcpyHostToDevice, stream));
        e = launch_wavefront_cached(sc->dev(), slot, b, stream, launches);
    }
    return cuda_status(e);
}

// A scene's queries share its counters and engine scratch.  A query on a
// stream other than the previous query's is ordered after that query's work;
// a stream under capture is left to the captured graph's own order.
int query_begin(cgs_scene* s, cudaStream_t st, bool& captured)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CGS_TRY(cudaStreamIsCapturing(st, &cs));
    captured = cs != cudaStreamCaptureStatusNone;
    if (!captured && s->queryIssued && st != s->queryStream) CGS_TRY(cudaStreamWaitEvent(st, s->queryDone, 0));
    return CGS_OK;
}

void query_end(cgs_scene* s, cudaStream_t st, bool captured)
{
    s->lastStream = st;
    s->lastCounters = s->counters.p;
    if (!captured && cudaEventRecord(s->queryDone, st) == cudaSuccess)
    {
        s->queryStream = st;
        s->queryIssued = true;
    }
}

}  // namespace cgs

extern "C" {

int cgs_debug_fail_allocation(uint32_t nth)
{
    cgs::g_failAllocation.store(nth, std::memory_order_relaxed);
    return CGS_OK;
}

int cgs_intersect(cgs_scene* s, const cgs_rays* rays, uint32_t n, int method, int precision, float tol, int any_hit,
                  const cgs_hits* hits, void* stream)
{
    if (!s || !rays || !hits || !valid_query(method, precision) || !(tol > 0.0f)) return CGS_ERR_INVALID_ARGUMENT;
    if (n && (!hits->patch || (!any_hit && (!hits->t || !hits->u || !hits->v || !hits->object))))
        return CGS_ERR_INVALID_ARGUMENT;
    if (n && (!rays->ox || !rays->oy || !rays->oz || !rays->dx || !rays->dy || !rays->dz))
        return CGS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    if (!s->hashed) return CGS_ERR_NOT_BUILT;
    if (n == 0) return CGS_OK;
    CGS_TRY(cudaSetDevice(s->device));
    cudaStream_t st = (cudaStream_t)stream;
    bool captured = false;
    if (int er = query_begin(s, st, captured)) return er;
    CGS_TRY(cudaMemsetAsync(s->counters.p, 0, sizeof(Counters), st));
    RaysSoA r {rays->ox, rays->oy, rays->oz, rays->dx, rays->dy, rays->dz, rays->tmax, rays->group};
    Query q {method, precision, tol};
    s->launches = 0;
    {
        int er = ensure_engine(s, n);
        if (er) return er;
    }
    cudaError_t e = run_query(s->dev(), r, n, nullptr, q, any_hit != 0,
                              HitsSoA {hits->t, hits->u, hits->v, hits->patch, hits->object}, hits->patch,
                              s->engine.p, s->engineCapacity, kEnginePasses, s->counters.p, st, &s->launches);
    query_end(s, st, captured);
    return cuda_status(e);
}

int cgs_traverse(cgs_scene* s, const cgs_rays* rays, uint32_t n, int any_hit, uint32_t* list_lengths, void* stream)
{
    if (!s || !rays) return CGS_ERR_INVALID_ARGUMENT;
    if (n && (!rays->ox || !rays->oy || !rays->oz || !rays->dx || !rays->dy || !rays->dz))
        return CGS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    if (!s->hashed) return CGS_ERR_NOT_BUILT;
    if (n == 0) return CGS_OK;
    CGS_TRY(cudaSetDevice(s->device));
    cudaStream_t st = (cudaStream_t)stream;
    bool captured = false;
    if (int er = query_begin(s, st, captured)) return er;
    CGS_TRY(cudaMemsetAsync(s->counters.p, 0, sizeof(Counters), st));
    RaysSoA r {rays->ox, rays->oy, rays->oz, rays->dx, rays->dy, rays->dz, rays->tmax, rays->group};
    s->launches = 0;
    {
        int er = ensure_engine(s, n);
        if (er) return er;
    }
    cudaError_t e = run_traverse(s->dev(), r, n, any_hit != 0, s->engine.p, s->engineCapacity, s->counters.p, st,
                                 list_lengths, &s->launches);
    query_end(s, st, captured);
    return cuda_status(e);
}

int cgs_intersect_host(cgs_scene* s, const cgs_rays* rays, uint32_t n, int method, int precision, float tol,
                       int any_hit, const cgs_hits* hits, void* stream)
{
    if (!s || !rays || !hits) return CGS_ERR_INVALID_ARGUMENT;
    if (n == 0) return CGS_OK;
    std::lock_guard<std::mutex> hg(s->hostMu);  // the staging buffers are in use until the call returns
    cudaStream_t st = (cudaStream_t)stream;
    cgs_rays dr {};
    cgs_hits dh {};
    {
        std::lock_guard<std::mutex> g(s->mu);
        CGS_TRY(cudaSetDevice(s->device));
        CGS_TRY(s->rayStage.reserve(7ull * n));
        CGS_TRY(s->hitF.reserve(3ull * n));
        CGS_TRY(s->hitI.reserve(2ull * n));
        const float* src[7] = {rays->ox, rays->oy, rays->oz, rays->dx, rays->dy, rays->dz, rays->tmax};
        for (int k = 0; k < 7; k++)
        {
            if (!src[k]) { if (k == 6) continue; return CGS_ERR_INVALID_ARGUMENT; }
            CGS_TRY(cudaMemcpyAsync(s->rayStage.p + size_t(k) * n, src[k], n * sizeof(float), cudaMemcpyHostToDevice, st));
        }
        float* R = s->rayStage.p;
        dr = cgs_rays {R, R + n, R + 2ull * n, R + 3ull * n, R + 4ull * n, R + 5ull * n,
                       rays->tmax ? R + 6ull * n : nullptr, nullptr};
        if (rays->group)
        {
            CGS_TRY(s->groupStage.reserve(n));
            CGS_TRY(cudaMemcpyAsync(s->groupStage.p, rays->group, n * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
            dr.group = s->groupStage.p;
        }
        dh = cgs_hits {s->hitF.p, s->hitF.p + n, s->hitF.p + 2ull * n, s->hitI.p, s->hitI.p + n};
    }
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
    bool captured = false;
    if (int er = query_begin(s, st, captured)) return er;
    CGS_TRY(cudaMemsetAsync(s->counters.p, 0, sizeof(Counters), st));
    RaysSoA r {rays->ox, rays->oy, rays->oz, rays->dx, rays->dy, rays->dz, rays->tmax, nullptr};
    Query q {method, 0, tol};
    s->launches = 1;
    const cudaError_t e = launch_patch_pairs(s->dev(), surface, s->surfaces[surface].patchCount(), r, pids, n, q,
                                             HitsSoA {hits->t, hits->u, hits->v, hits->patch, hits->object},
                                             s->counters.p, st);
    query_end(s, st, captured);
    return cuda_status(e);
}

int cgs_patch_normal(cgs_scene* s, uint32_t surface, const uint32_t* pids, const float* u, const float* v, uint32_t n,
                     float* normals, void* stream)
{
    if (!s || (n && (!pids || !u || !v || !normals))) return CGS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    if (!s->uploaded) return CGS_ERR_NOT_BUILT;
    if (surface >= s->surfaces.size()) return CGS_ERR_INVALID_ARGUMENT;
    if (n == 0) return CGS_OK;
    CGS_TRY(cudaSetDevice(s->device));
    cudaStream_t st = (cudaStream_t)stream;
    bool captured = false;
    if (int er = query_begin(s, st, captured)) return er;
    CGS_TRY(cudaMemsetAsync(s->counters.p, 0, sizeof(Counters), st));
    s->launches = 1;
    const cudaError_t e = launch_patch_normals(s->dev(), surface, s->surfaces[surface].patchCount(), pids, u, v, n,
                                               normals, s->counters.p, st);
    query_end(s, st, captured);
    return cuda_status(e);
}

// RayTracer::render (src/rt/RayTracer.cu:107-180) for a batch of requests;
// refuses while the previous batch of this scene is in flight, as the
// reference's render refuses while its worker thread runs.
int cgs_render_batch(cgs_scene* s, const cgs_render_request* reqs, uint32_t n, const cgs_render_options* opt,
                     void* stream)
{
    if (!s) return CGS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    std::vector<DevRequest> host;
    RenderBatch b;
    int r = prepare_batch(s, reqs, n, opt, host, b);
    if (r) return r;
    if (!s->hashed) return CGS_ERR_NOT_BUILT;
    CGS_TRY(cudaSetDevice(s->device));
    if (cudaEventQuery(s->finished) == cudaErrorNotReady) return CGS_ERR_BUSY;
    cudaStream_t st = (cudaStream_t)stream;
    s->launches = 0;
    r = run_batch(s, s->slot, host, b, opt->schedule, st, &s->launches);
    if (r) return r;
    CGS_TRY(cudaEventRecord(s->finished, st));
    s->lastStream = st;
    s->lastCounters = s->slot.counters.p;
    return CGS_OK;
}

int cgs_render(cgs_scene* s, const cgs_camera* cam, uint32_t w, uint32_t h, const cgs_render_options* opt,
               uint32_t* fb, uint32_t stride, float* linear, void* stream)
{
    if (!s || !cam || !opt || w == 0 || h == 0 || (!fb && !linear) || (fb && stride < w)) return CGS_ERR_INVALID_ARGUMENT;
    if (opt->recursion_depth < 0 || opt->recursion_depth > 64) return CGS_ERR_INVALID_ARGUMENT;
    cgs_render_request req {};
    req.group = 0;
    req.camera = *cam;
    req.width = w; req.height = h; req.spp = 1;
    req.recursion_depth = opt->recursion_depth;
    req.framebuffer = fb; req.linear_rgb = linear;
    std::lock_guard<std::mutex> g(s->mu);
    std::vector<DevRequest> host;
    RenderBatch b;
    int r = prepare_batch(s, &req, 1, opt, host, b);
    if (r) return r;
    host[0].stride = fb ? stride : w;
    if (!s->hashed) return CGS_ERR_NOT_BUILT;
    CGS_TRY(cudaSetDevice(s->device));
    if (cudaEventQuery(s->finished) == cudaErrorNotReady) return CGS_ERR_BUSY;
    cudaStream_t st = (cudaStream_t)stream;
    s->launches = 0;
    r = run_batch(s, s->slot, host, b, opt->schedule, st, &s->launches);
    if (r) return r;
    CGS_TRY(cudaEventRecord(s->finished, st));
    s->lastStream = st;
    s->lastCounters = s->slot.counters.p;
    return CGS_OK;
}

int cgs_render_host(cgs_scene* s, const cgs_camera* cam, uint32_t w, uint32_t h, const cgs_render_options* opt,
                    uint32_t* fb, float* linear, void* stream)
{
    if (!s || (!fb && !linear) || w == 0 || h == 0) return CGS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> hg(s->hostMu);  // the staging buffers are in use until the call returns
    cudaStream_t st = (cudaStream_t)stream;
    {
        std::lock_guard<std::mutex> g(s->mu);
        CGS_TRY(cudaSetDevice(s->device));
        if (cudaEventQuery(s->finished) == cudaErrorNotReady) return CGS_ERR_BUSY;
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

int cgs_camera_rays(const cgs_camera* cam, uint32_t w, uint32_t h, int flip_y, float* rays, void* stream)
{
    if (!cam || !rays || w == 0 || h == 0 || uint64_t(w) * h >= (1ull << 32)) return CGS_ERR_INVALID_ARGUMENT;
    CameraSetup c;
    camera_setup(*cam, w, h, flip_y, c);
    return cuda_status(launch_camera_rays(c, w, h, rays, (cudaStream_t)stream));
}

static cgs_engine_config to_c(const EngineConfig& c)
{
    return cgs_engine_config {c.passes,         c.collectThreads,  c.resolveThreads, c.collectOccupancy,
                              c.resolveOccupancy, c.backtrackCache, c.compressedNodes, c.queueChunk,
                              c.packetWidth,      c.rayOrder,       c.originLast,      c.subdivLevels};
}

int cgs_engine_config_get(cgs_engine_config* out)
{
    if (!out) return CGS_ERR_INVALID_ARGUMENT;
    const EngineConfig c = engine_config();
    *out = to_c(c);
    return CGS_OK;
}

int cgs_engine_config_set(const cgs_engine_config* in)
{
    if (!in) return CGS_ERR_INVALID_ARGUMENT;
    const EngineConfig c {in->passes,          in->collect_threads, in->resolve_threads,
                          in->collect_occupancy, in->resolve_occupancy, in->backtrack_cache,
                          in->compressed_nodes,  in->queue_chunk,     in->packet_width,
                          in->ray_order,         in->origin_last,     in->subdiv_levels};
    return set_engine_config(c) ? CGS_OK : CGS_ERR_INVALID_ARGUMENT;
}

// The autotuner: a coordinate descent over the engine settings.  Each
// candidate renders the batch (wavefront schedule) `repeats` + 2 times, the
// last `repeats` timed with CUDA events on `stream`; its median is its score.
// Two rounds visit the knobs in turn, each set to its fastest value with the
// others held; scores are kept, so a setting is timed once.
int cgs_autotune_render(cgs_scene* s, const cgs_render_request* reqs, uint32_t n, const cgs_render_options* opt,
                        int repeats, cgs_engine_config* best, double* best_ms, void* stream)
{
    if (!s || !opt || repeats < 1 || repeats > 64) return CGS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    std::vector<DevRequest> host;
    RenderBatch b;
    int r = prepare_batch(s, reqs, n, opt, host, b);
    if (r) return r;
    if (!s->hashed) return CGS_ERR_NOT_BUILT;
    CGS_TRY(cudaSetDevice(s->device));
    if (cudaEventQuery(s->finished) == cudaErrorNotReady) return CGS_ERR_BUSY;
    cudaStream_t st = (cudaStream_t)stream;
    const EngineConfig saved = engine_config();
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CGS_TRY(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) { cudaEventDestroy(e0); return CGS_ERR_CUDA; }
    int status = CGS_OK;

    // the knobs; `capped` stands for the traversal's blocks per SM: as many as
    // fit (0), or three quarters of that (768 threads per SM), which leaves
    // room for the overlapping queries
    struct Point { int passes, ct, rt, capped, cq, chunk, width, order, olast, levels; };
    auto config = [&](const Point& p) {
        EngineConfig c = saved;
        c.passes = p.passes; c.collectThreads = p.ct; c.resolveThreads = p.rt;
        c.collectOccupancy = p.capped ? 768 / p.ct : 0; c.resolveOccupancy = 0;
        c.compressedNodes = p.cq; c.queueChunk = p.chunk; c.packetWidth = p.width; c.rayOrder = p.order;
        c.originLast = p.olast; c.subdivLevels = p.levels;
        return c;
    };
    auto key = [](const Point& p) {
        return ((((((((int64_t(p.passes) * 512 + p.ct) * 256 + p.rt) * 2 + p.capped) * 2 + p.cq) * 128 + p.chunk) * 64 +
                  p.width) * 2 + p.order) * 2 + p.olast) * 128 + p.levels;
    };
    std::map<int64_t, double> scores;
    auto score = [&](const Point& p) -> double {
        const auto it = scores.find(key(p));
        if (it != scores.end()) return it->second;
        if (!set_engine_config(config(p))) return 1e300;
        std::vector<float> ms;
        for (int k = 0; k < repeats + 2 && status == CGS_OK; k++)
        {
            RenderBatch bk = b;
            if (k >= 2 && cudaEventRecord(e0, st) != cudaSuccess) status = CGS_ERR_CUDA;
            if (status == CGS_OK) status = run_batch(s, s->slot, host, bk, CGS_SCHED_WAVEFRONT, st, &s->launches);
            if (status == CGS_OK && k >= 2)
            {
                float t = 0.0f;
                if (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                    cudaEventElapsedTime(&t, e0, e1) != cudaSuccess)
                    status = CGS_ERR_CUDA;
                ms.push_back(t);
            }
            else if (status == CGS_OK && cudaStreamSynchronize(st) != cudaSuccess)
                status = CGS_ERR_CUDA;
        }
        if (status != CGS_OK || ms.empty()) return 1e300;
        std::sort(ms.begin(), ms.end());
        return scores[key(p)] = ms[ms.size() / 2];
    };

    // start from the current setting, rounded onto the search grid
    Point cur {saved.passes, saved.collectThreads, saved.resolveThreads, saved.collectOccupancy != 0 ? 1 : 0,
               saved.compressedNodes, saved.queueChunk, saved.packetWidth, saved.rayOrder, saved.originLast,
               saved.subdivLevels};
    double curMs = score(cur);
    std::vector<std::pair<int Point::*, std::vector<int>>> knobs {
        {&Point::passes, {1, 2, 4, 8}}, {&Point::ct, {128, 256}},   {&Point::rt, {64, 128}},
        {&Point::capped, {0, 1}},       {&Point::cq, {0, 1}},       {&Point::chunk, {8, 16, 32, 64}},
        {&Point::width, {1, 8, 16}},    {&Point::order, {0, 1}},    {&Point::olast, {0, 1}}};
    // the subdivision levels per round matter only to a subdivision batch
    if (opt->method == CGS_METHOD_SUBDIV) knobs.push_back({&Point::levels, {1, 4, 16, 64}});
    for (int round = 0; round < 2 && status == CGS_OK; round++)
        for (const auto& [field, values] : knobs)
            for (int v : values)
            {
                if (status != CGS_OK) break;
                Point p = cur;
                p.*field = v;
                const double ms = score(p);
                if (ms < curMs) { curMs = ms; cur = p; }
            }
    // the pass count and the first chunk act together (a small chunk needs the
    // passes to resume its rays), so a last stage tries them as pairs
    for (int passes : {2, 4, 8})
        for (int chunk : {8, 16, 32, 64})
        {
            if (status != CGS_OK) break;
            Point p = cur;
            p.passes = passes;
            p.chunk = chunk;
            const double ms = score(p);
            if (ms < curMs) { curMs = ms; cur = p; }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const EngineConfig winner = config(cur);
    set_engine_config(status == CGS_OK ? winner : saved);
    if (status != CGS_OK) return status;
    if (best) *best = to_c(winner);
    if (best_ms) *best_ms = curMs;
    s->lastStream = st;
    s->lastCounters = s->slot.counters.p;
    return CGS_OK;
}

int cgs_render_running(cgs_scene* s)
{
    if (!s) return 0;
    std::lock_guard<std::mutex> g(s->mu);
    if (cudaSetDevice(s->device) != cudaSuccess) return 0;
    return cudaEventQuery(s->finished) == cudaErrorNotReady ? 1 : 0;
}

int cgs_perfect_hash_build(const uint32_t* keys, uint32_t n, uint32_t* disp, uint32_t dcap, uint32_t* table,
                           uint32_t tcap, uint32_t params[5], void* stream)
{
    if (!keys || !disp || !table || !params || n == 0) return CGS_ERR_INVALID_ARGUMENT;
    if (dcap < displ_size(n) || tcap < table_capacity(n)) return CGS_ERR_INVALID_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    if (n <= kHashGlobalBlockMaxKeys)
    {
        // one CTA builds the table, its scratch in shared memory up to
        // kHashBlockMaxKeys keys, else in global memory (hash_build_blocks)
        HashJob J {};
        J.n = n; J.tableCap = tcap; J.mask = displ_size(n) - 1;
        hash_coefficients(n, J.A, J.B);
        uint32_t* dj = nullptr;
        const size_t jobWords = (sizeof(HashJob) + 3) / 4 + 1;
        const size_t scratch = n > kHashBlockMaxKeys ? size_t(hash_block_scratch_words(n)) + 2 : 0;
        CGS_TRY(cudaMallocAsync(&dj, (jobWords + 8 + scratch) * sizeof(uint32_t), st));
        uint32_t res[8] = {};
        uint32_t* gs = scratch ? dj + ((jobWords + 8 + 1) & ~size_t(1)) : nullptr;
        cudaError_t e = cudaMemcpyAsync(dj, &J, sizeof J, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = hash_build_blocks(keys, reinterpret_cast<const HashJob*>(dj), 1, n, disp, table, dj + jobWords, st,
                                  gs);
        if (e == cudaSuccess) e = cudaMemcpyAsync(res, dj + jobWords, sizeof res, cudaMemcpyDeviceToHost, st);
        cudaFreeAsync(dj, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return CGS_ERR_CUDA;
        for (int k = 0; k < 5; k++) params[k] = res[1 + k];
        if (res[0] == 4) return CGS_ERR_HASH_BUCKET_OVERFLOW;
        if (res[0]) return CGS_ERR_HASH_FAILED;
        return CGS_OK;
    }
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
