// server.cu -- the request server of libcgspline_gb300.so (cgs_server_*):
// a scheduler thread that cuts submitted render / ray-query requests into
// chunks, packs queued chunks into batches and runs each batch on the first
// free slot (a stream with its own working buffers), so that batches overlap
// on the device and requests that arrive meanwhile join the next batch.
#include <chrono>
#include <condition_variable>
#include <deque>
#include <thread>
#include <unordered_map>

#include "scene_impl.h"

using namespace cgs;

namespace {

constexpr uint32_t kMaxSlots = 16;
constexpr uint32_t kDefaultBatchChunks = 256;
constexpr uint32_t kMaxUnits = 1u << 30;  // samples or rays in one batch

enum Kind : int { kRender = 0, kClosest = 1, kAnyHit = 2 };

// Device bytes of a query batch of n rays: staged rays (7 floats), group,
// hits (3 floats + 2 ints) and the query engine's scratch.
uint64_t query_bytes(uint32_t n)
{
    return uint64_t(n) * (7 + 1 + 3 + 2) * 4 + uint64_t(engine_words(n, kEnginePasses)) * 4;
}

// Largest n <= hi with bytes(n) <= budget (bytes non-decreasing), or 0.
template<class F> uint32_t largest_fit(F bytes, uint64_t budget, uint32_t hi)
{
    if (hi == 0 || bytes(1) > budget) return 0;
    uint32_t lo = 1;
    while (lo < hi)
    {
        const uint32_t mid = lo + (hi - lo + 1) / 2;
        if (bytes(mid) <= budget) lo = mid; else hi = mid - 1;
    }
    return lo;
}

struct Request
{
    cgs_request_info info {};
    uint32_t pending = 0;  // chunks not finished
    uint32_t waiters = 0;
    bool done = false;
};

struct Chunk
{
    uint64_t ticket;
    int kind;
    uint32_t units;  // samples (render) or rays (query)
    DevRequest render;
    QueryChunk query;
};

struct Slot
{
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    RenderSlot rs;
    DBuf<float> qrays, qhitF;
    DBuf<uint32_t> qgroup;
    DBuf<int32_t> qhitI;
    DBuf<QueryChunk> qtab;
    DBuf<uint32_t> qhdr;             // (chunks, rays) of a query batch
    DevRequest* hostReq = nullptr;   // pinned request table of the batch
    QueryChunk* hostQuery = nullptr; // pinned query table of the batch
    RenderBatch* hostBatch = nullptr;
    uint32_t* hostHdr = nullptr;
    Counters* hostCnt = nullptr;     // pinned copy of the batch's counters
    std::vector<Chunk> chunks;       // the batch on this slot
    bool busy = false;
    int launches = 0;

    uint32_t qcap = 0;               // query staging capacity (rays)

    uint64_t query_held() const { return qrays.bytes() + qhitF.bytes() + qgroup.bytes() + qhitI.bytes() + qtab.bytes(); }
    uint64_t bytes() const { return rs.bytes() + query_held(); }
    void release_query()
    {
        qrays.release(); qhitF.release(); qgroup.release(); qhitI.release(); qtab.release();
        qcap = 0;
    }
};

}  // namespace

struct cgs_server
{
    cgs_scene* scene = nullptr;
    cgs_server_options opt {};
    bool plain = false;
    uint32_t ngroups = 0, maxLights = 1, maxRender = 0, maxQuery = 0, maxChunks = kDefaultBatchChunks;
    uint64_t share = 0;  // device bytes per slot
    std::vector<Slot> slots;
    std::chrono::steady_clock::time_point t0;

    std::mutex mu;
    std::condition_variable wake, finished;
    std::deque<Chunk> queue;
    std::unordered_map<uint64_t, Request> requests;
    uint64_t nextTicket = 1;
    bool stop = false;
    std::thread worker;

    cgs_server_stats stats {};
    uint32_t inflight = 0;
    double busySince = 0.0;

    double clock() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
    void run();
    int grow(Slot& s, int kind, uint32_t units, uint32_t nchunks);
    cudaError_t launch(Slot& s);
    void reap(Slot& s, cudaError_t e);
    void release_slots();
};

// Working buffers of slot s for a batch of `units` samples or rays of one
// kind, within the slot's share of the budget: the other kind's buffers are
// released first when both would not fit.  Worker thread only.
int cgs_server::grow(Slot& s, int kind, uint32_t units, uint32_t nchunks)
{
    if (plain)
    {
        CGS_TRY(s.rs.counters.reserve(1));
        return CGS_OK;
    }
    if (kind == kRender)
    {
        if (s.query_held() + RenderSlot::bytes_for(units, maxLights) > share) s.release_query();
        CGS_TRY(s.rs.batch.reserve(1));
        return s.rs.ensure(units, maxLights, std::max(nchunks, maxChunks));
    }
    // staging grows in powers of two up to the batch limit, so that a slot
    // settles on one capacity (and one captured graph per query kind)
    if (units > maxQuery) return CGS_ERR_INVALID_ARGUMENT;  // batches are packed within maxQuery
    uint32_t cap = std::max(s.qcap, std::min(1024u, maxQuery));
    while (cap < units) cap = cap * 2 > maxQuery ? maxQuery : cap * 2;
    if (s.rs.bytes() - s.rs.engine.bytes() + query_bytes(cap) > share) s.rs.release();
    if (cap != s.qcap)
    {
        s.qcap = 0;  // a reserve that fails frees its old buffer
        CGS_TRY(s.qrays.reserve(7ull * cap));
        CGS_TRY(s.qgroup.reserve(cap));
        CGS_TRY(s.qhitF.reserve(3ull * cap));
        CGS_TRY(s.qhitI.reserve(2ull * cap));
        s.qcap = cap;
    }
    CGS_TRY(s.qtab.reserve(maxChunks));
    CGS_TRY(s.qhdr.reserve(2));
    CGS_TRY(s.rs.counters.reserve(1));
    return s.rs.ensure_engine(cap);
}

// Enqueues the batch s.chunks on slot s's stream and records s.done.
// Worker thread, without the lock.
cudaError_t cgs_server::launch(Slot& s)
{
    const DevScene S = scene->dev();
    const cgs_render_options& ro = opt.render;
    const Query q {ro.method, ro.precision, ro.tol};
    const int kind = s.chunks.front().kind;
    const uint32_t n = uint32_t(s.chunks.size());
    uint32_t units = 0;
    for (const Chunk& c : s.chunks) units += c.units;
    s.launches = 0;
    if (int st = grow(s, kind, units, n)) return st == CGS_ERR_OUT_OF_MEMORY ? cudaErrorMemoryAllocation : cudaErrorUnknown;
    Counters* cnt = s.rs.counters.p;
    cudaError_t e = cudaMemsetAsync(cnt, 0, sizeof(Counters), s.stream);
    if (e != cudaSuccess) return e;
    if (kind == kRender)
    {
        RenderBatch b {};
        uint32_t sb = 0, pb = 0;
        int maxDepth = 0;
        for (uint32_t k = 0; k < n; k++)
        {
            DevRequest d = s.chunks[k].render;
            d.sampleBase = sb; d.pixelBase = pb;
            sb += d.width * d.height * d.spp;
            pb += d.width * d.height;
            maxDepth = std::max(maxDepth, d.depth);
            s.hostReq[k] = d;
        }
        b.nreq = n; b.samples = sb; b.pixels = pb; b.maxDepth = maxDepth; b.eps = ro.eps; b.q = q;
        b.sampling = ro.sampling;
        if (plain)
            e = launch_render_plain(S, b, s.hostReq, cnt, s.stream, &s.launches);
        else
        {
            b.req = s.rs.req.p;
            *s.hostBatch = b;
            e = cudaMemcpyAsync(s.rs.req.p, s.hostReq, n * sizeof(DevRequest), cudaMemcpyHostToDevice, s.stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(s.rs.batch.p, s.hostBatch, sizeof(RenderBatch), cudaMemcpyHostToDevice, s.stream);
            if (e == cudaSuccess) e = launch_wavefront_cached(S, s.rs, b, s.stream, &s.launches);
        }
    }
    else
    {
        const bool any = kind == kAnyHit;
        if (plain)
        {
            // one request; the plain kernel reads and writes its arrays in place
            const QueryChunk& c = s.chunks.front().query;
            const RaysSoA r {c.src[0], c.src[1], c.src[2], c.src[3], c.src[4], c.src[5], c.src[6], nullptr};
            e = launch_query_plain(S, r, c.n, c.group, q, any, c.out, cnt, s.stream);
            s.launches++;
        }
        else
        {
            for (uint32_t k = 0, base = 0; k < n; k++)
            {
                s.hostQuery[k] = s.chunks[k].query;
                s.hostQuery[k].base = base;
                base += s.chunks[k].units;
            }
            s.hostHdr[0] = n;
            s.hostHdr[1] = units;
            e = cudaMemcpyAsync(s.qtab.p, s.hostQuery, n * sizeof(QueryChunk), cudaMemcpyHostToDevice, s.stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(s.qhdr.p, s.hostHdr, 2 * sizeof(uint32_t), cudaMemcpyHostToDevice, s.stream);
            // the sequence reads the batch size from qhdr: one graph per (slot capacity, kind)
            Slot* sp = &s;
            const uint32_t cap = s.qcap;
            const uint64_t key = key_of({scene_key(S), query_key(q), uint64_t(any), engine_config_generation(),
                                         key_of(s.qrays.p),
                                         key_of(s.qhitF.p), key_of(s.qhitI.p), key_of(s.qgroup.p), key_of(s.qtab.p),
                                         key_of(s.qhdr.p), key_of(s.rs.engine.p), s.rs.engineCapacity, cap,
                                         key_of(cnt)});
            if (e == cudaSuccess)
                e = run_cached(s.rs.graphs, key, s.stream, &s.launches, [&](cudaStream_t st, int* nl) {
                    float* R = sp->qrays.p;
                    const RaysSoA rays {R, R + cap, R + 2ull * cap, R + 3ull * cap, R + 4ull * cap, R + 5ull * cap,
                                        R + 6ull * cap, sp->qgroup.p};
                    const HitsSoA hits {sp->qhitF.p, sp->qhitF.p + cap, sp->qhitF.p + 2ull * cap, sp->qhitI.p,
                                        sp->qhitI.p + cap};
                    cudaError_t r = launch_gather_rays(sp->qtab.p, sp->qhdr.p, cap, sp->qrays.p, sp->qgroup.p, st);
                    if (r == cudaSuccess)
                        r = run_query(S, rays, cap, sp->qhdr.p + 1, q, any, hits, hits.patch, sp->rs.engine.p,
                                      sp->rs.engineCapacity, kEnginePasses, cnt, st, nl);
                    if (r == cudaSuccess) r = launch_scatter_hits(sp->qtab.p, sp->qhdr.p, cap, hits, any, st);
                    *nl += 2;
                    return r;
                });
        }
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(s.hostCnt, cnt, sizeof(Counters), cudaMemcpyDeviceToHost, s.stream);
    if (e == cudaSuccess) e = cudaEventRecord(s.done, s.stream);
    return e;
}

// Completes the batch of slot s (lock held).
void cgs_server::reap(Slot& s, cudaError_t e)
{
    const double t = clock();
    if (e == cudaSuccess) stats.rays_traced += s.hostCnt->rays;
    stats.kernel_launches += uint64_t(s.launches);
    for (const Chunk& c : s.chunks)
    {
        auto it = requests.find(c.ticket);
        if (it == requests.end()) continue;
        Request& r = it->second;
        if (e != cudaSuccess && r.info.status == CGS_OK) r.info.status = cuda_status(e);
        if (--r.pending == 0)
        {
            r.done = true;
            r.info.finish_s = t;
            stats.finished++;
        }
    }
    s.chunks.clear();
    s.busy = false;
    if (--inflight == 0) stats.busy_s += t - busySince;
    finished.notify_all();
}

void cgs_server::run()
{
    cudaSetDevice(scene->device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;)
    {
        bool progress = false;
        for (Slot& s : slots)
        {
            if (!s.busy) continue;
            const cudaError_t qe = cudaEventQuery(s.done);
            if (qe == cudaErrorNotReady) continue;
            reap(s, qe);
            progress = true;
        }
        for (Slot& s : slots)
        {
            if (s.busy || queue.empty()) continue;
            const int kind = queue.front().kind;
            const uint32_t limit = kind == kRender ? maxRender : maxQuery;
            uint32_t units = 0;
            while (!queue.empty() && queue.front().kind == kind && s.chunks.size() < maxChunks)
            {
                const Chunk& c = queue.front();
                if (!s.chunks.empty() && (plain || units + c.units > limit)) break;
                units += c.units;
                s.chunks.push_back(c);
                queue.pop_front();
            }
            s.busy = true;
            const double t = clock();
            if (inflight++ == 0) busySince = t;
            stats.batches++;
            stats.chunks += s.chunks.size();
            for (const Chunk& c : s.chunks)
            {
                auto it = requests.find(c.ticket);
                if (it != requests.end() && it->second.info.start_s < 0.0) it->second.info.start_s = t;
            }
            lk.unlock();
            const cudaError_t e = launch(s);
            // a batch that failed part-way may have work on the stream: let it
            // drain before its requests are reported finished, so that callers
            // may free their buffers
            if (e != cudaSuccess) cudaStreamSynchronize(s.stream);
            lk.lock();
            uint64_t held = 0;
            for (const Slot& x : slots) held += x.bytes();
            stats.slot_bytes = held;
            stats.peak_slot_bytes = std::max(stats.peak_slot_bytes, held);
            if (e != cudaSuccess)
            {
                cudaGetLastError();
                reap(s, e);
            }
            progress = true;
        }
        if (stop && queue.empty() && inflight == 0) break;
        if (!progress)
        {
            if (inflight > 0)
                wake.wait_for(lk, std::chrono::microseconds(20));
            else
                wake.wait(lk, [&] { return stop || !queue.empty(); });
        }
    }
}

void cgs_server::release_slots()
{
    cudaSetDevice(scene->device);
    for (Slot& s : slots)
    {
        if (s.stream) cudaStreamSynchronize(s.stream);
        s.rs.release();
        s.release_query();
        if (s.hostReq) cudaFreeHost(s.hostReq);
        if (s.hostQuery) cudaFreeHost(s.hostQuery);
        if (s.hostCnt) cudaFreeHost(s.hostCnt);
        if (s.hostBatch) cudaFreeHost(s.hostBatch);
        if (s.hostHdr) cudaFreeHost(s.hostHdr);
        s.qhdr.release();
        if (s.done) cudaEventDestroy(s.done);
        if (s.stream) cudaStreamDestroy(s.stream);
        s = Slot {};
    }
}

extern "C" {

int cgs_server_create(cgs_server** out, cgs_scene* scene, const cgs_server_options* o)
{
    if (!out || !scene || !o) return CGS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    const cgs_render_options& ro = o->render;
    if (o->slots == 0 || o->slots > kMaxSlots || !valid_query(ro.method, ro.precision) || !(ro.tol > 0.0f) ||
        (ro.schedule != CGS_SCHED_PLAIN && ro.schedule != CGS_SCHED_WAVEFRONT) ||
        (ro.sampling != CGS_SAMPLING_MIRROR && ro.sampling != CGS_SAMPLING_MONTE_CARLO) || ro.recursion_depth < 0 ||
        ro.recursion_depth > 64)
        return CGS_ERR_INVALID_ARGUMENT;
    auto* sv = new (std::nothrow) cgs_server();
    if (!sv) return CGS_ERR_OUT_OF_MEMORY;
    {
        std::lock_guard<std::mutex> g(scene->mu);
        if (!scene->hashed) { delete sv; return CGS_ERR_NOT_BUILT; }
        sv->ngroups = uint32_t(scene->groups.size());
        sv->maxLights = scene->maxLights();
    }
    sv->scene = scene;
    sv->opt = *o;
    sv->plain = ro.schedule == CGS_SCHED_PLAIN;
    const uint32_t nslots = sv->plain ? 1u : o->slots;
    sv->maxChunks = sv->plain ? 1u : (o->max_batch_requests ? std::min(o->max_batch_requests, 4096u) : kDefaultBatchChunks);
    if (sv->plain)
    {
        sv->maxRender = sv->maxQuery = kMaxUnits;
    }
    else
    {
        sv->share = o->memory_budget / nslots;
        const uint32_t L = sv->maxLights, C = sv->maxChunks;
        const uint32_t hiR = std::min<uint64_t>(kMaxUnits, ((1ull << 31) - 1) / L);
        sv->maxRender = largest_fit([&](uint32_t s) { return RenderSlot::bytes_for(s, L) + uint64_t(C) * sizeof(DevRequest); },
                                    sv->share, hiR);
        sv->maxQuery = largest_fit([&](uint32_t n) { return query_bytes(n) + uint64_t(C) * sizeof(QueryChunk); }, sv->share,
                                   kMaxUnits);
        if (o->max_batch_samples)
        {
            sv->maxRender = std::min(sv->maxRender, o->max_batch_samples);
            sv->maxQuery = std::min(sv->maxQuery, o->max_batch_samples);
        }
        if (sv->maxRender == 0 || sv->maxQuery == 0) { delete sv; return CGS_ERR_ADMISSION; }
    }
    if (cudaSetDevice(scene->device) != cudaSuccess) { delete sv; return CGS_ERR_CUDA; }
    sv->slots.resize(nslots);
    for (Slot& s : sv->slots)
    {
        cudaError_t e = cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaMallocHost(&s.hostReq, sv->maxChunks * sizeof(DevRequest));
        if (e == cudaSuccess) e = cudaMallocHost(&s.hostQuery, sv->maxChunks * sizeof(QueryChunk));
        if (e == cudaSuccess) e = cudaMallocHost(&s.hostCnt, sizeof(Counters));
        if (e == cudaSuccess) e = cudaMallocHost(&s.hostBatch, sizeof(RenderBatch));
        if (e == cudaSuccess) e = cudaMallocHost(&s.hostHdr, 2 * sizeof(uint32_t));
        if (e != cudaSuccess)
        {
            sv->release_slots();
            delete sv;
            return cuda_status(e);
        }
    }
    sv->stats.max_batch_samples = sv->maxRender;
    sv->t0 = std::chrono::steady_clock::now();
    sv->worker = std::thread([sv] { sv->run(); });
    *out = sv;
    return CGS_OK;
}

int cgs_server_destroy(cgs_server* sv)
{
    if (!sv) return CGS_ERR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::mutex> g(sv->mu);
        sv->stop = true;
    }
    sv->wake.notify_all();
    if (sv->worker.joinable()) sv->worker.join();
    sv->release_slots();
    delete sv;
    return CGS_OK;
}

int cgs_server_submit_render(cgs_server* sv, const cgs_render_request* r, uint64_t* ticket)
{
    if (!sv || !r || !ticket) return CGS_ERR_INVALID_ARGUMENT;
    const int depth = r->recursion_depth < 0 ? sv->opt.render.recursion_depth : r->recursion_depth;
    if (r->width == 0 || r->height == 0 || r->spp == 0 || r->spp > 4096 || (!r->framebuffer && !r->linear_rgb) ||
        r->group >= sv->ngroups || depth > 64)
        return CGS_ERR_INVALID_ARGUMENT;
    const uint64_t row = uint64_t(r->width) * r->spp;
    const uint64_t total = row * r->height;
    if (total >= (1ull << 31) || row > sv->maxRender)
    {
        std::lock_guard<std::mutex> g(sv->mu);
        sv->stats.rejected++;
        return CGS_ERR_ADMISSION;
    }
    const uint32_t rows = sv->plain ? r->height : uint32_t(std::min<uint64_t>(r->height, sv->maxRender / row));
    DevRequest d {};
    camera_setup(r->camera, r->width, r->height, sv->opt.render.flip_y, d.cam);
    d.group = r->group; d.width = r->width; d.spp = r->spp; d.depth = depth; d.stride = r->width;
    {
        std::lock_guard<std::mutex> g(sv->mu);
        const uint64_t t = sv->nextTicket++;
        Request& R = sv->requests[t];
        R.info.status = CGS_OK;
        R.info.submit_s = sv->clock();
        R.info.start_s = -1.0;
        R.info.samples = total;
        for (uint32_t y = 0; y < r->height; y += rows)
        {
            Chunk c {};
            c.ticket = t;
            c.kind = kRender;
            c.render = d;
            c.render.row0 = y;
            c.render.height = std::min(rows, r->height - y);
            c.render.fb = r->framebuffer ? r->framebuffer + size_t(y) * r->width : nullptr;
            c.render.linear = r->linear_rgb ? r->linear_rgb + 3ull * y * r->width : nullptr;
            c.units = uint32_t(row * c.render.height);
            sv->queue.push_back(c);
            R.pending++;
        }
        R.info.chunks = R.pending;
        sv->stats.submitted++;
        *ticket = t;
    }
    sv->wake.notify_one();
    return CGS_OK;
}

int cgs_server_submit_query(cgs_server* sv, const cgs_query_request* q, uint64_t* ticket)
{
    if (!sv || !q || !ticket) return CGS_ERR_INVALID_ARGUMENT;
    const cgs_rays& R = q->rays;
    const cgs_hits& H = q->hits;
    if (q->n == 0 || q->group >= sv->ngroups || !R.ox || !R.oy || !R.oz || !R.dx || !R.dy || !R.dz || !H.patch ||
        (!q->any_hit && (!H.t || !H.u || !H.v || !H.object)))
        return CGS_ERR_INVALID_ARGUMENT;
    const uint32_t step = sv->plain ? q->n : sv->maxQuery;
    {
        std::lock_guard<std::mutex> g(sv->mu);
        const uint64_t t = sv->nextTicket++;
        Request& Rq = sv->requests[t];
        Rq.info.status = CGS_OK;
        Rq.info.submit_s = sv->clock();
        Rq.info.start_s = -1.0;
        Rq.info.samples = q->n;
        for (uint32_t i = 0; i < q->n; i += step)
        {
            const uint32_t m = std::min(step, q->n - i);
            Chunk c {};
            c.ticket = t;
            c.kind = q->any_hit ? kAnyHit : kClosest;
            c.units = m;
            const float* src[7] = {R.ox, R.oy, R.oz, R.dx, R.dy, R.dz, R.tmax};
            for (int k = 0; k < 7; k++) c.query.src[k] = src[k] ? src[k] + i : nullptr;
            c.query.group = q->group;
            c.query.n = m;
            c.query.out = HitsSoA {H.t ? H.t + i : nullptr, H.u ? H.u + i : nullptr, H.v ? H.v + i : nullptr,
                                   H.patch + i, H.object ? H.object + i : nullptr};
            sv->queue.push_back(c);
            Rq.pending++;
        }
        Rq.info.chunks = Rq.pending;
        sv->stats.submitted++;
        *ticket = t;
    }
    sv->wake.notify_one();
    return CGS_OK;
}

int cgs_server_wait(cgs_server* sv, uint64_t ticket, double timeout_s, cgs_request_info* info)
{
    if (!sv) return CGS_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(sv->mu);
    auto it = sv->requests.find(ticket);
    if (it == sv->requests.end()) return CGS_ERR_NOT_FOUND;
    Request* r = &it->second;  // stable until erased below
    r->waiters++;
    bool ok = true;
    if (timeout_s < 0.0)
        sv->finished.wait(lk, [&] { return r->done; });
    else
        ok = sv->finished.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] { return r->done; });
    r->waiters--;
    if (!ok) return CGS_ERR_BUSY;
    if (info) *info = r->info;
    if (r->waiters == 0) sv->requests.erase(ticket);
    return CGS_OK;
}

double cgs_server_clock(const cgs_server* sv)
{
    return sv ? sv->clock() : 0.0;
}

int cgs_server_stats_get(cgs_server* sv, cgs_server_stats* out)
{
    if (!sv || !out) return CGS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(sv->mu);
    *out = sv->stats;
    out->queued = uint32_t(sv->queue.size());
    if (sv->inflight > 0) out->busy_s += sv->clock() - sv->busySince;
    return CGS_OK;
}

}  // extern "C"
