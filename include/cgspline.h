/*
 * cgspline.h -- C ABI of libcgspline_gb300.so, a GB300 (sm_103a) implementation
 * of the ray--bicubic-patch path of MachSilva/cgspline.
 *
 * All entry points return an int status (CGS_OK == 0); nothing aborts, traps
 * or throws across this boundary.  Pointers documented as "device" are CUDA
 * device pointers on the scene's device; "host" pointers are ordinary host
 * memory.  Streams are cudaStream_t passed as void* (NULL = legacy default
 * stream).  Reference paths below are relative to the reference project root.
 */
#ifndef CGSPLINE_GB300_H
#define CGSPLINE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------- status -- */
enum cgs_status {
    CGS_OK = 0,
    CGS_ERR_INVALID_ARGUMENT = 1,
    CGS_ERR_CUDA = 2,              /* a CUDA runtime call failed (the reference aborts: src/rt/CUDAUtility.cpp:8-22) */
    CGS_ERR_OUT_OF_MEMORY = 3,
    CGS_ERR_NOT_BUILT = 4,         /* scene used before cgs_scene_build */
    CGS_ERR_HASH_BUCKET_OVERFLOW = 5, /* > 4 keys share a displacement bucket (reference: __trap, src/rt/PerfectHashFunction.cu:44-46) */
    CGS_ERR_HASH_FAILED = 6,       /* no perfect hash in 16 trials (reference: src/rt/BVH.cpp:26-28 throws) */
    CGS_ERR_EMPTY_LEAF = 7,        /* BVH leaf without elements (reference: src/rt/BVH.cpp:85-87 throws) */
    CGS_ERR_BUSY = 8,              /* a render is still in flight (reference: src/rt/RayTracer.cu:110-116 warns and returns) */
    CGS_ERR_DEVICE_LIMIT = 9,      /* a kernel hit a bounded loop or stack limit (reference: __trap, src/Spline_BezierClipping.cu:736-737) */
    CGS_ERR_ADMISSION = 10,        /* serving: request does not fit the HBM budget */
    CGS_ERR_NOT_FOUND = 11,
    CGS_ERR_CAPACITY = 12          /* input larger than a fixed-capacity entry point accepts */
};

const char* cgs_status_string(int status);
int cgs_version(void);

/* ----------------------------------------------------------- options -- */
enum cgs_method { CGS_METHOD_CLIP = 0, CGS_METHOD_SUBDIV = 1 };
/* Precision of closest-hit searches.  FP32: the reference's arithmetic.
 * FP32_POLISH64: FP32 search and traversal, then an FP64 Newton polish of
 * (u,v,t) of the winning hit.  FP32_GRAZE64 (the full precision form):
 * FP32_POLISH64, and candidates the ray meets within 30 degrees of grazing
 * (of the plane of the patch's diagonals or of a cell of its control net), or
 * whose control net folds over the ray (a silhouette), are searched on a net
 * projected in FP64 from the ray in double, with FP64 fat-line bounds to
 * tolerance 2^-20.  FP64: the whole search in FP64 (traversal, clipping to
 * 1e-9, every root polished), the comparison run of the precision form.
 * Any-hit searches (shadow rays, any_hit queries) always run in FP32. */
enum cgs_precision { CGS_PREC_FP32 = 0, CGS_PREC_FP32_POLISH64 = 1, CGS_PREC_FP64 = 2, CGS_PREC_FP32_GRAZE64 = 3 };
/* Split axis of the BVH build.  REFERENCE: BVH::split's axis, taken from a
 * box that is never inflated (src/rt/BVH.cpp:46-52) and so always y -- the
 * reference's topology, bit for bit.  LONGEST: the longest axis of the
 * elements' centroid box, everything else unchanged: the same hits (up to
 * ties between equally distant candidates) with far fewer node visits.
 * MIRROR: queries and renders traverse the LONGEST build, while
 * cgs_bvh_sizes / cgs_bvh_export give the REFERENCE topology and its hash
 * table (built again on the host, and hashed by cgs_perfect_hash_build, at
 * each call). */
enum cgs_bvh_split { CGS_SPLIT_REFERENCE = 0, CGS_SPLIT_LONGEST = 1, CGS_SPLIT_MIRROR = 2 };
/* PLAIN: one thread per pixel runs the whole bounce chain (the reference's
 * launch shape, src/rt/RayTracer.cu:171-178).  WAVEFRONT: persistent,
 * stage-separated kernels over compacted ray queues. */
enum cgs_schedule { CGS_SCHED_PLAIN = 0, CGS_SCHED_WAVEFRONT = 1 };
/* MIRROR: the reference's default shading, one mirror bounce per level
 * weighted by the specular reflectance (src/rt/RayTracer.cu:523-542).
 * MONTE_CARLO: its sampled path (USE_MONTECARLO_SAMPLING,
 * src/rt/RayTracer.cu:473-521): a GGX microfacet normal per bounce; the
 * random numbers come from Philox4x32-10 keyed by (image sample, depth)
 * instead of the reference's curand states, so they do not depend on the
 * batch a request runs in. */
enum cgs_sampling { CGS_SAMPLING_MIRROR = 0, CGS_SAMPLING_MONTE_CARLO = 1 };

/* src/rt/Scene.h:79-95 */
typedef struct cgs_material {
    float diffuse[3];
    float specular[3];   /* f0 */
    float metalness;
    float roughness;
} cgs_material;

/* src/rt/Scene.h:47-77: angle < 0.01 directional, > 1.57 point, else spot */
typedef struct cgs_light {
    float color[3];
    float strength;
    float position[3];
    float range;         /* 0 = infinite (inverse-square falloff) */
    float direction[3];
    float angle;
} cgs_light;

/* src/rt/Scene.h:16-45: camera looks down its local -z with +y up */
typedef struct cgs_camera {
    float rotation[4];   /* quaternion x, y, z, w */
    float position[3];
    float scale[3];
    float fovy;          /* radians */
} cgs_camera;

/* src/rt/RayTracer.h:26-34 plus this library's search, precision, schedule and sampling choices */
typedef struct cgs_render_options {
    int recursion_depth; /* mirror bounces after the primary hit (reference GPU default 6) */
    float eps;           /* shadow / bounce ray offset (reference 1e-4) */
    int flip_y;
    int method;          /* enum cgs_method */
    int precision;       /* enum cgs_precision */
    float tol;           /* search tolerance on the projected net (reference 2^-12) */
    int schedule;        /* enum cgs_schedule */
    int sampling;        /* enum cgs_sampling */
} cgs_render_options;

/* Rays as structure of arrays; direction must be unit length. */
typedef struct cgs_rays {
    const float* ox; const float* oy; const float* oz;
    const float* dx; const float* dy; const float* dz;
    const float* tmax;     /* ray.max (src/rt/Intersection.h:16-24) */
    const uint32_t* group; /* nullable: the scene group of each ray (default group 0) */
} cgs_rays;

/* Closest-hit results (src/rt/Intersection.h:28-34); patch = object = -1 on a miss.
 * For any-hit queries only patch is written (0 = occluded, -1 = free). */
typedef struct cgs_hits {
    float* t; float* u; float* v;
    int32_t* patch;
    int32_t* object;
} cgs_hits;

typedef struct cgs_counters {
    uint64_t rays;            /* rays traced by the last call (all kinds) */
    uint64_t primary_rays, bounce_rays, shadow_rays;
    uint64_t nodes;           /* inner BVH nodes visited */
    uint64_t hash_lookups;    /* stackless backtracks (each one a perfect-hash lookup in
                                 BVH::hashIntersect) */
    uint64_t candidates;      /* (ray, patch) pairs searched */
    uint64_t iterations;      /* clip / subdivision iterations */
    uint64_t device_errors;   /* bit mask: 1 clip stack full, 2 clip iteration limit,
                                 4 traversal step limit, 8 ray of an unknown group,
                                 16 a patch id past its surface's patch count */
    uint64_t kernel_launches;
    uint64_t hash_table_reads; /* backtracks answered through the perfect hash; the rest
                                  came from the traversal's backtrack cache */
} cgs_counters;

/* -------------------------------------------------------------- scene -- */
typedef struct cgs_scene cgs_scene;

int cgs_scene_create(cgs_scene** out, int device);
int cgs_scene_destroy(cgs_scene* scene);

/* A BezierSurface (src/rt/Primitive.h:90-116): points are xyzw float4, each
 * patch is 16 uint32 indices, point (i,j) at 4*j+i. */
int cgs_scene_add_surface(cgs_scene* scene, const float* points_xyzw, uint32_t npoints,
                          const uint32_t* indices, uint32_t nindices, uint32_t* surface_id);

/* One row of the Scene object arrays (src/rt/Scene.h:99-112).  Matrices are
 * column-major.  patch_material (nullable, one entry per patch) indexes
 * materials[] and overrides `material` per patch. */
int cgs_scene_add_object(cgs_scene* scene, uint32_t surface, const float local2world[16],
                         const float world2local[16], const cgs_material* material,
                         const uint32_t* patch_material, const cgs_material* materials,
                         uint32_t nmaterials, uint32_t* object_id);

/* Lights, background and ambient colour of the current group (rt::Scene::lights,
 * backgroundColor, ambientLight, src/rt/Scene.h:113-119). */
int cgs_scene_set_lights(cgs_scene* scene, const cgs_light* lights, uint32_t n);
int cgs_scene_set_environment(cgs_scene* scene, const float background[3], const float ambient[3]);

/* Groups: several independent scenes (each an rt::Scene with its own objects,
 * object-level BVH, lights and environment) resident in one store, so that
 * one launch can trace rays of different scenes.  A store starts with group 0
 * current; cgs_scene_add_group makes a new group current (or returns the
 * current one if nothing was added to it yet).  Objects, lights and
 * environment calls apply to the current group; surfaces are shared. */
int cgs_scene_add_group(cgs_scene* scene, uint32_t* group_id);

/* Split axis (enum cgs_bvh_split) of the next cgs_bvh_build; default REFERENCE. */
int cgs_scene_set_bvh_split(cgs_scene* scene, int mode);

/* BVH::build for every surface (BezierSurface::buildBVH, src/rt/Primitive.cu:199-220)
 * and the object level (Scene::buildBVH, src/rt/Scene.cu:218-232): host median
 * split, one element per leaf (src/rt/BVH.cpp:9-124). */
int cgs_bvh_build(cgs_scene* scene);

/* BVH::buildHashTable for every BVH (src/rt/BVH.cpp:24-38) with the GPU
 * perfect-hash build (PerfectHashFunction::build, src/rt/PerfectHashFunction.cu:229-503),
 * made deterministic. */
int cgs_hash_build(cgs_scene* scene, void* stream);

/* cgs_bvh_build + device upload + cgs_hash_build (MainWindow::convertScene's
 * acceleration steps, src/MainWindow.cpp:479-491). */
int cgs_scene_build(cgs_scene* scene, void* stream);

/* Device bytes held by a built scene. */
int cgs_scene_footprint(const cgs_scene* scene, uint64_t* bytes);

/* Scene blobs (no counterpart in the reference): cgs_scene_save writes a built
 * store -- surfaces, objects, groups, BVHs and their perfect-hash tables -- to
 * a file; cgs_scene_load reads it back onto `device` without the BVH and hash
 * builds.  The loader checks every count, index and link against the data,
 * and every key's hash slot, before anything reaches the device:
 * CGS_ERR_INVALID_ARGUMENT for a damaged file, CGS_ERR_NOT_FOUND for a
 * missing one. */
int cgs_scene_save(cgs_scene* scene, const char* path);
int cgs_scene_load(cgs_scene** scene, const char* path, int device);

/* which = surface id, or -1 - g for the object-level BVH of group g.
 * sizes = nodes, indices, table size, displacement size, keys. */
int cgs_bvh_sizes(const cgs_scene* scene, int32_t which, uint32_t sizes[5]);
/* nodes: 14 uint32 per node = leftBox lo,hi; rightBox lo,hi (float bits); left; right|first
 * (src/rt/BVH.h:23-39).  params = A, B, N (table size), mask.  Tables are read
 * back from the device. */
int cgs_bvh_export(const cgs_scene* scene, int32_t which, uint32_t* nodes, uint32_t* keys,
                   uint32_t* indices, uint32_t* table, uint32_t* disp, uint32_t params[4]);

/* ------------------------------------------------------------ queries -- */
/* Closest hit (BVH::hashIntersect + rt::intersect, src/rt/BVH.h:178-266,
 * src/rt/Primitive.cu:222-248, Context::intersect src/rt/RayTracer.cu:295-349)
 * or any hit (src/rt/BVH.h:268-350, src/rt/Primitive.cu:250-268) for n rays.
 * rays and hits are device pointers.  Asynchronous on `stream`.
 * CGS_METHOD_CLIP keeps the reference's fat-line hull scan
 * (src/Spline_BezierClipping.cu:655-693), which on some nets excludes a root:
 * on a 1920x1080 frame of a 16,384-patch torus about 2.5e-4 of the hit rays
 * report a farther surface than subdivision finds, at every precision. */
int cgs_intersect(cgs_scene* scene, const cgs_rays* rays, uint32_t n, int method, int precision,
                  float tol, int any_hit, const cgs_hits* hits, void* stream);

/* Same with host rays / hits: copies in, runs, copies out, synchronises. */
int cgs_intersect_host(cgs_scene* scene, const cgs_rays* rays, uint32_t n, int method, int precision,
                       float tol, int any_hit, const cgs_hits* hits, void* stream);

/* The traversal kernel alone: the query engine's first collect pass over n
 * device rays (the stackless hashed walk of BVH::hashIntersect,
 * src/rt/BVH.h:178-350, nested per object as in Context::intersect,
 * src/rt/RayTracer.cu:295-383), with no clipping.  list_lengths (device,
 * may be NULL) receives each ray's candidate-list length for that pass:
 * patches plus object enter / leave markers, at most 64 (a ray with more is
 * parked where its list filled).  The counters of the call count its node
 * visits and backtracks.  Exists so the traversal can be timed and profiled
 * on its own; hits come from cgs_intersect.  Asynchronous on `stream`. */
int cgs_traverse(cgs_scene* scene, const cgs_rays* rays, uint32_t n, int any_hit, uint32_t* list_lengths,
                 void* stream);

/* spline::doBezierClipping / doSubdivision on explicit (ray, patch) pairs
 * (src/Spline.h:488-508): ray k against patch patch_ids[k] of `surface`.
 * hits->t is hit.distance (in: current best, out: closer hit if found);
 * hits->patch is set to 1 when a closer hit was found, else 0; a patch id at or
 * past the surface's patch count is a miss and sets device_errors bit 16.
 * Device pointers. */
int cgs_patch_intersect(cgs_scene* scene, uint32_t surface, const cgs_rays* rays,
                        const uint32_t* patch_ids, uint32_t n, int method, float tol,
                        const cgs_hits* hits, void* stream);

/* rt::normal(const BezierSurface&, const rt::Intersection&) (src/rt/Primitive.cu:270-275):
 * the unit normal of patch patch_ids[k] of `surface` at (u[k], v[k]), in the
 * surface's own space (mat::normal normalized, src/SplineMat.h:178-187).
 * normals receives 3 n floats as nx | ny | nz.  A patch id at or past the
 * surface's patch count gives (0, 0, 0) and device_errors bit 16.  Device
 * pointers; asynchronous on `stream`. */
int cgs_patch_normal(cgs_scene* scene, uint32_t surface, const uint32_t* patch_ids, const float* u, const float* v,
                     uint32_t n, float* normals, void* stream);

/* ------------------------------------------------------------- render -- */
/* RayTracer::render (src/rt/RayTracer.cu:107-180): width x height pixels,
 * one primary ray each, PBR shading with shadow rays and
 * options->recursion_depth mirror bounces.  framebuffer: device RGBA8 sRGB,
 * row stride `stride` pixels (>= width).  linear_rgb: optional device float
 * (height, width, 3) clamped to [0,1].  Asynchronous; returns CGS_ERR_BUSY if
 * the scene's previous render has not finished. */
int cgs_render(cgs_scene* scene, const cgs_camera* camera, uint32_t width, uint32_t height,
               const cgs_render_options* options, uint32_t* framebuffer, uint32_t stride,
               float* linear_rgb, void* stream);

/* Same with host framebuffer / linear_rgb (either may be NULL); synchronises. */
int cgs_render_host(cgs_scene* scene, const cgs_camera* camera, uint32_t width, uint32_t height,
                    const cgs_render_options* options, uint32_t* framebuffer, float* linear_rgb,
                    void* stream);

/* A render request of a batch: `spp` jittered primary samples per pixel,
 * averaged (sample s offset by (s/spp, vdc(s)) as src/rt/RayTracer.cu:226-236;
 * spp = 1 is the unjittered pixel centre of the reference's default path). */
typedef struct cgs_render_request {
    uint32_t group;
    cgs_camera camera;
    uint32_t width, height, spp;
    int recursion_depth;
    uint32_t* framebuffer;   /* device RGBA8 sRGB, row stride = width (nullable) */
    float* linear_rgb;       /* device (height, width, 3) (nullable) */
} cgs_render_request;

/* Render n requests of any groups together.  options supplies eps, method,
 * precision, tol and schedule; a request's negative recursion_depth takes
 * options->recursion_depth.
 * With CGS_SCHED_WAVEFRONT all samples of all requests share one wavefront;
 * with CGS_SCHED_PLAIN each request is its own launch (the plain
 * one-request-per-launch path).  Asynchronous; CGS_ERR_BUSY while the
 * scene's previous render is in flight. */
int cgs_render_batch(cgs_scene* scene, const cgs_render_request* requests, uint32_t n,
                     const cgs_render_options* options, void* stream);

/* The primary rays of RayTracer::render (src/rt/RayTracer.cu:59-71,152-163):
 * one ray per pixel centre of a width x height image, written to the device
 * array rays as SoA (7, width*height) = ox oy oz dx dy dz tmax (= +inf).
 * Asynchronous on `stream`. */
int cgs_camera_rays(const cgs_camera* camera, uint32_t width, uint32_t height, int flip_y, float* rays,
                    void* stream);

/* -------------------------------------------------- engine settings -- */
/* Runtime settings of the query engine (no counterpart in the reference):
 * collect / resolve passes before the inline fallback (1..8), block sizes
 * (collect 128 or 256, resolve 64 or 128) and resident blocks per SM
 * (0 = as many as fit, else at most 32).  Process-wide. */
typedef struct cgs_engine_config {
    int passes;
    int collect_threads;
    int resolve_threads;
    int collect_occupancy;
    int resolve_occupancy;
    /* 1 (default): the traversal kernel keeps the node indices of the last 8
     * postponed siblings of each ray in a ring in shared memory and answers a
     * backtrack from it when the entry is still there; 0: every backtrack
     * goes through the perfect hash, as in BVH::hashIntersect.  Both visit
     * the same nodes in the same order and give the same hits. */
    int backtrack_cache;
    /* 1: the traversal kernel reads a 32-byte compressed copy of each BVH
     * node (child boxes on an 8-bit grid of the node's box, widened outward
     * so that they contain the exact boxes); 0 (default): the exact 64-byte
     * records.  The compressed boxes are met wherever the exact ones are, so
     * both settings give the same hits; the exported BVH is the exact one.
     * The autotuner tries both. */
    int compressed_nodes;
    /* Candidate-list entries a ray may fill in the first collect pass before
     * it parks (4..64, a multiple of 4; default 64); each later pass doubles
     * it, up to 64.  A small first chunk parks a ray after its nearest few
     * candidates, so that the next pass walks the rest of the tree culled by
     * the hit the clip found among them. */
    int queue_chunk;
    /* Packet refill (1..32; default 8): the traversal kernel gives a warp's
     * idle lanes new rays only once at least this many are idle, or none of
     * its lanes is busy, so that rays enter a warp in packets of adjacent
     * pixels; 1 refills every idle lane at once. */
    int packet_width;
    /* Order of a render's primary rays in the ray queue (0: scanline; 1, the
     * default: 8 x 4 pixel tiles, so that a warp's rays are neighbours in both
     * directions).  Every ray keeps its sample index, so frames are the
     * same under both. */
    int ray_order;
    /* Any-hit queries (shadow rays): 1 searches a ray's candidates whose leaf
     * box holds its origin after the others (0 default: in traversal order).
     * A shadow ray starts on the surface it leaves, and the search of that
     * patch converges on the root just behind the origin before rejecting
     * it; an occluder found first ends the ray without it.  The order does
     * not change an any-hit answer. */
    int origin_last;
    /* Subdivision searches (CGS_METHOD_SUBDIV): bisection levels a lane
     * runs before the clip kernel's next round (1..64; default 4).  The
     * search is resumable, so a lane that ends its search takes the next
     * candidate or ray while its warp's other lanes go on; the levels only
     * set how often the warp meets to refill.  Hits do not change. */
    int subdiv_levels;
} cgs_engine_config;
int cgs_engine_config_get(cgs_engine_config* config);
int cgs_engine_config_set(const cgs_engine_config* config);

/* The autotuner: renders the batch (wavefront schedule) and times `repeats`
 * renders of it with CUDA events per candidate setting, keeping the fastest
 * (median) as the process-wide setting.  The search is a coordinate descent
 * from the current setting, two rounds over the knobs in turn (passes 1, 2,
 * 4, 8; collect 128, 256 and resolve 64, 128 threads; traversal blocks per SM
 * as many as fit or 768 threads' worth; exact or compressed nodes; queue
 * chunk 8, 16, 32, 64; packet width 1, 8, 16; scanline or tiled ray order;
 * any-hit candidates in traversal order or origin boxes last; for a
 * subdivision batch, 1, 4, 16 or 64 subdivision levels per round),
 * then passes 2, 4, 8 x first chunk 8, 16, 32, 64 as pairs, each knob set to its fastest
 * value with the others held; a setting already timed is not timed again.
 * Synchronises `stream`. */
int cgs_autotune_render(cgs_scene* scene, const cgs_render_request* requests, uint32_t n,
                        const cgs_render_options* options, int repeats, cgs_engine_config* best,
                        double* best_ms, void* stream);

/* RayTracer::running (src/rt/RayTracer.h:45-48): 1 while a render is in flight. */
int cgs_render_running(cgs_scene* scene);

/* Counters of the scene's last query or render (synchronises the stream it ran on). */
int cgs_scene_counters(cgs_scene* scene, cgs_counters* out);

/* Failure injection on the host, for tests of the out-of-memory paths: the
 * nth growth of a working buffer from now on (scratch, staging and slot
 * buffers of queries, renders and servers; 1 = the next) frees the old
 * buffer and reports CGS_ERR_OUT_OF_MEMORY without calling the allocator.
 * 0 cancels.  No device work is involved; the calls that fail return the
 * status, and the next call grows its buffers again. */
int cgs_debug_fail_allocation(uint32_t nth);

/* ------------------------------------------------------ perfect hash -- */
/* PerfectHashFunction::build on n device keys (src/rt/PerfectHashFunction.cu:229-503).
 * Outputs (device): disp[displ_capacity], table[table_capacity] with
 * table[h(keys[i])] = i; params (host) = A, B, N, mask, trials.
 * displacement size = bit_floor(max(2, (n-1)>>1)); table_capacity must be at
 * least n + 15*max(4, 0.05n).  Up to 131,072 keys one thread block builds the
 * table in one launch (its scratch in shared memory up to 8,192 keys);
 * larger inputs run the multi-launch build (two launches per round).  All
 * give the same tables.  Synchronises `stream`. */
int cgs_perfect_hash_build(const uint32_t* keys, uint32_t n, uint32_t* disp, uint32_t displ_capacity,
                           uint32_t* table, uint32_t table_capacity, uint32_t params[5], void* stream);

/* cgs_perfect_hash_build without any device allocation.  This entry point
 * has no counterpart in the reference.  It exists for callers that cannot
 * allocate device memory when they need a table: code inside an allocator
 * callback (allocating there would re-enter the allocator) or a service that
 * reserves its device memory at start-up and must not grow the device heap
 * afterwards.  Its working memory is a fixed array inside the library (about
 * 6.9 MB, held on every GPU that loads the library until the process exits),
 * so n is limited to CGS_NOALLOC_MAX_KEYS; larger inputs return
 * CGS_ERR_CAPACITY.  The caller still provides keys, disp and table (device)
 * and params (host), exactly as for cgs_perfect_hash_build, and gets the same
 * results and status codes.  Each call looks the array's device address up
 * for the current device.  All calls on a device share the array: each call
 * clears the parts that must start from zero, but calls that overlap on the
 * GPU race and must be serialised by the caller.  Synchronises `stream`. */
#define CGS_NOALLOC_MAX_KEYS 262144u
int cgs_perfect_hash_build_noalloc(const uint32_t* keys, uint32_t n, uint32_t* disp, uint32_t displ_capacity,
                                   uint32_t* table, uint32_t table_capacity, uint32_t params[5], void* stream);

/* ------------------------------------------------------------ serving -- */
/* A request server over a built scene store.  Render and ray-query requests
 * of any groups are queued on submit, cut into chunks (row ranges of an image,
 * ranges of a ray array) that fit one slot's share of the device-memory
 * budget, and packed into batches that run on `slots` concurrent streams.  A
 * batch starts as soon as a slot is free, so requests that arrive while
 * others run are admitted and overlap with them on the device (continuous
 * batching).  Every sample and ray is computed exactly as by cgs_render_batch
 * and cgs_intersect, so a request's result does not depend on what it was
 * batched with.  The reference has no counterpart: its RayTracer renders one
 * frame at a time on a worker thread (src/rt/RayTracer.cu:107-180); with
 * schedule CGS_SCHED_PLAIN the server behaves that way (one slot, one request
 * per launch, the plain kernel, no chunking), which is the per-request
 * baseline.  The scene store must not change while a server uses it. */
typedef struct cgs_server cgs_server;

typedef struct cgs_server_options {
    uint32_t slots;              /* concurrent batches (streams), 1..16 */
    uint64_t memory_budget;      /* device bytes for all slots' working buffers
                                    (the resident scenes are not counted) */
    uint32_t max_batch_samples;  /* primary samples or query rays per batch; 0 = what a slot's share holds */
    uint32_t max_batch_requests; /* chunks per batch; 0 = 256 */
    cgs_render_options render;   /* eps, flip_y, method, precision, tol, schedule for every request */
} cgs_server_options;

/* A ray query: closest or any hit of n rays (device SoA) in one group. */
typedef struct cgs_query_request {
    uint32_t group;
    uint32_t n;
    int any_hit;
    cgs_rays rays;   /* device; rays.group is ignored (the request's group applies) */
    cgs_hits hits;   /* device; any_hit writes only hits.patch (0 occluded, -1 free) */
} cgs_query_request;

typedef struct cgs_request_info {
    int status;          /* CGS_OK, or the error that ended the request */
    uint32_t chunks;     /* chunks the request was cut into */
    double submit_s;     /* server clock at submit, first launch and completion */
    double start_s;
    double finish_s;
    uint64_t samples;    /* primary samples (renders) or rays (queries) */
} cgs_request_info;

typedef struct cgs_server_stats {
    uint64_t submitted, finished, rejected;
    uint64_t batches, chunks;
    uint64_t rays_traced;        /* every ray the device traced (primary, bounce, shadow, query) */
    uint64_t slot_bytes;         /* device bytes held by the slots now */
    uint64_t peak_slot_bytes;
    uint64_t kernel_launches;
    double busy_s;               /* time with at least one batch in flight */
    uint32_t max_batch_samples;  /* the per-batch limit in force */
    uint32_t queued;             /* chunks waiting */
} cgs_server_stats;

int cgs_server_create(cgs_server** server, cgs_scene* scene, const cgs_server_options* options);
/* Finishes every submitted request, then frees the server.  No other thread
 * may be inside, or call, a cgs_server_* function of this server meanwhile or
 * afterwards. */
int cgs_server_destroy(cgs_server* server);
/* Queue a request; *ticket identifies it.  CGS_ERR_ADMISSION when one row
 * (render) or one ray (query) cannot fit a slot's memory share, or when the
 * request needs more lights than the slots were sized for. */
int cgs_server_submit_render(cgs_server* server, const cgs_render_request* request, uint64_t* ticket);
int cgs_server_submit_query(cgs_server* server, const cgs_query_request* request, uint64_t* ticket);
/* Wait up to timeout_s seconds (< 0: without limit) for a request.  CGS_OK
 * with its info once it has finished (the ticket is then released),
 * CGS_ERR_BUSY on timeout, CGS_ERR_NOT_FOUND for an unknown ticket.  The
 * server keeps a finished request's info until its ticket is waited on. */
int cgs_server_wait(cgs_server* server, uint64_t ticket, double timeout_s, cgs_request_info* info);
/* Seconds since the server was created (the clock of cgs_request_info). */
double cgs_server_clock(const cgs_server* server);
int cgs_server_stats_get(cgs_server* server, cgs_server_stats* stats);

#ifdef __cplusplus
}
#endif

#endif /* CGSPLINE_GB300_H */
