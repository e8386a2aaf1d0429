// device.cuh -- device-side data layout and routines of the ray--bicubic-patch
// path: hashed stackless BVH traversal, Bezier clipping / subdivision on the
// projected control net, FP64 Newton polish, PBR shading.
//
// Reference citations are relative to the MachSilva/cgspline project root.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace cgs {

constexpr uint32_t EMPTY = 0xFFFFFFFFu;
constexpr int kClipStack = 32;          // reference stack depth, src/Spline_BezierClipping.cu:577
constexpr int kMaxClipIterations = 4096;
constexpr int kMaxTraversalSteps = 1 << 20;
constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.318309886183790671538f;

// Error bits reported through Counters::errors.
enum : uint32_t { kErrClipStack = 1u, kErrClipIterations = 2u, kErrTraversal = 4u, kErrGroup = 8u, kErrPatchId = 16u };

// ------------------------------------------------------------ data layout --
// One BVH (a surface's patch BVH or the object-level BVH).  Node offsets in
// the nodes / indices are relative to nodeBase / indexBase, as the
// reference's Node::left/right/first are relative to its own arrays
// (src/rt/BVH.h:23-39).
struct DevBVH
{
    uint32_t nodeBase, indexBase, tableBase, dispBase;
    uint32_t A, B, N, mask;  // h(k) = (A k + B + disp[k & mask]) mod N, src/rt/PerfectHashFunction.h:58-63
    unsigned long long Nmagic;  // ceil(2^64 / N): x mod N by multiplication (fastmod_u32)
    uint32_t compressed;        // 1: every node has a record in the compressed mirror
};

// x mod N for 32-bit x and N >= 1 with M = ceil(2^64 / N) (Lemire, Kaser,
// Kurz, "Faster remainder by direct computation", 2019): the low 64 bits of
// M*x, times N, keep the remainder in their high 64 bits.
__host__ __device__ __forceinline__ unsigned long long fastmod_magic(uint32_t N)
{
    return ~0ull / N + 1ull;
}
__device__ __forceinline__ uint32_t fastmod(uint32_t x, uint32_t N, unsigned long long M)
{
    unsigned long long low = M * x;
    return uint32_t(__umul64hi(low, N));
}

struct DevObject  // one row of Scene::ObjectArrays, src/rt/Scene.h:109-112
{
    float w2l[16];            // column-major world -> local
    uint32_t surface;
    uint32_t material;        // index into materials
    int32_t patchMaterialBase;  // >= 0: per-patch material indices start here
    uint32_t pad;
};

struct DevMaterial { float diffuse[3]; float specular[3]; float metalness; float roughness; };
struct DevLight { float color[3]; float strength; float position[3]; float range; float direction[3]; float angle; };

// Scene in HBM.  Nodes are 64 B (4 x float4):
//   q0 = leftBox.lo.xyz, leftBox.hi.x   q1 = leftBox.hi.yz, rightBox.lo.xy
//   q2 = rightBox.lo.z, rightBox.hi.xyz q3 = left, right|first (uint bits), 0, 0
// Patches are de-indexed: 16 float4 (256 B) per patch, point (i,j) at 4j+i.
struct DevScene
{
    const float4* patches;
    const float4* nodes;
    const uint4* qnodes;       // 32-byte compressed mirror of nodes (two uint4 per node)
    const uint32_t* indices;
    const uint32_t* tables;
    const uint32_t* disps;
    const DevBVH* bvhs;        // [nsurfaces] patch BVHs, then the object-level BVH
    const uint32_t* patchBase; // first global patch of each surface
    const DevObject* objects;
    const DevMaterial* materials;
    const uint32_t* patchMaterial;
    const DevLight* lights;
    // Groups: independent scenes that share the store.  Group g has its own
    // object-level BVH bvhs[groupTop[g]], lights lights[groupLights[g].x ..
    // + groupLights[g].y) and background / ambient colours groupEnv[6g..6g+5].
    const uint32_t* groupTop;
    const uint2* groupLights;
    const float* groupEnv;
    uint32_t nobjects, nsurfaces, ngroups;
};

__device__ __forceinline__ float3 group_background(const DevScene& S, uint32_t g)
{
    const float* e = S.groupEnv + 6ull * g;
    return make_float3(__ldg(e), __ldg(e + 1), __ldg(e + 2));
}
__device__ __forceinline__ float3 group_ambient(const DevScene& S, uint32_t g)
{
    const float* e = S.groupEnv + 6ull * g;
    return make_float3(__ldg(e + 3), __ldg(e + 4), __ldg(e + 5));
}

struct Counters
{
    unsigned long long nodes, hashLookups, candidates, iterations, rays, errors, tableReads;
};

struct LocalCounters
{
    uint32_t nodes = 0, hashLookups = 0, candidates = 0, iterations = 0;
    uint32_t errors = 0, tableReads = 0;
};

// One 32-byte load through the read-only path (a 256-bit vector load, sm_100
// and later): p must be 32-byte aligned and the data unchanged while the
// kernel runs.  A warp's divergent lanes then touch each 32-byte sector of a
// BVH node with one request instead of two.
__device__ __forceinline__ void ldg256(const float4* p, float4& a, float4& b)
{
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}

__device__ __forceinline__ void ldg256u(const uint4* p, uint4& a, uint4& b)
{
    asm("ld.global.nc.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=r"(a.x), "=r"(a.y), "=r"(a.z), "=r"(a.w), "=r"(b.x), "=r"(b.y), "=r"(b.z), "=r"(b.w)
        : "l"(p));
}

// ------------------------------------------------------------ float math --
__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return f3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float len(float3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ float3 cross(float3 a, float3 b)
{
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float3 versor(float3 a)
{
    float l = len(a);
    if (l != 0.0f) { float k = 1.0f / l; a = a * k; }
    return a;
}
__device__ __forceinline__ float vmax3(float3 a) { return fmaxf(fmaxf(a.x, a.y), a.z); }
__device__ __forceinline__ float3 xyz(float4 p) { return f3(p.x, p.y, p.z); }
__device__ __forceinline__ float3 project(float4 p) { return f3(p.x / p.w, p.y / p.w, p.z / p.w); }  // src/AlignedTypes.h:63-66

__device__ __forceinline__ float2 operator+(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 operator-(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 operator*(float2 a, float2 b) { return make_float2(a.x * b.x, a.y * b.y); }
__device__ __forceinline__ float dot2(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }
__device__ __forceinline__ float len2(float2 a) { return sqrtf(dot2(a, a)); }

// Column-major 4x4 times (x,y,z,1) / times (x,y,z,0).
__device__ __forceinline__ float4 m4_point(const float* m, float3 p)
{
    return make_float4(p.x * m[0] + p.y * m[4] + p.z * m[8] + m[12], p.x * m[1] + p.y * m[5] + p.z * m[9] + m[13],
                       p.x * m[2] + p.y * m[6] + p.z * m[10] + m[14], p.x * m[3] + p.y * m[7] + p.z * m[11] + m[15]);
}
__device__ __forceinline__ float3 m3_vec(const float* m, float3 v)
{
    return f3(v.x * m[0] + v.y * m[4] + v.z * m[8], v.x * m[1] + v.y * m[5] + v.z * m[9],
              v.x * m[2] + v.y * m[6] + v.z * m[10]);
}
__device__ __forceinline__ float3 m3T_vec(const float* m, float3 v)  // mat3(M)^T * v
{
    return f3(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[4] * v.x + m[5] * v.y + m[6] * v.z,
              m[8] * v.x + m[9] * v.y + m[10] * v.z);
}

// ------------------------------------------------ power-basis evaluation --
// Bernstein weights as CUBIC_BASE * [1 t t^2 t^3] (src/SplineMat.h:22-28,101-105)
__device__ __forceinline__ float4 basis(float t)
{
    float t2 = t * t, t3 = t2 * t;
    return make_float4(1.0f - 3.0f * t + 3.0f * t2 - t3, 3.0f * t - 6.0f * t2 + 3.0f * t3, 3.0f * t2 - 3.0f * t3, t3);
}
// CUBIC_DERIVATIVE_BASE * [1 t t^2 0] (src/SplineMat.h:38-44,107-110)
__device__ __forceinline__ float4 dbasis(float t)
{
    float t2 = t * t;
    return make_float4(-3.0f + 6.0f * t - 3.0f * t2, 3.0f - 12.0f * t + 9.0f * t2, 6.0f * t - 9.0f * t2, 3.0f * t2);
}
__device__ __forceinline__ float4 comb(float4 w, float4 a, float4 b, float4 c, float4 d)
{
    return make_float4(w.x * a.x + w.y * b.x + w.z * c.x + w.w * d.x, w.x * a.y + w.y * b.y + w.z * c.y + w.w * d.y,
                       w.x * a.z + w.y * b.z + w.z * c.z + w.w * d.z, w.x * a.w + w.y * b.w + w.z * c.w + w.w * d.w);
}
// mat::interpolate (src/SplineMat.h:125-140); wu weights along u (i), wv along v (j)
__device__ __forceinline__ float4 tensor_eval(const float4* __restrict__ P, float4 wu, float4 wv)
{
    float4 A0 = comb(wu, __ldg(P + 0), __ldg(P + 1), __ldg(P + 2), __ldg(P + 3));
    float4 A1 = comb(wu, __ldg(P + 4), __ldg(P + 5), __ldg(P + 6), __ldg(P + 7));
    float4 A2 = comb(wu, __ldg(P + 8), __ldg(P + 9), __ldg(P + 10), __ldg(P + 11));
    float4 A3 = comb(wu, __ldg(P + 12), __ldg(P + 13), __ldg(P + 14), __ldg(P + 15));
    return comb(wv, A0, A1, A2, A3);
}
// mat::normal (src/SplineMat.h:178-187), not normalized
__device__ __forceinline__ float3 patch_normal(const float4* __restrict__ P, float u, float v)
{
    float4 dU = tensor_eval(P, dbasis(u), basis(v));
    float4 dV = tensor_eval(P, basis(u), dbasis(v));
    return cross(xyz(dU), xyz(dV));
}

// ------------------------------------------------------------- slicing --
// mat::slice_matrix (src/SplineMat.h:64-82) applied as mat::slice
// (src/SplineMat.h:189-206): P_j <- sum_k M[j][k] P_k, M's columns below.
struct SliceM { float m[4][4]; };
__device__ __forceinline__ SliceM slice_matrix(float a, float b)
{
    const float a2 = a * a, b2 = b * b, ia = 1.0f - a, ib = 1.0f - b, ia2 = ia * ia, ib2 = ib * ib,
                k1 = a + 2.0f * b - 3.0f * a * b, k2 = 2.0f * a + b - 3.0f * a * b;
    SliceM M;
    M.m[0][0] = ia2 * ia; M.m[0][1] = 3.0f * a * ia2; M.m[0][2] = 3.0f * a2 * ia; M.m[0][3] = a2 * a;
    M.m[1][0] = ia2 * ib; M.m[1][1] = ia * k2; M.m[1][2] = a * k1; M.m[1][3] = a2 * b;
    M.m[2][0] = ia * ib2; M.m[2][1] = ib * k1; M.m[2][2] = b * k2; M.m[2][3] = a * b2;
    M.m[3][0] = ib2 * ib; M.m[3][1] = 3.0f * b * ib2; M.m[3][2] = 3.0f * b2 * ib; M.m[3][3] = b2 * b;
    return M;
}
template<int stride> __device__ __forceinline__ void apply_slice(float2* c, const SliceM& M)
{
    float2 p0 = c[0], p1 = c[stride], p2 = c[2 * stride], p3 = c[3 * stride];
#pragma unroll
    for (int j = 0; j < 4; j++)
    {
        float2 r;
        r.x = M.m[j][0] * p0.x + M.m[j][1] * p1.x + M.m[j][2] * p2.x + M.m[j][3] * p3.x;
        r.y = M.m[j][0] * p0.y + M.m[j][1] * p1.y + M.m[j][2] * p2.y + M.m[j][3] * p3.y;
        c[j * stride] = r;
    }
}
// mat::subpatchU / subpatchV (src/SplineMat.h:221-233)
__device__ __forceinline__ void subpatchU(float2* p, float a, float b)
{
    SliceM M = slice_matrix(a, b);
#pragma unroll
    for (int i = 0; i < 4; i++) apply_slice<1>(p + 4 * i, M);
}
__device__ __forceinline__ void subpatchV(float2* p, float a, float b)
{
    SliceM M = slice_matrix(a, b);
#pragma unroll
    for (int i = 0; i < 4; i++) apply_slice<4>(p + i, M);
}

// -------------------------------------------------------- clip helpers --
// xAxisIntersection, src/Spline_BezierClipping.cu:127-156
__device__ __forceinline__ bool xAxisIntersection(float& lo, float& hi, float2 A, float2 B)
{
    const float eps = 1.1920928955078125e-07f;  // FLT_EPSILON
    float q = A.y - B.y;
    if (fabsf(q) > eps)
    {
        float t = A.y / q;
        if (0.0f <= t && t <= 1.0f)
        {
            float s = (1.0f - t) * A.x + t * B.x;
            lo = s; hi = s;
            return true;
        }
    }
    else if (fabsf(A.y) <= eps)
    {
        lo = fminf(A.x, B.x); hi = fmaxf(A.x, B.x);
        return true;
    }
    return false;
}

// triangleOriginIntersection, src/Spline.h:709-737
__device__ __forceinline__ bool triangleOriginIntersection(float2& coord, float2 P, float2 A, float2 B)
{
    float2 p = A - P, q = B - P;
    float det = p.x * q.y - q.x * p.y;
    if (fabsf(det) < 0x1p-80f) return false;
    det = 1.0f / det;
    float u = det * (q.y * -P.x + -q.x * -P.y);
    if (u < 0.0f || u > 1.0f) return false;
    float v = det * (-p.y * -P.x + p.x * -P.y);
    if (v < 0.0f || u + v > 1.0f) return false;
    coord = make_float2(u, v);
    return true;
}

// Fat-line clip range of a sub-net (src/Spline_BezierClipping.cu:610-701):
// distance patch against the line through the net's diagonals, column
// extremes, convex-hull scan against the x axis, anti-sliver shrink.
__device__ __forceinline__ void clip_range(const float2* p, int cutside, float& lower, float& upper)
{
    lower = 1.0f; upper = 0.0f;
    float2 L = p[15] - p[0];
    float2 D = p[12] - p[3];
    L = cutside == 0 ? L + D : L - D;
    {
        float l = len2(L);
        if (l != 0.0f) { float k = 1.0f / l; L = make_float2(L.x * k, L.y * k); }
    }
    const float2 N = make_float2(-L.y, L.x);
    float ytop[4], ybot[4];
#pragma unroll
    for (int i = 0; i < 4; i++)
    {
        float y0, y1, y2, y3;
        if (cutside == 0)
        { y0 = dot2(N, p[i]); y1 = dot2(N, p[4 + i]); y2 = dot2(N, p[8 + i]); y3 = dot2(N, p[12 + i]); }
        else
        { y0 = dot2(N, p[4 * i]); y1 = dot2(N, p[4 * i + 1]); y2 = dot2(N, p[4 * i + 2]); y3 = dot2(N, p[4 * i + 3]); }
        ybot[i] = fminf(fminf(y0, y1), fminf(y2, y3));
        ytop[i] = fmaxf(fmaxf(y0, y1), fmaxf(y2, y3));
    }
    const float o1 = 1.0f / 3.0f, o2 = 2.0f / 3.0f;
    const float2 hull[7] = {make_float2(o2, ybot[2]), make_float2(1.0f, ybot[3]), make_float2(1.0f, ytop[3]),
                            make_float2(o2, ytop[2]), make_float2(o1, ytop[1]), make_float2(0.0f, ytop[0]),
                            make_float2(0.0f, ybot[0])};
    float2 P1 = make_float2(0.0f, ybot[0]), P2 = make_float2(o1, ybot[1]);
#pragma unroll
    for (int k = 0; k < 7; k++)
    {
        float2 P3 = hull[k];
        float2 a = P2 - P1, b = P3 - P1;
        if (a.x * b.y - a.y * b.x >= 0.0f)
        {
            float lo, hi;
            if (xAxisIntersection(lo, hi, P1, P2)) { lower = fminf(lower, lo); upper = fmaxf(upper, hi); }
            P1 = P2;
        }
        P2 = P3;
    }
    {
        float lo, hi;
        if (xAxisIntersection(lo, hi, P1, P2)) { lower = fminf(lower, lo); upper = fmaxf(upper, hi); }
    }
    lower = lower * 0x0FFp-8f;
    upper = upper + (1.0f - upper) * 0x001p-8f;
}

// onHit of doBezierClipping (src/Spline_BezierClipping.cu:94-112): keep the
// surface point closest to the origin and in front of it.
struct HitSink
{
    const float4* P;
    float3 o, d;
    float dist;
    float2 uv;
    __device__ __forceinline__ bool operator()(float2 e)
    {
        float3 V = project(tensor_eval(P, basis(e.x), basis(e.y))) - o;
        float t = len(V);
        if (t < dist && dot(V, d) > 0.0f) { dist = t; uv = e; return true; }
        return false;
    }
};

// approximateIntersection, src/Spline.h:739-765, on the net's corner points
// p0 = p[0], p3 = p[3], p12 = p[12], p15 = p[15]
__device__ __forceinline__ bool approximateIntersection(HitSink& sink, float2 p0, float2 p3, float2 p12, float2 p15,
                                                        float2 pmin, float2 pmax)
{
    bool found = false;
    float2 coord, psize = pmax - pmin;
    if (triangleOriginIntersection(coord, p0, p3, p12)) found |= sink(pmin + coord * psize);
    if (triangleOriginIntersection(coord, p15, p12, p3)) found |= sink(pmax - coord * psize);
    return found;
}
__device__ __forceinline__ bool approximateIntersection(HitSink& sink, const float2* p, float2 pmin, float2 pmax)
{
    return approximateIntersection(sink, p[0], p[3], p[12], p[15], pmin, pmax);
}

// Project the 16 control points onto two planes containing the ray
// (src/Spline_BezierClipping.cu:53-83).
__device__ __forceinline__ void project_net(float2* net, const float4* __restrict__ P, float3 o, float3 d)
{
    const float3 a0 = versor(cross(d, d + f3(0.0f, 0.0f, 8.0f)));
    const float3 a1 = versor(cross(d, a0));
#pragma unroll
    for (int i = 0; i < 16; i++)
    {
        float3 Q = xyz(__ldg(P + i)) - o;
        net[i] = make_float2(dot(a0, Q), dot(a1, Q));
    }
}

// ------------------------------------- FP64 fat-line bounds (grazing) --
// The precision form searches near-grazing candidates (the ray within 30
// degrees of the plane of the patch's diagonals) on a net projected in FP64
// (rounded to FP32), with the fat-line bounds of every FP32 sub-net computed
// in FP64 (distances, hull scan, DBL_EPSILON) and rounded outward, to the
// tolerance 2^-20: FP32 sub-nets near the ray are small, so FP32 holds them,
// while the FP32 bounds and the 2^-12 tolerance lose near-tangent roots.
constexpr float kGrazeTol = 0x1p-20f;
// A near-grazing search stops after this many iterations and keeps what it
// found (the 2^-20 tolerance can be out of FP32 reach far from the ray).
constexpr int kGrazeIterations = 1024;

// Precision levels (enum cgs_precision) of closest-hit searches: 0 FP32;
// 1 FP32 + FP64 polish; 2 pure FP64; 3 as 1, with the FP64 bounds for
// candidates within 30 degrees of grazing.  Internal level 5: the search of
// 3 without the polish (closest-hit passes whose polish runs separately).
// Any-hit searches run at level 0.
__host__ __device__ __forceinline__ bool polishes(int precision) { return precision == 1 || precision == 3; }
__host__ __device__ __forceinline__ float graze_sin(int precision)
{
    return (precision == 3 || precision == 5) ? 0.5f : 0.0f;  // sin 30 degrees
}
__host__ __device__ __forceinline__ int search_only(int precision)
{
    return precision == 3 ? 5 : precision == 5 ? 5 : 0;
}

__device__ __forceinline__ double2 operator+(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 operator-(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 operator*(double2 a, double2 b) { return make_double2(a.x * b.x, a.y * b.y); }
__device__ __forceinline__ double len2d(double2 a) { return sqrt(a.x * a.x + a.y * a.y); }

// xAxisIntersection in double with DBL_EPSILON (src/Spline_BezierClipping.cu:127-156)
__device__ __forceinline__ bool x_axis_d(double& lo, double& hi, double2 A, double2 B)
{
    const double eps = 2.220446049250313e-16;
    const double q = A.y - B.y;
    if (fabs(q) > eps)
    {
        const double t = A.y / q;
        if (0.0 <= t && t <= 1.0) { lo = hi = (1.0 - t) * A.x + t * B.x; return true; }
    }
    else if (fabs(A.y) <= eps)
    {
        lo = fmin(A.x, B.x); hi = fmax(A.x, B.x);
        return true;
    }
    return false;
}

// clip_range in double (src/Spline_BezierClipping.cu:610-701)
__device__ __forceinline__ void clip_range_d(const double2* p, int cutside, double& lower, double& upper)
{
    lower = 1.0; upper = 0.0;
    double2 L = p[15] - p[0];
    const double2 D = p[12] - p[3];
    L = cutside == 0 ? L + D : L - D;
    {
        const double l = len2d(L);
        if (l != 0.0) L = make_double2(L.x / l, L.y / l);
    }
    const double2 N = make_double2(-L.y, L.x);
    double ytop[4], ybot[4];
#pragma unroll
    for (int i = 0; i < 4; i++)
    {
        double y[4];
#pragma unroll
        for (int k = 0; k < 4; k++)
        {
            const double2 q = cutside == 0 ? p[4 * k + i] : p[4 * i + k];
            y[k] = N.x * q.x + N.y * q.y;
        }
        ybot[i] = fmin(fmin(y[0], y[1]), fmin(y[2], y[3]));
        ytop[i] = fmax(fmax(y[0], y[1]), fmax(y[2], y[3]));
    }
    const double o1 = 1.0 / 3.0, o2 = 2.0 / 3.0;
    const double2 hull[7] = {make_double2(o2, ybot[2]), make_double2(1.0, ybot[3]), make_double2(1.0, ytop[3]),
                             make_double2(o2, ytop[2]), make_double2(o1, ytop[1]), make_double2(0.0, ytop[0]),
                             make_double2(0.0, ybot[0])};
    double2 P1 = make_double2(0.0, ybot[0]), P2 = make_double2(o1, ybot[1]);
#pragma unroll
    for (int k = 0; k < 7; k++)
    {
        const double2 P3 = hull[k];
        const double2 a = P2 - P1, b = P3 - P1;
        if (a.x * b.y - a.y * b.x >= 0.0)
        {
            double lo, hi;
            if (x_axis_d(lo, hi, P1, P2)) { lower = fmin(lower, lo); upper = fmax(upper, hi); }
            P1 = P2;
        }
        P2 = P3;
    }
    double lo, hi;
    if (x_axis_d(lo, hi, P1, P2)) { lower = fmin(lower, lo); upper = fmax(upper, hi); }
    lower = lower * 0x0FFp-8;
    upper = upper + (1.0 - upper) * 0x001p-8;
}

// FP64 bounds of an FP32 sub-net, rounded outward.
__device__ __forceinline__ void clip_range64(const float2* p, int cutside, float& lower, float& upper)
{
    double2 q[16];
#pragma unroll
    for (int i = 0; i < 16; i++) q[i] = make_double2(p[i].x, p[i].y);
    double lo, hi;
    clip_range_d(q, cutside, lo, hi);
    lower = __double2float_rd(lo);
    upper = __double2float_ru(hi);
}

__device__ __forceinline__ double dot_d(double3 a, double3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ double3 cross_d(double3 a, double3 b)
{
    return make_double3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double3 unit3d(double3 a)
{
    const double l = sqrt(dot_d(a, a));
    return l != 0.0 ? make_double3(a.x / l, a.y / l, a.z / l) : a;
}

// project_net with the axes and dot products in double, rounded to float, on
// a ray given in double.
__device__ __forceinline__ void project_net64(float2* net, const float4* __restrict__ P, double3 o, double3 dd)
{
    const double3 a0 = unit3d(cross_d(dd, make_double3(dd.x, dd.y, dd.z + 8.0)));
    const double3 a1 = unit3d(cross_d(dd, a0));
#pragma unroll
    for (int i = 0; i < 16; i++)
    {
        const float4 q = __ldg(P + i);
        const double3 Q = make_double3(double(q.x) - o.x, double(q.y) - o.y, double(q.z) - o.z);
        net[i] = make_float2(float(dot_d(a0, Q)), float(dot_d(a1, Q)));
    }
}

// A ray in an object's space computed in double from the FP32 world ray: the
// origin through the world-to-object matrix, the direction through its 3x3
// part, normalised.  The FP32 object-space ray rounds each of these, and on a
// near-grazing ray that one-ulp turn of the direction moves the line across a
// tangent root; the precision form projects near-grazing candidates from
// this ray instead.
struct Ray64 { double3 o, d; };
__device__ __forceinline__ Ray64 to_local64(const DevObject& ob, float3 o, float3 d)
{
    const float* m = ob.w2l;
    const double ox = o.x, oy = o.y, oz = o.z, dx = d.x, dy = d.y, dz = d.z;
    Ray64 r;
    r.o = make_double3(ox * m[0] + oy * m[4] + oz * m[8] + m[12], ox * m[1] + oy * m[5] + oz * m[9] + m[13],
                       ox * m[2] + oy * m[6] + oz * m[10] + m[14]);
    if (!(m[3] == 0.0f && m[7] == 0.0f && m[11] == 0.0f && m[15] == 1.0f))
    {
        const double lw = ox * m[3] + oy * m[7] + oz * m[11] + m[15];
        r.o = make_double3(r.o.x / lw, r.o.y / lw, r.o.z / lw);
    }
    const double3 ld = make_double3(dx * m[0] + dy * m[4] + dz * m[8], dx * m[1] + dy * m[5] + dz * m[9],
                                    dx * m[2] + dy * m[6] + dz * m[10]);
    const double il = 1.0 / sqrt(ld.x * ld.x + ld.y * ld.y + ld.z * ld.z);
    r.d = make_double3(ld.x * il, ld.y * il, ld.z * il);
    return r;
}

// The precision form's near-grazing test of a candidate: the ray within
// asin(sinmax) of the plane of the patch's diagonals or of any of the nine
// cells of its control net (a cell's normal: the cross product of its edges
// along u and v at its first corner), or those ten normals on both sides of
// the ray (the patch folds over the ray's direction: a silhouette).  The
// cells' normals bound the patch's, interior control points included, so a
// bumpy patch tangent to the ray somewhere inside is caught even where its
// diagonals and corners are not.
__device__ __forceinline__ bool near_grazing(const float4* __restrict__ P, float3 d, float sinmax)
{
    bool pos = false, neg = false, near = false;
    auto test = [&](float3 n) {
        const float l = len(n);
        if (!(l > 0.0f)) return;
        const float c = dot(n, d);
        if (fabsf(c) < sinmax * l) near = true;
        if (c > 0.0f) pos = true;
        else neg = true;
    };
    test(cross(xyz(__ldg(P + 15)) - xyz(__ldg(P)), xyz(__ldg(P + 12)) - xyz(__ldg(P + 3))));
#pragma unroll
    for (int j = 0; j < 3; j++)
    {
#pragma unroll
        for (int i = 0; i < 3; i++)
        {
            const float3 p = xyz(__ldg(P + 4 * j + i));
            test(cross(xyz(__ldg(P + 4 * j + i + 1)) - p, xyz(__ldg(P + 4 * (j + 1) + i)) - p));
        }
    }
    return near || (pos && neg);
}

// doBezierClipping2D_device (src/Spline_BezierClipping.cu:547-828) with the
// half-precision (mid,len) stack replaced by a full-precision (min,max)
// stack of the same depth.  Popped sub-nets are re-derived from the
// original net (patchCopy, src/SplineMat.h:248-257), which is re-projected
// from the patch so that it need not stay in registers.  Stack overflow and
// the iteration cap end the search with an error bit instead of __trap().
//
// The search is resumable: clip_begin sets up the state, each clip_step runs
// one iteration of the reference loop and returns false when the search is
// over, so a persistent kernel can interleave candidates lane by lane.
struct ClipState
{
    float2 buf[16];
    float2 emin, emax;
    int cutsideStack, sl, it;
    float tol;
    bool found, b64;  // b64: FP64 projection and fat-line bounds (near-grazing)
    bool fresh;       // the net is still to be projected (the search's first step)
    bool tposed;      // buf holds the transposed net (left so by a cut along v)
    // The resumable subdivision search (subdiv_step) keeps its walk in the
    // same state: the bit trail in cutsideStack, the level in sl, the
    // sub-domain's integer coordinates in the bits of emin (which it does not
    // use otherwise), and `fresh` as its reload flag.
};

// grazeSin > 0: the precision form (candidates within asin(grazeSin) of
// grazing get the FP64 bounds).  kG64 = false compiles the FP64 path out
// (searches that never take it: a smaller loop body for the instruction
// cache).
// ob, wo, wd: the candidate's object and the world ray, from which a
// near-grazing candidate's ray is recomputed in double (to_local64); a null
// ob projects it from the FP32 ray in the sink.  ray64: where that ray
// (origin, direction) is kept for the search's projections, a six-double
// array in local memory (read only where a projection starts, it would
// otherwise hold twelve registers through the whole search).
template<bool kG64 = true>
__device__ __forceinline__ void clip_begin(ClipState& c, const HitSink& sink, float tol, float grazeSin,
                                           volatile double* ray64, const DevObject* ob = nullptr, float3 wo = {},
                                           float3 wd = {})
{
    c.b64 = kG64 && grazeSin > 0.0f && near_grazing(sink.P, sink.d, grazeSin);
    c.tol = c.b64 ? kGrazeTol : tol;
    if (kG64 && c.b64)
    {
        Ray64 r;
        if (ob) r = to_local64(*ob, wo, wd);
        else r = Ray64 {make_double3(sink.o.x, sink.o.y, sink.o.z), make_double3(sink.d.x, sink.d.y, sink.d.z)};
        ray64[0] = r.o.x; ray64[1] = r.o.y; ray64[2] = r.o.z;
        ray64[3] = r.d.x; ray64[4] = r.d.y; ray64[5] = r.d.z;
    }
    c.fresh = true;  // the first clip_step projects the net
    c.tposed = false;
    c.emin = make_float2(0.0f, 0.0f);
    c.emax = make_float2(1.0f, 1.0f);
    c.cutsideStack = 0;
    c.sl = 0;
    c.it = 0;
    c.found = false;
}

// Transposes the 4x4 net in registers where t holds.  A cut along v
// (subpatchV, fat line of side 1) is a cut along u (subpatchU, side 0) of the
// transposed net, bit for bit, so one code path serves both sides and the
// lanes of a warp do not split on the side they cut.
__device__ __forceinline__ void transpose_if(float2* p, bool t)
{
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = i + 1; j < 4; j++)
        {
            const float2 a = p[4 * i + j], b = p[4 * j + i];
            p[4 * i + j] = t ? b : a;
            p[4 * j + i] = t ? a : b;
        }
}

// One step of the search.  The first step of a search only projects the net
// (clip_begin leaves that to it), at the same place in the code as the
// re-projection after a pop, so lanes starting a search and lanes popping a
// sub-net share those instructions; it is not counted as an iteration.
// A cut along v leaves the net transposed (c.tposed); the next step
// transposes it only if its own cut needs the other orientation, so a step
// moves the net at most once, and the sub-net of a pop is derived in the
// natural orientation.  A loop iteration costs the union of the paths its
// lanes take, so the transposes are kept off the paths that differ.
template<bool kG64 = true>
__device__ __forceinline__ bool clip_step(ClipState& c, float4* st, HitSink& sink, LocalCounters& lc,
                                          const volatile double* ray64)
{
    const bool b64 = kG64 && c.b64;
    const bool fresh = c.fresh;
    bool pop = false, tr = false;
    float a = 0.0f, b = 1.0f;  // the cut, on the (transposed) net's u axis
    if (!fresh)
    {
        if (b64 && c.it >= kGrazeIterations) return false;
        if (c.it++ >= kMaxClipIterations) { lc.errors |= kErrClipIterations; return false; }
        lc.iterations++;
        tr = (c.cutsideStack & 1) != 0;  // this step cuts along v
        pop = true;
        // the corners in the natural orientation (a transpose swaps p3 and p12)
        const float2 p3 = c.tposed ? c.buf[12] : c.buf[3], p12 = c.tposed ? c.buf[3] : c.buf[12];
        if (len2(p3 - p12) < c.tol && len2(c.buf[15] - c.buf[0]) < c.tol)
            c.found |= approximateIntersection(sink, c.buf[0], p3, p12, c.buf[15], c.emin, c.emax);
        else
        {
            transpose_if(c.buf, tr != c.tposed);
            c.tposed = tr;
            float lower, upper;
            if (b64) clip_range64(c.buf, 0, lower, upper);
            else clip_range(c.buf, 0, lower, upper);
            const float delta = upper - lower;
            const float lo = tr ? c.emin.y : c.emin.x, hi = tr ? c.emax.y : c.emax.x;
            if (delta > 0.8f)
            {
                // split in halves: keep the upper half, push the lower
                const float h = 0.5f * (lo + hi);
                const float4 pushed = tr ? make_float4(c.emin.x, c.emin.y, c.emax.x, h)
                                         : make_float4(c.emin.x, c.emin.y, h, c.emax.y);
                if (tr) c.emin.y = h; else c.emin.x = h;
                c.cutsideStack = tr ? ((c.cutsideStack << 1) & ~3) : ((c.cutsideStack << 1) | 3);
                if (c.sl >= kClipStack) { lc.errors |= kErrClipStack; return false; }
                st[c.sl++] = pushed;
                a = 0.5f; b = 1.0f;
                pop = false;
            }
            else if (delta > 0.0f)
            {
                const float sz = hi - lo;
                const float n0 = lo + sz * lower, n1 = hi - sz * (1.0f - upper);
                if (tr) { c.emin.y = n0; c.emax.y = n1; } else { c.emin.x = n0; c.emax.x = n1; }
                c.cutsideStack ^= 1;
                a = lower; b = upper;
                pop = false;
            }
        }
        if (pop)
        {
            c.cutsideStack >>= 1;
            if (--c.sl < 0) return false;
            const float4 e = st[c.sl];
            c.emin = make_float2(e.x, e.y);
            c.emax = make_float2(e.z, e.w);
            a = c.emin.x; b = c.emax.x;
        }
    }
    if (fresh || pop)
    {
        if (b64)
            project_net64(c.buf, sink.P, make_double3(ray64[0], ray64[1], ray64[2]),
                          make_double3(ray64[3], ray64[4], ray64[5]));
        else project_net(c.buf, sink.P, sink.o, sink.d);
        c.tposed = false;
    }
    if (fresh)
    {
        c.fresh = false;
        return true;
    }
    subpatchU(c.buf, a, b);  // every lane: the cut, or the u range of the popped sub-net
    if (pop) subpatchV(c.buf, c.emin.y, c.emax.y);
    return true;
}

// anyHit: stop at the first root found.  An any-hit query only asks whether
// the patch has a root before sink.dist, which the first one answers; the
// reference's search runs on to the closest root and returns the same flag.
static __device__ __noinline__ bool clip_patch(HitSink& sink, float tol, float grazeSin, LocalCounters& lc,
                                               bool anyHit = false, const DevObject* ob = nullptr, float3 wo = {},
                                               float3 wd = {})
{
    float4 st[kClipStack];
    ClipState c;
    volatile double ray64[6];
    clip_begin(c, sink, tol, grazeSin, ray64, ob, wo, wd);
    while (clip_step(c, st, sink, lc, ray64) && !(anyHit && c.found)) {}
    return c.found;
}

// Stackless 2-D subdivision (doSubdivision2D_device,
// src/Spline_Subdivision.cu:16-109): bisect alternately along u and v, lower
// half first, bit trails instead of a stack, re-derive the sub-net after each
// backtrack, accept a leaf whose bounding box strictly contains the origin
// once both diagonals are below tol (or after 31 halvings).  The sub-domain
// follows the buffer: after k halvings su = 2^-ceil(k/2), sv = 2^-floor(k/2).
// subdiv_patch as a resumable search for the query engine: subdiv_begin
// projects the net; each subdiv_step runs up to `levels` iterations of the
// same loop and returns false when the search is over (c.found: a root was
// kept), so lanes of a warp interleave their searches and refill from the
// queue one search at a time.  The iterations are subdiv_patch's, in the same
// order, so the results are the same bit for bit.
__device__ __forceinline__ void subdiv_begin(ClipState& c, const HitSink& sink, float tol)
{
    project_net(c.buf, sink.P, sink.o, sink.d);
    c.cutsideStack = 0; c.sl = 0; c.it = 0;
    c.emin = make_float2(__uint_as_float(0u), __uint_as_float(0u));  // tu, tv
    c.fresh = false; c.found = false; c.tol = tol;
}
__device__ __forceinline__ bool subdiv_step(ClipState& c, HitSink& sink, LocalCounters& lc, int levels)
{
    uint32_t trail = uint32_t(c.cutsideStack), tu = __float_as_uint(c.emin.x), tv = __float_as_uint(c.emin.y);
    int k = c.sl;
    bool more = true;
    for (int s = 0; s < levels; s++)
    {
        if (c.it >= 4 * kMaxClipIterations) { lc.errors |= kErrClipIterations; more = false; break; }
        c.it++;
        lc.iterations++;
        const float su = ldexpf(1.0f, -((k + 1) >> 1)), sv = ldexpf(1.0f, -(k >> 1));
        const float2 emin = make_float2(float(tu) * su, float(tv) * sv);
        const float2 emax = make_float2(emin.x + su, emin.y + sv);
        if (c.fresh)
        {
            project_net(c.buf, sink.P, sink.o, sink.d);
            subpatchU(c.buf, emin.x, emax.x);
            subpatchV(c.buf, emin.y, emax.y);
        }
        float2 bmin = c.buf[0], bmax = c.buf[0];
#pragma unroll
        for (int i = 1; i < 16; i++)
        {
            bmin = make_float2(fminf(bmin.x, c.buf[i].x), fminf(bmin.y, c.buf[i].y));
            bmax = make_float2(fmaxf(bmax.x, c.buf[i].x), fmaxf(bmax.y, c.buf[i].y));
        }
        if (bmin.x < 0.0f && bmin.y < 0.0f && bmax.x > 0.0f && bmax.y > 0.0f)
        {
            if ((len2(c.buf[3] - c.buf[12]) < c.tol && len2(c.buf[15] - c.buf[0]) < c.tol) || k >= 31)
                c.found |= approximateIntersection(sink, c.buf, emin, emax);
            else
            {
                c.fresh = false;
                if ((k & 1) == 0) { subpatchU(c.buf, 0.0f, 0.5f); tu <<= 1; }
                else { subpatchV(c.buf, 0.0f, 0.5f); tv <<= 1; }
                trail <<= 1;
                ++k;
                continue;
            }
        }
        const int ones = __clz(__brev(~trail));
        if (ones >= k) { more = false; break; }
        const int hi = k - 1, lo = k - ones;
        const int evens = (hi / 2) - ((lo + 1) / 2) + 1;
        tu >>= evens;
        tv >>= (ones - evens);
        k -= ones;
        trail = (trail >> ones) | 1u;
        if (((k - 1) & 1) == 0) tu |= 1u; else tv |= 1u;
        c.fresh = true;
    }
    c.cutsideStack = int(trail); c.emin = make_float2(__uint_as_float(tu), __uint_as_float(tv)); c.sl = k;
    return more;
}

static __device__ __noinline__ bool subdiv_patch(HitSink& sink, float tol, LocalCounters& lc)
{
    float2 buf[16];
    project_net(buf, sink.P, sink.o, sink.d);
    uint32_t trail = 0, tu = 0, tv = 0;
    int k = 0;
    bool reload = false, found = false;
    for (int it = 0;; it++)
    {
        if (it >= 4 * kMaxClipIterations) { lc.errors |= kErrClipIterations; break; }
        lc.iterations++;
        const float su = ldexpf(1.0f, -((k + 1) >> 1)), sv = ldexpf(1.0f, -(k >> 1));
        const float2 emin = make_float2(float(tu) * su, float(tv) * sv);
        const float2 emax = make_float2(emin.x + su, emin.y + sv);
        if (reload)
        {
            project_net(buf, sink.P, sink.o, sink.d);
            subpatchU(buf, emin.x, emax.x);
            subpatchV(buf, emin.y, emax.y);
        }
        float2 bmin = buf[0], bmax = buf[0];
#pragma unroll
        for (int i = 1; i < 16; i++)
        {
            bmin = make_float2(fminf(bmin.x, buf[i].x), fminf(bmin.y, buf[i].y));
            bmax = make_float2(fmaxf(bmax.x, buf[i].x), fmaxf(bmax.y, buf[i].y));
        }
        if (bmin.x < 0.0f && bmin.y < 0.0f && bmax.x > 0.0f && bmax.y > 0.0f)
        {
            if ((len2(buf[3] - buf[12]) < tol && len2(buf[15] - buf[0]) < tol) || k >= 31)
                found |= approximateIntersection(sink, buf, emin, emax);
            else
            {
                reload = false;
                if ((k & 1) == 0) { subpatchU(buf, 0.0f, 0.5f); tu <<= 1; }
                else { subpatchV(buf, 0.0f, 0.5f); tv <<= 1; }
                trail <<= 1;
                ++k;
                continue;
            }
        }
        int ones = __clz(__brev(~trail));
        if (ones >= k) break;
        // levels k-1 .. k-ones are undone: even levels were u cuts
        const int hi = k - 1, lo = k - ones;         // inclusive range of undone cut levels
        const int evens = (hi / 2) - ((lo + 1) / 2) + 1;  // even levels in [lo, hi] were u cuts
        tu >>= evens;
        tv >>= (ones - evens);
        k -= ones;
        trail = (trail >> ones) | 1u;
        if (((k - 1) & 1) == 0) tu |= 1u; else tv |= 1u;
        reload = true;
    }
    return found;
}

// ----------------------------------------------------------- FP64 polish --
__device__ __forceinline__ void basis_d(double t, double* w)
{
    double s = 1.0 - t;
    w[0] = s * s * s; w[1] = 3.0 * t * s * s; w[2] = 3.0 * t * t * s; w[3] = t * t * t;
}
__device__ __forceinline__ void dbasis_d(double t, double* w)
{
    double s = 1.0 - t;
    w[0] = -3.0 * s * s; w[1] = 3.0 * s * s - 6.0 * t * s; w[2] = 6.0 * t * s - 3.0 * t * t; w[3] = 3.0 * t * t;
}

// Newton polish of S(u,v) = o + t d on the winning hit, first as
// mixed-precision iterative refinement: the residual S(u,v) - (o + t d) is
// evaluated in FP64 (Bernstein weights and the tensor sum in double), the 3x3
// Jacobian [dS/du dS/dv -d] and its solve stay in FP32, and (u,v,t)
// accumulate in FP64.  An FP32 Jacobian is accurate to ~1e-7 relative, so a
// step from an error e leaves about 1e-7 x cond x e + c e^2 (Newton's
// quadratic term).  The iteration stops once the update is below 1e-9 of t,
// or after a step whose update was at most kPolishAccept (relative in t,
// absolute in u + v) on a well-conditioned system (|det| at least
// kPolishMinSin of |dS/du| |dS/dv|, the ray's direction being a unit vector):
// the error left is then ~1e-10 relative, far below FP32 resolution, and the
// step that would only confirm it (a second FP64 residual, the dominant cost
// on a GPU whose FP64 rate is 1/64 of its FP32 rate) is skipped.  Hits where
// kPolishSteps such steps do not converge (ill-conditioned, e.g. grazing)
// continue with up to kPolishSteps64 full-FP64 Newton steps (FP64 Jacobian,
// as the oracle's polish).  The result is kept if it is finite and lies
// inside the patch domain (1e-6 slack) in front of the origin.
constexpr int kPolishSteps = 3;
constexpr int kPolishSteps64 = 10;
constexpr double kPolishAccept = 1e-5;
constexpr float kPolishMinSin = 1e-3f;

// Projected surface point and partials at (U, V) in FP64.
__device__ __forceinline__ void surface_d(const float4* __restrict__ P, double U, double V, double3& Sp, double3& Su,
                                          double3& Sv)
{
    double wu[4], wv[4], du[4], dv[4];
    basis_d(U, wu); basis_d(V, wv); dbasis_d(U, du); dbasis_d(V, dv);
    double H[4] = {0, 0, 0, 0}, Hu[4] = {0, 0, 0, 0}, Hv[4] = {0, 0, 0, 0};
#pragma unroll
    for (int j = 0; j < 4; j++)
    {
        double r[4] = {0, 0, 0, 0}, ru[4] = {0, 0, 0, 0};
#pragma unroll
        for (int i = 0; i < 4; i++)
        {
            const float4 q = __ldg(P + 4 * j + i);
            r[0] += wu[i] * q.x; r[1] += wu[i] * q.y; r[2] += wu[i] * q.z; r[3] += wu[i] * q.w;
            ru[0] += du[i] * q.x; ru[1] += du[i] * q.y; ru[2] += du[i] * q.z; ru[3] += du[i] * q.w;
        }
#pragma unroll
        for (int k = 0; k < 4; k++) { H[k] += wv[j] * r[k]; Hu[k] += wv[j] * ru[k]; Hv[k] += dv[j] * r[k]; }
    }
    const double iw = 1.0 / H[3];
    Sp = make_double3(H[0] * iw, H[1] * iw, H[2] * iw);
    Su = make_double3((Hu[0] - Hu[3] * Sp.x) * iw, (Hu[1] - Hu[3] * Sp.y) * iw, (Hu[2] - Hu[3] * Sp.z) * iw);
    Sv = make_double3((Hv[0] - Hv[3] * Sp.x) * iw, (Hv[1] - Hv[3] * Sp.y) * iw, (Hv[2] - Hv[3] * Sp.z) * iw);
}

static __device__ __noinline__ bool newton_polish64(const float4* __restrict__ P, double3 o, double3 d, double& t,
                                                    double& u, double& v)
{
    double U = u, V = v, T = t;
    const float3 df = f3(float(d.x), float(d.y), float(d.z));
    bool converged = false;
    for (int it = 0; it < kPolishSteps; it++)
    {
        double wu[4], wv[4];
        basis_d(U, wu);
        basis_d(V, wv);
        double S[4] = {0, 0, 0, 0};
#pragma unroll
        for (int j = 0; j < 4; j++)
        {
            double r[4] = {0, 0, 0, 0};
#pragma unroll
            for (int i = 0; i < 4; i++)
            {
                const float4 q = __ldg(P + 4 * j + i);
                r[0] += wu[i] * q.x; r[1] += wu[i] * q.y; r[2] += wu[i] * q.z; r[3] += wu[i] * q.w;
            }
            S[0] += wv[j] * r[0]; S[1] += wv[j] * r[1]; S[2] += wv[j] * r[2]; S[3] += wv[j] * r[3];
        }
        const double iw = 1.0 / S[3];
        const double px = S[0] * iw, py = S[1] * iw, pz = S[2] * iw;
        const float fx = float(px - (o.x + T * d.x)), fy = float(py - (o.y + T * d.y)), fz = float(pz - (o.z + T * d.z));
        // FP32 Jacobian of the projected surface at (U, V)
        const float uf = float(U), vf = float(V);
        const float4 Hu = tensor_eval(P, dbasis(uf), basis(vf));
        const float4 Hv = tensor_eval(P, basis(uf), dbasis(vf));
        const float4 H = tensor_eval(P, basis(uf), basis(vf));
        const float ih = 1.0f / H.w;
        const float3 Pf = f3(H.x * ih, H.y * ih, H.z * ih);
        const float3 Su = (xyz(Hu) - Hu.w * Pf) * ih, Sv = (xyz(Hv) - Hv.w * Pf) * ih;
        const float3 c = -df;
        const float3 svxc = cross(Sv, c);
        const float det = dot(Su, svxc);
        if (!(fabsf(det) > 1e-30f)) break;
        const float3 mF = f3(-fx, -fy, -fz);
        const float idet = 1.0f / det;
        const double dU = double(dot(mF, svxc) * idet);
        const double dV = double(dot(Su, cross(mF, c)) * idet);
        const double dT = double(dot(Su, cross(Sv, mF)) * idet);
        U += dU; V += dV; T += dT;
        if (!isfinite(U + V + T)) { U = u; V = v; T = t; break; }
        // the last step bounds the error of the previous iterate and contracts
        // by ~1e-7 x the Jacobian's condition: below 1e-9 the result is FP32-exact
        if (fabs(dT) <= 1e-9 * fabs(T) && fabs(dU) + fabs(dV) <= 1e-9) { converged = true; break; }
        // a small step on a well-conditioned system: the next would only confirm it
        if (fabs(dT) <= kPolishAccept * fabs(T) && fabs(dU) + fabs(dV) <= kPolishAccept &&
            fabsf(det) >= kPolishMinSin * len(Su) * len(Sv))
        {
            converged = true;
            break;
        }
    }
    if (!converged)
    {
        // the oracle's polish: FP64 Jacobian and solve
        const double3 c = make_double3(-d.x, -d.y, -d.z);
        for (int it = 0; it < kPolishSteps64; it++)
        {
            double3 Sp, Su, Sv;
            surface_d(P, U, V, Sp, Su, Sv);
            const double3 mF = make_double3(o.x + T * d.x - Sp.x, o.y + T * d.y - Sp.y, o.z + T * d.z - Sp.z);
            const double3 svxc = cross_d(Sv, c);
            const double det = dot_d(Su, svxc);
            if (!(fabs(det) > 1e-300)) return false;
            const double dU = dot_d(mF, svxc) / det;
            const double dV = dot_d(Su, cross_d(mF, c)) / det;
            const double dT = dot_d(Su, cross_d(Sv, mF)) / det;
            U += dU; V += dV; T += dT;
            if (!isfinite(U + V + T)) return false;
            if (fabs(dU) + fabs(dV) < 1e-15 && fabs(dT) < 1e-15 * fabs(T)) { converged = true; break; }
        }
    }
    if (U < -1e-6 || U > 1.0 + 1e-6 || V < -1e-6 || V > 1.0 + 1e-6 || T <= 0.0) return false;
    t = T; u = U; v = V;
    return true;
}

// ----------------------------------------------------------- traversal --
__device__ __forceinline__ uint32_t hash_slot(const DevScene& S, const DevBVH& b, uint32_t key)
{
    uint32_t disp = __ldg(S.disps + b.dispBase + (key & b.mask));
    return fastmod(b.A * key + b.B + disp, b.N, b.Nmagic);
}

// _node_intersect, src/rt/BVH.h:147-176
__device__ __forceinline__ bool slab(float& tMin, float3 lo, float3 hi, float3 o, float3 inv)
{
    // `if (a > tm) tm = a` and `if (b < tM) tM = b` as one max / min each:
    // tm and tM start at -inf / +inf and never become NaN, and fmaxf / fminf
    // skip a NaN argument just as the comparison does.
    float tm = -INFINITY, tM = INFINITY;
    {
        float t0 = (lo.x - o.x) * inv.x, t1 = (hi.x - o.x) * inv.x;
        bool s = signbit(inv.x);
        tm = fmaxf(tm, s ? t1 : t0);
        tM = fminf(tM, s ? t0 : t1);
    }
    {
        float t0 = (lo.y - o.y) * inv.y, t1 = (hi.y - o.y) * inv.y;
        bool s = signbit(inv.y);
        tm = fmaxf(tm, s ? t1 : t0);
        tM = fminf(tM, s ? t0 : t1);
    }
    {
        float t0 = (lo.z - o.z) * inv.z, t1 = (hi.z - o.z) * inv.z;
        bool s = signbit(inv.z);
        tm = fmaxf(tm, s ? t1 : t0);
        tM = fminf(tM, s ? t0 : t1);
    }
    tMin = tm;
    return tm < tM && tM > 0.0001f;
}

// Box tests on the compressed node mirror (32 bytes per node, written by
// pack_qnodes in scene.cu): the entry distances of a node's two child boxes,
// or for a leaf of its own box (left slot).  A grid byte q of an axis stands
// for the coordinate P + q s, s = 2^(e-127); its slab distance
// (P + q s - o) inv is evaluated as fma(2^23 + q, s inv, (P - o) inv - 2^23 s inv),
// where 2^23 + q is q placed in a float's mantissa by a byte permute (exact,
// no integer-to-float conversion).  Subtracting 2^23 s inv costs at most half
// a grid step of rounding (for nodes within 2^23 grid steps of the ray's
// origin; beyond that the rounding of (P - o) inv dominates, as it does in
// the exact test), and the encoder widens every box by at least one step, so
// a ray meets each decoded box wherever it meets the exact one, entering no
// later.  A ray parallel to an axis (inv = +-inf) gets NaN distances on
// that axis, which fmaxf / fminf skip: the axis then accepts, conservatively.
constexpr uint32_t kQNodeLeaf = 1u;

__device__ __forceinline__ void qslab_axis(uint32_t Pbits, uint32_t sbits, uint32_t q, float o, float inv,
                                           float& tmL, float& tML, float& tmR, float& tMR)
{
    const float step = __uint_as_float(sbits) * inv;
    const float base = fmaf(-8388608.0f, step, (__uint_as_float(Pbits) - o) * inv);
    const float lLo = fmaf(__uint_as_float(__byte_perm(q, 0x4B000000u, 0x7540u)), step, base);
    const float lHi = fmaf(__uint_as_float(__byte_perm(q, 0x4B000000u, 0x7541u)), step, base);
    const float rLo = fmaf(__uint_as_float(__byte_perm(q, 0x4B000000u, 0x7542u)), step, base);
    const float rHi = fmaf(__uint_as_float(__byte_perm(q, 0x4B000000u, 0x7543u)), step, base);
    const bool s = signbit(inv);
    tmL = fmaxf(tmL, s ? lHi : lLo);
    tML = fminf(tML, s ? lLo : lHi);
    tmR = fmaxf(tmR, s ? rHi : rLo);
    tMR = fminf(tMR, s ? rLo : rHi);
}

// a = words 0-3 (origins, scale exponents, flags), b = words 4-7 (grid
// bytes per axis, right child / first element).  Returns the two boxes'
// entries and whether the ray meets them (the exact test's condition).
__device__ __forceinline__ void qslab2(const uint4& a, const uint4& b, float3 o, float3 inv, float& L0, bool& iL,
                                       float& R0, bool& iR)
{
    float tmL = -INFINITY, tML = INFINITY, tmR = -INFINITY, tMR = INFINITY;
    qslab_axis(a.x, (a.w << 23) & 0x7F800000u, b.x, o.x, inv.x, tmL, tML, tmR, tMR);
    qslab_axis(a.y, (a.w << 15) & 0x7F800000u, b.y, o.y, inv.y, tmL, tML, tmR, tMR);
    qslab_axis(a.z, (a.w << 7) & 0x7F800000u, b.z, o.z, inv.z, tmL, tML, tmR, tMR);
    L0 = tmL;
    R0 = tmR;
    iL = tmL < tML && tML > 0.0001f;
    iR = tmR < tMR && tMR > 0.0001f;
}

// BVH::hashIntersect (src/rt/BVH.h:178-350): stackless descent that visits
// the nearer child first and records a postponed sibling as a 1 bit; going
// up shifts the bits out, flips to the sibling key and finds its node through
// the perfect hash.  kAny returns at the first accepted leaf element.
// `limit` is hit.t (closest) or ray.max (any); leaf(p) returns true on a hit
// and may lower `limit`.
template<bool kAny, class Leaf>
__device__ __forceinline__ bool hash_traverse(const DevScene& S, const DevBVH& b, float3 o, float3 inv, float& limit,
                                              Leaf&& leaf, LocalCounters& lc)
{
    const float4* __restrict__ nodes = S.nodes + 4ull * b.nodeBase;
    const uint32_t* __restrict__ indices = S.indices + b.indexBase;
    const uint32_t* __restrict__ table = S.tables + b.tableBase;
    uint32_t node = 0, key = 1, postponed = 0;
    bool result = false;
    for (int step = 0;; step++)
    {
        if (step >= kMaxTraversalSteps) { lc.errors |= kErrTraversal; break; }
        const float4* q = nodes + 4ull * node;
        float4 q0, q1, q2, q3;
        ldg256(q, q0, q1);
        ldg256(q + 2, q2, q3);
        uint32_t left = __float_as_uint(q3.x), right = __float_as_uint(q3.y);
        if (left != EMPTY)
        {
            lc.nodes++;
            float L0, R0;
            bool iL = slab(L0, f3(q0.x, q0.y, q0.z), f3(q0.w, q1.x, q1.y), o, inv) && L0 < limit;
            bool iR = slab(R0, f3(q1.z, q1.w, q2.x), f3(q2.y, q2.z, q2.w), o, inv) && R0 < limit;
            if (iL || iR) postponed <<= 1;
            if (iL)
            {
                if (iR)
                {
                    postponed |= 1u;
                    if (L0 < R0) { key = key << 1; node = left; }
                    else { key = (key << 1) ^ 1u; node = right; }
                }
                else { key = key << 1; node = left; }
                continue;
            }
            else if (iR) { key = (key << 1) ^ 1u; node = right; continue; }
        }
        else
        {
            for (uint32_t i = right;; i++)
            {
                uint32_t p = __ldg(indices + i);
                if (p == EMPTY) break;
                bool h = leaf(p);
                if (kAny && h) return true;
                result |= h;
            }
        }
        if (!postponed) break;
        int levels = __ffs(postponed) - 1;
        postponed >>= levels;
        key = (key >> levels) ^ 1u;
        postponed ^= 1u;
        lc.hashLookups++;
        lc.tableReads++;
        node = __ldg(table + hash_slot(S, b, key));
    }
    return kAny ? false : result;
}

struct Query { int method; int precision; float tol; };

struct HitRecord { float t, u, v; int32_t patch, object; };

// World -> object space ray (Context::intersect, src/rt/RayTracer.cu:305-314).
__device__ __forceinline__ void to_local(const DevObject& ob, float3 o, float3 d, float tmax, float3& lo, float3& ld,
                                         float& lmax, float& scale_inv)
{
    float4 o4 = m4_point(ob.w2l, o);
    lo = project(o4);
    ld = m3_vec(ob.w2l, d);
    float s = len(ld);
    lmax = tmax * s;
    s = 1.0f / s;
    ld = ld * s;
    scale_inv = s;
}

__device__ __forceinline__ bool search_patch(HitSink& sink, const Query& q, LocalCounters& lc, bool anyHit = false,
                                             const DevObject* ob = nullptr, float3 wo = {}, float3 wd = {})
{
    lc.candidates++;
    return q.method == 0 ? clip_patch(sink, q.tol, graze_sin(q.precision), lc, anyHit, ob, wo, wd)
                         : subdiv_patch(sink, q.tol, lc);
}

// FP64 Newton polish of a world-space hit, done in the object's space.
__device__ __forceinline__ void polish_hit(const DevScene& S, float3 o, float3 d, HitRecord& hit)
{
    const DevObject& ob = S.objects[hit.object];
    const float4* P = S.patches + 16ull * (__ldg(S.patchBase + ob.surface) + uint32_t(hit.patch));
    const float* m = ob.w2l;
    double ox = o.x, oy = o.y, oz = o.z, dx = d.x, dy = d.y, dz = d.z;
    double3 lo = make_double3(ox * m[0] + oy * m[4] + oz * m[8] + m[12], ox * m[1] + oy * m[5] + oz * m[9] + m[13],
                              ox * m[2] + oy * m[6] + oz * m[10] + m[14]);
    // an affine world-to-object matrix (the usual case) has w = 1: no division
    if (!(m[3] == 0.0f && m[7] == 0.0f && m[11] == 0.0f && m[15] == 1.0f))
    {
        const double lw = ox * m[3] + oy * m[7] + oz * m[11] + m[15];
        lo = make_double3(lo.x / lw, lo.y / lw, lo.z / lw);
    }
    double3 ld = make_double3(dx * m[0] + dy * m[4] + dz * m[8], dx * m[1] + dy * m[5] + dz * m[9],
                              dx * m[2] + dy * m[6] + dz * m[10]);
    const double sc = sqrt(ld.x * ld.x + ld.y * ld.y + ld.z * ld.z), isc = 1.0 / sc;
    ld = make_double3(ld.x * isc, ld.y * isc, ld.z * isc);
    double t = double(hit.t) * sc, u = hit.u, v = hit.v;
    if (newton_polish64(P, lo, ld, t, u, v)) { hit.t = float(t * isc); hit.u = float(u); hit.v = float(v); }
}

// Closest hit over the object-level BVH and each object's patch BVH
// (Context::intersect, src/rt/RayTracer.cu:295-349; rt::intersect,
// src/rt/Primitive.cu:222-248).  hit.t must hold ray.max on entry.
__device__ __forceinline__ int scene_closest(const DevScene& S, uint32_t group, float3 o, float3 d, float tmax,
                                             const Query& q, HitRecord& hit, LocalCounters& lc)
{
    int nearest = -1;
    float limit = tmax;
    const float3 inv = f3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    auto objfn = [&](uint32_t oi) -> bool {
        const DevObject& ob = S.objects[oi];
        float3 lo, ld; float lmax, sinv;
        to_local(ob, o, d, tmax, lo, ld, lmax, sinv);
        const float4* patches = S.patches + 16ull * __ldg(S.patchBase + ob.surface);
        float lt = lmax, lu = 0.0f, lv = 0.0f;
        uint32_t lp = 0;
        const float3 linv = f3(1.0f / ld.x, 1.0f / ld.y, 1.0f / ld.z);
        auto leaf = [&](uint32_t p) -> bool {
            HitSink sink {patches + 16ull * p, lo, ld, lt, make_float2(lu, lv)};
            if (search_patch(sink, q, lc, false, &ob, o, d))
            {
                lt = sink.dist; lu = sink.uv.x; lv = sink.uv.y; lp = p;
                return true;
            }
            return false;
        };
        bool b = hash_traverse<false>(S, S.bvhs[ob.surface], lo, linv, lt, leaf, lc);
        if (b)
        {
            float t = lt * sinv;
            if (t < limit)
            {
                hit.t = t; hit.u = lu; hit.v = lv; hit.patch = int32_t(lp); hit.object = int32_t(oi);
                limit = t; nearest = int(oi);
                return true;
            }
        }
        return false;
    };
    hash_traverse<false>(S, S.bvhs[S.groupTop[group]], o, inv, limit, objfn, lc);
    if (nearest >= 0 && polishes(q.precision)) polish_hit(S, o, d, hit);
    return nearest;
}

// Any hit (Context::intersect(const Ray&), src/rt/RayTracer.cu:351-383;
// rt::intersect(const BezierSurface&, const Ray&), src/rt/Primitive.cu:250-268).
__device__ __forceinline__ bool scene_any(const DevScene& S, uint32_t group, float3 o, float3 d, float tmax,
                                          const Query& qin, LocalCounters& lc)
{
    const Query q {qin.method, 0, qin.tol};  // any-hit searches run at level 0
    float limit = tmax;
    const float3 inv = f3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    auto objfn = [&](uint32_t oi) -> bool {
        const DevObject& ob = S.objects[oi];
        float3 lo, ld; float lmax, sinv;
        to_local(ob, o, d, tmax, lo, ld, lmax, sinv);
        const float4* patches = S.patches + 16ull * __ldg(S.patchBase + ob.surface);
        const float3 linv = f3(1.0f / ld.x, 1.0f / ld.y, 1.0f / ld.z);
        float llimit = lmax;
        auto leaf = [&](uint32_t p) -> bool {
            HitSink sink {patches + 16ull * p, lo, ld, lmax, make_float2(0.0f, 0.0f)};
            return search_patch(sink, q, lc, true);
        };
        return hash_traverse<true>(S, S.bvhs[ob.surface], lo, linv, llimit, leaf, lc);
    };
    return hash_traverse<true>(S, S.bvhs[S.groupTop[group]], o, inv, limit, objfn, lc);
}

// --------------------------------------------------------------- shading --
// src/rt/PBR.h:21-176, src/rt/PBR.cu:198-242
__device__ __forceinline__ bool lightVector(float& dist, float3& L, float3 P, const DevLight& l)
{
    if (l.angle < 0.01f) { L = -f3(l.direction[0], l.direction[1], l.direction[2]); dist = INFINITY; return true; }
    L = f3(l.position[0], l.position[1], l.position[2]) - P;
    dist = len(L);
    if (dist < 1e-14f || (l.range > 0.0f && dist > l.range)) return false;
    L = L * (1.0f / dist);
    if (l.angle > 1.57f) return true;
    float DL = dot(f3(l.direction[0], l.direction[1], l.direction[2]), L);
    return DL < 0.0f && l.angle > 2.0f * acosf(DL);
}
__device__ __forceinline__ float3 lightColor(float dist, const DevLight& l)
{
    float3 c = f3(l.color[0], l.color[1], l.color[2]);
    if (l.angle < 0.01f) return c;
    float f;
    if (l.range == 0.0f) { f = 1.0f / dist; f *= f; }
    else { f = dist / l.range; f = 1.0f + f * (f - 2.0f); }
    return c * f;
}
__device__ __forceinline__ float3 schlick(float3 f0, float dotLH)
{
    float b = 1.0f - dotLH, b2 = b * b;
    return f0 + (f3(1.0f, 1.0f, 1.0f) - f0) * (b2 * b2 * b);
}
__device__ __forceinline__ float G1(float x, float k) { return x / (x * (1.0f - k) + k); }
__device__ __forceinline__ float Gsmith(float nl, float nv, float r)
{
    float r1 = r + 1.0f, k = r1 * r1 * 0.125f;
    return G1(nl, k) * G1(nv, k);
}
__device__ __forceinline__ float Dggx(float nh, float r)
{
    r = fmaxf(r, 1e-3f);
    float a = r * r, a2 = a * a, dd = nh * nh * (a2 - 1.0f) + 1.0f;
    return a2 / (kPi * dd * dd);
}
__device__ __forceinline__ float3 BRDF_specular(float hl, float hn, float nv, float nl, float r, float3 f0)
{
    return schlick(f0, hl) * (Gsmith(nl, nv, r) * Dggx(hn, r) / (4.0f * nl * nv));
}

__device__ __forceinline__ const DevMaterial& hit_material(const DevScene& S, const DevObject& ob, uint32_t patch)
{
    if (ob.patchMaterialBase >= 0) return S.materials[__ldg(S.patchMaterial + ob.patchMaterialBase + patch)];
    return S.materials[ob.material];
}

// sRGB encode (IEC 61966-2-1) and RGBA8 packing.
__device__ __forceinline__ uint32_t srgb8(float c)
{
    float x = c <= 0.0031308f ? 12.92f * c : 1.055f * powf(c, 1.0f / 2.4f) - 0.055f;
    int v = __float2int_rn(x * 255.0f);
    return uint32_t(min(255, max(0, v)));
}
__device__ __forceinline__ uint32_t pack_srgb(float3 c)
{
    return srgb8(c.x) | (srgb8(c.y) << 8) | (srgb8(c.z) << 16) | 0xFF000000u;
}

// ---------------------------------------------------- warp-level helpers --
__device__ __forceinline__ unsigned lane_id()
{
    unsigned id;
    asm volatile("mov.u32 %0, %%laneid;" : "=r"(id));
    return id;
}

// Warp-aggregated atomic increment: every active lane with `want` gets a slot.
__device__ __forceinline__ uint32_t warp_push(uint32_t* counter, bool want)
{
    unsigned mask = __activemask();
    unsigned ballot = __ballot_sync(mask, want);
    if (!ballot) return EMPTY;
    int leader = __ffs(ballot) - 1;
    uint32_t base = 0;
    if ((int)lane_id() == leader) base = atomicAdd(counter, (uint32_t)__popc(ballot));
    base = __shfl_sync(mask, base, leader);
    return want ? base + __popc(ballot & ((1u << lane_id()) - 1u)) : EMPTY;
}

__device__ __forceinline__ void flush_counters(Counters* c, const LocalCounters& lc, uint32_t rays)
{
    if (!c) return;
    unsigned mask = __activemask();
    unsigned long long v[6] = {lc.nodes, lc.hashLookups, lc.candidates, lc.iterations, rays, lc.tableReads};
    uint32_t err = lc.errors;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
    {
#pragma unroll
        for (int k = 0; k < 6; k++) v[k] += __shfl_down_sync(mask, v[k], off);
        err |= __shfl_down_sync(mask, err, off);
    }
    if (lane_id() == (unsigned)(__ffs(mask) - 1))
    {
        atomicAdd(&c->nodes, v[0]); atomicAdd(&c->hashLookups, v[1]); atomicAdd(&c->candidates, v[2]);
        atomicAdd(&c->iterations, v[3]); atomicAdd(&c->rays, v[4]); atomicAdd(&c->tableReads, v[5]);
        if (err) atomicOr(&c->errors, (unsigned long long)err);
    }
}

}  // namespace cgs
