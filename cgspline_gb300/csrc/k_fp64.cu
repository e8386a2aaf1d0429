// k_fp64.cu -- the pure-FP64 search on the GPU (precision 2): the two-level
// hashed traversal, Bezier clipping of the projected net and the Newton
// polish of every root, all in double, one thread per ray.  It is the
// comparison run of the precision form: the FP32 paths report their t error
// and hit/miss disagreement against it.  The FP64 oracle restates the same
// search (FP64 traversal, clipping to tolerance 1e-9, each root polished and
// the closest polished root kept); the clip here follows the device variant
// of doBezierClipping2D (src/Spline_BezierClipping.cu:547-828: interval stack,
// sub-nets re-derived from the projected net), as the FP32 kernels do.
#include "kernels.h"

namespace cgs {

namespace {

constexpr int kThreads64 = 128;

struct Interval64 { double x0, y0, x1, y1; };  // a pushed sub-domain (min, max)

__device__ __forceinline__ double3 sub3(double3 a, double3 b) { return make_double3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ double len3d(double3 a) { return sqrt(dot_d(a, a)); }

// mat::slice_matrix / mat::slice in double (src/SplineMat.h:64-82,189-233)
struct SliceD { double m[4][4]; };
__device__ __forceinline__ SliceD slice_matrix_d(double a, double b)
{
    const double a2 = a * a, b2 = b * b, ia = 1.0 - a, ib = 1.0 - b, ia2 = ia * ia, ib2 = ib * ib,
                 k1 = a + 2.0 * b - 3.0 * a * b, k2 = 2.0 * a + b - 3.0 * a * b;
    SliceD M;
    M.m[0][0] = ia2 * ia; M.m[0][1] = 3.0 * a * ia2; M.m[0][2] = 3.0 * a2 * ia; M.m[0][3] = a2 * a;
    M.m[1][0] = ia2 * ib; M.m[1][1] = ia * k2; M.m[1][2] = a * k1; M.m[1][3] = a2 * b;
    M.m[2][0] = ia * ib2; M.m[2][1] = ib * k1; M.m[2][2] = b * k2; M.m[2][3] = a * b2;
    M.m[3][0] = ib2 * ib; M.m[3][1] = 3.0 * b * ib2; M.m[3][2] = 3.0 * b2 * ib; M.m[3][3] = b2 * b;
    return M;
}
template<int stride> __device__ __forceinline__ void apply_slice_d(double2* c, const SliceD& M)
{
    const double2 p0 = c[0], p1 = c[stride], p2 = c[2 * stride], p3 = c[3 * stride];
#pragma unroll
    for (int j = 0; j < 4; j++)
        c[j * stride] = make_double2(M.m[j][0] * p0.x + M.m[j][1] * p1.x + M.m[j][2] * p2.x + M.m[j][3] * p3.x,
                                     M.m[j][0] * p0.y + M.m[j][1] * p1.y + M.m[j][2] * p2.y + M.m[j][3] * p3.y);
}
__device__ __forceinline__ void subU_d(double2* p, double a, double b)
{
    const SliceD M = slice_matrix_d(a, b);
#pragma unroll
    for (int i = 0; i < 4; i++) apply_slice_d<1>(p + 4 * i, M);
}
__device__ __forceinline__ void subV_d(double2* p, double a, double b)
{
    const SliceD M = slice_matrix_d(a, b);
#pragma unroll
    for (int i = 0; i < 4; i++) apply_slice_d<4>(p + i, M);
}

// triangleOriginIntersection with the FP64 restatement's determinant floor
// 2^-200 (xAxisIntersection and the fat-line bounds in double are shared
// with the FP32 search's near-grazing variant).
__device__ __forceinline__ bool tri_origin_d(double2& coord, double2 P, double2 A, double2 B)
{
    const double2 p = A - P, q = B - P;
    double det = p.x * q.y - q.x * p.y;
    if (fabs(det) < 0x1p-200) return false;
    det = 1.0 / det;
    const double u = det * (q.y * -P.x + -q.x * -P.y);
    if (u < 0.0 || u > 1.0) return false;
    const double v = det * (-p.y * -P.x + p.x * -P.y);
    if (v < 0.0 || u + v > 1.0) return false;
    coord = make_double2(u, v);
    return true;
}

// The oracle's polish (FP64 Jacobian, up to 12 steps); leaves the inputs
// when it fails.
__device__ __forceinline__ bool polish_full(const float4* P, double3 o, double3 d, double& t, double& u, double& v)
{
    double U = u, V = v, T = t;
    const double3 c = make_double3(-d.x, -d.y, -d.z);
    for (int it = 0; it < 12; it++)
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
        if (fabs(dU) + fabs(dV) < 1e-15 && fabs(dT) < 1e-15 * fabs(T)) break;
    }
    if (U < -1e-6 || U > 1.0 + 1e-6 || V < -1e-6 || V > 1.0 + 1e-6 || T <= 0.0) return false;
    u = U; v = V; t = T;
    return true;
}

// Every root of the patch is polished; the closest polished one is kept.
struct Sink64
{
    const float4* P;
    double3 o, d;
    double best, bu, bv;
    bool any;
    __device__ __forceinline__ bool operator()(double2 e)
    {
        double3 Sp, Su, Sv;
        surface_d(P, e.x, e.y, Sp, Su, Sv);
        const double3 V = sub3(Sp, o);
        if (dot_d(V, d) <= 0.0) return false;
        double uu = e.x, vv = e.y, tt = len3d(V);
        polish_full(P, o, d, tt, uu, vv);
        if (tt < best) { best = tt; bu = uu; bv = vv; any = true; return true; }
        return false;
    }
};

__device__ __forceinline__ void project_d(double2* net, const float4* P, double3 o, double3 d)
{
    const double3 a0 = unit3d(cross_d(d, make_double3(d.x, d.y, d.z + 8.0)));
    const double3 a1 = unit3d(cross_d(d, a0));
#pragma unroll
    for (int i = 0; i < 16; i++)
    {
        const float4 q = __ldg(P + i);
        const double3 Q = make_double3(double(q.x) - o.x, double(q.y) - o.y, double(q.z) - o.z);
        net[i] = make_double2(dot_d(a0, Q), dot_d(a1, Q));
    }
}

__device__ __forceinline__ bool approx_d(Sink64& sink, const double2* p, double2 emin, double2 emax)
{
    bool found = false;
    double2 coord;
    const double2 size = emax - emin;
    if (tri_origin_d(coord, p[0], p[3], p[12])) found |= sink(emin + coord * size);
    if (tri_origin_d(coord, p[15], p[12], p[3])) found |= sink(emax - coord * size);
    return found;
}

__device__ __noinline__ bool clip64(Sink64& sink, double tol, LocalCounters& lc)
{
    double2 buf[16];
    Interval64 st[kClipStack];
    project_d(buf, sink.P, sink.o, sink.d);
    double2 emin = make_double2(0.0, 0.0), emax = make_double2(1.0, 1.0);
    int cutsideStack = 0, sl = 0;
    bool found = false;
    for (int it = 0;; it++)
    {
        if (it >= 4 * kMaxClipIterations) { lc.errors |= kErrClipIterations; break; }
        lc.iterations++;
        const int cutside = cutsideStack & 1;
        if (len2d(buf[3] - buf[12]) < tol && len2d(buf[15] - buf[0]) < tol)
            found |= approx_d(sink, buf, emin, emax);
        else
        {
            double lower, upper;
            clip_range_d(buf, cutside, lower, upper);
            const double delta = upper - lower;
            if (delta > 0.8)
            {
                Interval64 pushed;
                if (cutside == 0)
                {
                    const double hx = 0.5 * (emin.x + emax.x);
                    pushed = Interval64 {emin.x, emin.y, hx, emax.y};
                    emin.x = hx;
                    cutsideStack = (cutsideStack << 1) | 3;
                    subU_d(buf, 0.5, 1.0);
                }
                else
                {
                    const double hy = 0.5 * (emin.y + emax.y);
                    pushed = Interval64 {emin.x, emin.y, emax.x, hy};
                    emin.y = hy;
                    cutsideStack = (cutsideStack << 1) & ~3;
                    subV_d(buf, 0.5, 1.0);
                }
                if (sl >= kClipStack) { lc.errors |= kErrClipStack; break; }
                st[sl++] = pushed;
                continue;
            }
            if (delta > 0.0)
            {
                if (cutside == 0)
                {
                    const double sx = emax.x - emin.x;
                    const double u0 = emin.x + sx * lower, u1 = emax.x - sx * (1.0 - upper);
                    subU_d(buf, lower, upper);
                    emin.x = u0; emax.x = u1;
                }
                else
                {
                    const double sy = emax.y - emin.y;
                    const double v0 = emin.y + sy * lower, v1 = emax.y - sy * (1.0 - upper);
                    subV_d(buf, lower, upper);
                    emin.y = v0; emax.y = v1;
                }
                cutsideStack ^= 1;
                continue;
            }
        }
        cutsideStack >>= 1;
        if (--sl < 0) break;
        const Interval64 e = st[sl];
        emin = make_double2(e.x0, e.y0);
        emax = make_double2(e.x1, e.y1);
        project_d(buf, sink.P, sink.o, sink.d);
        subU_d(buf, emin.x, emax.x);
        subV_d(buf, emin.y, emax.y);
    }
    return found;
}

// _node_intersect in double (box corners are the FP32 node boxes).
__device__ __forceinline__ bool slab_d(double& tMin, const float* lo, const float* hi, double3 o, double3 inv)
{
    double tm = -INFINITY, tM = INFINITY;
    const double O[3] = {o.x, o.y, o.z}, I[3] = {inv.x, inv.y, inv.z};
#pragma unroll
    for (int k = 0; k < 3; k++)
    {
        const double t0 = (double(lo[k]) - O[k]) * I[k], t1 = (double(hi[k]) - O[k]) * I[k];
        const bool s = signbit(I[k]);
        const double a = s ? t1 : t0, b = s ? t0 : t1;
        if (a > tm) tm = a;
        if (b < tM) tM = b;
    }
    tMin = tm;
    return tm < tM && tM > double(0.0001f);
}

// BVH::hashIntersect (closest) in double.
template<class Leaf>
__device__ __forceinline__ bool traverse_d(const DevScene& S, const DevBVH& b, double3 o, double3 inv, double& limit,
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
        const uint32_t left = __float_as_uint(q3.x), right = __float_as_uint(q3.y);
        if (left != EMPTY)
        {
            lc.nodes++;
            const float lL[3] = {q0.x, q0.y, q0.z}, hL[3] = {q0.w, q1.x, q1.y};
            const float lR[3] = {q1.z, q1.w, q2.x}, hR[3] = {q2.y, q2.z, q2.w};
            double L0, R0;
            const bool iL = slab_d(L0, lL, hL, o, inv) && L0 < limit;
            const bool iR = slab_d(R0, lR, hR, o, inv) && R0 < limit;
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
                const uint32_t p = __ldg(indices + i);
                if (p == EMPTY) break;
                result |= leaf(p);
            }
        }
        if (!postponed) break;
        const int levels = __ffs(postponed) - 1;
        postponed >>= levels;
        key = (key >> levels) ^ 1u;
        postponed ^= 1u;
        lc.hashLookups++;
        lc.tableReads++;
        node = __ldg(table + hash_slot(S, b, key));
    }
    return result;
}

__global__ void __launch_bounds__(kThreads64) k_query_fp64(DevScene S, RaysSoA rays, uint32_t n0, const uint32_t* nDev,
                                                           double tol, HitsSoA hits, Counters* cnt)
{
    LocalCounters lc;
    const uint32_t n = nDev ? *nDev : n0;
    uint32_t nrays = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        nrays++;
        const double3 o = make_double3(rays.ox[i], rays.oy[i], rays.oz[i]);
        const double3 d = make_double3(rays.dx[i], rays.dy[i], rays.dz[i]);
        const double tmax = rays.tmax ? double(rays.tmax[i]) : double(INFINITY);
        const uint32_t g = rays.group ? rays.group[i] : 0u;
        int nearest = -1;
        double limit = tmax, bt = tmax, bu = 0.0, bv = 0.0;
        uint32_t bp = 0;
        if (g < S.ngroups)
        {
            const double3 inv = make_double3(1.0 / d.x, 1.0 / d.y, 1.0 / d.z);
            auto objfn = [&](uint32_t oi) -> bool {
                const DevObject& ob = S.objects[oi];
                const float* m = ob.w2l;
                const double lw = o.x * m[3] + o.y * m[7] + o.z * m[11] + m[15];
                const double3 lo = make_double3((o.x * m[0] + o.y * m[4] + o.z * m[8] + m[12]) / lw,
                                                (o.x * m[1] + o.y * m[5] + o.z * m[9] + m[13]) / lw,
                                                (o.x * m[2] + o.y * m[6] + o.z * m[10] + m[14]) / lw);
                double3 ld = make_double3(d.x * m[0] + d.y * m[4] + d.z * m[8], d.x * m[1] + d.y * m[5] + d.z * m[9],
                                          d.x * m[2] + d.y * m[6] + d.z * m[10]);
                const double sc = len3d(ld);
                ld = make_double3(ld.x / sc, ld.y / sc, ld.z / sc);
                const double3 linv = make_double3(1.0 / ld.x, 1.0 / ld.y, 1.0 / ld.z);
                const float4* patches = S.patches + 16ull * __ldg(S.patchBase + ob.surface);
                double lt = tmax * sc, lu = 0.0, lv = 0.0;
                uint32_t lp = 0;
                auto leaf = [&](uint32_t p) -> bool {
                    lc.candidates++;
                    Sink64 sink {patches + 16ull * p, lo, ld, lt, 0.0, 0.0, false};
                    clip64(sink, tol, lc);
                    if (sink.any) { lt = sink.best; lu = sink.bu; lv = sink.bv; lp = p; }
                    return sink.any;
                };
                if (!traverse_d(S, S.bvhs[ob.surface], lo, linv, lt, leaf, lc)) return false;
                const double t = lt / sc;
                if (!(t < limit)) return false;
                limit = t; nearest = int(oi); bt = t; bu = lu; bv = lv; bp = lp;
                return true;
            };
            traverse_d(S, S.bvhs[S.groupTop[g]], o, inv, limit, objfn, lc);
        }
        else
            lc.errors |= kErrGroup;
        hits.t[i] = nearest >= 0 ? float(bt) : float(tmax);
        hits.u[i] = float(bu); hits.v[i] = float(bv);
        hits.patch[i] = nearest >= 0 ? int32_t(bp) : -1;
        hits.object[i] = nearest;
    }
    flush_counters(cnt, lc, nrays);
}

}  // namespace

cudaError_t launch_query_fp64(const DevScene& S, RaysSoA rays, uint32_t n, const uint32_t* nDev, double tol,
                              HitsSoA hits, Counters* counters, cudaStream_t stream)
{
    if (n == 0) return cudaSuccess;
    k_query_fp64<<<(n + kThreads64 - 1) / kThreads64, kThreads64, 0, stream>>>(S, rays, n, nDev, tol, hits, counters);
    return cudaGetLastError();
}

}  // namespace cgs
