// cgs_oracle.cpp -- TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.
//
// A CPU restatement of the ray--bicubic-patch path of MachSilva/cgspline, used
// only to verify the CUDA implementation in cgspline_gb300/.  Only
// tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg may load this
// library.  Every function cites the reference file:line it restates (paths are
// relative to the reference project's root).
//
// Parity unpinned: the reference program itself cannot be compiled here (see
// below) and holds no tests or golden vectors, so this restatement is pinned
// only by analytic known-answer patches, the reference's own BVH and hash
// invariants, and the agreement of its FP32 variants with its FP64 search.
//
// The reference depends on an un-vendored submodule ("Ds", .gitmodules:1-3)
// for its vector/box types.  The semantics chosen here for those types are:
//   * vector ops are component-wise, dot products sum x,y,z(,w) left to right;
//   * length = sqrt(dot(v,v)); normalize multiplies by 1/length when length!=0;
//   * an empty Bounds3 has min=+inf, max=-inf (so size() = -inf per axis);
//   * mat4 is column-major and M*v = v.x*c0 + v.y*c1 + v.z*c2 + v.w*c3.
// The library is compiled with -ffp-contract=off so that results are the
// same on x86-64 and aarch64 hosts.
//
// Precision: every geometric routine is a template over the real type so the
// same code gives the FP32 reference semantics and the FP64 "true t" oracle.

#include <algorithm>
#include <atomic>
#include <bit>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <mutex>
#include <numeric>
#include <random>
#include <thread>
#include <type_traits>
#include <vector>

namespace ora {

// ---------------------------------------------------------------- vectors --
template<class R> struct V2 { R x, y; };
template<class R> struct V3 { R x, y, z; };
template<class R> struct V4 { R x, y, z, w; };

template<class R> inline V2<R> operator+(V2<R> a, V2<R> b) { return {a.x + b.x, a.y + b.y}; }
template<class R> inline V2<R> operator-(V2<R> a, V2<R> b) { return {a.x - b.x, a.y - b.y}; }
template<class R> inline V2<R> operator*(R s, V2<R> a) { return {s * a.x, s * a.y}; }
template<class R> inline V2<R> operator*(V2<R> a, V2<R> b) { return {a.x * b.x, a.y * b.y}; }
template<class R> inline R dot(V2<R> a, V2<R> b) { return a.x * b.x + a.y * b.y; }
template<class R> inline R length(V2<R> a) { return std::sqrt(dot(a, a)); }
template<class R> inline V2<R> normalized(V2<R> a)
{
    R l = length(a);
    if (l != R(0)) { R k = R(1) / l; a = {a.x * k, a.y * k}; }
    return a;
}

template<class R> inline V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template<class R> inline V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template<class R> inline V3<R> operator-(V3<R> a) { return {-a.x, -a.y, -a.z}; }
template<class R> inline V3<R> operator*(R s, V3<R> a) { return {s * a.x, s * a.y, s * a.z}; }
template<class R> inline V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template<class R> inline V3<R> operator*(V3<R> a, V3<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template<class R> inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template<class R> inline R length(V3<R> a) { return std::sqrt(dot(a, a)); }
template<class R> inline V3<R> cross(V3<R> a, V3<R> b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template<class R> inline V3<R> versor(V3<R> a)
{
    R l = length(a);
    if (l != R(0)) { R k = R(1) / l; a = {a.x * k, a.y * k, a.z * k}; }
    return a;
}
template<class R> inline R vmax(V3<R> a) { return std::max(std::max(a.x, a.y), a.z); }

template<class R> inline V4<R> operator+(V4<R> a, V4<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
template<class R> inline V4<R> operator*(R s, V4<R> a) { return {s * a.x, s * a.y, s * a.z, s * a.w}; }
template<class R> inline V3<R> project(V4<R> p) { return {p.x / p.w, p.y / p.w, p.z / p.w}; }  // src/AlignedTypes.h:63-66
template<class R> inline V3<R> xyz(V4<R> p) { return {p.x, p.y, p.z}; }

template<class R, class S> inline V3<R> cast3(V3<S> a) { return {R(a.x), R(a.y), R(a.z)}; }
template<class R, class S> inline V4<R> cast4(V4<S> a) { return {R(a.x), R(a.y), R(a.z), R(a.w)}; }

// Column-major 4x4 and 3x3 matrices (src/AlignedTypes.h:83-216).
template<class R> struct M4 { V4<R> c[4]; };
template<class R> struct M3 { V3<R> c[3]; };

template<class R> inline V4<R> mul(const M4<R>& m, V4<R> v)  // src/AlignedTypes.h:185-188
{
    return ((v.x * m.c[0] + v.y * m.c[1]) + v.z * m.c[2]) + v.w * m.c[3];
}
template<class R> inline V3<R> mul(const M3<R>& m, V3<R> v)  // src/AlignedTypes.h:127-130
{
    return (v.x * m.c[0] + v.y * m.c[1]) + v.z * m.c[2];
}
template<class R> inline M3<R> upper3(const M4<R>& m)  // src/AlignedTypes.h:195-198
{
    return {{xyz(m.c[0]), xyz(m.c[1]), xyz(m.c[2])}};
}
template<class R> inline M3<R> transposed(const M3<R>& m)  // src/AlignedTypes.h:147-151
{
    const auto& a = m.c[0]; const auto& b = m.c[1]; const auto& c = m.c[2];
    return {{{a.x, b.x, c.x}, {a.y, b.y, c.y}, {a.z, b.z, c.z}}};
}
template<class R> inline M4<R> load_m4(const float* p)  // 16 floats, column-major
{
    M4<R> m;
    for (int k = 0; k < 4; k++)
        m.c[k] = {R(p[4 * k]), R(p[4 * k + 1]), R(p[4 * k + 2]), R(p[4 * k + 3])};
    return m;
}

// ------------------------------------------------------------------ boxes --
struct Box
{
    V3<float> lo {INFINITY, INFINITY, INFINITY};
    V3<float> hi {-INFINITY, -INFINITY, -INFINITY};
    void inflate(V3<float> p)
    {
        lo = {std::min(lo.x, p.x), std::min(lo.y, p.y), std::min(lo.z, p.z)};
        hi = {std::max(hi.x, p.x), std::max(hi.y, p.y), std::max(hi.z, p.z)};
    }
    void inflate(const Box& b) { inflate(b.lo); inflate(b.hi); }
    V3<float> size() const { return hi - lo; }
    V3<float> center() const { return 0.5f * (lo + hi); }
};

// ------------------------------------------------- power-basis evaluation --
// CUBIC_BASE and CUBIC_DERIVATIVE_BASE as columns (src/SplineMat.h:22-44).
template<class R> inline V4<R> basis(R t)  // CUBIC_BASE * _eval_vec(t), src/SplineMat.h:101-105
{
    const R t2 = t * t;
    const V4<R> e {R(1), t, t2, t2 * t};
    const M4<R> B {{{1, 0, 0, 0}, {-3, 3, 0, 0}, {3, -6, 3, 0}, {-1, 3, -3, 1}}};
    return mul(B, e);
}
template<class R> inline V4<R> dbasis(R t)  // CUBIC_DERIVATIVE_BASE * _eval_vec_dt(t), src/SplineMat.h:107-110
{
    const V4<R> e {R(1), t, t * t, R(0)};
    const M4<R> C {{{-3, 3, 0, 0}, {6, -12, 6, 0}, {-3, 9, -9, 3}, {0, 0, 0, 0}}};
    return mul(C, e);
}
template<class R> inline V4<R> comb4(const V4<R>* s, int i0, int stride, V4<R> w)
{
    return ((w.x * s[i0] + w.y * s[i0 + stride]) + w.z * s[i0 + 2 * stride]) + w.w * s[i0 + 3 * stride];
}
// mat::interpolate(S,u,v), src/SplineMat.h:125-140
template<class R> V4<R> interpolate(const V4<R> s[16], R u, R v)
{
    V4<R> x = basis(u), y = basis(v);
    V4<R> A[4];
    for (int j = 0; j < 4; j++) A[j] = comb4(s, 4 * j, 1, x);
    return comb4(A, 0, 1, y);
}
// mat::derivativeU, src/SplineMat.h:142-158
template<class R> V4<R> derivativeU(const V4<R> s[16], R u, R v)
{
    V4<R> x = dbasis(u), y = basis(v);
    V4<R> A[4];
    for (int j = 0; j < 4; j++) A[j] = comb4(s, 4 * j, 1, x);
    return comb4(A, 0, 1, y);
}
// mat::derivativeV, src/SplineMat.h:160-176
template<class R> V4<R> derivativeV(const V4<R> s[16], R u, R v)
{
    V4<R> x = basis(u), y = dbasis(v);
    V4<R> A[4];
    for (int i = 0; i < 4; i++) A[i] = comb4(s, i, 4, y);
    return comb4(A, 0, 1, x);
}
// mat::normal, src/SplineMat.h:178-187 (not normalized)
template<class R> V3<R> patch_normal(const V4<R> s[16], R u, R v)
{
    return cross(xyz(derivativeU(s, u, v)), xyz(derivativeV(s, u, v)));
}

// ------------------------------------------------------- curve slicing --
// spline::slice (de Casteljau split1 then split0), src/Spline.h:324-364.
// Used by the host clipping path (src/Spline_BezierClipping.cu:388-426).
template<class R, int stride> inline void slice_dc(V2<R>* c, R u, R v)
{
    auto C = [&](int i) -> V2<R>& { return c[i * stride]; };
    R iu = R(1) - u;
    R vv = (v - u) / iu;
    R ivv = R(1) - vv;
    V2<R> P5, P6, P8;
    P6 = u * C(1) + iu * C(0);
    P5 = u * C(2) + iu * C(1);
    C(2) = u * C(3) + iu * C(2);
    P8 = u * P5 + iu * P6;
    C(1) = u * C(2) + iu * P5;
    C(0) = u * C(1) + iu * P8;
    P6 = ivv * C(2) + vv * C(3);
    P5 = ivv * C(1) + vv * C(2);
    C(1) = ivv * C(0) + vv * C(1);
    P8 = ivv * P5 + vv * P6;
    C(2) = ivv * C(1) + vv * P5;
    C(3) = ivv * C(2) + vv * P8;
}
template<class R> inline void subpatchU_dc(V2<R>* p, R a, R b)  // src/Spline.h:366-373
{
    for (int i = 0; i < 4; i++) slice_dc<R, 1>(p + 4 * i, a, b);
}
template<class R> inline void subpatchV_dc(V2<R>* p, R a, R b)  // src/Spline.h:375-382
{
    for (int i = 0; i < 4; i++) slice_dc<R, 4>(p + i, a, b);
}

// mat::slice_matrix (columns), src/SplineMat.h:64-82.
template<class R> inline M4<R> slice_matrix(R a, R b)
{
    const R a2 = a * a, b2 = b * b, ia = R(1) - a, ib = R(1) - b, ia2 = ia * ia, ib2 = ib * ib,
            _a_2b_3ab = a + R(2) * b - R(3) * a * b, _2a_b_3ab = R(2) * a + b - R(3) * a * b;
    return {{{ia2 * ia, R(3) * a * ia2, R(3) * a2 * ia, a2 * a},
             {ia2 * ib, ia * _2a_b_3ab, a * _a_2b_3ab, a2 * b},
             {ia * ib2, ib * _a_2b_3ab, b * _2a_b_3ab, a * b2},
             {ib2 * ib, R(3) * b * ib2, R(3) * b2 * ib, b2 * b}}};
}
// mat::slice<stride>(vec2*), src/SplineMat.h:189-206: P_j <- sum_k M[j][k] P_k.
template<class R, int stride> inline void slice_mat(V2<R>* c, R a, R b)
{
    M4<R> M = slice_matrix(a, b);
    V4<R> x {c[0].x, c[stride].x, c[2 * stride].x, c[3 * stride].x};
    V4<R> y {c[0].y, c[stride].y, c[2 * stride].y, c[3 * stride].y};
    // M^T * x, written out as M^T's column combination (src/AlignedTypes.h:185-188)
    M4<R> T {{{M.c[0].x, M.c[1].x, M.c[2].x, M.c[3].x},
              {M.c[0].y, M.c[1].y, M.c[2].y, M.c[3].y},
              {M.c[0].z, M.c[1].z, M.c[2].z, M.c[3].z},
              {M.c[0].w, M.c[1].w, M.c[2].w, M.c[3].w}}};
    V4<R> X = mul(T, x), Y = mul(T, y);
    c[0] = {X.x, Y.x};
    c[stride] = {X.y, Y.y};
    c[2 * stride] = {X.z, Y.z};
    c[3 * stride] = {X.w, Y.w};
}
template<class R> inline void subpatchU_mat(V2<R>* p, R a, R b)  // src/SplineMat.h:221-226
{
    for (int i = 0; i < 4; i++) slice_mat<R, 1>(p + 4 * i, a, b);
}
template<class R> inline void subpatchV_mat(V2<R>* p, R a, R b)  // src/SplineMat.h:228-233
{
    for (int i = 0; i < 4; i++) slice_mat<R, 4>(p + i, a, b);
}
template<class R> inline void patchCopy(V2<R>* q, const V2<R>* p, V2<R> lo, V2<R> hi)  // src/SplineMat.h:248-257
{
    for (int i = 0; i < 16; i++) q[i] = p[i];
    subpatchU_mat(q, lo.x, hi.x);
    subpatchV_mat(q, lo.y, hi.y);
}

// ------------------------------------------------------ clipping helpers --
template<class R> struct Eps;
// v: xAxisIntersection's epsilon (FLT_EPSILON in the reference).  det: the
// smallest |det| triangleOriginIntersection accepts (0x1p-80f in the
// reference); the FP64 oracle scales it to double range because its sub-nets
// get far thinner than FP32 ones.
template<> struct Eps<float> { static constexpr float v = FLT_EPSILON; static constexpr float det = 0x1p-80f; };
template<> struct Eps<double> { static constexpr double v = DBL_EPSILON; static constexpr double det = 0x1p-200; };

// xAxisIntersection, src/Spline_BezierClipping.cu:127-156
template<class R> inline bool xAxisIntersection(V2<R>& result, V2<R> A, V2<R> B)
{
    const R eps = Eps<R>::v;
    R q = A.y - B.y;
    if (std::fabs(q) > eps)
    {
        R t = A.y / q;
        if (R(0) <= t && t <= R(1))
        {
            R s = (R(1) - t) * A.x + t * B.x;
            result = {s, s};
            return true;
        }
    }
    else if (std::fabs(A.y) <= eps)
    {
        result = {std::fmin(A.x, B.x), std::fmax(A.x, B.x)};
        return true;
    }
    return false;
}
template<class R> inline R isCCW(V2<R> P, V2<R> Q) { return P.x * Q.y - P.y * Q.x; }  // :161-165

// triangleOriginIntersection, src/Spline.h:709-737
template<class R> inline bool triangleOriginIntersection(V2<R>& coord, V2<R> P, V2<R> A, V2<R> B)
{
    V2<R> p = A - P, q = B - P;
    R det = p.x * q.y - q.x * p.y;
    if (std::fabs(det) < Eps<R>::det) return false;
    det = R(1) / det;
    V2<R> m0 {q.y, -q.x}, m1 {-p.y, p.x};
    V2<R> mP {-P.x, -P.y};
    R u = det * dot(m0, mP);
    if (u < 0 || u > 1) return false;
    R v = det * dot(m1, mP);
    if (v < 0 || u + v > 1) return false;
    coord = {u, v};
    return true;
}
// approximateIntersection, src/Spline.h:739-765
template<class R, class F> inline bool approximateIntersection(F& onHit, const V2<R>* p, V2<R> pmin, V2<R> pmax, V2<R> psize)
{
    bool found = false;
    V2<R> p00 = p[0], p10 = p[3], p01 = p[12], p11 = p[15];
    V2<R> coord;
    if (triangleOriginIntersection(coord, p00, p10, p01)) found |= onHit(pmin + coord * psize);
    if (triangleOriginIntersection(coord, p11, p01, p10)) found |= onHit(pmax - coord * psize);
    return found;
}

// The x-axis range of the true convex hull of the bound points (x_i, ybot_i)
// and (x_i, ytop_i): the lower chain of the bottoms and the upper chain of the
// tops, each a monotone-chain hull (Andrew's algorithm), closed by the sides
// at x = 0 and x = 1.  Not in the reference: its scan (clip_range below) walks
// the points once and never revisits an accepted edge, so on some nets its
// polygon leaves out part of the hull and the clip drops a root.
template<class R> inline void hull_range_exact(const R* ybot, const R* ytop, R& lower, R& upper)
{
    const R xs[4] {R(0), R(1) / R(3), R(2) / R(3), R(1)};
    V2<R> lo[4], up[4];
    int nl = 0, nu = 0;
    for (int i = 0; i < 4; i++)
    {
        const V2<R> q {xs[i], ybot[i]};
        while (nl >= 2 && isCCW(lo[nl - 1] - lo[nl - 2], q - lo[nl - 2]) <= 0) nl--;
        lo[nl++] = q;
    }
    for (int i = 3; i >= 0; i--)
    {
        const V2<R> q {xs[i], ytop[i]};
        while (nu >= 2 && isCCW(up[nu - 1] - up[nu - 2], q - up[nu - 2]) <= 0) nu--;
        up[nu++] = q;
    }
    lower = R(1); upper = R(0);
    auto edge = [&](V2<R> A, V2<R> B) {
        V2<R> s;
        if (xAxisIntersection(s, A, B)) { lower = std::fmin(lower, s.x); upper = std::fmax(upper, s.y); }
    };
    for (int k = 0; k + 1 < nl; k++) edge(lo[k], lo[k + 1]);
    edge(lo[nl - 1], up[0]);
    for (int k = 0; k + 1 < nu; k++) edge(up[k], up[k + 1]);
    edge(up[nu - 1], lo[0]);
}

// Fat-line clip of one sub-net: returns (lower, upper) after the anti-sliver
// shrink.  src/Spline_BezierClipping.cu:250-353 (host) / :610-701 (device).
// kExact: the true hull's range (hull_range_exact) in place of the
// reference's scan.
template<class R, bool kExact = false> inline void clip_range(const V2<R>* p, int cutside, R& lower, R& upper)
{
    const R over3[] {R(0), R(1) / R(3), R(2) / R(3), R(1)};
    lower = R(1); upper = R(0);
    R ytop[4], ybot[4];
    {
        V2<R> L = p[15] - p[0];
        V2<R> D = p[12] - p[3];
        L = cutside == 0 ? L + D : L - D;
        L = normalized(L);
        const V2<R> N {-L.y, L.x};
        R d[16];
        for (int i = 0; i < 16; i++) d[i] = dot(N, p[i]);
        for (int i = 0; i < 4; i++)
        {
            R y0 = cutside == 0 ? d[i] : d[4 * i];
            ytop[i] = ybot[i] = y0;
            for (int k = 1; k < 4; k++)
            {
                R y = cutside == 0 ? d[4 * k + i] : d[4 * i + k];
                ytop[i] = std::fmax(ytop[i], y);
                ybot[i] = std::fmin(ybot[i], y);
            }
        }
    }
    if constexpr (kExact)
    {
        hull_range_exact(ybot, ytop, lower, upper);
        lower = lower * R(0x0FFp-8);
        upper = upper + (R(1) - upper) * R(0x001p-8);
        return;
    }
    const V2<R> hull[] {{over3[2], ybot[2]}, {over3[3], ybot[3]}, {over3[3], ytop[3]}, {over3[2], ytop[2]},
                        {over3[1], ytop[1]}, {over3[0], ytop[0]}, {over3[0], ybot[0]}};
    V2<R> P1 {over3[0], ybot[0]}, P2 {over3[1], ybot[1]};
    for (const V2<R>& P3 : hull)
    {
        if (isCCW(P2 - P1, P3 - P1) >= 0)
        {
            V2<R> s;
            if (xAxisIntersection(s, P1, P2)) { lower = std::fmin(lower, s.x); upper = std::fmax(upper, s.y); }
            P1 = P2;
        }
        P2 = P3;
    }
    V2<R> s;
    if (xAxisIntersection(s, P1, P2)) { lower = std::fmin(lower, s.x); upper = std::fmax(upper, s.y); }
    lower = lower * R(0x0FFp-8);
    upper = upper + (R(1) - upper) * R(0x001p-8);
}

struct ClipStats { uint64_t iterations = 0, pushes = 0, maxDepth = 0, overflow = 0; };

// doBezierClipping2D_host, src/Spline_BezierClipping.cu:174-445 (the CPU
// path of the reference: full sub-nets on an unbounded stack).
template<class R, class F, bool kExact = false> bool clip2d_host(F& onHit, const V2<R>* patch, R tol, ClipStats* st)
{
    struct State { V2<R> patch[16]; V2<R> min, max, size; int cutside; };
    bool found = false;
    std::vector<State> S;
    S.reserve(16);
    S.push_back({});
    {
        auto& b = S.back();
        for (int i = 0; i < 16; i++) b.patch[i] = patch[i];
        b.min = {0, 0}; b.max = {1, 1}; b.size = {1, 1}; b.cutside = 0;
    }
    do
    {
        if (st) st->iterations++;
        auto& e = S.back();
        const V2<R>* p = e.patch;
        R d0 = length(p[3] - p[12]);
        R d1 = length(p[15] - p[0]);
        if (d0 < tol && d1 < tol)
        {
            found |= approximateIntersection(onHit, p, e.min, e.max, e.size);
            S.pop_back();
            continue;
        }
        R lower, upper;
        clip_range<R, kExact>(p, e.cutside, lower, upper);
        R delta = upper - lower;
        if (delta < 0)
            S.pop_back();
        else if (delta > R(0.8f))
        {
            State s1;
            for (int i = 0; i < 16; i++) s1.patch[i] = e.patch[i];
            if (e.cutside == 0)
            {
                R hs = R(0.5f) * e.size.x, hx = e.min.x + hs;
                s1.max = e.max; s1.min = {hx, e.min.y};
                e.max = {hx, e.max.y};
                s1.size = e.size = {hs, e.size.y};
                s1.cutside = e.cutside = 1;
                subpatchU_dc(e.patch, R(0), R(0.5f));
                subpatchU_dc(s1.patch, R(0.5f), R(1));
            }
            else
            {
                R hs = R(0.5f) * e.size.y, hy = e.min.y + hs;
                s1.max = e.max; s1.min = {e.min.x, hy};
                e.max = {e.max.x, hy};
                s1.size = e.size = {e.size.x, hs};
                s1.cutside = e.cutside = 0;
                subpatchV_dc(e.patch, R(0), R(0.5f));
                subpatchV_dc(s1.patch, R(0.5f), R(1));
            }
            S.push_back(s1);
            if (st) { st->pushes++; st->maxDepth = std::max<uint64_t>(st->maxDepth, S.size()); }
        }
        else
        {
            if (e.cutside == 0)
            {
                R u0 = e.min.x + e.size.x * lower, u1 = e.max.x - e.size.x * (R(1) - upper);
                subpatchU_dc(e.patch, lower, upper);
                e.min.x = u0; e.max.x = u1; e.size.x = u1 - u0; e.cutside = 1;
            }
            else
            {
                R v0 = e.min.y + e.size.y * lower, v1 = e.max.y - e.size.y * (R(1) - upper);
                subpatchV_dc(e.patch, lower, upper);
                e.min.y = v0; e.max.y = v1; e.size.y = v1 - v0; e.cutside = 0;
            }
        }
    } while (!S.empty());
    return found;
}

// doBezierClipping2D_device, src/Spline_BezierClipping.cu:547-828, with the
// half-precision (mid,len) stack replaced by a full-precision (min,max) stack
// of the same depth (32).  The CUDA product follows this structure; this copy
// lets the tests compare against it directly.
// FP64 fat-line bounds of an FP32 sub-net (the precision form's variant for
// near-grazing candidates): the distances, hull scan and epsilons of
// clip_range in double, the interval rounded outward to float.
inline void clip_range_f64(const V2<float>* p, int cutside, float& lower, float& upper)
{
    V2<double> q[16];
    for (int i = 0; i < 16; i++) q[i] = {double(p[i].x), double(p[i].y)};
    double lo, hi;
    clip_range<double>(q, cutside, lo, hi);
    lower = float(lo);
    if (double(lower) > lo) lower = std::nextafter(lower, -INFINITY);
    upper = float(hi);
    if (double(upper) < hi) upper = std::nextafter(upper, INFINITY);
}
inline void clip_range_f64(const V2<double>* p, int cutside, double& lower, double& upper)
{
    clip_range<double>(p, cutside, lower, upper);
}

template<class R, class F, bool kBounds64 = false> bool clip2d_device(F& onHit, const V2<R>* patch, R tol, ClipStats* st)
{
    struct State { V2<R> min, max; };
    bool found = false;
    int cutsideStack = 0;
    State S[32];
    int S_len = 0;
    State e {{0, 0}, {1, 1}};
    V2<R> buf[16];
    for (int i = 0; i < 16; i++) buf[i] = patch[i];
    int it = 0;
    do
    {
        // the near-grazing variant keeps what it found after 1024 iterations
        if (kBounds64 && it++ >= 1024) return found;
        if (st) st->iterations++;
        const int cutside = cutsideStack & 1;
        R d0 = length(buf[3] - buf[12]);
        R d1 = length(buf[15] - buf[0]);
        if (d0 < tol && d1 < tol)
            found |= approximateIntersection(onHit, buf, e.min, e.max, e.max - e.min);
        else
        {
            R lower, upper;
            if constexpr (kBounds64) clip_range_f64(buf, cutside, lower, upper);
            else clip_range(buf, cutside, lower, upper);
            R delta = upper - lower;
            if (delta > R(0.8f))
            {
                State s1;
                if (cutside == 0)
                {
                    R hx = R(0.5f) * (e.min.x + e.max.x);
                    s1.max = e.max; s1.min = {hx, e.min.y};
                    e.max.x = hx;
                    cutsideStack = (cutsideStack << 1) | 3;
                    subpatchU_mat(buf, R(0.5f), R(1));
                }
                else
                {
                    R hy = R(0.5f) * (e.min.y + e.max.y);
                    s1.max = e.max; s1.min = {e.min.x, hy};
                    e.max.y = hy;
                    cutsideStack = (cutsideStack << 1) & ~3;
                    subpatchV_mat(buf, R(0.5f), R(1));
                }
                if (S_len >= 32) { if (st) st->overflow++; return found; }
                S[S_len++] = e;
                if (st) { st->pushes++; st->maxDepth = std::max<uint64_t>(st->maxDepth, S_len); }
                e = s1;
                continue;
            }
            else if (delta > 0)
            {
                if (cutside == 0)
                {
                    R sx = e.max.x - e.min.x;
                    R u0 = e.min.x + sx * lower, u1 = e.max.x - sx * (R(1) - upper);
                    subpatchU_mat(buf, lower, upper);
                    e.min.x = u0; e.max.x = u1;
                }
                else
                {
                    R sy = e.max.y - e.min.y;
                    R v0 = e.min.y + sy * lower, v1 = e.max.y - sy * (R(1) - upper);
                    subpatchV_mat(buf, lower, upper);
                    e.min.y = v0; e.max.y = v1;
                }
                cutsideStack ^= 1;
                continue;
            }
        }
        cutsideStack >>= 1;
        if (--S_len >= 0)
        {
            e = S[S_len];
            patchCopy(buf, patch, e.min, e.max);
        }
    } while (S_len >= 0);
    return found;
}

// Stackless 2-D subdivision.  Restates doSubdivision2D_device
// (src/Spline_Subdivision.cu:16-109): bisect alternately along u then v,
// descend into the lower half first, keep only bit trails, re-derive a
// sub-net from the original net after every backtrack, accept a leaf when
// the sub-net's bounding box strictly contains the origin and both diagonals
// are shorter than tol (or 31 levels are reached).  The reference derives
// the sub-domain extents from a negative depth with truncating division
// (:39-42), which puts the v extent one halving ahead of the buffer; here the
// domain follows the buffer exactly: after k halvings su = 2^-ceil(k/2),
// sv = 2^-floor(k/2).
template<class R, class F> bool subdiv2d(F& onHit, const V2<R>* patch, R tol, ClipStats* st)
{
    bool found = false;
    uint32_t trail = 0, tu = 0, tv = 0;
    int k = 0;           // number of halvings of the current sub-domain
    bool reload = false;
    V2<R> buf[16];
    for (int i = 0; i < 16; i++) buf[i] = patch[i];
    for (;;)
    {
        if (st) st->iterations++;
        const R su = std::ldexp(R(1), -((k + 1) / 2));
        const R sv = std::ldexp(R(1), -(k / 2));
        const V2<R> emin {R(tu) * su, R(tv) * sv};
        const V2<R> emax {emin.x + su, emin.y + sv};
        if (reload) patchCopy(buf, patch, emin, emax);
        V2<R> bmin = buf[0], bmax = buf[0];
        for (int i = 1; i < 16; i++)
        {
            bmin = {std::fmin(bmin.x, buf[i].x), std::fmin(bmin.y, buf[i].y)};
            bmax = {std::fmax(bmax.x, buf[i].x), std::fmax(bmax.y, buf[i].y)};
        }
        if (bmin.x < 0 && bmin.y < 0 && bmax.x > 0 && bmax.y > 0)
        {
            R d0 = length(buf[3] - buf[12]);
            R d1 = length(buf[15] - buf[0]);
            if ((d0 < tol && d1 < tol) || k >= 31)
                found |= approximateIntersection(onHit, buf, emin, emax, emax - emin);
            else
            {
                reload = false;
                if ((k & 1) == 0) { subpatchU_mat(buf, R(0), R(0.5f)); tu <<= 1; }
                else              { subpatchV_mat(buf, R(0), R(0.5f)); tv <<= 1; }
                trail <<= 1;
                ++k;
                if (st) st->maxDepth = std::max<uint64_t>(st->maxDepth, k);
                continue;
            }
        }
        // go up past every level where we were the upper half, then step to
        // the upper sibling of the first lower half
        int ones = std::countr_zero(~trail);
        if (ones >= k) break;  // back above the root: done
        for (int m = 0; m < ones; m++)
        {
            int level = k - 1 - m;  // the cut that produced this level
            if ((level & 1) == 0) tu >>= 1; else tv >>= 1;
        }
        k -= ones;
        trail >>= ones;
        trail |= 1;
        if (((k - 1) & 1) == 0) tu |= 1; else tv |= 1;
        reload = true;
    }
    return found;
}

// --------------------------------------------------- ray/patch front end --
template<class R> struct Ray { V3<R> o, d; R max; };
struct PatchHit { float t; float u, v; };

// kClipDeviceB64: kClipDevice with FP64 fat-line bounds; kClipDeviceB64P:
// the same on a net projected in FP64 (rounded to the search type).
// kClipGraze: the precision form's clip (CGS_PREC_FP32_GRAZE64) --
// kClipDevice, except that a near-grazing candidate (grazing(): within
// asin(g_grazeSin) = 30 degrees of a control-net normal, or a silhouette)
// gets kClipDeviceB64P with tolerance 2^-20.
// kClipExactHull: the host clip with the true convex hull (hull_range_exact),
// an oracle-only variant that shows the roots the reference's scan drops.
enum Method { kClipHost = 0, kClipDevice = 1, kSubdiv = 2, kClipDeviceB64 = 3, kClipDeviceB64P = 4, kClipGraze = 5,
              kClipExactHull = 6 };
static float g_grazeSin = 0.5f;
constexpr float kGrazeTol = 0x1p-20f;
// The precision form's near-grazing test of a candidate (restates
// near_grazing in the CUDA path).  Mode 1 (the default): the ray within
// asin(g_grazeSin) of the plane of the patch's diagonals or of any of the
// nine cells of its control net (each cell's normal: the cross product of
// its edges along u and v at its first corner), or those ten normals on both
// sides of the ray (the patch folds over the ray's direction somewhere: a
// silhouette).  The cells' normals bound the patch's, interior control
// points included, so a bumpy patch tangent to the ray inside is caught even
// where its diagonals and corners are not.  Mode 0: the diagonals' plane
// alone (the earlier test, for comparison).
static int g_grazeMode = 1;
template<class R> inline bool grazing(const V4<R> P[16], V3<R> d)
{
    bool pos = false, neg = false;
    auto test = [&](V3<R> nn) {
        const R ln = length(nn);
        if (!(ln > R(0))) return false;
        const R c = dot(nn, d);
        if (std::fabs(c) < R(g_grazeSin) * ln) return true;
        (c > 0 ? pos : neg) = true;
        return false;
    };
    if (test(cross(xyz(P[15]) - xyz(P[0]), xyz(P[12]) - xyz(P[3])))) return true;
    if (g_grazeMode == 0) return false;
    for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++)
        {
            const V3<R> tu = xyz(P[4 * j + i + 1]) - xyz(P[4 * j + i]);
            const V3<R> tv = xyz(P[4 * (j + 1) + i]) - xyz(P[4 * j + i]);
            if (test(cross(tu, tv))) return true;
        }
    return pos && neg;
}

// spline::doBezierClipping / doSubdivision_device front end,
// src/Spline_BezierClipping.cu:46-114 and src/Spline_Subdivision.cu:111-165:
// project the 16 points onto two planes that contain the ray, then run the
// 2-D search with an onHit that keeps the closest point in front.
// ray64 (optional): the same ray in object space computed in double from the
// world ray; a near-grazing candidate's FP64 projection then starts from it
// instead of from the FP32 object-space ray (restates to_local64 and its use
// in the CUDA path's precision form; 0 gives the projection from the FP32
// ray, for comparison).
static int g_graze64Ray = 1;
template<class R>
bool intersect_patch(R& distance, V2<R>& uv, const Ray<R>& ray, const V4<R> P[16], R tol, int method, ClipStats* st,
                     const Ray<double>* ray64 = nullptr)
{
    const V3<R> d = ray.d;
    const V3<R> axis0 = versor(cross(d, d + V3<R>{0, 0, 8}));
    const V3<R> axis1 = versor(cross(d, axis0));
    V2<R> net[16];
    if (method == kClipGraze)
    {
        if (grazing(P, d)) { method = kClipDeviceB64P; tol = R(kGrazeTol); }
        else method = kClipDevice;
    }
    if (method == kClipDeviceB64P)
    {
        const V3<double> dd = ray64 ? ray64->d : cast3<double>(d), oo = ray64 ? ray64->o : cast3<double>(ray.o);
        const V3<double> a0 = versor(cross(dd, dd + V3<double>{0, 0, 8}));
        const V3<double> a1 = versor(cross(dd, a0));
        for (int i = 0; i < 16; i++)
        {
            V3<double> Q = cast3<double>(xyz(P[i])) - oo;
            net[i] = {R(dot(a0, Q)), R(dot(a1, Q))};
        }
    }
    else
        for (int i = 0; i < 16; i++)
        {
            V3<R> Q = xyz(P[i]);
            net[i] = {dot(axis0, Q - ray.o), dot(axis1, Q - ray.o)};
        }
    auto onHit = [&](V2<R> e) -> bool {
        V3<R> V = project(interpolate(P, e.x, e.y)) - ray.o;
        R t = length(V);
        if (t < distance && dot(V, ray.d) > 0) { distance = t; uv = e; return true; }
        return false;
    };
    switch (method)
    {
    case kClipHost: return clip2d_host(onHit, net, tol, st);
    case kClipExactHull: return clip2d_host<R, decltype(onHit), true>(onHit, net, tol, st);
    case kClipDevice: return clip2d_device(onHit, net, tol, st);
    case kClipDeviceB64:
    case kClipDeviceB64P: return clip2d_device<R, decltype(onHit), true>(onHit, net, tol, st);
    default: return subdiv2d(onHit, net, tol, st);
    }
}

// ------------------------------------------------ host subdivision (3-D) --
// doSubdivision_host, src/Spline_Subdivision.cu:166-288: the CPU variant,
// which subdivides the 3-D net itself rather than a 2-D projection.  A stack
// of parameter rectangles starts with u in [0, 1/2] and [1/2, 1]; each popped
// rectangle's sub-net (subpatchV then subpatchU by de Casteljau slicing of
// the homogeneous points, src/Spline.h:398-478) is bounded by the box of its
// projected points; a box the ray misses is dropped; a rectangle smaller than
// the threshold in both u and v (2^-4 by default, src/Spline.h:496-500) is
// replaced by the two triangles of its corner points, and the nearer triangle
// hit in front of the current best gives t and the rectangle's centre as
// (u, v); otherwise it is halved along u or v alternately.  The box and
// triangle tests come from the un-vendored Ds library; the semantics chosen
// for them (also those of oracle/ds_compat) are a slab test clipped to the
// ray's [tMin, tMax], and the Moller--Trumbore ray/triangle test with
// |det| >= 1e-12 and t in [tMin, tMax].
struct RayI { V3<float> o, d; float tmin, tmax; };

inline bool box_hit(const Box& b, const RayI& r)  // Bounds3::intersect (Ds)
{
    float tMin = r.tmin, tMax = r.tmax;
    const float lo[3] = {b.lo.x, b.lo.y, b.lo.z}, hi[3] = {b.hi.x, b.hi.y, b.hi.z};
    const float o[3] = {r.o.x, r.o.y, r.o.z}, d[3] = {r.d.x, r.d.y, r.d.z};
    for (int i = 0; i < 3; i++)
    {
        const float inv = 1.0f / d[i];
        float t0 = (lo[i] - o[i]) * inv, t1 = (hi[i] - o[i]) * inv;
        if (t0 > t1) std::swap(t0, t1);
        if (t0 > tMin) tMin = t0;
        if (t1 < tMax) tMax = t1;
        if (tMin > tMax) return false;
    }
    return true;
}

inline bool triangle_hit(const RayI& r, V3<float> p0, V3<float> p1, V3<float> p2, float& t)  // triangle::intersect (Ds)
{
    const V3<float> e1 = p1 - p0, e2 = p2 - p0;
    const V3<float> pv = cross(r.d, e2);
    const float det = dot(e1, pv);
    if (det > -1e-12f && det < 1e-12f) return false;
    const float inv = 1.0f / det;
    const V3<float> sv = r.o - p0;
    const float u = dot(sv, pv) * inv;
    if (u < 0 || u > 1) return false;
    const V3<float> q = cross(sv, e1);
    const float v = dot(r.d, q) * inv;
    if (v < 0 || u + v > 1) return false;
    const float tt = dot(e2, q) * inv;
    if (tt < r.tmin || tt > r.tmax) return false;
    t = tt;
    return true;
}

// spline::slice on homogeneous points (src/Spline.h:324-364)
template<int stride> inline void slice_dc4(V4<float>* c, float u, float v)
{
    auto C = [&](int i) -> V4<float>& { return c[i * stride]; };
    const float iu = 1.0f - u;
    const float vv = (v - u) / iu;
    const float ivv = 1.0f - vv;
    V4<float> P5, P6, P8;
    P6 = u * C(1) + iu * C(0);
    P5 = u * C(2) + iu * C(1);
    C(2) = u * C(3) + iu * C(2);
    P8 = u * P5 + iu * P6;
    C(1) = u * C(2) + iu * P5;
    C(0) = u * C(1) + iu * P8;
    P6 = ivv * C(2) + vv * C(3);
    P5 = ivv * C(1) + vv * C(2);
    C(1) = ivv * C(0) + vv * C(1);
    P8 = ivv * P5 + vv * P6;
    C(2) = ivv * C(1) + vv * P5;
    C(3) = ivv * C(2) + vv * P8;
}

inline Box projected_box(const V4<float>* p)  // spline::boundingbox, src/Spline.h:398-414
{
    Box b;
    for (int i = 0; i < 16; i++) b.inflate(project(p[i]));
    return b;
}

bool subdiv_host(float& distance, V2<float>& uv, const RayI& ray, const V4<float> P[16], float threshold)
{
    struct State { V2<float> min, max; bool cutside; };
    if (!box_hit(projected_box(P), ray)) return false;
    std::vector<State> st;
    st.push_back({{0.0f, 0.0f}, {0.5f, 1.0f}, false});
    st.push_back({{0.5f, 0.0f}, {1.0f, 1.0f}, false});
    bool found = false;
    V4<float> sub[16];
    while (!st.empty())
    {
        const State e = st.back();
        st.pop_back();
        // spline::subpatchBoundingbox, src/Spline.h:464-478
        for (int i = 0; i < 16; i++) sub[i] = P[i];
        for (int i = 0; i < 4; i++) slice_dc4<4>(sub + i, e.min.y, e.max.y);
        for (int i = 0; i < 4; i++) slice_dc4<1>(sub + 4 * i, e.min.x, e.max.x);
        if (!box_hit(projected_box(sub), ray)) continue;
        const float x = 0.5f * (e.min.x + e.max.x);
        const float y = 0.5f * (e.min.y + e.max.y);
        if ((e.max.x - e.min.x) < threshold && (e.max.y - e.min.y) < threshold)
        {
            const V3<float> p00 = project(sub[0]), p10 = project(sub[3]), p01 = project(sub[12]),
                            p11 = project(sub[15]);
            float t = 0, t1 = 0;
            bool b0 = triangle_hit(ray, p10, p01, p00, t);
            const bool b1 = triangle_hit(ray, p01, p10, p11, t1);
            if (b0) { if (b1 && t1 < t) t = t1; }
            else if (b1) { t = t1; b0 = true; }
            if (b0 && t < distance)
            {
                distance = t;
                uv = {x, y};
                found = true;
            }
        }
        else if (e.cutside)
        {
            st.push_back({{e.min.x, e.min.y}, {x, e.max.y}, !e.cutside});
            st.push_back({{x, e.min.y}, {e.max.x, e.max.y}, !e.cutside});
        }
        else
        {
            st.push_back({{e.min.x, e.min.y}, {e.max.x, y}, !e.cutside});
            st.push_back({{e.min.x, y}, {e.max.x, e.max.y}, !e.cutside});
        }
    }
    return found;
}

// Newton polish of (u,v,t) on S(u,v) = o + t d in FP64.  Starts from the
// search result; returns false (and leaves the inputs) if it diverges or
// leaves the patch domain by more than 1e-6.
inline bool newton_polish(double& t, double& u, double& v, const Ray<double>& ray, const V4<double> P[16])
{
    double U = u, Vv = v, T = t;
    for (int it = 0; it < 12; it++)
    {
        V4<double> H = interpolate(P, U, Vv), Hu = derivativeU(P, U, Vv), Hv = derivativeV(P, U, Vv);
        double iw = 1.0 / H.w;
        V3<double> S {H.x * iw, H.y * iw, H.z * iw};
        V3<double> Su = (xyz(Hu) - Hu.w * S) * iw;
        V3<double> Sv = (xyz(Hv) - Hv.w * S) * iw;
        V3<double> F = S - (ray.o + T * ray.d);
        V3<double> c3 = -ray.d;
        // solve [Su Sv c3] x = -F by Cramer's rule
        double det = dot(Su, cross(Sv, c3));
        if (!(std::fabs(det) > 1e-300)) return false;
        V3<double> mF = -F;
        double du = dot(mF, cross(Sv, c3)) / det;
        double dv = dot(Su, cross(mF, c3)) / det;
        double dt = dot(Su, cross(Sv, mF)) / det;
        U += du; Vv += dv; T += dt;
        if (!std::isfinite(U + Vv + T)) return false;
        if (std::fabs(du) + std::fabs(dv) < 1e-15 && std::fabs(dt) < 1e-15 * std::fabs(T)) break;
    }
    if (U < -1e-6 || U > 1 + 1e-6 || Vv < -1e-6 || Vv > 1 + 1e-6 || T <= 0) return false;
    u = U; v = Vv; t = T;
    return true;
}

// ------------------------------------------------------------------- BVH --
static constexpr uint32_t EMPTY = 0xFFFFFFFFu;

struct Node { Box leftBox, rightBox; uint32_t left, right; };
struct Element { Box bounds; V3<float> centroid; uint32_t index; };

struct Hash
{
    uint32_t A = 31, B = 19, N = 0, mask = 0;
    std::vector<uint32_t> disp;
    uint32_t operator()(uint32_t key) const { return (A * key + B + disp[key & mask]) % N; }  // PerfectHashFunction.h:58-63
};

struct BVH
{
    std::vector<Node> nodes;
    std::vector<uint32_t> keys, indices, table;
    Hash hash;
    uint32_t elementsPerNode = 1;
    int splitMode = 0;  // 0: the reference's axis (an empty box: y); 1: longest axis of the centroid box

    // BVH::wrap, src/rt/BVH.cpp:82-108
    uint32_t wrap(Element* e, size_t count, uint32_t key)
    {
        if (count == 0) throw std::logic_error("invalid");
        Box box;
        size_t idx = indices.size();
        indices.resize(idx + count + 1);
        for (size_t i = 0; i < count; i++) { indices[idx + i] = e[i].index; box.inflate(e[i].bounds); }
        indices[idx + count] = EMPTY;
        keys.push_back(key);
        nodes.push_back({box, Box{}, EMPTY, uint32_t(idx)});
        return uint32_t(nodes.size() - 1);
    }
    // BVH::split, src/rt/BVH.cpp:40-80 (the split axis is computed from a box
    // that is never inflated, so with an empty box it is always y).
    uint32_t split(Element* e, size_t count, uint32_t key)
    {
        if (count <= elementsPerNode || (key & (1u << 31))) return wrap(e, count, key);
        Box box;  // never inflated in the reference (src/rt/BVH.cpp:46-52)
        if (splitMode == 1)
            for (size_t i = 0; i < count; i++) box.inflate(e[i].centroid);
        V3<float> v = box.size();
        int dim = v.z > v.y ? (v.x > v.z ? 0 : 2) : (v.x > v.y ? 0 : 1);
        size_t middle = count / 2;
        std::nth_element(e, e + middle, e + count, [=](const Element& a, const Element& b) {
            const float* ca = &a.centroid.x; const float* cb = &b.centroid.x;
            return ca[dim] < cb[dim];
        });
        keys.push_back(key);
        size_t idx = nodes.size();
        nodes.push_back({});
        uint32_t l = split(e, middle, key << 1);
        uint32_t r = split(e + middle, count - middle, (key << 1) ^ 1u);
        Node& node = nodes[idx];
        node.left = l; node.right = r;
        const Node& L = nodes[l]; const Node& Rn = nodes[r];
        node.leftBox = L.leftBox;
        node.rightBox = Rn.leftBox;
        if (L.left != EMPTY) node.leftBox.inflate(L.rightBox);
        if (Rn.left != EMPTY) node.rightBox.inflate(Rn.rightBox);
        return uint32_t(idx);
    }
    // BVH::build, src/rt/BVH.cpp:9-22 (link() only validates, :110-124)
    void build(std::vector<Element>& el, uint32_t perNode = 1)
    {
        keys.clear(); nodes.clear(); indices.clear();
        keys.reserve(2 * el.size()); nodes.reserve(2 * el.size()); indices.reserve(el.size());
        elementsPerNode = perNode;
        split(el.data(), el.size(), 1u);
    }
};

// ------------------------------------------------------------ perfect hash --
// Deterministic restatement of PerfectHashFunction::build,
// src/rt/PerfectHashFunction.cu:229-503.  Same table sizing, bucket capacity
// (4), coefficient draws (std::mt19937 seeded 42 and
// std::uniform_int_distribution<uint32_t>(0,n), gcd(n,A)=1), 32 attempts per
// bucket with displacement += rank+1, at most 16 trials growing the table by
// max(4, 0.05n).  The reference resolves the buckets of one size class
// concurrently with atomicInc races (:147-227), so its tables differ run to
// run.  Here a size class resolves in synchronous rounds: every unplaced
// bucket whose slots are all free (and pairwise distinct) bids for them; the
// lowest rank (position of the bucket id among the buckets of that size,
// ascending) wins a slot; a bucket that wins all of its slots is placed; the
// others add rank+1 to their displacement.  The CUDA build reproduces this
// exactly.
// Returns 0 on success, 1 on bucket overflow, 2 if no trial succeeded,
// 3 on a duplicate (the reference's injectivity check, :486-503).
int hash_build(Hash& h, std::vector<uint32_t>& table, const uint32_t* keys, uint32_t n, uint32_t* trials_used = nullptr)
{
    constexpr uint32_t kCap = 4;
    int s = int(n - 1) >> 1;
    if (s < 2) s = 2;
    const uint32_t displSize = std::bit_floor(uint32_t(s));
    h.disp.assign(displSize, 0);
    h.mask = displSize - 1;
    h.N = n;
    const uint32_t step = std::max<uint32_t>(4u, uint32_t(0.05f * float(n)));

    std::vector<uint32_t> bsize(displSize, 0), bkeys(size_t(displSize) * kCap, 0);
    for (uint32_t i = 0; i < n; i++)
    {
        uint32_t j = keys[i] & h.mask;
        if (bsize[j] >= kCap) return 1;
        bkeys[size_t(j) * kCap + bsize[j]++] = keys[i];
    }
    std::vector<uint32_t> classes[kCap + 1];
    for (uint32_t b = 0; b < displSize; b++) classes[bsize[b]].push_back(b);
    int maxSize = 0;
    for (int c = 0; c <= int(kCap); c++) if (!classes[c].empty()) maxSize = c;

    std::mt19937 mt(42);
    std::uniform_int_distribution<uint32_t> dist(0, n);
    bool ok = false;
    uint32_t trial = 0;
    for (trial = 0; trial < 16; trial++)
    {
        uint32_t cof;
        do
        {
            h.A = dist(mt);
            if (h.A == 0) h.A = 31;
            h.B = dist(mt);
            cof = std::gcd(n, h.A);
        } while (cof > 1);

        const uint32_t N = h.N;
        std::vector<uint8_t> occ(N, 0);
        std::vector<uint32_t> owner(N, EMPTY);
        std::fill(h.disp.begin(), h.disp.end(), 0u);
        uint32_t failures = 0;
        for (int c = maxSize; c >= 1; c--)
        {
            const auto& list = classes[c];
            const uint32_t m = uint32_t(list.size());
            std::vector<uint32_t> d(m, 0);
            std::vector<uint8_t> active(m, 1), feas(m, 0);
            std::vector<uint32_t> slots(size_t(m) * kCap);
            uint32_t remaining = m;
            for (int round = 0; round < 32 && remaining; round++)
            {
                for (uint32_t g = 0; g < m; g++)
                {
                    feas[g] = 0;
                    if (!active[g]) continue;
                    const uint32_t b = list[g];
                    bool f = true;
                    for (int k = 0; k < c; k++)
                    {
                        uint32_t key = bkeys[size_t(b) * kCap + k];
                        uint32_t sl = (h.A * key + h.B + d[g]) % N;
                        slots[size_t(g) * kCap + k] = sl;
                        if (occ[sl]) f = false;
                        for (int q = 0; q < k; q++) if (slots[size_t(g) * kCap + q] == sl) f = false;
                    }
                    if (f)
                    {
                        feas[g] = 1;
                        for (int k = 0; k < c; k++)
                        {
                            uint32_t sl = slots[size_t(g) * kCap + k];
                            owner[sl] = std::min(owner[sl], g);
                        }
                    }
                }
                for (uint32_t g = 0; g < m; g++)
                {
                    if (!active[g]) continue;
                    bool win = feas[g];
                    if (win)
                        for (int k = 0; k < c; k++)
                            if (owner[slots[size_t(g) * kCap + k]] != g) win = false;
                    if (win)
                    {
                        for (int k = 0; k < c; k++) occ[slots[size_t(g) * kCap + k]] = 1;
                        h.disp[list[g]] = d[g];
                        active[g] = 0;
                        remaining--;
                    }
                    else
                        d[g] += g + 1;
                }
                for (uint32_t g = 0; g < m; g++)
                    if (feas[g])
                        for (int k = 0; k < c; k++) owner[slots[size_t(g) * kCap + k]] = EMPTY;
            }
            failures += remaining;
        }
        if (failures == 0) { ok = true; break; }
        h.N = h.N + step;
    }
    if (trials_used) *trials_used = trial;
    if (!ok) return 2;
    // injectivity check and table fill (src/rt/BVH.cpp:24-38)
    table.assign(h.N, EMPTY);
    for (uint32_t i = 0; i < n; i++)
    {
        uint32_t v = h(keys[i]);
        if (table[v] != EMPTY) return 3;
        table[v] = i;
    }
    return 0;
}

// -------------------------------------------------------------- traversal --
// _node_intersect, src/rt/BVH.h:147-176
template<class R> inline bool node_intersect(R& tMin, R& tMax, const Box& b, V3<R> o, V3<R> inv)
{
    tMin = -std::numeric_limits<R>::infinity();
    tMax = std::numeric_limits<R>::infinity();
    const R O[3] {o.x, o.y, o.z}, I[3] {inv.x, inv.y, inv.z};
    const float lo[3] {b.lo.x, b.lo.y, b.lo.z}, hi[3] {b.hi.x, b.hi.y, b.hi.z};
    for (int i = 0; i < 3; i++)
    {
        int s = std::signbit(I[i]);
        R t[2];
        t[0] = (R(lo[i]) - O[i]) * I[i];
        t[1] = (R(hi[i]) - O[i]) * I[i];
        if (t[0 + s] > tMin) tMin = t[0 + s];
        if (t[1 - s] < tMax) tMax = t[1 - s];
    }
    return tMin < tMax && tMax > R(0.0001f);
}

struct TraversalStats { uint64_t nodes = 0, leaves = 0, hashLookups = 0; };

// BVH::hashIntersect (closest / any), src/rt/BVH.h:178-350.  `limit` is the
// current best t (closest) or ray.max (any); `fn` returns true for a hit and
// may lower `limit` (closest) / ends the walk (any).
template<class R, bool kAny, class F>
bool hash_intersect(const BVH& bvh, const Ray<R>& ray, R& limit, F&& fn, TraversalStats* ts)
{
    const V3<R> inv {R(1) / ray.d.x, R(1) / ray.d.y, R(1) / ray.d.z};
    const Node* node = bvh.nodes.data();
    uint32_t key = 1, postponed = 0;
    bool result = false;
    for (;;)
    {
        if (node->left != EMPTY)
        {
            if (ts) ts->nodes++;
            R L0, L1, R0, R1;
            bool iL = node_intersect(L0, L1, node->leftBox, ray.o, inv) && L0 < limit;
            bool iR = node_intersect(R0, R1, node->rightBox, ray.o, inv) && R0 < limit;
            if (iL || iR) postponed <<= 1;
            if (iL)
            {
                if (iR)
                {
                    postponed |= 1;
                    if (L0 < R0) { key = key << 1; node = bvh.nodes.data() + node->left; }
                    else { key = (key << 1) ^ 1u; node = bvh.nodes.data() + node->right; }
                }
                else { key = key << 1; node = bvh.nodes.data() + node->left; }
                continue;
            }
            else if (iR) { key = (key << 1) ^ 1u; node = bvh.nodes.data() + node->right; continue; }
        }
        else
        {
            if (ts) ts->leaves++;
            uint32_t i = node->right;
            while (bvh.indices[i] != EMPTY)
            {
                bool b = fn(bvh.indices[i++]);
                if (kAny && b) return true;
                result |= b;
            }
        }
        if (!postponed) break;
        int levels = std::countr_zero(postponed);
        postponed >>= levels;
        key = (key >> levels) ^ 1u;
        postponed ^= 1;
        if (ts) ts->hashLookups++;
        node = bvh.nodes.data() + bvh.table[bvh.hash(key)];
    }
    return kAny ? false : result;
}

// ------------------------------------------------------------------ scene --
struct Material { V3<float> diffuse, specular; float metalness, roughness; };  // src/rt/Scene.h:79-95
struct Light                                                                     // src/rt/Scene.h:47-77
{
    V3<float> color; float strength; V3<float> position; float range; V3<float> direction; float angle;
    bool isDirectional() const { return angle < 0.01f; }
    bool isPoint() const { return angle > 1.57f; }
};

struct Surface
{
    std::vector<V4<float>> points;
    std::vector<uint32_t> indices;
    BVH bvh;
    uint32_t patchCount() const { return uint32_t(indices.size() / 16); }
    void patch(uint32_t i, V4<float> out[16]) const
    {
        for (int k = 0; k < 16; k++) out[k] = points[indices[16 * i + k]];
    }
};

struct Object
{
    int surface;
    float l2w[16], w2l[16];
    Material material;
    std::vector<uint32_t> patchMaterial;  // optional per-patch material index
    std::vector<Material> materials;
};

struct Scene
{
    std::vector<Surface> surfaces;
    std::vector<Object> objects;
    std::vector<Light> lights;
    BVH top;
    V3<float> background {0.1f, 0.1f, 0.1f}, ambient {0.1f, 0.1f, 0.1f};
    int built = 0;

    // BezierSurface::buildBVH, src/rt/Primitive.cu:199-220
    static void build_surface_bvh(Surface& s)
    {
        std::vector<Element> el(s.patchCount());
        for (uint32_t i = 0; i < el.size(); i++)
        {
            Element& e = el[i];
            e.bounds = Box{};
            e.centroid = {0, 0, 0};
            e.index = i;
            const float inv = 1.0f / 16.0f;
            for (int j = 0; j < 16; j++)
            {
                V3<float> p = project(s.points[s.indices[16 * i + j]]);
                e.bounds.inflate(p);
                e.centroid = e.centroid + inv * p;
            }
        }
        s.bvh.build(el, 1);
    }
    // Scene::buildBVH, src/rt/Scene.cu:218-232 with BezierSurface::bounds(M),
    // src/rt/Primitive.cu:172-179
    void build_top()
    {
        std::vector<Element> el(objects.size());
        for (uint32_t i = 0; i < el.size(); i++)
        {
            const Object& ob = objects[i];
            const Surface& s = surfaces[ob.surface];
            M4<float> M = load_m4<float>(ob.l2w);
            Box b;
            for (uint32_t idx : s.indices) b.inflate(project(mul(M, s.points[idx])));
            el[i].index = i;
            el[i].bounds = b;
            el[i].centroid = b.center();
        }
        top.build(el, 1);
    }
    int splitMode = 0;
    int build()
    {
        for (auto& s : surfaces)
        {
            s.bvh.splitMode = splitMode;
            build_surface_bvh(s);
            int e = hash_build(s.bvh.hash, s.bvh.table, s.bvh.keys.data(), uint32_t(s.bvh.keys.size()));
            if (e) return 10 + e;
        }
        if (objects.empty()) return 1;
        top.splitMode = splitMode;
        build_top();
        int e = hash_build(top.hash, top.table, top.keys.data(), uint32_t(top.keys.size()));
        if (e) return 20 + e;
        built = 1;
        return 0;
    }
};

struct Hit { int object = -1; uint32_t patch = 0; float t = INFINITY; float u = 0, v = 0; };

struct QueryOpts { int method = kClipHost; float tol = 0x1p-12f; };

struct Counters { TraversalStats ts; ClipStats cs; uint64_t candidates = 0; };

// Context::intersect (closest), src/rt/RayTracer.cu:295-349 /
// CPURayTracer::intersect, src/rt/CPURayTracer.cpp:221-258, with
// rt::intersect(const BezierSurface&,...), src/rt/Primitive.cu:222-248.
// FP32 reference semantics.
inline int scene_intersect(const Scene& sc, Hit& hit0, const Ray<float>& ray0, const QueryOpts& q, Counters* cn)
{
    int nearest = -1;
    float limit = hit0.t;
    auto fn = [&](uint32_t i) -> bool {
        const Object& ob = sc.objects[i];
        const Surface& s = sc.surfaces[ob.surface];
        M4<float> M_1 = load_m4<float>(ob.w2l);
        Ray<float> lr;
        V4<float> o4 {ray0.o.x, ray0.o.y, ray0.o.z, 1.0f};
        lr.o = project(mul(M_1, o4));
        lr.d = mul(upper3(M_1), ray0.d);
        float d = length(lr.d);
        lr.max = ray0.max * d;
        d = 1 / d;
        lr.d = lr.d * d;
        float lt = lr.max;
        Ray<double> lr64;
        const bool use64 = g_graze64Ray && q.method == kClipGraze;
        if (use64)
        {
            M4<double> M64 = load_m4<double>(ob.w2l);
            V4<double> o64 {double(ray0.o.x), double(ray0.o.y), double(ray0.o.z), 1.0};
            lr64.o = project(mul(M64, o64));
            lr64.d = mul(upper3(M64), cast3<double>(ray0.d));
            lr64.d = lr64.d * (1.0 / length(lr64.d));
        }
        uint32_t lpatch = 0; V2<float> luv {0, 0};
        auto leaf = [&](uint32_t p) -> bool {
            if (cn) cn->candidates++;
            V4<float> P[16];
            s.patch(p, P);
            float dist = lt; V2<float> uv = luv;
            if (intersect_patch<float>(dist, uv, lr, P, q.tol, q.method, cn ? &cn->cs : nullptr,
                                       use64 ? &lr64 : nullptr))
            {
                lpatch = p; lt = dist; luv = uv;
                return true;
            }
            return false;
        };
        bool b = hash_intersect<float, false>(s.bvh, lr, lt, leaf, cn ? &cn->ts : nullptr);
        if (b)
        {
            float t = lt * d;
            if (t < limit)
            {
                hit0.u = luv.x; hit0.v = luv.y; hit0.patch = lpatch; hit0.object = int(i);
                hit0.t = t; limit = t; nearest = int(i);
                return true;
            }
        }
        return false;
    };
    hash_intersect<float, false>(sc.top, ray0, limit, fn, cn ? &cn->ts : nullptr);
    return nearest;
}

// Context::intersect (any hit), src/rt/RayTracer.cu:351-383 with
// rt::intersect(const BezierSurface&, const Ray&), src/rt/Primitive.cu:250-268
inline bool scene_occluded(const Scene& sc, const Ray<float>& ray0, const QueryOpts& q, Counters* cn)
{
    float limit = ray0.max;
    auto fn = [&](uint32_t i) -> bool {
        const Object& ob = sc.objects[i];
        const Surface& s = sc.surfaces[ob.surface];
        M4<float> M_1 = load_m4<float>(ob.w2l);
        Ray<float> lr;
        V4<float> o4 {ray0.o.x, ray0.o.y, ray0.o.z, 1.0f};
        lr.o = project(mul(M_1, o4));
        lr.d = mul(upper3(M_1), ray0.d);
        float d = length(lr.d);
        lr.max = ray0.max * d;
        d = 1 / d;
        lr.d = lr.d * d;
        float llimit = lr.max;
        auto leaf = [&](uint32_t p) -> bool {
            if (cn) cn->candidates++;
            V4<float> P[16];
            s.patch(p, P);
            float dist = lr.max; V2<float> uv {0, 0};
            return intersect_patch<float>(dist, uv, lr, P, q.tol, q.method, cn ? &cn->cs : nullptr);
        };
        return hash_intersect<float, true>(s.bvh, lr, llimit, leaf, cn ? &cn->ts : nullptr);
    };
    return hash_intersect<float, true>(sc.top, ray0, limit, fn, cn ? &cn->ts : nullptr);
}

// FP64 "true t": the same two-level traversal and search in double with a
// tight tolerance, followed by a Newton polish.  The ray is the FP32 input
// promoted; hit.t is the ray parameter of the polished root.  exactHull: the
// search clips with the true convex hull (hull_range_exact) instead of the
// reference's scan.
inline int scene_intersect_f64(const Scene& sc, double& t_out, double& u_out, double& v_out, uint32_t& patch_out,
                               const Ray<float>& rayf, double tol, bool exactHull = false)
{
    Ray<double> ray0 {cast3<double>(rayf.o), cast3<double>(rayf.d), double(rayf.max)};
    int nearest = -1;
    double limit = ray0.max;
    auto fn = [&](uint32_t i) -> bool {
        const Object& ob = sc.objects[i];
        const Surface& s = sc.surfaces[ob.surface];
        M4<double> M_1 = load_m4<double>(ob.w2l);
        Ray<double> lr;
        V4<double> o4 {ray0.o.x, ray0.o.y, ray0.o.z, 1.0};
        lr.o = project(mul(M_1, o4));
        lr.d = mul(upper3(M_1), ray0.d);
        double d = length(lr.d);
        lr.max = ray0.max * d;
        d = 1 / d;
        lr.d = lr.d * d;
        double lt = lr.max;
        uint32_t lpatch = 0; double lu = 0, lv = 0;
        auto leaf = [&](uint32_t p) -> bool {
            V4<float> Pf[16]; V4<double> P[16];
            s.patch(p, Pf);
            for (int k = 0; k < 16; k++) P[k] = cast4<double>(Pf[k]);
            double dist = INFINITY; V2<double> uv {0, 0};
            // every root of the patch is visited; keep the closest polished one
            bool any = false;
            double best = lt, bu = 0, bv = 0;
            auto onHit = [&](V2<double> e) -> bool {
                V3<double> V = project(interpolate(P, e.x, e.y)) - lr.o;
                double t = length(V);
                if (dot(V, lr.d) <= 0) return false;
                double uu = e.x, vv = e.y, tt = t;
                newton_polish(tt, uu, vv, lr, P);
                if (tt < best) { best = tt; bu = uu; bv = vv; any = true; return true; }
                return false;
            };
            const V3<double> dd = lr.d;
            const V3<double> axis0 = versor(cross(dd, dd + V3<double>{0, 0, 8}));
            const V3<double> axis1 = versor(cross(dd, axis0));
            V2<double> net[16];
            for (int k = 0; k < 16; k++)
            {
                V3<double> Q = xyz(P[k]);
                net[k] = {dot(axis0, Q - lr.o), dot(axis1, Q - lr.o)};
            }
            if (exactHull) clip2d_host<double, decltype(onHit), true>(onHit, net, tol, nullptr);
            else clip2d_host(onHit, net, tol, nullptr);
            (void)dist; (void)uv;
            if (any) { lt = best; lpatch = p; lu = bu; lv = bv; }
            return any;
        };
        bool b = hash_intersect<double, false>(s.bvh, lr, lt, leaf, nullptr);
        if (b)
        {
            double t = lt * d;
            if (t < limit) { limit = t; nearest = int(i); t_out = t; u_out = lu; v_out = lv; patch_out = lpatch; return true; }
        }
        return false;
    };
    hash_intersect<double, false>(sc.top, ray0, limit, fn, nullptr);
    return nearest;
}

// ----------------------------------------------------------------- shading --
// src/rt/PBR.h:21-176, src/rt/PBR.cu:9-64
constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.318309886183790671538f;

inline bool lightVector(float& d, V3<float>& L, V3<float> P, const Light& light)  // PBR.cu:198-220
{
    if (light.isDirectional()) { L = -light.direction; d = INFINITY; return true; }
    L = light.position - P;
    d = length(L);
    if (d < 1e-14f || (light.range > 0 && d > light.range)) return false;
    L = L * (1 / d);
    if (light.isPoint()) return true;
    float DL = dot(light.direction, L);
    return DL < 0 && light.angle > 2 * std::acos(DL);
}
inline V3<float> lightColor(float d, const Light& light)  // PBR.cu:222-242
{
    if (light.isDirectional()) return light.color;
    float range = light.range, f;
    if (range == 0) { f = 1 / d; f *= f; }
    else { f = d / range; f = 1 + f * (f - 2); }
    return light.color * f;
}
inline V3<float> schlick(V3<float> f0, float dotLH)  // PBR.h:53-61
{
    float b = 1 - dotLH, b2 = b * b;
    return f0 + (V3<float>{1, 1, 1} - f0) * (b2 * b2 * b);
}
inline float G1(float dotNX, float k) { return dotNX / (dotNX * (1 - k) + k); }  // PBR.h:72-76
inline float Gsmith(float dotNL, float dotNV, float r)                            // PBR.h:78-85
{
    const float r1 = r + 1;
    const float k = float(double(r1 * r1) * 0.125);
    return G1(dotNL, k) * G1(dotNV, k);
}
inline float Dggx(float dotNH, float r)  // PBR.h:87-96
{
    r = std::fmax(r, 1e-3f);
    float a = r * r, a2 = a * a;
    float d = dotNH * dotNH * (a2 - 1) + 1;
    return a2 / (kPi * d * d);
}
inline float BRDF_microfacet(float dotNV, float dotNL, float dotNH, float r)  // PBR.h:98-107
{
    return Gsmith(dotNL, dotNV, r) * Dggx(dotNH, r) / (4 * dotNL * dotNV);
}
inline V3<float> BRDF_specular(float dotHL, float dotHN, float dotNV, float dotNL, float r, V3<float> f0)  // PBR.h:131-141
{
    return schlick(f0, dotHL) * BRDF_microfacet(dotNV, dotNL, dotHN, r);
}

struct Camera { float rot[4]; float pos[3]; float scale[3]; float fovy; };

struct RenderOpts { int depth = 1; float eps = 1e-4f; int method = kClipHost; float tol = 0x1p-12f; int mc = 0; };

// Philox4x32-10 (Salmon, Moraes, Dror & Shaw, SC 2011), the product's
// counter-based generator for the Monte-Carlo path.
inline void philox(uint32_t c[4], uint32_t k0, uint32_t k1)
{
    for (int r = 0; r < 10; r++)
    {
        const uint64_t p0 = uint64_t(0xD2511F53u) * c[0], p1 = uint64_t(0xCD9E8D57u) * c[2];
        const uint32_t hi0 = uint32_t(p0 >> 32), lo0 = uint32_t(p0), hi1 = uint32_t(p1 >> 32), lo1 = uint32_t(p1);
        const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}
inline float u01(uint32_t x) { return float(x >> 8) * 0x1p-24f + 0x1p-25f; }

// sRGB encode of a [0,1] value to 8 bits (the reference's pack_sRGB comes
// from the un-vendored Ds library; IEC 61966-2-1 is used here).
inline uint32_t srgb8(float c)
{
    double x = c <= 0.0031308f ? 12.92 * c : 1.055 * std::pow(double(c), 1.0 / 2.4) - 0.055;
    int v = int(x * 255.0 + 0.5);
    return uint32_t(std::min(255, std::max(0, v)));
}

struct Renderer
{
    const Scene& sc;
    RenderOpts op;
    QueryOpts q;
    M4<float> cameraToWorld;
    V3<float> camPos;
    V2<float> tl;
    float half_dx, half_dy;
    uint32_t w, h;

    Renderer(const Scene& s, const Camera& cam, uint32_t W, uint32_t H, const RenderOpts& o) : sc(s), op(o), w(W), h(H)
    {
        q.method = o.method; q.tol = o.tol;
        // Transform::matrix() = T*R*S; rotation matrix as src/AlignedTypes.h:99-115
        float i = cam.rot[0], j = cam.rot[1], k = cam.rot[2], r = cam.rot[3];
        float ii = 2 * i * i, ij = 2 * i * j, ik = 2 * i * k, jj = 2 * j * j, jk = 2 * j * k, kk = 2 * k * k,
              ri = 2 * r * i, rj = 2 * r * j, rk = 2 * r * k;
        V3<float> c0 {1 - jj - kk, ij + rk, ik - rj}, c1 {ij - rk, 1 - ii - kk, jk + ri}, c2 {ik + rj, jk - ri, 1 - ii - jj};
        c0 = c0 * cam.scale[0]; c1 = c1 * cam.scale[1]; c2 = c2 * cam.scale[2];
        cameraToWorld = {{{c0.x, c0.y, c0.z, 0}, {c1.x, c1.y, c1.z, 0}, {c2.x, c2.y, c2.z, 0},
                          {cam.pos[0], cam.pos[1], cam.pos[2], 1}}};
        camPos = {cam.pos[0], cam.pos[1], cam.pos[2]};
        // RayTracer::render camera set-up, src/rt/RayTracer.cu:152-163
        float halfHeight = std::tan(0.5f * cam.fovy);
        half_dy = halfHeight / float(h);
        half_dx = half_dy;
        tl.x = -half_dx * float(w - 1);
        tl.y = halfHeight - half_dy;
    }
    // pixelRayDirection, src/rt/CPURayTracer.h:96-107
    V3<float> pixelRayDirection(float x, float y) const
    {
        V4<float> P {tl.x + half_dx * (2 * x), tl.y - half_dy * (2 * y), -1.0f, 1.0f};
        P = mul(cameraToWorld, P);
        return versor(project(P) - camPos);
    }
    const Material& material(const Hit& hit) const
    {
        const Object& ob = sc.objects[hit.object];
        if (!ob.patchMaterial.empty()) return ob.materials[ob.patchMaterial[hit.patch]];
        return ob.material;
    }
    // CPURayTracer::trace / closestHit (non Monte-Carlo),
    // src/rt/CPURayTracer.cpp:199-219, 291-440
    V3<float> trace(const Ray<float>& ray, V3<float> att, int depth, Counters* cn, uint64_t* nrays,
                    uint32_t imageSample = 0) const
    {
        if (nrays) nrays[depth == op.depth ? 0 : 1]++;
        Hit hit; hit.t = ray.max;
        int nearest = scene_intersect(sc, hit, ray, q, cn);
        if (nearest < 0) return att * sc.background;
        const Object& ob = sc.objects[nearest];
        const Material& m = material(hit);
        M4<float> M_1 = load_m4<float>(ob.w2l);
        const V3<float> diffuse = (1 - m.metalness) * (m.diffuse * kInvPi);
        V3<float> color = sc.ambient * diffuse;
        V3<float> V = -ray.d;
        V4<float> P16[16];
        sc.surfaces[ob.surface].patch(hit.patch, P16);
        V3<float> N = versor(patch_normal<float>(P16, hit.u, hit.v));  // src/rt/Primitive.cu:270-275
        N = versor(mul(transposed(upper3(M_1)), N));
        float dotNV = dot(N, V);
        if (dotNV < 0) { N = -N; dotNV = -dotNV; }
        V3<float> P = ray.o + hit.t * ray.d;
        for (const Light& light : sc.lights)
        {
            V3<float> L; float d;
            if (!lightVector(d, L, P, light)) continue;
            const float dotNL = dot(N, L);
            if (dotNL < 1e-14f) continue;
            Ray<float> r1 {P + op.eps * L, L, d};
            if (nrays) nrays[2]++;
            if (scene_occluded(sc, r1, q, cn)) continue;
            V3<float> H = versor(L + V);
            float dotHN = dot(H, N), dotHL = dot(H, L);
            V3<float> I = lightColor(d, light);
            color = color + (I * dotNL) * (diffuse + m.metalness * BRDF_specular(dotHL, dotHN, dotNV, dotNL, m.roughness, m.specular));
        }
        color = color * (kPi * att);
        if (depth <= 0) return color;
        if (op.mc)
        {
            // the sampled path, src/rt/RayTracer.cu:473-521; microfacet, src/rt/PBR.h:165-176
            uint32_t c[4] = {imageSample, uint32_t(depth), 0u, 0u};
            philox(c, 42u, 0u);
            const float x = u01(c[0]), y = u01(c[1]);
            const float alpha = m.roughness * m.roughness;
            const float theta = std::atan2(alpha * std::sqrt(x), std::sqrt(1.0f - x)), phi = 2.0f * kPi * y;
            const V3<float> ts = versor(cross(N, V)), tp = versor(cross(N, ts));
            const float st = std::sin(theta), ct = std::cos(theta), sp = std::sin(phi), cp = std::cos(phi);
            const V3<float> M = versor((st * cp) * ts + (st * sp) * tp + ct * N);
            const float dotMV = dot(M, V);
            const V3<float> reflectance = schlick(m.specular, dotMV);
            const V3<float> R = (-V) - (2 * (-dotMV)) * M;
            const float dotMN = dot(M, N), dotNR = dot(N, R);
            if (dotNR < 1e-14f) return color;
            const float g = Gsmith(dotNR, dotNV, m.roughness) * dotMV / (dotNV * dotMN);
            const V3<float> kd = m.diffuse * kInvPi, ks = reflectance * g;
            const V3<float> a = att * (kd * (1.0f - m.metalness) + ks * m.metalness);
            if (vmax(a) > 0x1p-8f)
            {
                Ray<float> r {P + op.eps * R, R, INFINITY};
                color = color + trace(r, a, depth - 1, cn, nrays, imageSample);
            }
            return color;
        }
        V3<float> reflectance = schlick(m.specular, dotNV);
        V3<float> R = (-V) - (2 * (-dotNV)) * N;
        float g = Gsmith(dotNV, dotNV, m.roughness);
        V3<float> brdf = (dotNV * (diffuse + m.metalness * (reflectance * g))) * ((1 - m.roughness) * (1 - m.roughness));
        V3<float> a = att * brdf;
        if (vmax(a) > 0x1p-8f)
        {
            Ray<float> r {P + op.eps * R, R, INFINITY};
            color = color + trace(r, a, depth - 1, cn, nrays);
        }
        return color;
    }
};

}  // namespace ora

// =================================================================== C API --
using namespace ora;

static void unpack_ray(const float* rays, uint64_t n, uint64_t i, Ray<float>& r)
{
    r.o = {rays[0 * n + i], rays[1 * n + i], rays[2 * n + i]};
    r.d = {rays[3 * n + i], rays[4 * n + i], rays[5 * n + i]};
    r.max = rays[6 * n + i];
}

template<class F> static void parallel_for(uint64_t n, int nthreads, F&& f)
{
    if (nthreads <= 1 || n < 64) { for (uint64_t i = 0; i < n; i++) f(i, 0); return; }
    std::atomic<uint64_t> next {0};
    const uint64_t chunk = 64;
    std::vector<std::thread> th;
    for (int w = 0; w < nthreads; w++)
        th.emplace_back([&, w] {
            for (;;)
            {
                uint64_t b = next.fetch_add(chunk);
                if (b >= n) return;
                uint64_t e = std::min(n, b + chunk);
                for (uint64_t i = b; i < e; i++) f(i, w);
            }
        });
    for (auto& t : th) t.join();
}

extern "C" {

int ora_version(void) { return 3; }

void* ora_scene_new(void) { return new Scene(); }
void ora_scene_free(void* s) { delete static_cast<Scene*>(s); }

int ora_scene_add_surface(void* s_, const float* points4, uint32_t npoints, const uint32_t* indices, uint32_t nindices)
{
    auto* s = static_cast<Scene*>(s_);
    if (nindices == 0 || nindices % 16) return -1;
    for (uint32_t i = 0; i < nindices; i++) if (indices[i] >= npoints) return -2;
    Surface sf;
    sf.points.resize(npoints);
    std::memcpy(sf.points.data(), points4, sizeof(float) * 4 * npoints);
    sf.indices.assign(indices, indices + nindices);
    s->surfaces.push_back(std::move(sf));
    return int(s->surfaces.size() - 1);
}

// material8 = diffuse[3], specular[3], metalness, roughness
int ora_scene_add_object(void* s_, int surface, const float* l2w, const float* w2l, const float* material8,
                         const uint32_t* patch_material, const float* materials8, uint32_t nmaterials)
{
    auto* s = static_cast<Scene*>(s_);
    if (surface < 0 || surface >= int(s->surfaces.size())) return -1;
    Object ob;
    ob.surface = surface;
    std::memcpy(ob.l2w, l2w, sizeof ob.l2w);
    std::memcpy(ob.w2l, w2l, sizeof ob.w2l);
    auto mat = [](const float* m) {
        return Material{{m[0], m[1], m[2]}, {m[3], m[4], m[5]}, m[6], m[7]};
    };
    ob.material = mat(material8);
    if (patch_material && materials8 && nmaterials)
    {
        uint32_t P = s->surfaces[surface].patchCount();
        ob.patchMaterial.assign(patch_material, patch_material + P);
        for (uint32_t i = 0; i < nmaterials; i++) ob.materials.push_back(mat(materials8 + 8 * i));
        for (uint32_t i = 0; i < P; i++) if (ob.patchMaterial[i] >= nmaterials) return -2;
    }
    s->objects.push_back(std::move(ob));
    return int(s->objects.size() - 1);
}

// light12 = color[3], strength, position[3], range, direction[3], angle
int ora_scene_set_lights(void* s_, const float* lights12, uint32_t n)
{
    auto* s = static_cast<Scene*>(s_);
    s->lights.clear();
    for (uint32_t i = 0; i < n; i++)
    {
        const float* l = lights12 + 12 * i;
        s->lights.push_back({{l[0], l[1], l[2]}, l[3], {l[4], l[5], l[6]}, l[7], {l[8], l[9], l[10]}, l[11]});
    }
    return 0;
}

void ora_scene_set_env(void* s_, const float* bg3, const float* amb3)
{
    auto* s = static_cast<Scene*>(s_);
    s->background = {bg3[0], bg3[1], bg3[2]};
    s->ambient = {amb3[0], amb3[1], amb3[2]};
}

int ora_scene_build(void* s_) { return static_cast<Scene*>(s_)->build(); }
void ora_scene_set_split(void* s_, int mode) { static_cast<Scene*>(s_)->splitMode = mode; }
// Philox4x32-10 of the Monte-Carlo path, exposed for known-answer tests.
void ora_philox(uint32_t* ctr4, uint32_t k0, uint32_t k1) { philox(ctr4, k0, k1); }
// the grazing margin of kClipGraze (process-wide; not thread-safe against running queries)
void ora_set_graze_sin(float s) { g_grazeSin = s; }
// the near-grazing test of CLIP_GRAZE64 (process-wide; see grazing())
void ora_set_graze_mode(int m) { g_grazeMode = m; }
// CLIP_GRAZE64: project a near-grazing candidate from the object-space ray
// computed in double (1, the default) or from the FP32 one (0)
void ora_set_graze64_ray(int m) { g_graze64Ray = m; }

static const BVH* pick_bvh(const Scene* s, int which)
{
    if (which < 0) return &s->top;
    if (which >= int(s->surfaces.size())) return nullptr;
    return &s->surfaces[which].bvh;
}

// sizes[0..4] = nodes, indices, tableSize, displSize, keys
int ora_bvh_sizes(void* s_, int which, uint32_t* sizes)
{
    const BVH* b = pick_bvh(static_cast<Scene*>(s_), which);
    if (!b) return -1;
    sizes[0] = uint32_t(b->nodes.size());
    sizes[1] = uint32_t(b->indices.size());
    sizes[2] = uint32_t(b->table.size());
    sizes[3] = uint32_t(b->hash.disp.size());
    sizes[4] = uint32_t(b->keys.size());
    return 0;
}

// nodes: 14 u32 per node = leftBox(lo,hi) rightBox(lo,hi) as float bits, left, right
// params[0..3] = A, B, N, mask
int ora_bvh_export(void* s_, int which, uint32_t* nodes, uint32_t* keys, uint32_t* indices, uint32_t* table,
                   uint32_t* disp, uint32_t* params)
{
    const BVH* b = pick_bvh(static_cast<Scene*>(s_), which);
    if (!b) return -1;
    for (size_t i = 0; i < b->nodes.size(); i++)
    {
        const Node& n = b->nodes[i];
        float f[12] = {n.leftBox.lo.x, n.leftBox.lo.y, n.leftBox.lo.z, n.leftBox.hi.x, n.leftBox.hi.y, n.leftBox.hi.z,
                       n.rightBox.lo.x, n.rightBox.lo.y, n.rightBox.lo.z, n.rightBox.hi.x, n.rightBox.hi.y, n.rightBox.hi.z};
        std::memcpy(nodes + 14 * i, f, sizeof f);
        nodes[14 * i + 12] = n.left;
        nodes[14 * i + 13] = n.right;
    }
    std::copy(b->keys.begin(), b->keys.end(), keys);
    std::copy(b->indices.begin(), b->indices.end(), indices);
    std::copy(b->table.begin(), b->table.end(), table);
    std::copy(b->hash.disp.begin(), b->hash.disp.end(), disp);
    params[0] = b->hash.A; params[1] = b->hash.B; params[2] = b->hash.N; params[3] = b->hash.mask;
    return 0;
}

// Stand-alone perfect hash over arbitrary keys.  out_params = A, B, N, mask, trials.
int ora_hash_build(const uint32_t* keys, uint32_t n, uint32_t* out_params, uint32_t* disp, uint32_t disp_cap,
                   uint32_t* table, uint32_t table_cap)
{
    Hash h; std::vector<uint32_t> t; uint32_t trials = 0;
    int e = hash_build(h, t, keys, n, &trials);
    out_params[0] = h.A; out_params[1] = h.B; out_params[2] = h.N; out_params[3] = h.mask; out_params[4] = trials;
    if (e) return e;
    if (h.disp.size() > disp_cap || t.size() > table_cap) return -1;
    std::copy(h.disp.begin(), h.disp.end(), disp);
    std::copy(t.begin(), t.end(), table);
    return 0;
}

// rays: SoA (7, n) = ox oy oz dx dy dz tmax.  precision: 0 FP32 reference,
// 1 FP32 + FP64 Newton polish of the winning hit, 2 FP64 search + polish.
// out_f: (3, n) = t u v; out_i: (2, n) = patch object (-1 = miss).
// counters (optional, 8 u64): nodes, leaves, hash lookups, candidates,
// clip iterations, pushes, max depth, stack overflows.
int ora_intersect(void* s_, const float* rays, uint64_t n, int method, int precision, float tol, double tol64,
                  int any_hit, float* out_f, int32_t* out_i, uint64_t* counters, int nthreads)
{
    auto* s = static_cast<Scene*>(s_);
    if (!s->built) return -1;
    std::vector<Counters> cn(std::max(1, nthreads));
    QueryOpts q; q.method = method; q.tol = tol;
    parallel_for(n, nthreads, [&](uint64_t i, int w) {
        Ray<float> r; unpack_ray(rays, n, i, r);
        Counters* c = counters ? &cn[w] : nullptr;
        if (any_hit)
        {
            bool occ = scene_occluded(*s, r, q, c);
            out_i[i] = occ ? 0 : -1; out_i[n + i] = occ ? 0 : -1;
            out_f[i] = 0; out_f[n + i] = 0; out_f[2 * n + i] = 0;
            return;
        }
        if (precision == 2)
        {
            double t = 0, u = 0, v = 0; uint32_t p = 0;
            int ob = scene_intersect_f64(*s, t, u, v, p, r, tol64, method == kClipExactHull);
            out_f[i] = ob >= 0 ? float(t) : INFINITY;
            out_f[n + i] = float(u); out_f[2 * n + i] = float(v);
            out_i[i] = ob >= 0 ? int32_t(p) : -1; out_i[n + i] = ob;
            return;
        }
        Hit hit; hit.t = r.max;
        int ob = scene_intersect(*s, hit, r, q, c);
        if (ob >= 0 && precision == 1)
        {
            const Object& o = s->objects[ob];
            const Surface& sf = s->surfaces[o.surface];
            M4<double> M_1 = load_m4<double>(o.w2l);
            Ray<double> lr;
            V4<double> o4 {double(r.o.x), double(r.o.y), double(r.o.z), 1.0};
            lr.o = project(mul(M_1, o4));
            lr.d = mul(upper3(M_1), cast3<double>(r.d));
            double sc = length(lr.d);
            lr.d = lr.d * (1.0 / sc);
            V4<float> Pf[16]; V4<double> P[16];
            sf.patch(hit.patch, Pf);
            for (int k = 0; k < 16; k++) P[k] = cast4<double>(Pf[k]);
            double t = double(hit.t) * sc, u = hit.u, v = hit.v;
            if (newton_polish(t, u, v, lr, P)) { hit.t = float(t / sc); hit.u = float(u); hit.v = float(v); }
        }
        out_f[i] = ob >= 0 ? hit.t : INFINITY;
        out_f[n + i] = hit.u; out_f[2 * n + i] = hit.v;
        out_i[i] = ob >= 0 ? int32_t(hit.patch) : -1; out_i[n + i] = ob;
    });
    if (counters)
    {
        std::memset(counters, 0, 8 * sizeof(uint64_t));
        for (auto& c : cn)
        {
            counters[0] += c.ts.nodes; counters[1] += c.ts.leaves; counters[2] += c.ts.hashLookups;
            counters[3] += c.candidates; counters[4] += c.cs.iterations; counters[5] += c.cs.pushes;
            counters[6] = std::max(counters[6], c.cs.maxDepth); counters[7] += c.cs.overflow;
        }
    }
    return 0;
}

// Per-ray work of a query (diagnostics): out (4, n) u32 = inner nodes,
// hash lookups, candidates, search iterations.
int ora_intersect_stats(void* s_, const float* rays, uint64_t n, int method, float tol, int any_hit, uint32_t* out,
                        int nthreads)
{
    auto* s = static_cast<Scene*>(s_);
    if (!s->built) return -1;
    QueryOpts q; q.method = method; q.tol = tol;
    parallel_for(n, nthreads, [&](uint64_t i, int) {
        Ray<float> r; unpack_ray(rays, n, i, r);
        Counters c;
        if (any_hit) scene_occluded(*s, r, q, &c);
        else { Hit hit; hit.t = r.max; scene_intersect(*s, hit, r, q, &c); }
        out[i] = uint32_t(c.ts.nodes); out[n + i] = uint32_t(c.ts.hashLookups);
        out[2 * n + i] = uint32_t(c.candidates); out[3 * n + i] = uint32_t(c.cs.iterations);
    });
    return 0;
}

// camera11 = rotation quaternion (x,y,z,w), position[3], scale[3], fovy
// Renders w x h pixels (one primary ray each, non Monte-Carlo shading) with
// 32x32 tiles handed to nthreads workers (src/rt/CPURayTracer.cpp:55-197).
// out_rgb: (h, w, 3) linear, clamped to [0,1]; out_packed: (h, w) sRGB RGBA8.
// ray_counts (optional, 3 u64): primary, bounce, shadow.
int ora_render_rows(void* s_, const float* camera11, uint32_t w, uint32_t h, uint32_t row0, uint32_t row_step,
                    int depth, float eps, int method, float tol, float* out_rgb, uint32_t* out_packed,
                    uint64_t* ray_counts, int nthreads, double* seconds);

int ora_render(void* s_, const float* camera11, uint32_t w, uint32_t h, int depth, float eps, int method, float tol,
               float* out_rgb, uint32_t* out_packed, uint64_t* ray_counts, int nthreads, double* seconds)
{
    return ora_render_rows(s_, camera11, w, h, 0, 1, depth, eps, method, tol, out_rgb, out_packed, ray_counts,
                           nthreads, seconds);
}

// Renders only rows row0, row0 + row_step, ... of the w x h image (a bounded
// sample of a frame for CPU timing); other pixels are left untouched.
int ora_render_rows(void* s_, const float* camera11, uint32_t w, uint32_t h, uint32_t row0, uint32_t row_step,
                    int depth, float eps, int method, float tol, float* out_rgb, uint32_t* out_packed,
                    uint64_t* ray_counts, int nthreads, double* seconds)
{
    if (row_step == 0) return -2;
    auto* s = static_cast<Scene*>(s_);
    if (!s->built) return -1;
    Camera cam;
    std::memcpy(cam.rot, camera11, 4 * sizeof(float));
    std::memcpy(cam.pos, camera11 + 4, 3 * sizeof(float));
    std::memcpy(cam.scale, camera11 + 7, 3 * sizeof(float));
    cam.fovy = camera11[10];
    RenderOpts op; op.depth = depth; op.eps = eps; op.method = method; op.tol = tol;
    Renderer R(*s, cam, w, h, op);
    const uint32_t tile = 32, cx = (w + tile - 1) / tile, cy = (h + tile - 1) / tile;
    std::vector<uint64_t> counts(3 * std::max(1, nthreads), 0);
    auto t0 = std::chrono::steady_clock::now();
    parallel_for(uint64_t(cx) * cy, std::max(1, nthreads), [&](uint64_t tix, int wk) {
        uint32_t x0 = uint32_t(tix % cx) * tile, y0 = uint32_t(tix / cx) * tile;
        uint32_t x1 = std::min(w, x0 + tile), y1 = std::min(h, y0 + tile);
        uint64_t* nr = ray_counts ? &counts[3 * wk] : nullptr;
        for (uint32_t j = y0; j < y1; j++)
            for (uint32_t i = x0; i < x1; i++)
            {
                if (j < row0 || (j - row0) % row_step) continue;
                Ray<float> pr {R.camPos, R.pixelRayDirection(float(i), float(j)), INFINITY};
                V3<float> c = R.trace(pr, V3<float>{1, 1, 1}, depth, nullptr, nr);
                c = {std::clamp(c.x, 0.0f, 1.0f), std::clamp(c.y, 0.0f, 1.0f), std::clamp(c.z, 0.0f, 1.0f)};
                size_t px = size_t(j) * w + i;
                if (out_rgb) { out_rgb[3 * px] = c.x; out_rgb[3 * px + 1] = c.y; out_rgb[3 * px + 2] = c.z; }
                if (out_packed) out_packed[px] = srgb8(c.x) | (srgb8(c.y) << 8) | (srgb8(c.z) << 16) | 0xFF000000u;
            }
    });
    auto t1 = std::chrono::steady_clock::now();
    if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
    if (ray_counts)
    {
        ray_counts[0] = ray_counts[1] = ray_counts[2] = 0;
        for (size_t k = 0; k < counts.size(); k++) ray_counts[k % 3] += counts[k];
    }
    return 0;
}

// Van der Corput radical inverse in base 2 (src/rt/PBR.h:143-157).
static float vdc(uint32_t i)
{
    i = (i << 16) | (i >> 16);
    i = ((i & 0x55555555u) << 1) | ((i & 0xAAAAAAAAu) >> 1);
    i = ((i & 0x33333333u) << 2) | ((i & 0xCCCCCCCCu) >> 2);
    i = ((i & 0x0F0F0F0Fu) << 4) | ((i & 0xF0F0F0F0u) >> 4);
    i = ((i & 0x00FF00FFu) << 8) | ((i & 0xFF00FF00u) >> 8);
    return float(i) * 0x1p-32f;
}

// spp jittered samples per pixel, averaged (mc: the Monte-Carlo bounce with
// the Philox counter (image sample px*spp + s, remaining depth)): sample s of pixel (i, j) traces
// the primary ray through (i + s/spp, j + vdc(s)) (the sampled path's jitter,
// src/rt/RayTracer.cu:226-236); spp = 1 is the unjittered pixel of ora_render.
// The sum runs over s in order and is scaled by 1/spp before clamping.
int ora_render_spp(void* s_, const float* camera11, uint32_t w, uint32_t h, uint32_t spp, int depth, float eps,
                   int method, float tol, int mc, float* out_rgb, uint32_t* out_packed, int nthreads)
{
    if (spp == 0) return -2;
    auto* s = static_cast<Scene*>(s_);
    if (!s->built) return -1;
    Camera cam;
    std::memcpy(cam.rot, camera11, 4 * sizeof(float));
    std::memcpy(cam.pos, camera11 + 4, 3 * sizeof(float));
    std::memcpy(cam.scale, camera11 + 7, 3 * sizeof(float));
    cam.fovy = camera11[10];
    RenderOpts op; op.depth = depth; op.eps = eps; op.method = method; op.tol = tol; op.mc = mc;
    Renderer R(*s, cam, w, h, op);
    parallel_for(uint64_t(w) * h, std::max(1, nthreads), [&](uint64_t px, int) {
        const uint32_t i = uint32_t(px % w), j = uint32_t(px / w);
        V3<float> c {0, 0, 0};
        for (uint32_t k = 0; k < spp; k++)
        {
            float x = float(i), y = float(j);
            if (spp > 1) { x = x + float(k) * (1.0f / float(spp)); y = y + vdc(k); }
            Ray<float> pr {R.camPos, R.pixelRayDirection(x, y), INFINITY};
            V3<float> ck = R.trace(pr, V3<float>{1, 1, 1}, depth, nullptr, nullptr, uint32_t(px * spp + k));
            c = {c.x + ck.x, c.y + ck.y, c.z + ck.z};
        }
        if (spp > 1)
        {
            const float inv = 1.0f / float(spp);
            c = {c.x * inv, c.y * inv, c.z * inv};
        }
        c = {std::clamp(c.x, 0.0f, 1.0f), std::clamp(c.y, 0.0f, 1.0f), std::clamp(c.z, 0.0f, 1.0f)};
        if (out_rgb) { out_rgb[3 * px] = c.x; out_rgb[3 * px + 1] = c.y; out_rgb[3 * px + 2] = c.z; }
        if (out_packed) out_packed[px] = srgb8(c.x) | (srgb8(c.y) << 8) | (srgb8(c.z) << 16) | 0xFF000000u;
    });
    return 0;
}

// Primary ray directions for a camera (the same set-up as ora_render), SoA (7, w*h).
int ora_camera_rays(const float* camera11, uint32_t w, uint32_t h, float* rays)
{
    Scene dummy;
    Camera cam;
    std::memcpy(cam.rot, camera11, 4 * sizeof(float));
    std::memcpy(cam.pos, camera11 + 4, 3 * sizeof(float));
    std::memcpy(cam.scale, camera11 + 7, 3 * sizeof(float));
    cam.fovy = camera11[10];
    Renderer R(dummy, cam, w, h, RenderOpts{});
    uint64_t n = uint64_t(w) * h;
    for (uint32_t j = 0; j < h; j++)
        for (uint32_t i = 0; i < w; i++)
        {
            uint64_t k = uint64_t(j) * w + i;
            V3<float> d = R.pixelRayDirection(float(i), float(j));
            rays[k] = R.camPos.x; rays[n + k] = R.camPos.y; rays[2 * n + k] = R.camPos.z;
            rays[3 * n + k] = d.x; rays[4 * n + k] = d.y; rays[5 * n + k] = d.z; rays[6 * n + k] = INFINITY;
        }
    return 0;
}

// Single (ray, patch) query: the drop-in for spline::doBezierClipping.
// ray7 = origin, unit direction, (unused) max; inout_t is hit.distance.
int ora_patch_intersect(const float* points4, const uint32_t* idx16, const float* ray7, float tol, int method,
                        float* inout_t, float* out_uv, uint64_t* stats4)
{
    V4<float> P[16];
    for (int k = 0; k < 16; k++)
    {
        const float* p = points4 + 4 * idx16[k];
        P[k] = {p[0], p[1], p[2], p[3]};
    }
    Ray<float> r {{ray7[0], ray7[1], ray7[2]}, {ray7[3], ray7[4], ray7[5]}, ray7[6]};
    float dist = *inout_t; V2<float> uv {0, 0};
    ClipStats cs;
    bool b = intersect_patch<float>(dist, uv, r, P, tol, method, &cs);
    if (b) { *inout_t = dist; out_uv[0] = uv.x; out_uv[1] = uv.y; }
    if (stats4) { stats4[0] = cs.iterations; stats4[1] = cs.pushes; stats4[2] = cs.maxDepth; stats4[3] = cs.overflow; }
    return b ? 1 : 0;
}

// doSubdivision_host on one (ray, patch) pair.  ray9 = origin, unit
// direction, tMin, tMax (and one unused slot); *inout_t is the current best
// distance in, the hit's distance out.
int ora_patch_subdiv_host(const float* points4, const uint32_t* idx16, const float* ray9, float threshold,
                          float* inout_t, float* out_uv)
{
    V4<float> P[16];
    for (int k = 0; k < 16; k++)
    {
        const float* p = points4 + 4 * idx16[k];
        P[k] = {p[0], p[1], p[2], p[3]};
    }
    const RayI r {{ray9[0], ray9[1], ray9[2]}, {ray9[3], ray9[4], ray9[5]}, ray9[6], ray9[7]};
    float dist = *inout_t;
    V2<float> uv {0, 0};
    const bool b = subdiv_host(dist, uv, r, P, threshold);
    if (b) { *inout_t = dist; out_uv[0] = uv.x; out_uv[1] = uv.y; }
    return b ? 1 : 0;
}

// Patch evaluation (mat::interpolate) and unit normal, for fixtures.
void ora_patch_eval(const float* points16x4, float u, float v, float* out_p3, float* out_n3)
{
    V4<float> P[16];
    for (int k = 0; k < 16; k++) P[k] = {points16x4[4 * k], points16x4[4 * k + 1], points16x4[4 * k + 2], points16x4[4 * k + 3]};
    V3<float> p = project(interpolate(P, u, v));
    V3<float> n = versor(patch_normal(P, u, v));
    out_p3[0] = p.x; out_p3[1] = p.y; out_p3[2] = p.z;
    out_n3[0] = n.x; out_n3[1] = n.y; out_n3[2] = n.z;
}

}  // extern "C"
