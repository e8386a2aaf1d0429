// TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT (ds_compat; see core/Globals.h).
//
// Ray--triangle intersection by the published algorithm of Moller and Trumbore
// ("Fast, minimum storage ray-triangle intersection", 1997): barycentric
// (u, v) of the hit with respect to (p1 - p0, p2 - p0), uvw = (u, v, 1-u-v),
// and t.  A hit needs |det| > 1e-12 (not parallel), u >= 0, v >= 0,
// u + v <= 1 and t inside the ray's [tMin, tMax].  normal() is the
// unnormalised face normal.
#pragma once

#include "../geometry/Bounds3.h"

namespace cg::triangle
{

template<typename T>
HOST DEVICE bool intersect(const Ray3<T>& ray, const Vector<T,3>& p0, const Vector<T,3>& p1,
                           const Vector<T,3>& p2, Vector<T,3>& uvw, T& t)
{
    const Vector<T,3> e1 = p1 - p0;
    const Vector<T,3> e2 = p2 - p0;
    const Vector<T,3> pv = ray.direction.cross(e2);
    const T det = e1.dot(pv);
    if (det > -T(1e-12) && det < T(1e-12)) return false;
    const T inv = T(1) / det;
    const Vector<T,3> s = ray.origin - p0;
    const T u = s.dot(pv) * inv;
    if (u < 0 || u > 1) return false;
    const Vector<T,3> q = s.cross(e1);
    const T v = ray.direction.dot(q) * inv;
    if (v < 0 || u + v > 1) return false;
    const T tt = e2.dot(q) * inv;
    if (tt < ray.tMin || tt > ray.tMax) return false;
    uvw.set(u, v, 1 - u - v);
    t = tt;
    return true;
}

// Unnormalised face normal (p1 - p0) x (p2 - p0).
template<typename T>
HOST DEVICE Vector<T,3> normal(const Vector<T,3>& p0, const Vector<T,3>& p1, const Vector<T,3>& p2)
{
    return (p1 - p0).cross(p2 - p0);
}

} // namespace cg::triangle
