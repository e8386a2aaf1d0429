// TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT (ds_compat; see core/Globals.h).
//
// Axis-aligned boxes and rays.  A default box is empty: min = +inf and
// max = -inf on every axis, so size() = max - min is -inf per axis; the
// reference's BVH split reads its axis from such a box (src/rt/BVH.cpp:46-52).
// inflate() takes the component-wise min/max with a point or a box; a
// homogeneous 4-vector is projected first.
// intersect(ray, tMin, tMax) is the slab test clipped to the ray's
// [tMin, tMax]; it reports the entry and exit distances and whether the
// clipped interval is non-empty.
#pragma once

#include <limits>
#include "../math/Vector.h"

namespace cg
{

template<typename T>
struct Ray3
{
    Vector<T,3> origin;
    Vector<T,3> direction;
    T tMin = T(0);
    T tMax = std::numeric_limits<T>::infinity();
};

using Ray3f = Ray3<float>;

template<typename T, int N>
struct BoundsN
{
    using vec = Vector<T,N>;

    HOST DEVICE constexpr BoundsN()
    {
        for (int i = 0; i < N; i++)
        {
            _p0[i] = +std::numeric_limits<T>::infinity();
            _p1[i] = -std::numeric_limits<T>::infinity();
        }
    }
    HOST DEVICE constexpr BoundsN(const vec& a, const vec& b)
    {
        for (int i = 0; i < N; i++)
        {
            _p0[i] = a[i] < b[i] ? a[i] : b[i];
            _p1[i] = a[i] < b[i] ? b[i] : a[i];
        }
    }

    HOST DEVICE constexpr const vec& min() const { return _p0; }
    HOST DEVICE constexpr const vec& max() const { return _p1; }
    HOST DEVICE constexpr vec size() const { return _p1 - _p0; }
    HOST DEVICE constexpr vec center() const { return T(0.5) * (_p0 + _p1); }
    HOST DEVICE constexpr bool empty() const
    {
        for (int i = 0; i < N; i++) if (_p0[i] > _p1[i]) return true;
        return false;
    }

    HOST DEVICE constexpr void inflate(const vec& p)
    {
        for (int i = 0; i < N; i++)
        {
            if (p[i] < _p0[i]) _p0[i] = p[i];
            if (p[i] > _p1[i]) _p1[i] = p[i];
        }
    }
    // A homogeneous point inflates the box by its projection (x/w, y/w, z/w).
    HOST DEVICE constexpr void inflate(const Vector<T,4>& p) requires (N == 3)
    {
        inflate(vec{p.x / p.w, p.y / p.w, p.z / p.w});
    }
    HOST DEVICE constexpr void inflate(const BoundsN& b)
    {
        for (int i = 0; i < N; i++)
        {
            if (b._p0[i] < _p0[i]) _p0[i] = b._p0[i];
            if (b._p1[i] > _p1[i]) _p1[i] = b._p1[i];
        }
    }

    HOST DEVICE bool intersect(const Ray3<T>& ray, T& tMin, T& tMax) const requires (N == 3)
    {
        tMin = ray.tMin;
        tMax = ray.tMax;
        for (int i = 0; i < 3; i++)
        {
            const T inv = T(1) / ray.direction[i];
            T t0 = (_p0[i] - ray.origin[i]) * inv;
            T t1 = (_p1[i] - ray.origin[i]) * inv;
            if (t0 > t1) { T s = t0; t0 = t1; t1 = s; }
            if (t0 > tMin) tMin = t0;
            if (t1 < tMax) tMax = t1;
            if (tMin > tMax) return false;
        }
        return true;
    }

protected:
    vec _p0;
    vec _p1;
};

template<typename T> using Bounds2 = BoundsN<T,2>;
template<typename T> using Bounds3 = BoundsN<T,3>;
using Bounds2f = Bounds2<float>;
using Bounds3f = Bounds3<float>;

} // namespace cg
