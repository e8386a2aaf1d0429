// TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT (ds_compat; see core/Globals.h).
//
// Column-major 3x3 and 4x4 matrices and a quaternion with public x, y, z, w,
// as the reference's AlignedTypes.h and Scene.cu use them: m[i] is column i,
// M * v = v.x*c0 + v.y*c1 + v.z*c2 (+ v.w*c3), and TRS(t, q, s) builds
// translate * rotate * scale.
#pragma once

#include "Vector.h"

namespace cg
{

template<typename T>
struct Quaternion
{
    T x, y, z, w;

    HOST DEVICE constexpr Quaternion() : x{}, y{}, z{}, w{1} {}
    HOST DEVICE constexpr Quaternion(T a, T b, T c, T d) : x{a}, y{b}, z{c}, w{d} {}
    HOST DEVICE constexpr Quaternion(const Vector<T,3>& v, T d) : x{v.x}, y{v.y}, z{v.z}, w{d} {}
    HOST DEVICE static constexpr Quaternion identity() { return {T(0), T(0), T(0), T(1)}; }
};

template<typename T>
struct Matrix3x3
{
    Vector<T,3> c[3];

    HOST DEVICE constexpr Matrix3x3() : c{} {}
    HOST DEVICE constexpr explicit Matrix3x3(T d) : c{{d, 0, 0}, {0, d, 0}, {0, 0, d}} {}
    HOST DEVICE constexpr Matrix3x3(const Vector<T,3>& c0, const Vector<T,3>& c1, const Vector<T,3>& c2)
        : c{c0, c1, c2} {}

    HOST DEVICE constexpr Vector<T,3>& operator[](int i) { return c[i]; }
    HOST DEVICE constexpr const Vector<T,3>& operator[](int i) const { return c[i]; }
    HOST DEVICE constexpr T& operator()(int i, int j) { return c[j][i]; }
    HOST DEVICE constexpr T operator()(int i, int j) const { return c[j][i]; }

    HOST DEVICE constexpr Vector<T,3> operator*(const Vector<T,3>& v) const
    {
        return v.x * c[0] + v.y * c[1] + v.z * c[2];
    }
    HOST DEVICE constexpr Matrix3x3 operator*(const Matrix3x3& m) const
    {
        return {(*this) * m[0], (*this) * m[1], (*this) * m[2]};
    }
    HOST DEVICE constexpr Matrix3x3 transposed() const
    {
        return {{c[0].x, c[1].x, c[2].x}, {c[0].y, c[1].y, c[2].y}, {c[0].z, c[1].z, c[2].z}};
    }
};

template<typename T>
struct Matrix4x4
{
    Vector<T,4> c[4];

    HOST DEVICE constexpr Matrix4x4() : c{} {}
    HOST DEVICE constexpr explicit Matrix4x4(T d) : c{{d, 0, 0, 0}, {0, d, 0, 0}, {0, 0, d, 0}, {0, 0, 0, d}} {}
    HOST DEVICE constexpr Matrix4x4(const Vector<T,4>& c0, const Vector<T,4>& c1, const Vector<T,4>& c2,
                                    const Vector<T,4>& c3)
        : c{c0, c1, c2, c3} {}

    HOST DEVICE constexpr Vector<T,4>& operator[](int i) { return c[i]; }
    HOST DEVICE constexpr const Vector<T,4>& operator[](int i) const { return c[i]; }
    HOST DEVICE constexpr T& operator()(int i, int j) { return c[j][i]; }
    HOST DEVICE constexpr T operator()(int i, int j) const { return c[j][i]; }

    HOST DEVICE constexpr Vector<T,4> operator*(const Vector<T,4>& v) const
    {
        return v.x * c[0] + v.y * c[1] + v.z * c[2] + v.w * c[3];
    }
    HOST DEVICE constexpr Matrix4x4 operator*(const Matrix4x4& m) const
    {
        return {(*this) * m[0], (*this) * m[1], (*this) * m[2], (*this) * m[3]};
    }
    HOST DEVICE constexpr Vector<T,3> transform(const Vector<T,3>& p) const
    {
        const Vector<T,4> r = (*this) * Vector<T,4>(p, T(1));
        return {r.x / r.w, r.y / r.w, r.z / r.w};
    }
    HOST DEVICE constexpr Vector<T,3> transformVector(const Vector<T,3>& v) const
    {
        const Vector<T,4> r = (*this) * Vector<T,4>(v, T(0));
        return {r.x, r.y, r.z};
    }
    HOST DEVICE constexpr Matrix4x4 transposed() const
    {
        Matrix4x4 r;
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) r(i, j) = (*this)(j, i);
        return r;
    }

    // translate(t) * rotate(q) * scale(s); the rotation columns use the
    // reference's own quaternion-to-matrix arithmetic (src/AlignedTypes.h:
    // 99-115), each column then multiplied by its scale factor.
    HOST DEVICE static Matrix4x4 TRS(const Vector<T,3>& t, const Quaternion<T>& q, const Vector<T,3>& s)
    {
        const T i = q.x, j = q.y, k = q.z, r = q.w;
        const T ii = 2 * i * i, ij = 2 * i * j, ik = 2 * i * k, jj = 2 * j * j, jk = 2 * j * k, kk = 2 * k * k;
        const T ri = 2 * r * i, rj = 2 * r * j, rk = 2 * r * k;
        const Vector<T,3> c0 = Vector<T,3>{1 - jj - kk, ij + rk, ik - rj} * s.x;
        const Vector<T,3> c1 = Vector<T,3>{ij - rk, 1 - ii - kk, jk + ri} * s.y;
        const Vector<T,3> c2 = Vector<T,3>{ik + rj, jk - ri, 1 - ii - jj} * s.z;
        return {Vector<T,4>(c0, 0), Vector<T,4>(c1, 0), Vector<T,4>(c2, 0), Vector<T,4>(t, 1)};
    }
};

using mat3f = Matrix3x3<float>;
using mat4f = Matrix4x4<float>;
using quatf = Quaternion<float>;

} // namespace cg
