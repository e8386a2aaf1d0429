// TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.
//
// cg::Vector<T,N> (N = 2, 3, 4) for the ds_compat stand-in of the Ds library.
// Public members x, y(, z, w) and nothing else, so that structured bindings
// work as the reference uses them (src/AlignedTypes.h:105,
// src/rt/Primitive.cu:272).  Arithmetic is component-wise; dot sums the
// products left to right (a.dot(b), or the static Vector::dot(a, b)); length = sqrt(dot(v, v)); versor() and normalize()
// multiply by 1/length when the length is not zero; inverse() is the
// component-wise reciprocal 1/x.  Vectors of two and three components convert
// into each other (dropping z, or adding z = 0); a three-component vector
// converts to four only with an explicit w and back only explicitly.
#pragma once

#include <cmath>
#include <type_traits>
#include "../core/Globals.h"

namespace cg
{

template<typename T, int N> struct Vector;

// Member operations shared by the three sizes (N components, self type V).
#define DS_COMPAT_VECTOR_MEMBERS(N)                                                   \
    HOST DEVICE constexpr T dot(const Vector& b) const                                \
    {                                                                                 \
        T s = (*this)[0] * b[0];                                                      \
        for (int i = 1; i < N; i++) s = s + (*this)[i] * b[i];                        \
        return s;                                                                     \
    }                                                                                 \
    HOST DEVICE static constexpr T dot(const Vector& a, const Vector& b)              \
    {                                                                                 \
        return a.dot(b);                                                              \
    }                                                                                 \
    HOST DEVICE constexpr T squaredNorm() const { return dot(*this); }               \
    HOST DEVICE T length() const { return std::sqrt(squaredNorm()); }                \
    HOST DEVICE Vector versor() const                                                 \
    {                                                                                 \
        const T l = length();                                                         \
        if (l == T(0)) return *this;                                                  \
        const T k = T(1) / l;                                                         \
        Vector r;                                                                     \
        for (int i = 0; i < N; i++) r[i] = (*this)[i] * k;                            \
        return r;                                                                     \
    }                                                                                 \
    HOST DEVICE Vector& normalize() { *this = versor(); return *this; }               \
    HOST DEVICE constexpr Vector inverse() const                                      \
    {                                                                                 \
        Vector r;                                                                     \
        for (int i = 0; i < N; i++) r[i] = T(1) / (*this)[i];                         \
        return r;                                                                     \
    }                                                                                 \
    HOST DEVICE constexpr T max() const                                               \
    {                                                                                 \
        T m = (*this)[0];                                                             \
        for (int i = 1; i < N; i++) if ((*this)[i] > m) m = (*this)[i];               \
        return m;                                                                     \
    }                                                                                 \
    HOST DEVICE constexpr T min() const                                               \
    {                                                                                 \
        T m = (*this)[0];                                                             \
        for (int i = 1; i < N; i++) if ((*this)[i] < m) m = (*this)[i];               \
        return m;                                                                     \
    }                                                                                 \
    HOST DEVICE Vector abs() const                                                    \
    {                                                                                 \
        Vector r;                                                                     \
        for (int i = 0; i < N; i++) r[i] = std::abs((*this)[i]);                      \
        return r;                                                                     \
    }

template<typename T>
struct Vector<T,2>
{
    using value_type = T;
    T x, y;

    HOST DEVICE constexpr Vector() : x{}, y{} {}
    HOST DEVICE constexpr explicit Vector(T s) : x{s}, y{s} {}
    HOST DEVICE constexpr Vector(T a, T b) : x{a}, y{b} {}
    HOST DEVICE constexpr Vector(const Vector<T,3>& v);
    HOST DEVICE constexpr Vector(const float2& v) requires std::is_same_v<T,float> : x{v.x}, y{v.y} {}

    HOST DEVICE constexpr T& operator[](int i) { return i == 0 ? x : y; }
    HOST DEVICE constexpr const T& operator[](int i) const { return i == 0 ? x : y; }
    HOST DEVICE constexpr void set(T a, T b) { x = a; y = b; }
    DS_COMPAT_VECTOR_MEMBERS(2)
};

template<typename T>
struct Vector<T,3>
{
    using value_type = T;
    T x, y, z;

    HOST DEVICE constexpr Vector() : x{}, y{}, z{} {}
    HOST DEVICE constexpr explicit Vector(T s) : x{s}, y{s}, z{s} {}
    HOST DEVICE constexpr Vector(T a, T b, T c) : x{a}, y{b}, z{c} {}
    HOST DEVICE constexpr Vector(const Vector<T,2>& v, T c = T(0)) : x{v.x}, y{v.y}, z{c} {}
    HOST DEVICE constexpr explicit Vector(const Vector<T,4>& v);
    HOST DEVICE constexpr Vector(const float3& v) requires std::is_same_v<T,float> : x{v.x}, y{v.y}, z{v.z} {}

    HOST DEVICE constexpr T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    HOST DEVICE constexpr const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    HOST DEVICE constexpr void set(T a, T b, T c) { x = a; y = b; z = c; }
    HOST DEVICE constexpr Vector cross(const Vector& b) const
    {
        return {y * b.z - z * b.y, z * b.x - x * b.z, x * b.y - y * b.x};
    }
    DS_COMPAT_VECTOR_MEMBERS(3)
};

template<typename T>
struct Vector<T,4>
{
    using value_type = T;
    T x, y, z, w;

    HOST DEVICE constexpr Vector() : x{}, y{}, z{}, w{} {}
    HOST DEVICE constexpr explicit Vector(T s) : x{s}, y{s}, z{s}, w{s} {}
    HOST DEVICE constexpr Vector(T a, T b, T c, T d) : x{a}, y{b}, z{c}, w{d} {}
    HOST DEVICE constexpr Vector(const Vector<T,3>& v, T d) : x{v.x}, y{v.y}, z{v.z}, w{d} {}
    HOST DEVICE constexpr Vector(const float4& v) requires std::is_same_v<T,float> : x{v.x}, y{v.y}, z{v.z}, w{v.w} {}

    HOST DEVICE constexpr T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    HOST DEVICE constexpr const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    HOST DEVICE constexpr void set(T a, T b, T c, T d) { x = a; y = b; z = c; w = d; }
    DS_COMPAT_VECTOR_MEMBERS(4)
};

template<typename T>
HOST DEVICE constexpr Vector<T,2>::Vector(const Vector<T,3>& v) : x{v.x}, y{v.y} {}

template<typename T>
HOST DEVICE constexpr Vector<T,3>::Vector(const Vector<T,4>& v) : x{v.x}, y{v.y}, z{v.z} {}

// ------------------------------------------------------------- arithmetic --

template<typename T, int N>
HOST DEVICE constexpr Vector<T,N> operator+(const Vector<T,N>& a, const Vector<T,N>& b)
{
    Vector<T,N> r;
    for (int i = 0; i < N; i++) r[i] = a[i] + b[i];
    return r;
}

template<typename T, int N>
HOST DEVICE constexpr Vector<T,N> operator-(const Vector<T,N>& a, const Vector<T,N>& b)
{
    Vector<T,N> r;
    for (int i = 0; i < N; i++) r[i] = a[i] - b[i];
    return r;
}

template<typename T, int N>
HOST DEVICE constexpr Vector<T,N> operator-(const Vector<T,N>& a)
{
    Vector<T,N> r;
    for (int i = 0; i < N; i++) r[i] = -a[i];
    return r;
}

template<typename T, int N>
HOST DEVICE constexpr Vector<T,N> operator*(const Vector<T,N>& a, const Vector<T,N>& b)
{
    Vector<T,N> r;
    for (int i = 0; i < N; i++) r[i] = a[i] * b[i];
    return r;
}

template<typename T, int N>
HOST DEVICE constexpr Vector<T,N> operator/(const Vector<T,N>& a, const Vector<T,N>& b)
{
    Vector<T,N> r;
    for (int i = 0; i < N; i++) r[i] = a[i] / b[i];
    return r;
}

template<typename S, typename T, int N>
requires std::is_arithmetic_v<S>
HOST DEVICE constexpr Vector<T,N> operator*(S s, const Vector<T,N>& a)
{
    Vector<T,N> r;
    for (int i = 0; i < N; i++) r[i] = T(s) * a[i];
    return r;
}

template<typename S, typename T, int N>
requires std::is_arithmetic_v<S>
HOST DEVICE constexpr Vector<T,N> operator*(const Vector<T,N>& a, S s)
{
    Vector<T,N> r;
    for (int i = 0; i < N; i++) r[i] = a[i] * T(s);
    return r;
}

template<typename S, typename T, int N>
requires std::is_arithmetic_v<S>
HOST DEVICE constexpr Vector<T,N> operator/(const Vector<T,N>& a, S s)
{
    Vector<T,N> r;
    for (int i = 0; i < N; i++) r[i] = a[i] / T(s);
    return r;
}

template<typename T, int N>
HOST DEVICE constexpr Vector<T,N>& operator+=(Vector<T,N>& a, const Vector<T,N>& b)
{
    for (int i = 0; i < N; i++) a[i] += b[i];
    return a;
}

template<typename T, int N>
HOST DEVICE constexpr Vector<T,N>& operator-=(Vector<T,N>& a, const Vector<T,N>& b)
{
    for (int i = 0; i < N; i++) a[i] -= b[i];
    return a;
}

template<typename T, int N>
HOST DEVICE constexpr Vector<T,N>& operator*=(Vector<T,N>& a, const Vector<T,N>& b)
{
    for (int i = 0; i < N; i++) a[i] *= b[i];
    return a;
}

template<typename S, typename T, int N>
requires std::is_arithmetic_v<S>
HOST DEVICE constexpr Vector<T,N>& operator*=(Vector<T,N>& a, S s)
{
    for (int i = 0; i < N; i++) a[i] *= T(s);
    return a;
}

template<typename S, typename T, int N>
requires std::is_arithmetic_v<S>
HOST DEVICE constexpr Vector<T,N>& operator/=(Vector<T,N>& a, S s)
{
    for (int i = 0; i < N; i++) a[i] /= T(s);
    return a;
}

template<typename T, int N>
HOST DEVICE constexpr bool operator==(const Vector<T,N>& a, const Vector<T,N>& b)
{
    for (int i = 0; i < N; i++) if (!(a[i] == b[i])) return false;
    return true;
}

using vec2f = Vector<float,2>;
using vec3f = Vector<float,3>;
using vec4f = Vector<float,4>;
using vec2d = Vector<double,2>;
using vec3d = Vector<double,3>;
using vec4d = Vector<double,4>;

} // namespace cg
