/*
 * Quaternions and view/projection helpers for the LightMath compatibility
 * shim (LightMath is an absent submodule of the reference tree), written for
 * building SoftLight's scene-graph sources as a CPU oracle. Conventions (the
 * ones the CPU oracle and the GPU scene kernels share; no reference test pins
 * them):
 *   quat_t{x, y, z, w}; a * b is the Hamilton product, each component summed
 *   left to right in the order w*, x*, y*, z* of the left operand;
 *   quat_to_mat3(q) has columns
 *     (1-2(yy+zz), 2(xy+wz), 2(xz-wy)), (2(xy-wz), 1-2(xx+zz), 2(yz+wx)),
 *     (2(xz+wy), 2(yz-wx), 1-2(xx+yy)), with xy = x*y and so on, and
 *   quat_to_mat4 embeds it with (0, 0, 0, 1) as the last column;
 *   get_x/y/z_axis(q) are the columns of quat_to_mat3(q);
 *   normalize(q) = q * (1/sqrt(dot(q, q))); mat3{mat4} keeps the upper-left
 *   3x3; perspective / ortho / look_at follow the OpenGL forms.
 */
#ifndef LS_SHIM_QUAT_H
#define LS_SHIM_QUAT_H

#include "_shim_math.h"

namespace ls
{
namespace math
{

template <typename T>
struct quat_t
{
    typedef T value_type;
    T q[4];
    quat_t() noexcept = default;
    constexpr quat_t(T x, T y, T z, T w) noexcept : q{x, y, z, w} {}
    T& operator[](std::size_t i) noexcept { return q[i]; }
    constexpr const T& operator[](std::size_t i) const noexcept { return q[i]; }
    quat_t operator*(const quat_t& b) const noexcept
    {
        const T ax = q[0], ay = q[1], az = q[2], aw = q[3];
        return quat_t{((aw * b.q[0] + ax * b.q[3]) + ay * b.q[2]) - az * b.q[1],
                      ((aw * b.q[1] - ax * b.q[2]) + ay * b.q[3]) + az * b.q[0],
                      ((aw * b.q[2] + ax * b.q[1]) - ay * b.q[0]) + az * b.q[3],
                      ((aw * b.q[3] - ax * b.q[0]) - ay * b.q[1]) - az * b.q[2]};
    }
    quat_t operator*(T s) const noexcept { return quat_t{q[0] * s, q[1] * s, q[2] * s, q[3] * s}; }
    quat_t operator+(const quat_t& b) const noexcept { return quat_t{q[0] + b.q[0], q[1] + b.q[1], q[2] + b.q[2], q[3] + b.q[3]}; }
    quat_t operator-(const quat_t& b) const noexcept { return quat_t{q[0] - b.q[0], q[1] - b.q[1], q[2] - b.q[2], q[3] - b.q[3]}; }
    quat_t operator-() const noexcept { return quat_t{-q[0], -q[1], -q[2], -q[3]}; }
    quat_t& operator*=(const quat_t& b) noexcept { return *this = *this * b; }
    bool operator==(const quat_t& b) const noexcept { return q[0] == b.q[0] && q[1] == b.q[1] && q[2] == b.q[2] && q[3] == b.q[3]; }
    bool operator!=(const quat_t& b) const noexcept { return !(*this == b); }
};

typedef quat_t<float> quat;

template <typename T> inline T dot(const quat_t<T>& a, const quat_t<T>& b) noexcept
{
    return ((a.q[0] * b.q[0] + a.q[1] * b.q[1]) + a.q[2] * b.q[2]) + a.q[3] * b.q[3];
}
template <typename T> inline T length(const quat_t<T>& a) noexcept { return std::sqrt(dot(a, a)); }
template <typename T> inline quat_t<T> normalize(const quat_t<T>& a) noexcept { return a * (T(1) / std::sqrt(dot(a, a))); }
template <typename T> inline quat_t<T> conjugate(const quat_t<T>& a) noexcept { return quat_t<T>{-a.q[0], -a.q[1], -a.q[2], a.q[3]}; }

template <typename T> inline mat3_t<T> quat_to_mat3(const quat_t<T>& a) noexcept
{
    const T x = a.q[0], y = a.q[1], z = a.q[2], w = a.q[3];
    const T xx = x * x, yy = y * y, zz = z * z, xy = x * y, xz = x * z, yz = y * z, wx = w * x, wy = w * y, wz = w * z;
    return mat3_t<T>{vec3_t<T>{T(1) - T(2) * (yy + zz), T(2) * (xy + wz), T(2) * (xz - wy)},
                     vec3_t<T>{T(2) * (xy - wz), T(1) - T(2) * (xx + zz), T(2) * (yz + wx)},
                     vec3_t<T>{T(2) * (xz + wy), T(2) * (yz - wx), T(1) - T(2) * (xx + yy)}};
}

template <typename T> inline mat4_t<T> quat_to_mat4(const quat_t<T>& a) noexcept
{
    const mat3_t<T> r = quat_to_mat3(a);
    return mat4_t<T>{vec4_t<T>{r.m[0].v[0], r.m[0].v[1], r.m[0].v[2], T(0)},
                     vec4_t<T>{r.m[1].v[0], r.m[1].v[1], r.m[1].v[2], T(0)},
                     vec4_t<T>{r.m[2].v[0], r.m[2].v[1], r.m[2].v[2], T(0)},
                     vec4_t<T>{T(0), T(0), T(0), T(1)}};
}

template <typename T> inline vec3_t<T> get_x_axis(const quat_t<T>& a) noexcept { return quat_to_mat3(a).m[0]; }
template <typename T> inline vec3_t<T> get_y_axis(const quat_t<T>& a) noexcept { return quat_to_mat3(a).m[1]; }
template <typename T> inline vec3_t<T> get_z_axis(const quat_t<T>& a) noexcept { return quat_to_mat3(a).m[2]; }

/* Shepperd's method on the largest of the trace and the diagonal */
template <typename T> inline quat_t<T> mat_to_quat(const mat3_t<T>& m) noexcept
{
    const T m00 = m.m[0].v[0], m11 = m.m[1].v[1], m22 = m.m[2].v[2];
    const T tr = (m00 + m11) + m22;
    if (tr > T(0))
    {
        const T s = std::sqrt(tr + T(1)) * T(2);
        return quat_t<T>{(m.m[1].v[2] - m.m[2].v[1]) / s, (m.m[2].v[0] - m.m[0].v[2]) / s, (m.m[0].v[1] - m.m[1].v[0]) / s, T(0.25) * s};
    }
    if (m00 > m11 && m00 > m22)
    {
        const T s = std::sqrt(((T(1) + m00) - m11) - m22) * T(2);
        return quat_t<T>{T(0.25) * s, (m.m[1].v[0] + m.m[0].v[1]) / s, (m.m[2].v[0] + m.m[0].v[2]) / s, (m.m[1].v[2] - m.m[2].v[1]) / s};
    }
    if (m11 > m22)
    {
        const T s = std::sqrt(((T(1) + m11) - m00) - m22) * T(2);
        return quat_t<T>{(m.m[1].v[0] + m.m[0].v[1]) / s, T(0.25) * s, (m.m[2].v[1] + m.m[1].v[2]) / s, (m.m[2].v[0] - m.m[0].v[2]) / s};
    }
    const T s = std::sqrt(((T(1) + m22) - m00) - m11) * T(2);
    return quat_t<T>{(m.m[2].v[0] + m.m[0].v[2]) / s, (m.m[2].v[1] + m.m[1].v[2]) / s, T(0.25) * s, (m.m[0].v[1] - m.m[1].v[0]) / s};
}

template <typename T> inline quat_t<T> lerp(const quat_t<T>& a, const quat_t<T>& b, T t) noexcept { return (b - a) * t + a; }

template <typename T> inline quat_t<T> slerp(const quat_t<T>& a, quat_t<T> b, T t) noexcept
{
    T c = dot(a, b);
    if (c < T(0)) { b = -b; c = -c; }
    if (c > T(0.9995)) return normalize(lerp(a, b, t));
    const T th = std::acos(c), s = std::sin(th);
    return a * (std::sin((T(1) - t) * th) / s) + b * (std::sin(t * th) / s);
}

template <typename T> inline T tan(T x) noexcept { return std::tan(x); }
template <typename T> inline T fmod(T x, T y) noexcept { return std::fmod(x, y); }

template <typename T> inline mat3_t<T> transpose(const mat3_t<T>& a) noexcept
{
    mat3_t<T> r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            r.m[i].v[j] = a.m[j].v[i];
    return r;
}

template <typename T> inline vec3_t<T> operator*(const mat3_t<T>& m, const vec3_t<T>& v) noexcept
{
    return (m.m[0] * v.v[0] + m.m[1] * v.v[1]) + m.m[2] * v.v[2];
}

template <typename T> inline mat4_t<T> perspective(T fov, T aspect, T zNear, T zFar) noexcept
{
    const T f = T(1) / std::tan(fov * T(0.5));
    return mat4_t<T>{f / aspect, T(0), T(0), T(0), T(0), f, T(0), T(0),
                     T(0), T(0), (zFar + zNear) / (zNear - zFar), T(-1),
                     T(0), T(0), (T(2) * zFar * zNear) / (zNear - zFar), T(0)};
}

template <typename T> inline mat4_t<T> infinite_perspective(T fov, T aspect, T zNear) noexcept
{
    const T f = T(1) / std::tan(fov * T(0.5));
    return mat4_t<T>{f / aspect, T(0), T(0), T(0), T(0), f, T(0), T(0), T(0), T(0), T(-1), T(-1), T(0), T(0), T(-2) * zNear, T(0)};
}

template <typename T> inline mat4_t<T> ortho(T l, T r, T b, T t) noexcept
{
    return mat4_t<T>{T(2) / (r - l), T(0), T(0), T(0), T(0), T(2) / (t - b), T(0), T(0), T(0), T(0), T(-1), T(0),
                     -(r + l) / (r - l), -(t + b) / (t - b), T(0), T(1)};
}

template <typename T> inline mat4_t<T> ortho(T l, T r, T b, T t, T n, T f) noexcept
{
    return mat4_t<T>{T(2) / (r - l), T(0), T(0), T(0), T(0), T(2) / (t - b), T(0), T(0), T(0), T(0), T(-2) / (f - n), T(0),
                     -(r + l) / (r - l), -(t + b) / (t - b), -(f + n) / (f - n), T(1)};
}

template <typename T> inline mat4_t<T> look_at(const vec3_t<T>& eye, const vec3_t<T>& target, const vec3_t<T>& up) noexcept
{
    const vec3_t<T> zAxis = normalize(eye - target);
    const vec3_t<T> xAxis = normalize(cross(up, zAxis));
    const vec3_t<T> yAxis = cross(zAxis, xAxis);
    return mat4_t<T>{xAxis.v[0], yAxis.v[0], zAxis.v[0], T(0), xAxis.v[1], yAxis.v[1], zAxis.v[1], T(0),
                     xAxis.v[2], yAxis.v[2], zAxis.v[2], T(0), -dot(xAxis, eye), -dot(yAxis, eye), -dot(zAxis, eye), T(1)};
}

template <typename T> inline mat4_t<T> look_from(const vec3_t<T>& eye, const vec3_t<T>& target, const vec3_t<T>& up) noexcept
{
    const vec3_t<T> zAxis = normalize(target - eye);
    const vec3_t<T> xAxis = normalize(cross(up, zAxis));
    const vec3_t<T> yAxis = cross(zAxis, xAxis);
    return mat4_t<T>{xAxis.v[0], yAxis.v[0], zAxis.v[0], T(0), xAxis.v[1], yAxis.v[1], zAxis.v[1], T(0),
                     xAxis.v[2], yAxis.v[2], zAxis.v[2], T(0), -dot(xAxis, eye), -dot(yAxis, eye), -dot(zAxis, eye), T(1)};
}

} // namespace math
} // namespace ls

#endif /* LS_SHIM_QUAT_H */
