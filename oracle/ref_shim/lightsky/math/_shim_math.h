/*
 * Compatibility shim for LightSky's "math" library (LightMath, an absent
 * submodule of the reference tree), written for building the reference's
 * draw-path sources as a CPU oracle. It provides the types and functions
 * those sources call, with these conventions (the same ones the CPU oracle
 * restatement and the GPU kernels use):
 *   fmadd(a,b,c) = a*b + c with two roundings (built with -ffp-contract=off);
 *   rcp(x) = 1/x; dot and horizontal sums fold left ((a0+a1)+a2)+a3;
 *   sum(a, b, c, ...) folds left; mix(a,b,t) = (b-a)*t + a;
 *   cross(vec4) = (a1*b2-a2*b1, a2*b0-a0*b2, a0*b1-a1*b0, 0);
 *   cross(vec2) = a0*b1 - a1*b0; max(a,b) = a<b ? b : a; min(a,b) = b<a ? b : a;
 *   vecN == / < / <= / > / >= hold when they hold for every component and
 *   != is the negation of ==; mat4 is column-major; mat4*vec4 sums the
 *   scaled columns left to right; vec4*mat4 is the dot product with each
 *   column; outer(a, b) has columns b*a[i]; normalize(v) = v * (1/sqrt(dot(v,v))).
 * These are choices made here: the library's own source is not available, so
 * no reference test pins them.
 */
#ifndef LS_SHIM_MATH_H
#define LS_SHIM_MATH_H

#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <type_traits>

#include "../setup/_shim_setup.h"

#include "../../../../include/slg_half.h"

namespace ls
{
namespace math
{

/*-----------------------------------------------------------------------------
 * half (IEEE binary16 storage)
-----------------------------------------------------------------------------*/
struct half
{
    uint16_t bits;

    half() noexcept = default;
    constexpr half(uint8_t hi, uint8_t lo) noexcept : bits((uint16_t)(((uint16_t)hi << 8) | lo)) {}
    half(float f) noexcept { bits = from_float(f); }
    half(double d) noexcept { bits = from_float((float)d); }
    half(int i) noexcept { bits = from_float((float)i); }
    half(unsigned i) noexcept { bits = from_float((float)i); }
    half(long i) noexcept { bits = from_float((float)i); }
    half(unsigned long i) noexcept { bits = from_float((float)i); }
    half(unsigned char i) noexcept { bits = from_float((float)i); }
    half(unsigned short i) noexcept { bits = from_float((float)i); }

    operator float() const noexcept { return to_float(bits); }

    /* IEEE binary16, round to nearest even (include/slg_half.h, shared with
     * the GPU kernels and the CPU checker) */
    static uint16_t from_float(float f) noexcept { return slg_float_to_half(f); }
    static float to_float(uint16_t h) noexcept { return slg_half_to_float(h); }
};

/*-----------------------------------------------------------------------------
 * fixed point (declared for SL_Sampler's fixed-point wrap functions)
-----------------------------------------------------------------------------*/
struct long_medp_t
{
    int64_t v; /* 32.32 */
    constexpr bool operator<(const long_medp_t& o) const noexcept { return v < o.v; }
    constexpr bool operator>(const long_medp_t& o) const noexcept { return v > o.v; }
    constexpr bool operator<=(const long_medp_t& o) const noexcept { return v <= o.v; }
    constexpr bool operator>=(const long_medp_t& o) const noexcept { return v >= o.v; }
    constexpr long_medp_t operator+(const long_medp_t& o) const noexcept { return long_medp_t{v + o.v}; }
    constexpr long_medp_t operator*(const long_medp_t& o) const noexcept { return long_medp_t{(int64_t)(((__int128)v * o.v) >> 32)}; }
};

/* 16.16 fixed point: named by SL_Plane's SL_Planex typedef only */
struct medp_t
{
    int32_t v;
};

template <typename fixed_t, typename T>
constexpr fixed_t fixed_cast(T n) noexcept { return fixed_t{(int64_t)((double)n * 4294967296.0)}; }

template <typename int_t, typename fixed_t>
constexpr int_t integer_cast(fixed_t f) noexcept { return (int_t)(f.v >> 32); }

/*-----------------------------------------------------------------------------
 * scalar helpers
-----------------------------------------------------------------------------*/
template <typename T> constexpr T min(T a, T b) noexcept { return (b < a) ? b : a; }
template <typename T> constexpr T max(T a, T b) noexcept { return (a < b) ? b : a; }
template <typename T> constexpr T min(T a, T b, T c) noexcept { return min(min(a, b), c); }
template <typename T> constexpr T max(T a, T b, T c) noexcept { return max(max(a, b), c); }
template <typename T> constexpr T clamp(T x, T lo, T hi) noexcept { return min(max(x, lo), hi); }
template <typename T> constexpr T abs(T x) noexcept { return (x < T(0)) ? T(-x) : x; }
inline float floor(float x) noexcept { return std::floor(x); }
inline double floor(double x) noexcept { return std::floor(x); }
inline float round(float x) noexcept { return std::round(x); }
inline double round(double x) noexcept { return std::round(x); }
template <typename T> constexpr T fmadd(T a, T b, T c) noexcept { return a * b + c; }
template <typename T> constexpr T fmsub(T a, T b, T c) noexcept { return a * b - c; }
template <typename T> constexpr T rcp(T x) noexcept { return T(1) / x; }
template <typename T> constexpr T mix(T a, T b, T t) noexcept { return (b - a) * t + a; }
template <typename T> constexpr T step(T edge, T x) noexcept { return (x < edge) ? T(0) : T(1); }
template <typename T> constexpr T saturate(T x) noexcept { return clamp<T>(x, T(0), T(1)); }
template <typename T> constexpr T radians(T x) noexcept { return x * T(0.01745329251994329577); }
inline float fmod_1(float x) noexcept { return std::fmod(x, 1.f); }
inline double fmod_1(double x) noexcept { return std::fmod(x, 1.0); }
template <typename T> inline T fast_sqrt(T x) noexcept { return (T)std::sqrt(x); }
inline float inversesqrt(float x) noexcept { return 1.f / std::sqrt(x); }
template <typename T> constexpr bool is_pow2(T x) noexcept { return x && !(x & (x - 1)); }
template <typename T> constexpr T gcd(T a, T b) noexcept { return b ? gcd<T>(b, a % b) : a; }
inline unsigned popcnt_u32(uint32_t x) noexcept { return (unsigned)__builtin_popcount(x); }
inline int sign_mask(float f) noexcept { uint32_t u; std::memcpy(&u, &f, 4); return (int)(u >> 31); }
inline int sign_mask(double d) noexcept { uint64_t u; std::memcpy(&u, &d, 8); return (int)(u >> 63); }
inline int sign_mask(int32_t i) noexcept { return (int)((uint32_t)i >> 31); }

/*-----------------------------------------------------------------------------
 * vectors
-----------------------------------------------------------------------------*/
#define LS_EPSILON 1.0e-6f

#define LS_SHIM_VEC_COMMON(N)                                                                          \
    typedef T value_type;                                                                              \
    static constexpr unsigned num_components() noexcept { return N; }                                 \
    T& operator[](std::size_t i) noexcept { return v[i]; }                                             \
    constexpr const T& operator[](std::size_t i) const noexcept { return v[i]; }                       \
    vecN_t operator-() const noexcept { vecN_t r; for (unsigned i = 0; i < N; ++i) r.v[i] = -v[i]; return r; } \
    vecN_t operator~() const noexcept { vecN_t r; for (unsigned i = 0; i < N; ++i) r.v[i] = ~v[i]; return r; } \
    LS_SHIM_VEC_BINOP(N, +) LS_SHIM_VEC_BINOP(N, -) LS_SHIM_VEC_BINOP(N, *) LS_SHIM_VEC_BINOP(N, /)     \
    LS_SHIM_VEC_BINOP(N, &) LS_SHIM_VEC_BINOP(N, |) LS_SHIM_VEC_BINOP(N, ^) LS_SHIM_VEC_BINOP(N, %)     \
    LS_SHIM_VEC_BINOP(N, <<) LS_SHIM_VEC_BINOP(N, >>)                                                  \
    bool operator==(const vecN_t& o) const noexcept { for (unsigned i = 0; i < N; ++i) if (!(v[i] == o.v[i])) return false; return true; } \
    bool operator!=(const vecN_t& o) const noexcept { return !(*this == o); }                          \
    bool operator<(const vecN_t& o) const noexcept { for (unsigned i = 0; i < N; ++i) if (!(v[i] < o.v[i])) return false; return true; } \
    bool operator<=(const vecN_t& o) const noexcept { for (unsigned i = 0; i < N; ++i) if (!(v[i] <= o.v[i])) return false; return true; } \
    bool operator>(const vecN_t& o) const noexcept { for (unsigned i = 0; i < N; ++i) if (!(v[i] > o.v[i])) return false; return true; } \
    bool operator>=(const vecN_t& o) const noexcept { for (unsigned i = 0; i < N; ++i) if (!(v[i] >= o.v[i])) return false; return true; }

#define LS_SHIM_VEC_BINOP(N, OP)                                                                       \
    vecN_t operator OP(const vecN_t& o) const noexcept { vecN_t r; for (unsigned i = 0; i < N; ++i) r.v[i] = (T)(v[i] OP o.v[i]); return r; } \
    vecN_t operator OP(const T s) const noexcept { vecN_t r; for (unsigned i = 0; i < N; ++i) r.v[i] = (T)(v[i] OP s); return r; } \
    vecN_t& operator OP##=(const vecN_t& o) noexcept { for (unsigned i = 0; i < N; ++i) v[i] = (T)(v[i] OP o.v[i]); return *this; } \
    vecN_t& operator OP##=(const T s) noexcept { for (unsigned i = 0; i < N; ++i) v[i] = (T)(v[i] OP s); return *this; }

template <typename T>
struct vec2_t
{
    typedef vec2_t vecN_t;
    T v[2];
    vec2_t() noexcept = default;
    constexpr vec2_t(T s) noexcept : v{s, s} {}
    constexpr vec2_t(T a, T b) noexcept : v{a, b} {}
    template <typename U> explicit constexpr operator vec2_t<U>() const noexcept { return vec2_t<U>{(U)v[0], (U)v[1]}; }
    LS_SHIM_VEC_COMMON(2)
};

template <typename T>
struct vec3_t
{
    typedef vec3_t vecN_t;
    T v[3];
    vec3_t() noexcept = default;
    constexpr vec3_t(T s) noexcept : v{s, s, s} {}
    constexpr vec3_t(T a, T b, T c) noexcept : v{a, b, c} {}
    template <typename U> explicit constexpr operator vec3_t<U>() const noexcept { return vec3_t<U>{(U)v[0], (U)v[1], (U)v[2]}; }
    LS_SHIM_VEC_COMMON(3)
};

template <typename T>
union vec4_t
{
    typedef vec4_t vecN_t;
    T v[4];
    vec4_t() noexcept = default;
    constexpr vec4_t(T s) noexcept : v{s, s, s, s} {}
    constexpr vec4_t(T a, T b, T c, T d) noexcept : v{a, b, c, d} {}
    template <typename U> explicit constexpr operator vec4_t<U>() const noexcept { return vec4_t<U>{(U)v[0], (U)v[1], (U)v[2], (U)v[3]}; }
    /* the address of a vec4 is the address of its first component (the
     * reference passes &vec4 where a float pointer is expected) */
    T* operator&() noexcept { return v; }
    const T* operator&() const noexcept { return v; }
    LS_SHIM_VEC_COMMON(4)
};

#undef LS_SHIM_VEC_COMMON
#undef LS_SHIM_VEC_BINOP

typedef vec2_t<float> vec2;
typedef vec3_t<float> vec3;
typedef vec4_t<float> vec4;
typedef vec2_t<int> vec2i;
typedef vec3_t<int> vec3i;
typedef vec4_t<int> vec4i;
typedef vec4_t<double> vec4d;

template <typename T> struct ls_ident { typedef T type; };

#define LS_SHIM_SCALAR_LHS(V, OP)                                                                     \
    template <typename T> inline V<T> operator OP(typename ls_ident<T>::type s, const V<T>& a) noexcept \
    { return V<T>(s) OP a; }
LS_SHIM_SCALAR_LHS(vec2_t, +) LS_SHIM_SCALAR_LHS(vec2_t, -) LS_SHIM_SCALAR_LHS(vec2_t, *) LS_SHIM_SCALAR_LHS(vec2_t, /)
LS_SHIM_SCALAR_LHS(vec3_t, +) LS_SHIM_SCALAR_LHS(vec3_t, -) LS_SHIM_SCALAR_LHS(vec3_t, *) LS_SHIM_SCALAR_LHS(vec3_t, /)
LS_SHIM_SCALAR_LHS(vec4_t, +) LS_SHIM_SCALAR_LHS(vec4_t, -) LS_SHIM_SCALAR_LHS(vec4_t, *) LS_SHIM_SCALAR_LHS(vec4_t, /)
#undef LS_SHIM_SCALAR_LHS

/* componentwise helpers */
#define LS_SHIM_VEC_FN1(NAME)                                                                         \
    template <typename T> inline vec2_t<T> NAME(const vec2_t<T>& a) noexcept { return vec2_t<T>{NAME(a.v[0]), NAME(a.v[1])}; } \
    template <typename T> inline vec3_t<T> NAME(const vec3_t<T>& a) noexcept { return vec3_t<T>{NAME(a.v[0]), NAME(a.v[1]), NAME(a.v[2])}; } \
    template <typename T> inline vec4_t<T> NAME(const vec4_t<T>& a) noexcept { return vec4_t<T>{NAME(a.v[0]), NAME(a.v[1]), NAME(a.v[2]), NAME(a.v[3])}; }
LS_SHIM_VEC_FN1(floor)
LS_SHIM_VEC_FN1(abs)
LS_SHIM_VEC_FN1(rcp)
LS_SHIM_VEC_FN1(round)
LS_SHIM_VEC_FN1(fmod_1)
#undef LS_SHIM_VEC_FN1

#define LS_SHIM_VEC_FN2(NAME)                                                                         \
    template <typename T> inline vec2_t<T> NAME(const vec2_t<T>& a, const vec2_t<T>& b) noexcept { return vec2_t<T>{NAME(a.v[0], b.v[0]), NAME(a.v[1], b.v[1])}; } \
    template <typename T> inline vec3_t<T> NAME(const vec3_t<T>& a, const vec3_t<T>& b) noexcept { return vec3_t<T>{NAME(a.v[0], b.v[0]), NAME(a.v[1], b.v[1]), NAME(a.v[2], b.v[2])}; } \
    template <typename T> inline vec4_t<T> NAME(const vec4_t<T>& a, const vec4_t<T>& b) noexcept { return vec4_t<T>{NAME(a.v[0], b.v[0]), NAME(a.v[1], b.v[1]), NAME(a.v[2], b.v[2]), NAME(a.v[3], b.v[3])}; }
LS_SHIM_VEC_FN2(min)
LS_SHIM_VEC_FN2(max)
LS_SHIM_VEC_FN2(step)
#undef LS_SHIM_VEC_FN2

template <typename T> inline vec4_t<T> min(const vec4_t<T>& a, const vec4_t<T>& b, const vec4_t<T>& c) noexcept { return min(min(a, b), c); }
template <typename T> inline vec4_t<T> max(const vec4_t<T>& a, const vec4_t<T>& b, const vec4_t<T>& c) noexcept { return max(max(a, b), c); }
template <typename T> inline vec2_t<T> clamp(const vec2_t<T>& x, const vec2_t<T>& lo, const vec2_t<T>& hi) noexcept { return min(max(x, lo), hi); }
template <typename T> inline vec3_t<T> clamp(const vec3_t<T>& x, const vec3_t<T>& lo, const vec3_t<T>& hi) noexcept { return min(max(x, lo), hi); }
template <typename T> inline vec4_t<T> clamp(const vec4_t<T>& x, const vec4_t<T>& lo, const vec4_t<T>& hi) noexcept { return min(max(x, lo), hi); }

template <typename T> inline vec2_t<T> fmadd(const vec2_t<T>& a, const vec2_t<T>& b, const vec2_t<T>& c) noexcept { return a * b + c; }
template <typename T> inline vec3_t<T> fmadd(const vec3_t<T>& a, const vec3_t<T>& b, const vec3_t<T>& c) noexcept { return a * b + c; }
template <typename T> inline vec4_t<T> fmadd(const vec4_t<T>& a, const vec4_t<T>& b, const vec4_t<T>& c) noexcept { return a * b + c; }
template <typename T> inline vec4_t<T> fmsub(const vec4_t<T>& a, const vec4_t<T>& b, const vec4_t<T>& c) noexcept { return a * b - c; }

template <typename T> inline vec2_t<T> mix(const vec2_t<T>& a, const vec2_t<T>& b, typename ls_ident<T>::type t) noexcept { return (b - a) * t + a; }
template <typename T> inline vec3_t<T> mix(const vec3_t<T>& a, const vec3_t<T>& b, typename ls_ident<T>::type t) noexcept { return (b - a) * t + a; }
template <typename T> inline vec4_t<T> mix(const vec4_t<T>& a, const vec4_t<T>& b, typename ls_ident<T>::type t) noexcept { return (b - a) * t + a; }

template <typename T> constexpr T dot(const vec2_t<T>& a, const vec2_t<T>& b) noexcept { return a.v[0] * b.v[0] + a.v[1] * b.v[1]; }
template <typename T> constexpr T dot(const vec3_t<T>& a, const vec3_t<T>& b) noexcept { return (a.v[0] * b.v[0] + a.v[1] * b.v[1]) + a.v[2] * b.v[2]; }
template <typename T> constexpr T dot(const vec4_t<T>& a, const vec4_t<T>& b) noexcept { return ((a.v[0] * b.v[0] + a.v[1] * b.v[1]) + a.v[2] * b.v[2]) + a.v[3] * b.v[3]; }

template <typename T> constexpr T cross(const vec2_t<T>& a, const vec2_t<T>& b) noexcept { return a.v[0] * b.v[1] - a.v[1] * b.v[0]; }
template <typename T> inline vec3_t<T> cross(const vec3_t<T>& a, const vec3_t<T>& b) noexcept
{
    return vec3_t<T>{a.v[1] * b.v[2] - a.v[2] * b.v[1], a.v[2] * b.v[0] - a.v[0] * b.v[2], a.v[0] * b.v[1] - a.v[1] * b.v[0]};
}
template <typename T> inline vec4_t<T> cross(const vec4_t<T>& a, const vec4_t<T>& b) noexcept
{
    return vec4_t<T>{a.v[1] * b.v[2] - a.v[2] * b.v[1], a.v[2] * b.v[0] - a.v[0] * b.v[2], a.v[0] * b.v[1] - a.v[1] * b.v[0], T(0)};
}

template <typename T> constexpr T sum(const vec2_t<T>& a) noexcept { return a.v[0] + a.v[1]; }
template <typename T> constexpr T sum(const vec3_t<T>& a) noexcept { return (a.v[0] + a.v[1]) + a.v[2]; }
template <typename T> constexpr T sum(const vec4_t<T>& a) noexcept { return ((a.v[0] + a.v[1]) + a.v[2]) + a.v[3]; }
template <typename V, typename... Vs> inline V sum(const V& a, const V& b, const Vs&... rest) noexcept
{
    if constexpr (sizeof...(rest) == 0) return a + b;
    else return sum(a + b, rest...);
}
template <typename T> constexpr T sum_inv(const vec4_t<T>& a) noexcept { return T(1) / sum(a); }

template <typename T> inline T length_squared(const vec4_t<T>& a) noexcept { return dot(a, a); }
template <typename T> inline T length_squared(const vec3_t<T>& a) noexcept { return dot(a, a); }
template <typename T> inline T length_squared(const vec2_t<T>& a) noexcept { return dot(a, a); }
template <typename T> inline T length(const vec4_t<T>& a) noexcept { return std::sqrt(dot(a, a)); }
template <typename T> inline T length(const vec3_t<T>& a) noexcept { return std::sqrt(dot(a, a)); }
template <typename T> inline T length(const vec2_t<T>& a) noexcept { return std::sqrt(dot(a, a)); }
template <typename T> inline vec4_t<T> normalize(const vec4_t<T>& a) noexcept { return a * (T(1) / std::sqrt(dot(a, a))); }
template <typename T> inline vec3_t<T> normalize(const vec3_t<T>& a) noexcept { return a * (T(1) / std::sqrt(dot(a, a))); }
template <typename T> inline vec2_t<T> normalize(const vec2_t<T>& a) noexcept { return a * (T(1) / std::sqrt(dot(a, a))); }

inline int sign_mask(const vec4_t<float>& a) noexcept
{
    return sign_mask(a.v[0]) | (sign_mask(a.v[1]) << 1) | (sign_mask(a.v[2]) << 2) | (sign_mask(a.v[3]) << 3);
}
inline int sign_mask(const vec4_t<int>& a) noexcept
{
    return sign_mask(a.v[0]) | (sign_mask(a.v[1]) << 1) | (sign_mask(a.v[2]) << 2) | (sign_mask(a.v[3]) << 3);
}

/* vector casts */
template <typename U, typename T> using ls_cast_t = typename std::conditional<std::is_void<U>::value, T, U>::type;
template <typename U = void, typename T> constexpr vec2_t<ls_cast_t<U, T>> vec2_cast(const vec3_t<T>& a) noexcept
{ return vec2_t<ls_cast_t<U, T>>{(ls_cast_t<U, T>)a.v[0], (ls_cast_t<U, T>)a.v[1]}; }
template <typename U = void, typename T> constexpr vec2_t<ls_cast_t<U, T>> vec2_cast(const vec4_t<T>& a) noexcept
{ return vec2_t<ls_cast_t<U, T>>{(ls_cast_t<U, T>)a.v[0], (ls_cast_t<U, T>)a.v[1]}; }
template <typename U = void, typename T> constexpr vec3_t<ls_cast_t<U, T>> vec3_cast(const vec4_t<T>& a) noexcept
{ return vec3_t<ls_cast_t<U, T>>{(ls_cast_t<U, T>)a.v[0], (ls_cast_t<U, T>)a.v[1], (ls_cast_t<U, T>)a.v[2]}; }
template <typename T> constexpr vec3_t<T> vec3_cast(const vec2_t<T>& a, typename ls_ident<T>::type z) noexcept { return vec3_t<T>{a.v[0], a.v[1], z}; }
template <typename T> constexpr vec4_t<T> vec4_cast(const vec3_t<T>& a, typename ls_ident<T>::type w) noexcept { return vec4_t<T>{a.v[0], a.v[1], a.v[2], w}; }
template <typename T> constexpr vec4_t<T> vec4_cast(const vec2_t<T>& a, typename ls_ident<T>::type z, typename ls_ident<T>::type w) noexcept { return vec4_t<T>{a.v[0], a.v[1], z, w}; }
template <typename T> constexpr vec4_t<T> vec4_cast(typename ls_ident<T>::type x, const vec2_t<T>& a, typename ls_ident<T>::type w) noexcept { return vec4_t<T>{x, a.v[0], a.v[1], w}; }

/*-----------------------------------------------------------------------------
 * matrices (column-major)
-----------------------------------------------------------------------------*/
template <typename T>
struct mat2_t
{
    vec2_t<T> m[2];
    mat2_t() noexcept = default;
    constexpr mat2_t(const vec2_t<T>& a, const vec2_t<T>& b) noexcept : m{a, b} {}
    vec2_t<T>& operator[](std::size_t i) noexcept { return m[i]; }
    constexpr const vec2_t<T>& operator[](std::size_t i) const noexcept { return m[i]; }
};

template <typename T> struct mat4_t;

template <typename T>
struct mat3_t
{
    vec3_t<T> m[3];
    mat3_t() noexcept = default;
    constexpr mat3_t(const vec3_t<T>& a, const vec3_t<T>& b, const vec3_t<T>& c) noexcept : m{a, b, c} {}
    explicit mat3_t(const mat4_t<T>& a) noexcept;   /* the upper-left 3x3 */
    vec3_t<T>& operator[](std::size_t i) noexcept { return m[i]; }
    constexpr const vec3_t<T>& operator[](std::size_t i) const noexcept { return m[i]; }
};

template <typename T>
struct mat4_t
{
    vec4_t<T> m[4];
    mat4_t() noexcept = default;
    constexpr explicit mat4_t(T s) noexcept : m{vec4_t<T>{s, T(0), T(0), T(0)}, vec4_t<T>{T(0), s, T(0), T(0)},
                                                  vec4_t<T>{T(0), T(0), s, T(0)}, vec4_t<T>{T(0), T(0), T(0), s}} {}
    constexpr mat4_t(const vec4_t<T>& a, const vec4_t<T>& b, const vec4_t<T>& c, const vec4_t<T>& d) noexcept : m{a, b, c, d} {}
    constexpr mat4_t(T a0, T a1, T a2, T a3, T b0, T b1, T b2, T b3, T c0, T c1, T c2, T c3, T d0, T d1, T d2, T d3) noexcept
        : m{vec4_t<T>{a0, a1, a2, a3}, vec4_t<T>{b0, b1, b2, b3}, vec4_t<T>{c0, c1, c2, c3}, vec4_t<T>{d0, d1, d2, d3}} {}
    vec4_t<T>& operator[](std::size_t i) noexcept { return m[i]; }
    constexpr const vec4_t<T>& operator[](std::size_t i) const noexcept { return m[i]; }

    vec4_t<T> operator*(const vec4_t<T>& v) const noexcept
    {
        return ((m[0] * v.v[0] + m[1] * v.v[1]) + m[2] * v.v[2]) + m[3] * v.v[3];
    }
    mat4_t operator*(const mat4_t& o) const noexcept { return mat4_t{*this * o.m[0], *this * o.m[1], *this * o.m[2], *this * o.m[3]}; }
    mat4_t operator*(T s) const noexcept { return mat4_t{m[0] * s, m[1] * s, m[2] * s, m[3] * s}; }
    mat4_t operator+(const vec4_t<T>& v) const noexcept { return mat4_t{m[0] + v, m[1] + v, m[2] + v, m[3] + v}; }
    mat4_t operator+(const mat4_t& o) const noexcept { return mat4_t{m[0] + o.m[0], m[1] + o.m[1], m[2] + o.m[2], m[3] + o.m[3]}; }
    mat4_t operator-(const mat4_t& o) const noexcept { return mat4_t{m[0] - o.m[0], m[1] - o.m[1], m[2] - o.m[2], m[3] - o.m[3]}; }
    mat4_t& operator+=(const vec4_t<T>& v) noexcept { for (int i = 0; i < 4; ++i) m[i] += v; return *this; }
    mat4_t& operator+=(const mat4_t& o) noexcept { for (int i = 0; i < 4; ++i) m[i] += o.m[i]; return *this; }
};

template <typename T> inline mat3_t<T>::mat3_t(const mat4_t<T>& a) noexcept
    : m{vec3_t<T>{a.m[0].v[0], a.m[0].v[1], a.m[0].v[2]}, vec3_t<T>{a.m[1].v[0], a.m[1].v[1], a.m[1].v[2]},
        vec3_t<T>{a.m[2].v[0], a.m[2].v[1], a.m[2].v[2]}}
{
}

typedef mat2_t<float> mat2;
typedef mat3_t<float> mat3;
typedef mat4_t<float> mat4;

template <typename T> inline vec4_t<T> operator*(const vec4_t<T>& v, const mat4_t<T>& m) noexcept
{
    return vec4_t<T>{dot(v, m.m[0]), dot(v, m.m[1]), dot(v, m.m[2]), dot(v, m.m[3])};
}

template <typename T> inline mat4_t<T> transpose(const mat4_t<T>& a) noexcept
{
    mat4_t<T> r;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            r.m[i].v[j] = a.m[j].v[i];
    return r;
}

template <typename T> inline mat4_t<T> outer(const vec4_t<T>& a, const vec4_t<T>& b) noexcept
{
    return mat4_t<T>{b * a.v[0], b * a.v[1], b * a.v[2], b * a.v[3]};
}

template <typename T> constexpr T determinant(const mat2_t<T>& a) noexcept { return a.m[0].v[0] * a.m[1].v[1] - a.m[0].v[1] * a.m[1].v[0]; }
template <typename T> inline T determinant(const mat3_t<T>& a) noexcept
{
    return dot(a.m[0], cross(a.m[1], a.m[2]));
}
template <typename T> inline T determinant(const mat4_t<T>& a) noexcept
{
    T det = T(0);
    for (int c = 0; c < 4; ++c)
    {
        mat3_t<T> sub;
        for (int i = 1, si = 0; i < 4; ++i, ++si)
            for (int j = 0, sj = 0; j < 4; ++j)
                if (j != c) sub.m[si].v[sj++] = a.m[i].v[j];
        const T s = determinant(sub) * a.m[0].v[c];
        det = (c & 1) ? det - s : det + s;
    }
    return det;
}

} // namespace math
} // namespace ls

namespace ls
{
namespace setup
{
template <> struct IsFloat<ls::math::half> : std::true_type {};
} // namespace setup
} // namespace ls

#endif
