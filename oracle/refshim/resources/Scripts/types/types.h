/*
 * OpenCL-C -> C++ shim for compiling the reference's own kernel sources on
 * the host CPU.  TEST INFRASTRUCTURE ONLY: this header is used exclusively by
 * oracle/refshim/ref_kernels.cpp to build the reference-kernel oracle under
 * oracle/_ref/; nothing in the product links it.
 *
 * It shadows the reference's `resources/Scripts/types/types.h` (the kernel
 * files include it by that path) and provides, in plain C++17:
 *   - the OpenCL vector types used by the hot-path kernels (float2/3/4,
 *     usize2/3/4) with the `.XYZ` swizzle the kernels use, implemented as a
 *     member call returning a write-through proxy;
 *   - the OpenCL built-ins the kernels call (dot, length, cross, min, max,
 *     sqrt, pow, fabs, isnan, isinf, get_global_id, get_local_id);
 *   - the neighbour-loop macros BEGIN_NEIGHS/END_NEIGHS with the visiting
 *     order of the reference (types/3D.h:197-219, types/2D.h:174-194):
 *     x offset outermost, then y, then z, particles of a cell in sorted order
 *     from ihoc[c] while icell[j] == c;
 *   - the vector constants (VEC_ZERO, VEC_INFINITY, ...) of types/2D.h and
 *     types/3D.h.
 * The kernel arithmetic itself (Wendland functions, interaction sums, EOS,
 * integrator, link-list hashing) is compiled from the reference files where
 * they lie, unmodified.
 *
 * Floating point: every operation is a single IEEE binary32 operation in
 * source order; the build uses -ffp-contract=off so no FMA contraction takes
 * place.  dot() sums left to right ((x*x + y*y) + z*z), length() is
 * sqrt(dot(v, v)).
 */
#pragma once

#include <cmath>
#include <cstdint>
#include <cfloat>

typedef unsigned long usize;
typedef long ssize;
typedef unsigned int uint;

/* ---------------------------------------------------------------- float2 */
struct float2
{
    float x, y;
    float2() = default;
    constexpr float2(float a, float b) : x(a), y(b) {}
    explicit constexpr float2(float s) : x(s), y(s) {}
    float2& xy_() { return *this; }
    const float2& xy_() const { return *this; }
};
/* ---------------------------------------------------------------- float3 */
struct float3
{
    float x, y, z;
    float3() = default;
    constexpr float3(float a, float b, float c) : x(a), y(b), z(c) {}
    explicit constexpr float3(float s) : x(s), y(s), z(s) {}
    float3& xyz_() { return *this; }
    const float3& xyz_() const { return *this; }
};

/* Write-through proxies for the .xyz / .xy swizzles of a float4 lvalue */
struct f4_xyz
{
    float* p;
    operator float3() const { return float3(p[0], p[1], p[2]); }
    f4_xyz& operator=(const float3& v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; return *this; }
    f4_xyz& operator=(const f4_xyz& o) { float3 v = o; return (*this = v); }
    f4_xyz& operator+=(const float3& v) { p[0] = p[0] + v.x; p[1] = p[1] + v.y; p[2] = p[2] + v.z; return *this; }
    f4_xyz& operator-=(const float3& v) { p[0] = p[0] - v.x; p[1] = p[1] - v.y; p[2] = p[2] - v.z; return *this; }
};
struct f4_xy
{
    float* p;
    operator float2() const { return float2(p[0], p[1]); }
    f4_xy& operator=(const float2& v) { p[0] = v.x; p[1] = v.y; return *this; }
    f4_xy& operator=(const f4_xy& o) { float2 v = o; return (*this = v); }
    f4_xy& operator+=(const float2& v) { p[0] = p[0] + v.x; p[1] = p[1] + v.y; return *this; }
    f4_xy& operator-=(const float2& v) { p[0] = p[0] - v.x; p[1] = p[1] - v.y; return *this; }
};

/* ---------------------------------------------------------------- float4 */
struct float4
{
    float x, y, z, w;
    float4() = default;
    constexpr float4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    /* OpenCL (float4)(s) broadcasts a scalar */
    constexpr float4(float s) : x(s), y(s), z(s), w(s) {}
    f4_xyz xyz_() { return f4_xyz{ &x }; }
    float3 xyz_() const { return float3(x, y, z); }
    f4_xy xy_() { return f4_xy{ &x }; }
    float2 xy_() const { return float2(x, y); }
};

struct float16
{
    float s[16];
};

/* Integer vectors (only the members the kernels touch) */
struct usize2 { usize x, y; };
struct usize3 { usize x, y, z; };
struct usize4 { usize x, y, z, w; };
struct uint4 { uint x, y, z, w; };
#define uivec4 uint4

/* ------------------------------------------------------ element-wise ops */
#define F2_BIN(OP) float2(a.x OP b.x, a.y OP b.y)
#define F3_BIN(OP) float3(a.x OP b.x, a.y OP b.y, a.z OP b.z)
#define F4_BIN(OP) float4(a.x OP b.x, a.y OP b.y, a.z OP b.z, a.w OP b.w)
#define F2_SCL(A, OP, S) float2(A.x OP S, A.y OP S)
#define F3_SCL(A, OP, S) float3(A.x OP S, A.y OP S, A.z OP S)
#define F4_SCL(A, OP, S) float4(A.x OP S, A.y OP S, A.z OP S, A.w OP S)
inline float2 operator+(const float2& a, const float2& b) { return F2_BIN(+); }
inline float2 operator-(const float2& a, const float2& b) { return F2_BIN(-); }
inline float2 operator*(const float2& a, const float2& b) { return F2_BIN(*); }
inline float2 operator/(const float2& a, const float2& b) { return F2_BIN(/); }
inline float2 operator*(const float2& a, float s) { return F2_SCL(a, *, s); }
inline float2 operator*(float s, const float2& a) { return float2(s * a.x, s * a.y); }
inline float2 operator/(const float2& a, float s) { return F2_SCL(a, /, s); }
inline float2 operator-(const float2& a) { return float2(-a.x, -a.y); }
inline float2& operator+=(float2& a, const float2& b) { a = a + b; return a; }
inline float2& operator-=(float2& a, const float2& b) { a = a - b; return a; }
inline float2& operator/=(float2& a, float s) { a = a / s; return a; }

inline float3 operator+(const float3& a, const float3& b) { return F3_BIN(+); }
inline float3 operator-(const float3& a, const float3& b) { return F3_BIN(-); }
inline float3 operator*(const float3& a, const float3& b) { return F3_BIN(*); }
inline float3 operator/(const float3& a, const float3& b) { return F3_BIN(/); }
inline float3 operator*(const float3& a, float s) { return F3_SCL(a, *, s); }
inline float3 operator*(float s, const float3& a) { return float3(s * a.x, s * a.y, s * a.z); }
inline float3 operator/(const float3& a, float s) { return F3_SCL(a, /, s); }
inline float3 operator-(const float3& a) { return float3(-a.x, -a.y, -a.z); }
inline float3& operator+=(float3& a, const float3& b) { a = a + b; return a; }
inline float3& operator-=(float3& a, const float3& b) { a = a - b; return a; }
inline float3& operator/=(float3& a, float s) { a = a / s; return a; }

inline float4 operator+(const float4& a, const float4& b) { return F4_BIN(+); }
inline float4 operator-(const float4& a, const float4& b) { return F4_BIN(-); }
inline float4 operator*(const float4& a, const float4& b) { return F4_BIN(*); }
inline float4 operator/(const float4& a, const float4& b) { return F4_BIN(/); }
inline float4 operator*(const float4& a, float s) { return F4_SCL(a, *, s); }
inline float4 operator*(float s, const float4& a) { return float4(s * a.x, s * a.y, s * a.z, s * a.w); }
inline float4 operator/(const float4& a, float s) { return F4_SCL(a, /, s); }
inline float4 operator-(const float4& a) { return float4(-a.x, -a.y, -a.z, -a.w); }
inline float4& operator+=(float4& a, const float4& b) { a = a + b; return a; }
inline float4& operator-=(float4& a, const float4& b) { a = a - b; return a; }
inline float4& operator/=(float4& a, float s) { a = a / s; return a; }


/* ------------------------------------------------------------- built-ins */
inline float dot(const float2& a, const float2& b) { return a.x * b.x + a.y * b.y; }
inline float dot(const float3& a, const float3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float dot(const float4& a, const float4& b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
inline float length(const float2& a) { return std::sqrt(dot(a, a)); }
inline float length(const float3& a) { return std::sqrt(dot(a, a)); }
inline float length(const float4& a) { return std::sqrt(dot(a, a)); }
inline float3 cross(const float3& a, const float3& b)
{
    return float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float4 cross(const float4& a, const float4& b)
{
    return float4(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x, 0.f);
}
/* OpenCL min/max for floats: y if y < x (resp. x < y), else x */
inline float min(float x, float y) { return (y < x) ? y : x; }
inline float max(float x, float y) { return (x < y) ? y : x; }
inline float sqrt(float x) { return std::sqrt(x); }
inline float pow(float x, float y) { return std::pow(x, y); }
inline float fabs(float x) { return std::fabs(x); }
inline bool isnan(float x) { return std::isnan(x); }
inline bool isinf(float x) { return std::isinf(x); }
/* The analytic Shepard factor of the BI walls (KernelFunctions/Wendland*D.hcl
 * kernelS_D) */
inline float sign(float x) { return (x > 0.f) ? 1.f : ((x < 0.f) ? -1.f : 0.f); }
inline float acospi(float x) { return std::acos(x) / 3.14159265f; }
inline float atan(float x) { return std::atan(x); }

/* Work-item index: the harness sets it before calling a kernel function */
extern thread_local usize aqr_gid;
#define get_global_id(d) (aqr_gid)
#define get_local_id(d) ((usize)0)

/* OpenCL address-space qualifiers */
#define __kernel
#define __global
#define __local
#define __constant const

#ifndef INFINITY
#define INFINITY FLT_MAX
#endif

/* ----------------------------------------------- dimension-dependent part */
#define vec2 float2
#define vec3 float3
#define vec4 float4
#define svec4 usize4

#ifdef HAVE_3D
#define vec float4
#define vec_xyz float3
#define svec_xyz usize3
#define matrix float16
#define XYZ xyz_()
#define VEC_ZERO (float4(0.f, 0.f, 0.f, 0.f))
#define VEC_ONE (float4(1.f, 1.f, 1.f, 0.f))
#define VEC_INFINITY (float4(INFINITY, INFINITY, INFINITY, 0.f))
#define VEC_NEG_INFINITY (-VEC_INFINITY)
inline float4 aqr_matrix_dot(const float16& m, const float4& v)
{
    return float4(m.s[0] * v.x + m.s[1] * v.y + m.s[2] * v.z,
                  m.s[4] * v.x + m.s[5] * v.y + m.s[6] * v.z,
                  m.s[8] * v.x + m.s[9] * v.y + m.s[10] * v.z,
                  0.f);
}
#define MATRIX_DOT(_M, _V) aqr_matrix_dot(_M, _V)
/* types/3D.h:197-219 -- 27 cells, x offset outermost, z innermost */
#define BEGIN_NEIGHS(CELL, NPARTS, NCELLS, ICELL, IHOC)                        \
    for (int __ci = -1; __ci <= 1; __ci++) {                                   \
        for (int __cj = -1; __cj <= 1; __cj++) {                               \
            for (int __ck = -1; __ck <= 1; __ck++) {                           \
                const uint __c_j = CELL + __ci + __cj * NCELLS.x +             \
                                   __ck * NCELLS.x * NCELLS.y;                 \
                uint j = IHOC[__c_j];                                          \
                while ((j < NPARTS) && (ICELL[j] == __c_j)) {
#define END_NEIGHS()                                                           \
                    j++;                                                       \
                }                                                              \
            }                                                                  \
        }                                                                      \
    }
#else
#define vec float2
#define vec_xyz float2
#define svec_xyz usize2
#define matrix float4
#define XYZ xy_()
#define VEC_ZERO (float2(0.f, 0.f))
#define VEC_ONE (float2(1.f, 1.f))
#define VEC_INFINITY (float2(INFINITY, INFINITY))
#define VEC_NEG_INFINITY (-VEC_INFINITY)
inline float2 aqr_matrix_dot(const float4& m, const float2& v)
{
    return float2(m.x * v.x + m.y * v.y, m.z * v.x + m.w * v.y);
}
#define MATRIX_DOT(_M, _V) aqr_matrix_dot(_M, _V)
/* types/2D.h:174-194 -- 9 cells, x offset outermost.  The cell index is
 * taken modulo 2^32, as the reference computes it where usize is 32 bits:
 * cfd/Boundary/BI/Interactions.cl passes n_cells as uivec4, so
 * `__cj * NCELLS.x` is 32-bit unsigned arithmetic, and with a 64-bit usize
 * the row below (__cj = -1) would land 2^32 cells past the table. */
#define BEGIN_NEIGHS(CELL, NPARTS, NCELLS, ICELL, IHOC)                        \
    for (int __ci = -1; __ci <= 1; __ci++) {                                   \
        for (int __cj = -1; __cj <= 1; __cj++) {                               \
            const usize __c_j = (uint)(CELL + __ci + __cj * NCELLS.x);         \
            usize j = IHOC[__c_j];                                             \
            while ((j < NPARTS) && (ICELL[j] == __c_j)) {
#define END_NEIGHS()                                                           \
                j++;                                                           \
            }                                                                  \
        }                                                                      \
    }
#endif

#define LINKLIST_LOCAL_PARAMS                                                  \
    const usize* icell, const usize* ihoc, usize4 n_cells
