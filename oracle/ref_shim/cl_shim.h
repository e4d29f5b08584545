/*
 * cl_shim.h -- OpenCL C 1.1 vocabulary for g++, so that the reference's own
 * device kernels (PCISPH/data/kernels/{grid_utils,sort_utils,pcisph}.cl) can be
 * compiled unmodified as C++ and run on the host.
 *
 * TEST INFRASTRUCTURE ONLY. This header and the library built with it
 * (oracle/_ref/) are checkers: they produce golden vectors and pin the
 * oracle restatement. Nothing in the pcisph_gb300 product links them.
 *
 * Only the subset the three .cl files use is provided:
 *   types      float3, int3, uint2, uint
 *   memory     vload2/vstore2 (uint), vload3/vstore3 (float)
 *   geometry   dot, distance, fast_length
 *   math       max(float,float)
 *   conversion convert_int3_sat_rtn
 *   work-item  get_global_id(0)  (a thread-local set by the host driver)
 *   qualifiers __kernel, __global, __constant
 *
 * Semantics chosen where OpenCL leaves room (recorded as parity sources):
 *   - dot(a,b) = (a.x*b.x + a.y*b.y) + a.z*b.z, no fused multiply-add
 *     (the build passes -ffp-contract=off).
 *   - distance / fast_length = sqrtf(dot(d,d)), correctly rounded. OpenCL allows
 *     fast_length to be approximate (half_sqrt); any device may differ there.
 *   - convert_int3_sat_rtn: floor, saturate to [INT_MIN, INT_MAX], NaN -> 0
 *     (OpenCL 1.1 section 6.2.3.3, "_sat" conversions).
 *   - max(x,y) for float returns y if x < y, else x (OpenCL 1.1 section 6.11.4).
 *
 * The OpenCL cast-literal form "(float3)(a,b,c)" is not C++; the build recipe
 * (oracle/build_ref.sh) rewrites it to "float3(a,b,c)" on the way into g++
 * through a pipe, so no rewritten copy of the reference sources is kept.
 */
#ifndef PCISPH_ORACLE_CL_SHIM_H
#define PCISPH_ORACLE_CL_SHIM_H

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <climits>

typedef unsigned int uint;

#define __kernel
#define __global
#define __constant const

struct float3 {
    float x, y, z;
    float3() : x(0.f), y(0.f), z(0.f) {}
    explicit float3(float s) : x(s), y(s), z(s) {}
    float3(float a, float b, float c) : x(a), y(b), z(c) {}
    float3& operator+=(const float3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    float3& operator-=(const float3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    float3& operator*=(float s) { x *= s; y *= s; z *= s; return *this; }
};
inline float3 operator+(const float3& a, const float3& b) { return float3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline float3 operator-(const float3& a, const float3& b) { return float3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline float3 operator-(const float3& a) { return float3(-a.x, -a.y, -a.z); }
inline float3 operator*(const float3& a, float s) { return float3(a.x * s, a.y * s, a.z * s); }
inline float3 operator*(float s, const float3& a) { return float3(s * a.x, s * a.y, s * a.z); }
inline float3 operator/(const float3& a, float s) { return float3(a.x / s, a.y / s, a.z / s); }

struct int3 {
    int x, y, z;
    int3() : x(0), y(0), z(0) {}
    int3(int a, int b, int c) : x(a), y(b), z(c) {}
};
/* OpenCL integer vector addition wraps; the build passes -fwrapv. */
inline int3 operator+(const int3& a, const int3& b) { return int3(a.x + b.x, a.y + b.y, a.z + b.z); }

struct uint2 {
    uint x, y;
    uint2() : x(0u), y(0u) {}
    explicit uint2(uint s) : x(s), y(s) {}
    uint2(uint a, uint b) : x(a), y(b) {}
};

inline float3 vload3(size_t i, const float* p) { return float3(p[3 * i + 0], p[3 * i + 1], p[3 * i + 2]); }
inline void vstore3(const float3& v, size_t i, float* p) { p[3 * i + 0] = v.x; p[3 * i + 1] = v.y; p[3 * i + 2] = v.z; }
inline uint2 vload2(size_t i, const uint* p) { return uint2(p[2 * i + 0], p[2 * i + 1]); }
inline void vstore2(const uint2& v, size_t i, uint* p) { p[2 * i + 0] = v.x; p[2 * i + 1] = v.y; }

inline float dot(const float3& a, const float3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float fast_length(const float3& d) { return std::sqrt(dot(d, d)); }
inline float distance(const float3& a, const float3& b) { return fast_length(a - b); }
inline float max(float x, float y) { return x < y ? y : x; }

inline int cl_convert_int_sat_rtn(float v) {
    if (std::isnan(v)) return 0;
    float f = std::floor(v);
    if (f >= 2147483648.0f) return INT_MAX;
    if (f < -2147483648.0f) return INT_MIN;
    return (int)f;
}
inline int3 convert_int3_sat_rtn(const float3& v) {
    return int3(cl_convert_int_sat_rtn(v.x), cl_convert_int_sat_rtn(v.y), cl_convert_int_sat_rtn(v.z));
}

/* One work-item per host loop iteration; the driver sets this before each call. */
extern thread_local size_t cl_shim_global_id;
inline size_t get_global_id(uint /*dim*/) { return cl_shim_global_id; }

#endif
