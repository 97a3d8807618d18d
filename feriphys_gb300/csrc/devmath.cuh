// Device vector arithmetic in the reference's evaluation order.
//
// The reference computes in cgmath 0.18 Vector3<f32>: dot = (x*x' + y*y') +
// z*z', magnitude = sqrt(dot(v, v)), normalize(v) = v * (1 / |v|),
// Vector3::angle(a, b) = atan2(|a x b|, a . b).  The library is compiled with
// -fmad=false so no a*b+c is fused, and '/' and sqrt are the IEEE-rounded
// operations; with the same operation order the results are bit-identical to
// the reference's f32 arithmetic except in the faces' corner angles: the
// atan2 is the library's own (angle.cuh), and the three corners share one
// cross-product magnitude (physics.cuh: face_corner_weight).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#if defined(__CUDACC__)
#include "angle.cuh"
#include "fastdiv.cuh"
#endif

namespace fgb {

template <class T>
struct V3 {
  T x, y, z;
};

struct __align__(16) Dbl4 {
  double x, y, z, w;
};

template <class T> struct Vec4Of;
template <> struct Vec4Of<float> { using type = float4; };
template <> struct Vec4Of<double> { using type = Dbl4; };
template <class T> using Vec4 = typename Vec4Of<T>::type;

template <class T> __device__ __forceinline__ V3<T> xyz(const Vec4<T>& v) { return {v.x, v.y, v.z}; }
template <class T> __device__ __forceinline__ Vec4<T> make4(V3<T> v, T w) {
  Vec4<T> r;
  r.x = v.x; r.y = v.y; r.z = v.z; r.w = w;
  return r;
}

template <class T> __device__ __forceinline__ V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> __device__ __forceinline__ V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> __device__ __forceinline__ V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> __device__ __forceinline__ V3<T> operator*(T s, V3<T> v) { return {s * v.x, s * v.y, s * v.z}; }
template <class T> __device__ __forceinline__ V3<T> operator*(V3<T> v, T s) { return {v.x * s, v.y * s, v.z * s}; }
template <class T> __device__ __forceinline__ V3<T> operator/(V3<T> v, T s) { return {v.x / s, v.y / s, v.z / s}; }
template <class T> __device__ __forceinline__ T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> __device__ __forceinline__ V3<T> cross(V3<T> a, V3<T> b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float sq_root(float v) { return sqrtf(v); }
__device__ __forceinline__ double sq_root(double v) { return sqrt(v); }
// atan2(y, x) for y >= 0 (the angle between two vectors: cgmath's
// Vector3::angle(a, b) = atan2(|a x b|, a . b)): the f32 form is angle.cuh's,
// the f64 form (the FP64 rerun) libm's.
#if defined(__CUDACC__)
__device__ __forceinline__ float angle_of(float y, float x) { return angle_pos(y, x); }
__device__ __forceinline__ double angle_of(double y, double x) { return atan2(y, x); }
// 1 / |v| for normalize: the f32 form without the IEEE reciprocal's range
// branch (fastdiv.cuh: rcp_of_root, the same bits)
__device__ __forceinline__ float inv_magnitude(float m) { return rcp_of_root(m); }
__device__ __forceinline__ double inv_magnitude(double m) { return 1.0 / m; }
#endif
__device__ __forceinline__ float abs_val(float v) { return fabsf(v); }
__device__ __forceinline__ double abs_val(double v) { return fabs(v); }
__device__ __forceinline__ float min_num(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ double min_num(double a, double b) { return fmin(a, b); }
template <class T> __device__ __forceinline__ T magnitude(V3<T> v) { return sq_root(dot(v, v)); }
template <class T> __device__ __forceinline__ V3<T> normalize(V3<T> v) { return v * inv_magnitude(magnitude(v)); }
template <class T> __device__ __forceinline__ bool is_zero(V3<T> v) { return v.x == T(0) && v.y == T(0) && v.z == T(0); }
template <class T> __device__ __forceinline__ bool finite3(V3<T> v) { return isfinite(v.x) && isfinite(v.y) && isfinite(v.z); }

// std::f32::consts::PI and the reference's collision offset consts::EPSILON.
constexpr float kPiF32 = 3.14159265358979323846f;
constexpr float kEpsilonF32 = 0.0001f;

}  // namespace fgb
