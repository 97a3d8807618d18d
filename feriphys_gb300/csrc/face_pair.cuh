// Drag + lift and the corner weights of two faces at once (the tiled grid
// kernel's quad: faces A and B), as the two lanes of packed f32x2
// arithmetic.  Each lane rounds exactly as the scalar instruction does, so
// every lane gives the bits of physics.cuh's face_total_force and
// face_corner_weight for its face (tests/test_gpu_math.py checks this).
#pragma once

#include "angle.cuh"
#include "devmath.cuh"
#include "fastdiv.cuh"

namespace fgb {

// A pair of 3-vectors, lane 0 and lane 1 of packed f32x2 registers: faces A
// and B of a quad run the same expression sequence, so one packed instruction
// does each step for both with the roundings of the scalar one.
struct V3x2 {
  f2 x, y, z;
};
__device__ __forceinline__ V3x2 pk3(V3<float> a, V3<float> b) { return {pk(a.x, b.x), pk(a.y, b.y), pk(a.z, b.z)}; }
__device__ __forceinline__ V3x2 add3(V3x2 a, V3x2 b) { return {add2(a.x, b.x), add2(a.y, b.y), add2(a.z, b.z)}; }
__device__ __forceinline__ V3x2 sub3(V3x2 a, V3x2 b) { return {sub2(a.x, b.x), sub2(a.y, b.y), sub2(a.z, b.z)}; }
// s * v (operator*(T, V3): s * v.x, ...) and v * s: the same products
__device__ __forceinline__ V3x2 scale3(f2 s, V3x2 v) { return {mul2(s, v.x), mul2(s, v.y), mul2(s, v.z)}; }
// (x x' + y y') + z z', every sum of products an fma with the unit `one`
// (angle.cuh: add_p2), so each product and each sum is rounded once
__device__ __forceinline__ f2 dot3(V3x2 a, V3x2 b, f2 one) {
  return add_p2(mul2(a.z, b.z), add_p2(mul2(a.x, b.x), mul2(a.y, b.y), one), one);
}
__device__ __forceinline__ V3x2 cross3(V3x2 a, V3x2 b, f2 one) {
  return {rsub_p2(mul2(a.z, b.y), mul2(a.y, b.z), one), rsub_p2(mul2(a.x, b.z), mul2(a.z, b.x), one),
          rsub_p2(mul2(a.y, b.x), mul2(a.x, b.y), one)};
}
__device__ __forceinline__ f2 sqrt2(f2 v) {
  const float2 u = upk(v);
  return pk(sqrtf(u.x), sqrtf(u.y));
}
__device__ __forceinline__ f2 magnitude3(V3x2 v, f2 one) { return sqrt2(dot3(v, v, one)); }
// rcp_of_root (fastdiv.cuh) in both lanes: 1 / magnitude with the bits of 1/x
__device__ __forceinline__ f2 rcp_of_root2(f2 x) {
  const float2 u = upk(x);
  const f2 y0 = pk(rcp_approx_ftz(u.x), rcp_approx_ftz(u.y));
  const f2 e = fma2(neg2(x), y0, dup2(1.0f));
  const float2 y1 = upk(fma2(y0, e, y0)), z = upk(y0);
  return pk(y1.x != y1.x ? z.x : y1.x, y1.y != y1.y ? z.y : y1.y);
}

// drag + lift (D) and the three corner weights angle_k / PI of two faces
// (springy_mesh.rs:629-654, 134-172), lane 0 and lane 1, as
// face_total_force and face_corner_weight compute them: corners 0 and 1 take
// y = |(x1-x0) x (x2-x0)| and their dot products (x0-x1 = -(x1-x0) exactly),
// corner 2 the rest of the unit share; the mean velocity and the shares by
// multiplication with RN(1/3) and RN(1/pi).
__device__ __forceinline__ void face_terms2(V3x2 x0, V3x2 x1, V3x2 x2, V3x2 v0, V3x2 v1, V3x2 v2, V3x2 wind,
                                            float neg_cd, float neg_lift, float one_rt, float4& DwA, float2& wA,
                                            float4& DwB, float2& wB) {
  const f2 one = dup2(one_rt);
  const V3x2 sum = add3(add3(v0, v1), v2);
  const f2 r3 = dup2(kRcp3);
  // rv = avg - wind with avg = sum * RN(1/3) kept rounded (add_p2)
  const V3x2 rv{add_p2(mul2(sum.x, r3), neg2(wind.x), one), add_p2(mul2(sum.y, r3), neg2(wind.y), one),
                add_p2(mul2(sum.z, r3), neg2(wind.z), one)};
  const V3x2 e1 = sub3(x1, x0), e2 = sub3(x2, x0), e3 = sub3(x2, x1);
  const V3x2 cr = cross3(e1, e2, one);
  const f2 mag = magnitude3(cr, one);
  const f2 area = mul2(mag, dup2(0.5f));  // mag / 2, exactly
  const f2 inv = rcp_of_root2(mag);
  const V3x2 n{mul2(cr.x, inv), mul2(cr.y, inv), mul2(cr.z, inv)};
  const f2 eff = mul2(area, abs2(dot3(n, rv, one)));
  const V3x2 drag = scale3(mul2(dup2(neg_cd), eff), rv);
  const f2 m2 = magnitude3(cross3(n, rv, one), one);
  const V3x2 lift = scale3(mul2(dup2(neg_lift), eff), V3x2{mul2(rv.x, m2), mul2(rv.y, m2), mul2(rv.z, m2)});
  const V3x2 D{add_p2(lift.x, drag.x, one), add_p2(lift.y, drag.y, one), add_p2(lift.z, drag.z, one)};
  const f2 a0 = angle_pos2(mag, dot3(e2, e1, one), one);
  const f2 a1 = angle_pos2(mag, neg2(dot3(e1, e3, one)), one);
  const f2 rpi = dup2(kRcpPi), mone = neg2(one);
  const f2 w0 = mul2(a0, rpi), w1 = mul2(a1, rpi);
  const f2 w2 = fma2(w1, mone, fma2(w0, mone, dup2(1.0f)));  // (1 - w0) - w1, the products kept rounded
  const float2 dx = upk(D.x), dy = upk(D.y), dz = upk(D.z), u0 = upk(w0), u1 = upk(w1), u2 = upk(w2);
  DwA = make_float4(dx.x, dy.x, dz.x, u0.x);
  DwB = make_float4(dx.y, dy.y, dz.y, u0.y);
  wA = make_float2(u1.x, u2.x);
  wB = make_float2(u1.y, u2.y);
}

}  // namespace fgb
