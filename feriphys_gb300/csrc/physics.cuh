// Per-vertex physics of one Simulation::step, shared by every kernel.
//
// Each function restates one piece of the reference's step with its
// expression order (file:line relative to the reference project root):
//   strut spring + damper          springy_mesh.rs:533-551
//   face drag + lift, angle split  springy_mesh.rs:629-654, 118-172
//   explicit Euler / "RK4"         state.rs:75-106 with Point, springy_mesh.rs:199-256
//   vertex-face collision          collidable_mesh.rs:107-169, springy_mesh.rs:437-481
#pragma once

#include "devmath.cuh"
#include "step_consts.h"

namespace fgb {

// Spring and damper force on the strut's first vertex (the second gets the
// negation, -1.0 * f, which is exact).  p0/v0 belong to strut vertex a,
// p1/v1 to b: u = normalize(p1 - p0).
template <class T>
__device__ __forceinline__ void strut_forces(V3<T> p0, V3<T> p1, V3<T> v0, V3<T> v1, T k, T c, T L, V3<T>& sf,
                                             V3<T>& df) {
  const V3<T> d = p1 - p0;
  const V3<T> u = normalize(d);
  sf = (k * (magnitude(d) - L)) * u;
  df = (c * dot(v1 - v0, u)) * u;
}

// drag + lift of one face (springy_mesh.rs:634-646).
template <class T>
__device__ __forceinline__ V3<T> face_total_force(V3<T> x0, V3<T> x1, V3<T> x2, V3<T> v0, V3<T> v1, V3<T> v2,
                                                  V3<T> wind, T neg_cd, T neg_cl) {
  const V3<T> avg = ((v0 + v1) + v2) / T(3);
  const V3<T> rv = avg - wind;
  const V3<T> cr = cross(x1 - x0, x2 - x0);
  const T area = magnitude(cr) / T(2);
  const V3<T> n = normalize(cr);
  const T eff = area * abs_val(dot(n, rv));
  const V3<T> drag = (neg_cd * eff) * rv;
  const V3<T> lift = (neg_cl * eff) * (rv * magnitude(cross(n, rv)));
  return drag + lift;
}

// Vertex angle of corner k over PI (springy_mesh.rs:134-172, 647-649).
template <class T>
__device__ __forceinline__ T face_corner_weight(V3<T> x0, V3<T> x1, V3<T> x2, int k) {
  T a;
  if (k == 0) a = vangle(x2 - x0, x1 - x0);
  else if (k == 1) a = vangle(x0 - x1, x2 - x1);
  else a = vangle(x1 - x2, x0 - x2);
  return a / T(kPiF32);
}

// State integration of one point with frozen force F.  m' = m + 0*h and
// F' = F + 0*h are kept (they only differ from m, F in the sign of zero).
template <class T>
__device__ __forceinline__ void integrate_point(int integration, T h, V3<T> p, V3<T> v, V3<T> F, T m, V3<T>& np,
                                                V3<T>& nv, V3<T>& nF) {
  const V3<T> z3{T(0), T(0), T(0)};
  if (integration == 0) {  // state.rs:75-83
    const V3<T> a = F / m;
    np = p + v * h;
    nv = v + a * h;
    nF = F + z3 * h;
  } else {  // state.rs:86-106: k1..k4 share the carried F, so only v stages differ
    const T hh = h * T(0.5);
    const V3<T> a1 = F / m;
    const V3<T> F2 = F + z3 * hh;
    const T m2 = m + T(0) * hh;
    const V3<T> v2 = v + a1 * hh;
    const V3<T> a2 = F2 / m2;
    const V3<T> F3 = F + z3 * hh;
    const T m3 = m + T(0) * hh;
    const V3<T> v3 = v + a2 * hh;
    const V3<T> a3 = F3 / m3;
    const V3<T> F4 = F + z3 * h;
    const T m4 = m + T(0) * h;
    const V3<T> v4 = v + a3 * h;
    const V3<T> a4 = F4 / m4;
    const T h6 = h / T(6), h3 = h / T(3);
    np = p + (((h6 * v + h3 * v2) + h3 * v3) + h6 * v4);
    nv = v + (((h6 * a1 + h3 * a2) + h3 * a3) + h6 * a4);
    const V3<T> zf = ((h6 * z3 + h3 * z3) + h3 * z3) + h6 * z3;
    nF = F + zf;
  }
}

// One obstacle face as stored on the device: v0 (w = drop axis 0/1/2 as
// float bits), v1, v2, unit normal (computed on the host exactly as
// collidable_mesh.rs:41-43 does).
struct ObsFace {
  float4 v0, v1, v2, n;
};

// The crossing test of one face (collidable_mesh.rs:107-145): signs of the
// plane distances differ and the projected point lies inside the triangle.
template <class T>
__device__ __forceinline__ bool face_hit(const ObsFace& F, V3<T> op, V3<T> np, T dtd, T& d_old, T& d_new) {
  const V3<T> v0{T(F.v0.x), T(F.v0.y), T(F.v0.z)};
  const V3<T> n{T(F.n.x), T(F.n.y), T(F.n.z)};
  d_old = dot(op - v0, n);
  d_new = dot(np - v0, n);
  if (signbit(d_old) == signbit(d_new)) return false;
  const V3<T> ovel = (np - op) / dtd;
  const T fr = d_old / (d_old - d_new);
  const V3<T> cp = op + (dtd * fr) * ovel;
  const V3<T> v1{T(F.v1.x), T(F.v1.y), T(F.v1.z)};
  const V3<T> v2{T(F.v2.x), T(F.v2.y), T(F.v2.z)};
  const int axis = __float_as_int(F.v0.w);
  V3<T> a = v0, b = v1, c = v2, p = cp;
  if (axis == 0) { a.x = T(0); b.x = T(0); c.x = T(0); p.x = T(0); }
  else if (axis == 1) { a.y = T(0); b.y = T(0); c.y = T(0); p.y = T(0); }
  else { a.z = T(0); b.z = T(0); c.z = T(0); p.z = T(0); }
  const bool o0 = !signbit(dot(cross(b - a, p - a), n));
  const bool o1 = !signbit(dot(cross(c - b, p - b), n));
  const bool o2 = !signbit(dot(cross(a - c, p - c), n));
  return o0 == o1 && o1 == o2;
}

// Collision response (springy_mesh.rs:444-480) for a hit on face F.
template <class T>
__device__ __forceinline__ void collision_response(const ObsFace& F, T d_old, T d_new, V3<T> op, V3<T> ov, V3<T> oF,
                                                   T om, T dt, T e, T mu, V3<T>& np, V3<T>& nv) {
  const V3<T> n{T(F.n.x), T(F.n.y), T(F.n.z)};
  const T fr = d_old / (d_old - d_new);
  const V3<T> cp = op + (dt * fr) * ov;
  const V3<T> vc = ov + ((dt * fr) * oF) / om;
  np = cp + n * T(kEpsilonF32);
  const V3<T> vcn = dot(vc, n) * n;
  const V3<T> vct = vc - vcn;
  const V3<T> vrn = (T(-1) * vcn) * e;
  V3<T> vrt{T(0), T(0), T(0)};
  const T mt = magnitude(vct);
  if (!(is_zero(vct) || isnan(mt))) vrt = vct - normalize(vct) * min_num(mu * magnitude(vcn), mt);
  nv = vrn + vrt;
}

// First hit over the flattened obstacle faces, then the response.  Returns
// true when the point collided.
template <class T>
__device__ __forceinline__ bool collide_point(const ObsFace* __restrict__ faces, int n_faces, V3<T> op, V3<T> ov,
                                              V3<T> oF, T om, V3<T>& np, V3<T>& nv, const StepConsts& c) {
  const T dtd = T(c.dt_duration);
  for (int f = 0; f < n_faces; ++f) {
    const ObsFace F = faces[f];
    T d_old, d_new;
    if (face_hit(F, op, np, dtd, d_old, d_new)) {
      collision_response(F, d_old, d_new, op, ov, oF, om, T(c.dt), T(c.restitution), T(c.friction), np, nv);
      return true;
    }
  }
  return false;
}

}  // namespace fgb
