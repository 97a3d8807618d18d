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
#include "fastdiv.cuh"
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

// drag + lift of one face (springy_mesh.rs:634-646).  The f32 step takes
// the mean velocity as the sum times RN(1/3) (the reference divides by 3: at
// most an ulp apart, in the face terms only); the FP64 rerun divides.
template <class T>
__device__ __forceinline__ V3<T> face_total_force(V3<T> x0, V3<T> x1, V3<T> x2, V3<T> v0, V3<T> v1, V3<T> v2,
                                                  V3<T> wind, T neg_cd, T neg_cl) {
  V3<T> avg;
  if constexpr (sizeof(T) == 8) avg = ((v0 + v1) + v2) / T(3);
  else avg = ((v0 + v1) + v2) * kRcp3;
  const V3<T> rv = avg - wind;
  const V3<T> cr = cross(x1 - x0, x2 - x0);
  const T area = magnitude(cr) / T(2);
  const V3<T> n = normalize(cr);
  const T eff = area * abs_val(dot(n, rv));
  const V3<T> drag = (neg_cd * eff) * rv;
  const V3<T> lift = (neg_cl * eff) * (rv * magnitude(cross(n, rv)));
  return drag + lift;
}

// Vertex angle of corner k over PI (springy_mesh.rs:134-172, 647-649).  The
// reference takes each corner's angle as atan2(|a x b|, a . b) of that
// corner's two edges; the FP64 rerun (T = double) does exactly that.  The f32
// step saves work the reference repeats: |a x b| is twice the face's area at
// every corner, so corners 0 and 1 take the one magnitude
// |(x1 - x0) x (x2 - x0)| the drag already needs, with their own dot products
// in the reference's order; the angles sum to pi, so corner 2's share is
// (1 - w0) - w1; and a share is the angle times RN(1/pi) instead of over pi.
// Each differs from the reference's per-corner computation by rounding only
// (about 1e-7 of the face's force), like the angle's own last bits.
template <class T>
__device__ __forceinline__ T corner_share(V3<T> x0, V3<T> x1, V3<T> x2, T y, int k) {
  const T x = k == 0 ? dot(x2 - x0, x1 - x0) : dot(x0 - x1, x2 - x1);
  return angle_of(y, x) * kRcpPi;
}
template <class T>
__device__ __forceinline__ T face_corner_weight(V3<T> x0, V3<T> x1, V3<T> x2, int k) {
  if constexpr (sizeof(T) == 8) {  // the reference's form
    V3<T> a, b;
    if (k == 0) { a = x2 - x0; b = x1 - x0; }
    else if (k == 1) { a = x0 - x1; b = x2 - x1; }
    else { a = x1 - x2; b = x0 - x2; }
    return angle_of(magnitude(cross(a, b)), dot(a, b)) / T(kPiF32);
  } else {
    const T y = magnitude(cross(x1 - x0, x2 - x0));
    if (k < 2) return corner_share(x0, x1, x2, y, k);
    return (T(1) - corner_share(x0, x1, x2, y, 0)) - corner_share(x0, x1, x2, y, 1);
  }
}

// F / m componentwise, exactly as IEEE division; the f32 form shares one
// correctly rounded reciprocal of m (fastdiv.cuh) and checks the three
// quotients with one guard.  A zero component (a flat cloth's out-of-plane
// force) is exactly a * RN(1/m), a zero of the right sign, and needs no
// slow path; Markstein's correction would turn -0 into +0.
struct MassDiv {
  float m, y;
  bool fast;
};
__device__ __forceinline__ MassDiv mass_div(float m) {
  const bool fast = rcp_usable(m);
  return {m, fast ? rcp_rn_fast(m) : 0.0f, fast};
}
static __device__ __noinline__ V3<float> div3_ieee_cold(V3<float> F, float m) { return F / m; }
// 2^-100 <= |x| <= 2^100 (the range div_known_rcp's fast path accepts)
__device__ __forceinline__ bool markstein_range(float x) {
  return ((__float_as_uint(x) & 0x7fffffffu) - 0x0d800000u) <= (0x71800000u - 0x0d800000u);
}
__device__ __forceinline__ float div_known_rcp_z(float a, float b, float y, bool& ok) {
  const float q = __fmul_rn(a, y);
  const float r = __fmaf_rn(-b, q, a);
  const float q2 = __fmaf_rn(r, y, q);
  const bool zero = a == 0.0f;
  ok = ok && (zero || (markstein_range(a) && markstein_range(q2)));
  return zero ? q : q2;
}
__device__ __forceinline__ V3<float> div_mass(V3<float> F, float m, const MassDiv& d) {
  if (d.fast && m == d.m) {
    bool ok = true;
    const V3<float> q{div_known_rcp_z(F.x, m, d.y, ok), div_known_rcp_z(F.y, m, d.y, ok),
                      div_known_rcp_z(F.z, m, d.y, ok)};
    if (ok) return q;
  }
  return div3_ieee_cold(F, m);
}
struct MassDivD {
  double m;
};
__device__ __forceinline__ MassDivD mass_div(double m) { return {m}; }
__device__ __forceinline__ V3<double> div_mass(V3<double> F, double m, const MassDivD&) { return F / m; }

template <class T>
struct Integrated {
  V3<T> p, v, F;
};

// state.rs:86-106: k1..k4 share the carried F, so only the v stages differ.
// Out of line: the Euler step is the common case and this branch, inlined,
// doubled the integration code of every step kernel.
template <class T>
static __device__ __noinline__ Integrated<T> integrate_rk4(T h, V3<T> p, V3<T> v, V3<T> F, T m) {
  const V3<T> z3{T(0), T(0), T(0)};
  const auto md = mass_div(m);
  Integrated<T> out;
  {
    const T hh = h * T(0.5);
    const V3<T> a1 = div_mass(F, m, md);
    const V3<T> F2 = F + z3 * hh;
    const T m2 = m + T(0) * hh;
    const V3<T> v2 = v + a1 * hh;
    const V3<T> a2 = div_mass(F2, m2, md);
    const V3<T> F3 = F + z3 * hh;
    const T m3 = m + T(0) * hh;
    const V3<T> v3 = v + a2 * hh;
    const V3<T> a3 = div_mass(F3, m3, md);
    const V3<T> F4 = F + z3 * h;
    const T m4 = m + T(0) * h;
    const V3<T> v4 = v + a3 * h;
    const V3<T> a4 = div_mass(F4, m4, md);
    const T h6 = h / T(6), h3 = h / T(3);
    out.p = p + (((h6 * v + h3 * v2) + h3 * v3) + h6 * v4);
    out.v = v + (((h6 * a1 + h3 * a2) + h3 * a3) + h6 * a4);
    const V3<T> zf = ((h6 * z3 + h3 * z3) + h3 * z3) + h6 * z3;
    out.F = F + zf;
  }
  return out;
}

// State integration of one point with frozen force F.  m' = m + 0*h and
// F' = F + 0*h are kept (they only differ from m, F in the sign of zero).
template <class T>
__device__ __forceinline__ void integrate_point(int integration, T h, V3<T> p, V3<T> v, V3<T> F, T m, V3<T>& np,
                                                V3<T>& nv, V3<T>& nF) {
  if (integration == 0) {  // state.rs:75-83
    const V3<T> z3{T(0), T(0), T(0)};
    const V3<T> a = div_mass(F, m, mass_div(m));
    np = p + v * h;
    nv = v + a * h;
    nF = F + z3 * h;
  } else {
    const Integrated<T> r = integrate_rk4<T>(h, p, v, F, m);
    np = r.p;
    nv = r.v;
    nF = r.F;
  }
}

// x unchanged, opaque to the compiler: an expression of it cannot be moved
// out of the branch it sits in.  The crossing test's divisions by dt depend
// only on the point, so without this the compiler hoists them out of the
// candidate loop and every point pays three IEEE divisions, crossing or not.
__device__ __forceinline__ float opaque(float x) {
  asm volatile("" : "+f"(x));
  return x;
}
__device__ __forceinline__ double opaque(double x) {
  asm volatile("" : "+d"(x));
  return x;
}

// The crossing test of one face (collidable_mesh.rs:107-145): signs of the
// plane distances differ and the projected point lies inside the triangle.
// The triangle's other vertices are only loaded once the plane is crossed.
template <class T>
__device__ __forceinline__ bool face_hit(const ObsFace* __restrict__ Fp, V3<T> op, V3<T> np, T dtd, T& d_old,
                                         T& d_new) {
  const float4 fv0 = Fp->v0, fn = Fp->n;
  const V3<T> v0{T(fv0.x), T(fv0.y), T(fv0.z)};
  const V3<T> n{T(fn.x), T(fn.y), T(fn.z)};
  d_old = dot(op - v0, n);
  d_new = dot(np - v0, n);
  if (signbit(d_old) == signbit(d_new)) return false;
  const V3<T> ovel = (np - op) / opaque(dtd);
  const T fr = d_old / (d_old - d_new);
  const V3<T> cp = op + (dtd * fr) * ovel;
  const float4 fv1 = Fp->v1, fv2 = Fp->v2;
  const V3<T> v1{T(fv1.x), T(fv1.y), T(fv1.z)};
  const V3<T> v2{T(fv2.x), T(fv2.y), T(fv2.z)};
  const int axis = __float_as_int(fv0.w);
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
__device__ __forceinline__ void collision_response(const ObsFace* __restrict__ Fp, T d_old, T d_new, V3<T> op,
                                                   V3<T> ov, V3<T> oF, T om, T dt, T e, T mu, V3<T>& np,
                                                   V3<T>& nv) {
  const float4 fn = Fp->n;
  const V3<T> n{T(fn.x), T(fn.y), T(fn.z)};
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

// Margin of the query box: the computed crossing point can leave the
// segment's box by a few ulps of the step and of the coordinates.  The
// margin 1e-5 |a - b| + 1e-5 max(|a|, |b|) covers that many times over;
// since |a - b| <= 2 max(|a|, |b|), 3.0001e-5 max(|a|, |b|) covers it too,
// in fewer operations (a larger box only adds candidates).
__device__ __forceinline__ float query_slack(float a, float b) {
  return 3.0001e-5f * fmaxf(fabsf(a), fabsf(b)) + 1e-30f;
}

// First hit with the broad phase: obstacles in order; within one, the faces
// of the query's cell merged with the always-tested faces in ascending
// index.  The narrow test is the same face_hit as the full search, so the
// result is identical.  Every candidate -- a linear range of faces (no
// broad phase, or a query box that fits no cell) or the merge of two sorted
// lists -- goes through one face_hit site, and the response is applied once
// after the search: the inlined code stays small.
template <class T>
__device__ __forceinline__ bool collide_point(const ObsFace* __restrict__ faces, int n_faces, V3<T> op, V3<T> ov,
                                              V3<T> oF, T om, V3<T>& np, V3<T>& nv, const StepConsts& c) {
  if (n_faces == 0) return false;
  const ObsAccel& A = c.accel;
  const bool bounded = A.enabled && finite3(op) && finite3(np);
  float lo[3], hi[3];
  {
    const float o3[3] = {float(op.x), float(op.y), float(op.z)};
    const float n3[3] = {float(np.x), float(np.y), float(np.z)};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const float s = query_slack(o3[d], n3[d]);
      lo[d] = fminf(o3[d], n3[d]) - s;
      hi[d] = fmaxf(o3[d], n3[d]) + s;
    }
  }
  const T dtd = T(c.dt_duration);
  const int n_seg = bounded ? A.n_grids : 1;
  int hit = -1;
  T d_old = T(0), d_new = T(0);
  for (int k = 0; k < n_seg && hit < 0; ++k) {
    int lb = 0, le = 0;          // linear range of faces
    int ba = 0, ea = 0, bb = 0, eb = 0;  // cell list [ba, ea) merged with the always list [bb, eb)
    if (!bounded) {
      le = n_faces;
    } else {
      const ObsGrid3& g = A.grids[k];
      bool all = false;
      const bool meets = g.n[0] > 0 && hi[0] >= g.lo[0] && lo[0] <= g.hi[0] && hi[1] >= g.lo[1] &&
                         lo[1] <= g.hi[1] && hi[2] >= g.lo[2] && lo[2] <= g.hi[2];
      if (!meets && g.n_always == 0) continue;  // no face of this obstacle can be hit
      if (meets) {
        int idx[3];
        bool fits = true;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          int i = int(floorf((0.5f * (lo[d] + hi[d]) - g.lo[d]) * g.inv[d]));
          i = min(max(i, 0), g.n[d] - 1);
          const float c0 = g.lo[d] + float(i) * g.cell[d] - g.slack;
          const float c1 = g.lo[d] + float(i + 1) * g.cell[d] + g.slack;
          fits = fits && lo[d] >= c0 && hi[d] <= c1;
          idx[d] = i;
        }
        if (fits) {
          const int cell = g.off_base + (idx[0] * g.n[1] + idx[1]) * g.n[2] + idx[2];
          ba = A.cell_off[cell];
          ea = A.cell_off[cell + 1];
        } else {
          all = true;
        }
      }
      if (all) {  // the box does not fit one cell: every face of this obstacle in order
        lb = g.face_base;
        le = g.face_base + g.n_faces;
      } else {
        bb = g.always_base;
        eb = g.always_base + g.n_always;
      }
    }
    while (true) {
      int f;
      if (lb < le) {
        f = lb++;
      } else if (ba < ea || bb < eb) {  // the union of two ascending lists in ascending order
        const int fa = ba < ea ? A.cell_faces[ba] : 0x7fffffff;
        const int fb = bb < eb ? A.always[bb] : 0x7fffffff;
        if (fa <= fb) { f = fa; ++ba; } else { f = fb; ++bb; }
      } else {
        break;
      }
      if (face_hit(faces + f, op, np, dtd, d_old, d_new)) {
        hit = f;
        break;
      }
    }
  }
  if (hit < 0) return false;
  collision_response(faces + hit, d_old, d_new, op, ov, oF, om, T(c.dt), T(c.restitution), T(c.friction), np, nv);
  return true;
}

}  // namespace fgb
