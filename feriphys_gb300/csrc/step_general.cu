// General-mesh step: a deterministic vertex-centric gather over CSR
// incidence lists (no float atomics).
//
// The reference accumulates forces by scattering over struts in strut order
// (springy_mesh.rs:533-551) and then over faces in face order (629-654).  For
// one vertex, its accumulator therefore receives: gravity, then for each
// incident strut in increasing strut index its spring term and its damper
// term, then for each incident face in increasing face index its corner
// share.  The incidence lists here are sorted exactly that way, so each
// vertex sums the same terms in the same order as the reference and the
// result is bit-identical (with -fmad=false) except in the face weights
// (physics.cuh: face_corner_weight; in f32 their corner angles differ from
// the reference's by rounding).
//
// Layout (one entry per incidence):
//   strut_off[v]..strut_off[v+1]  ->  strut_inc[e] = {other vertex, strut<<1 | role}
//                                     role 0: v is the strut's first vertex a, 1: its second b
//   strut_kcl[s]                  =   {stiffness, damping, rest length, 0}
//   face_off[v]..face_off[v+1]    ->  face_inc[e] = face<<2 | corner
//   face_vtx[f]                   =   {v0, v1, v2, 0}
// State: pos[v] = {x, y, z, mass}, vel[v] = {vx, vy, vz, pinned ? 1 : 0}.
//
// The compact forms (FORM 1 and 2; built by mesh_build.cpp's build_compact)
// carry the same lists in fewer bytes, which is what bounds this kernel's
// DRAM traffic: one word per strut incidence (the other vertex as an offset
// from v, the role, and the strut's rank among its first vertex's struts;
// 32 bits in form 1, 16 in form 2 when every offset and rank is small), the
// strut constants as three float arrays in owner order (struts grouped by
// first vertex, ascending id within a group: v's role-0 incidences take v's
// group in order, a role-1 incidence takes entry `rank` of its other
// vertex's group), and one 16-bit word per face incidence (the corner, and
// where the face's other two vertices sit in v's strut list): 2 or 4 bytes
// plus 12 / 2 per strut incidence and 2 per face incidence, instead of
// 8 + 16 and 4 + 16.  The terms and their order are the same, so are the
// bits.
#include "kernels.h"
#include "physics.cuh"

namespace fgb {

namespace {

// One strut term and one face term, added to F in the reference's order.
template <class T>
__device__ __forceinline__ void add_strut(V3<T>& F, V3<T> P, V3<T> V, V3<T> Po, V3<T> Vo, int role, float k,
                                          float cd, float L) {
  V3<T> sf, df;
  if (role == 0) {
    strut_forces<T>(P, Po, V, Vo, T(k), T(cd), T(L), sf, df);
    F = F + sf;
    F = F + df;
  } else {
    strut_forces<T>(Po, P, Vo, V, T(k), T(cd), T(L), sf, df);
    F = F + (T(-1) * sf);
    F = F + (T(-1) * df);
  }
}
template <class T>
__device__ __forceinline__ void add_face(V3<T>& F, int i0, int i1, int i2, int corner,
                                         const Vec4<T>* __restrict__ pos, const Vec4<T>* __restrict__ vel,
                                         V3<T> wind, const StepConsts& c) {
  const V3<T> x0 = xyz<T>(pos[i0]), x1 = xyz<T>(pos[i1]), x2 = xyz<T>(pos[i2]);
  const V3<T> v0 = xyz<T>(vel[i0]), v1 = xyz<T>(vel[i1]), v2 = xyz<T>(vel[i2]);
  const V3<T> total = face_total_force<T>(x0, x1, x2, v0, v1, v2, wind, T(c.neg_drag), T(c.neg_lift));
  const T w = face_corner_weight<T>(x0, x1, x2, corner);
  F = F + w * total;
}

// A strut word of form 1 (32 bits) or 2 (16 bits; a role-0 word has no rank
// and a 15-bit offset): other-vertex offset, rank, role.
template <int FORM>
__device__ __forceinline__ void strut_word(const GeneralTopo& t, int e, int& off, int& rank, int& role) {
  if (FORM == 2) {
    const uint32_t w = __ldg(t.strut_word16 + e);
    role = int(w & 1u);
    off = int(int16_t(uint16_t(w))) >> (role ? 4 : 1);
    rank = int((w >> 1) & 7u);  // meaningful for role 1 only
  } else {
    const uint32_t w = __ldg(t.strut_word + e);
    off = int(w) >> 6;
    rank = int((w >> 1) & 31u);
    role = int(w & 1u);
  }
}

template <class T, int FORM>
__device__ __forceinline__ V3<T> gather_forces(int v, V3<T> P, V3<T> V, V3<T> F, const Vec4<T>* __restrict__ pos,
                                               const Vec4<T>* __restrict__ vel, const GeneralTopo& t,
                                               const StepConsts& c) {
  const int s_beg = t.strut_off[v], s_end = t.strut_off[v + 1];
  const V3<T> wind{T(c.wind[0]), T(c.wind[1]), T(c.wind[2])};
  if constexpr (FORM != 0) {
    int own = t.own_off[v];  // owner position of v's next role-0 strut
    for (int e = s_beg; e < s_end; ++e) {
      int off, rank, role;
      strut_word<FORM>(t, e, off, rank, role);
      const int o = v + off;
      const int i = role ? __ldg(t.own_off + o) + rank : own++;
      add_strut<T>(F, P, V, xyz<T>(pos[o]), xyz<T>(vel[o]), role, __ldg(t.sk + i), __ldg(t.sc + i),
                   __ldg(t.sl + i));
    }
    const int f_beg = t.face_off[v], f_end = t.face_off[v + 1];
    for (int e = f_beg; e < f_end; ++e) {
      const uint32_t h = __ldg(t.face_word + e);
      const int corner = int(h & 3u);
      int o1, o2, rk, rl;
      strut_word<FORM>(t, s_beg + int((h >> 2) & 127u), o1, rk, rl);
      strut_word<FORM>(t, s_beg + int(h >> 9), o2, rk, rl);
      const int u1 = v + o1, u2 = v + o2;
      const int i0 = corner == 0 ? v : u1, i1 = corner == 0 ? u1 : (corner == 1 ? v : u2),
                i2 = corner == 2 ? v : u2;
      add_face<T>(F, i0, i1, i2, corner, pos, vel, wind, c);
    }
  } else {
    for (int e = s_beg; e < s_end; ++e) {
      const int2 inc = t.strut_inc[e];
      const float4 kcl = t.strut_kcl[inc.y >> 1];
      add_strut<T>(F, P, V, xyz<T>(pos[inc.x]), xyz<T>(vel[inc.x]), inc.y & 1, kcl.x, kcl.y, kcl.z);
    }
    const int f_beg = t.face_off[v], f_end = t.face_off[v + 1];
    for (int e = f_beg; e < f_end; ++e) {
      const int fc = t.face_inc[e];
      const int4 fv = t.face_vtx[fc >> 2];
      add_face<T>(F, fv.x, fv.y, fv.z, fc & 3, pos, vel, wind, c);
    }
  }
  return F;
}

__device__ __forceinline__ void flag_nonfinite(bool bad, unsigned* flags) {
  if (__any_sync(__activemask(), bad) && bad && flags) atomicOr(flags, 1u);
}

// Fused Simulation::step for one mesh (accumulate -> integrate -> collide ->
// pin restore -> clear), one thread per vertex.  The f32 form asks for 4
// blocks of 256 per SM (at most 64 registers: the gather is latency-bound, so
// resident warps count); the FP64 rerun keeps the registers it needs.
template <class T, int FORM>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 1) k_step_general(int n, const Vec4<T>* __restrict__ pos,
                                                      const Vec4<T>* __restrict__ vel,
                                                      const Vec4<T>* __restrict__ force_in,
                                                      Vec4<T>* __restrict__ pos_out, Vec4<T>* __restrict__ vel_out,
                                                      GeneralTopo t, StepConsts c) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  const Vec4<T> P4 = pos[v];
  const Vec4<T> V4 = vel[v];
  if (V4.w != T(0)) {  // pinned: update_points restores the old point (springy_mesh.rs:492-496)
    pos_out[v] = P4;
    vel_out[v] = V4;
    return;
  }
  const V3<T> P = xyz<T>(P4), V = xyz<T>(V4);
  const T m = P4.w;
  V3<T> F;
  if (force_in) {
    const V3<T> g{T(c.force0[0]), T(c.force0[1]), T(c.force0[2])};
    F = xyz<T>(force_in[v]) + g;
  } else {
    F = V3<T>{T(c.force0[0]), T(c.force0[1]), T(c.force0[2])};
  }
  F = gather_forces<T, FORM>(v, P, V, F, pos, vel, t, c);
  V3<T> np, nv, nF;
  integrate_point<T>(c.integration, T(c.dt), P, V, F, m, np, nv, nF);
  collide_point<T>(static_cast<const ObsFace*>(c.obstacle_faces), c.n_obstacle_faces, P, V, F, m, np, nv, c);
  pos_out[v] = make4<T>(np, m);
  vel_out[v] = make4<T>(nv, V4.w);
  flag_nonfinite(!(finite3(np) && finite3(nv)), c.flags);
}

// accumulate_forces: force[v] = force[v] + gravity + struts + faces; pins -> 0.
template <class T, int FORM>
__global__ void __launch_bounds__(256) k_accumulate(int n, const Vec4<T>* __restrict__ pos,
                                                    const Vec4<T>* __restrict__ vel, Vec4<T>* __restrict__ force,
                                                    GeneralTopo t, StepConsts c) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  const Vec4<T> V4 = vel[v];
  const V3<T> g{T(c.force0[0]), T(c.force0[1]), T(c.force0[2])};
  V3<T> F = xyz<T>(force[v]) + g;
  F = gather_forces<T, FORM>(v, xyz<T>(pos[v]), xyz<T>(V4), F, pos, vel, t, c);
  if (V4.w != T(0)) F = V3<T>{T(0), T(0), T(0)};
  force[v] = make4<T>(F, T(0));
}

// State::euler_step / rk4_step into the staging points.
template <class T>
__global__ void __launch_bounds__(256) k_integrate(int n, int integration, T h, const Vec4<T>* __restrict__ pos,
                                                   const Vec4<T>* __restrict__ vel,
                                                   const Vec4<T>* __restrict__ force, Vec4<T>* __restrict__ spos,
                                                   Vec4<T>* __restrict__ svel, Vec4<T>* __restrict__ sforce) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  const Vec4<T> P4 = pos[v], V4 = vel[v];
  V3<T> np, nv, nF;
  const T m = P4.w;
  integrate_point<T>(integration, h, xyz<T>(P4), xyz<T>(V4), xyz<T>(force[v]), m, np, nv, nF);
  spos[v] = make4<T>(np, m + T(0) * h);
  svel[v] = make4<T>(nv, V4.w);
  sforce[v] = make4<T>(nF, T(0));
}

// update_points with the staged points: collide, then restore pins.
template <class T>
__global__ void __launch_bounds__(256) k_update(int n, Vec4<T>* __restrict__ pos, Vec4<T>* __restrict__ vel,
                                                Vec4<T>* __restrict__ force, const Vec4<T>* __restrict__ spos,
                                                const Vec4<T>* __restrict__ svel,
                                                const Vec4<T>* __restrict__ sforce, StepConsts c) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  const Vec4<T> P4 = pos[v], V4 = vel[v];
  if (V4.w != T(0)) return;  // pinned: keep the old point
  const Vec4<T> nP4 = spos[v], nV4 = svel[v];
  V3<T> np = xyz<T>(nP4), nv = xyz<T>(nV4);
  collide_point<T>(static_cast<const ObsFace*>(c.obstacle_faces), c.n_obstacle_faces, xyz<T>(P4), xyz<T>(V4),
                   xyz<T>(force[v]), P4.w, np, nv, c);
  pos[v] = make4<T>(np, nP4.w);
  vel[v] = make4<T>(nv, V4.w);
  force[v] = sforce[v];
}

template <class T>
__global__ void k_zero4(int n, Vec4<T>* __restrict__ a) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < n) a[v] = make4<T>(V3<T>{T(0), T(0), T(0)}, T(0));
}

inline int blocks_for(int n, int bs) { return (n + bs - 1) / bs; }

}  // namespace

template <class T>
cudaError_t launch_step_general(int n, const void* pos, const void* vel, const void* force_in, void* pos_out,
                                void* vel_out, const GeneralTopo& t, const StepConsts& c, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  auto k = t.form == 2 ? k_step_general<T, 2> : (t.form == 1 ? k_step_general<T, 1> : k_step_general<T, 0>);
  k<<<blocks_for(n, 256), 256, 0, s>>>(n, static_cast<const Vec4<T>*>(pos), static_cast<const Vec4<T>*>(vel),
                                       static_cast<const Vec4<T>*>(force_in), static_cast<Vec4<T>*>(pos_out),
                                       static_cast<Vec4<T>*>(vel_out), t, c);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_accumulate(int n, const void* pos, const void* vel, void* force, const GeneralTopo& t,
                              const StepConsts& c, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  auto k = t.form == 2 ? k_accumulate<T, 2> : (t.form == 1 ? k_accumulate<T, 1> : k_accumulate<T, 0>);
  k<<<blocks_for(n, 256), 256, 0, s>>>(n, static_cast<const Vec4<T>*>(pos), static_cast<const Vec4<T>*>(vel),
                                       static_cast<Vec4<T>*>(force), t, c);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_integrate(int n, int integration, float h, const void* pos, const void* vel, const void* force,
                             void* spos, void* svel, void* sforce, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_integrate<T><<<blocks_for(n, 256), 256, 0, s>>>(
      n, integration, T(h), static_cast<const Vec4<T>*>(pos), static_cast<const Vec4<T>*>(vel),
      static_cast<const Vec4<T>*>(force), static_cast<Vec4<T>*>(spos), static_cast<Vec4<T>*>(svel),
      static_cast<Vec4<T>*>(sforce));
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_update(int n, void* pos, void* vel, void* force, const void* spos, const void* svel,
                          const void* sforce, const StepConsts& c, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_update<T><<<blocks_for(n, 256), 256, 0, s>>>(n, static_cast<Vec4<T>*>(pos), static_cast<Vec4<T>*>(vel),
                                                 static_cast<Vec4<T>*>(force), static_cast<const Vec4<T>*>(spos),
                                                 static_cast<const Vec4<T>*>(svel),
                                                 static_cast<const Vec4<T>*>(sforce), c);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_zero4(int n, void* a, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_zero4<T><<<blocks_for(n, 256), 256, 0, s>>>(n, static_cast<Vec4<T>*>(a));
  return cudaGetLastError();
}

#define FGB_INSTANTIATE(T)                                                                                        \
  template cudaError_t launch_step_general<T>(int, const void*, const void*, const void*, void*, void*,          \
                                              const GeneralTopo&, const StepConsts&, cudaStream_t);               \
  template cudaError_t launch_accumulate<T>(int, const void*, const void*, void*, const GeneralTopo&,            \
                                            const StepConsts&, cudaStream_t);                                     \
  template cudaError_t launch_integrate<T>(int, int, float, const void*, const void*, const void*, void*, void*, \
                                           void*, cudaStream_t);                                                  \
  template cudaError_t launch_update<T>(int, void*, void*, void*, const void*, const void*, const void*,         \
                                        const StepConsts&, cudaStream_t);                                         \
  template cudaError_t launch_zero4<T>(int, void*, cudaStream_t);
FGB_INSTANTIATE(float)
FGB_INSTANTIATE(double)

}  // namespace fgb
