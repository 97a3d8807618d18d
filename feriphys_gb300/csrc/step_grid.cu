// Grid-stencil step for meshes with Cloth::new's topology (cloth.rs:20-113).
//
// The neighbourhood of every vertex is implicit in (row, col): no index
// lists are read.  Strut constants live in 4 float4 planes indexed by the
// owning vertex (grid_order.h).  The force terms are summed in the exact
// order of the reference's scatter loops (strut ids ascending, then face ids
// ascending -- checked on the host against the real ids before this kernel is
// chosen), so the result is bit-identical to the general gather.
#include <cuda.h>

#include <cstring>
#include <mutex>

#include "fastdiv.cuh"
#include "face_pair.cuh"
#include "grid_order.h"
#include "kernels.h"
#include "per_device.h"
#include "physics.cuh"
#include "tc05.cuh"

namespace fgb {

namespace {

using namespace grid;

__device__ __forceinline__ float param(const float4* __restrict__ planes, int n, int owner, int kind, int field) {
  const int idx = param_index(kind, field);
  const float* plane = reinterpret_cast<const float*>(planes + size_t(idx >> 2) * n);
  return plane[4 * size_t(owner) + (idx & 3)];
}

__device__ __forceinline__ void strut_ends(int kind, int owner, int C, int& a, int& b) {
  switch (kind) {
    case KH: a = owner; b = owner + 1; break;
    case KV: a = owner; b = owner + C; break;
    case KS: a = owner + 1; b = owner + C; break;
    case KBH: a = owner; b = owner + 2; break;
    default: a = owner; b = owner + 2 * C; break;
  }
}

__global__ void __launch_bounds__(256) k_step_grid_v1(int R, int C, const float4* __restrict__ planes,
                                                      const float4* __restrict__ pos,
                                                      const float4* __restrict__ vel,
                                                      const float4* __restrict__ force_in,
                                                      float4* __restrict__ pos_out, float4* __restrict__ vel_out,
                                                      StepConsts c) {
  const int n = R * C;
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  const float4 P4 = pos[v], V4 = vel[v];
  if (V4.w != 0.0f) {
    pos_out[v] = P4;
    vel_out[v] = V4;
    return;
  }
  const int r = v / C, cc = v - r * C;
  const V3<float> P = xyz<float>(P4), V = xyz<float>(V4);
  V3<float> F{c.force0[0], c.force0[1], c.force0[2]};
  if (force_in) F = xyz<float>(force_in[v]) + F;
  for (int j = 0; j < N_SLOTS; ++j) {
    const SlotDesc d = slot_desc(slot_at(j, r, cc, R, C));
    const int ro = r + d.dr, co = cc + d.dc;
    if (!owned_exists(d.kind, ro, co, R, C)) continue;
    const int owner = ro * C + co;
    int a, b;
    strut_ends(d.kind, owner, C, a, b);
    const float k = param(planes, n, owner, d.kind, 0);
    const float cdmp = param(planes, n, owner, d.kind, 1);
    const float L = param(planes, n, owner, d.kind, 2);
    V3<float> sf, df;
    if (d.role == 0) {
      strut_forces<float>(P, xyz<float>(pos[b]), V, xyz<float>(vel[b]), k, cdmp, L, sf, df);
      F = F + sf;
      F = F + df;
    } else {
      strut_forces<float>(xyz<float>(pos[a]), P, xyz<float>(vel[a]), V, k, cdmp, L, sf, df);
      F = F + (-1.0f * sf);
      F = F + (-1.0f * df);
    }
  }
  const V3<float> wind{c.wind[0], c.wind[1], c.wind[2]};
  for (int s = 0; s < N_FACE_SLOTS; ++s) {
    const FaceDesc fd = face_desc(s);
    const int qr = r + fd.dr, qc = cc + fd.dc;
    if (!quad_exists(qr, qc, R, C)) continue;
    const int q = qr * C + qc;
    int i0, i1, i2;
    if (fd.is_b) { i0 = q + 1; i1 = q + C + 1; i2 = q + C; }
    else { i0 = q + 1; i1 = q + C; i2 = q; }
    const V3<float> x0 = xyz<float>(pos[i0]), x1 = xyz<float>(pos[i1]), x2 = xyz<float>(pos[i2]);
    const V3<float> v0 = xyz<float>(vel[i0]), v1 = xyz<float>(vel[i1]), v2 = xyz<float>(vel[i2]);
    const V3<float> total = face_total_force<float>(x0, x1, x2, v0, v1, v2, wind, c.neg_drag, c.neg_lift);
    F = F + face_corner_weight<float>(x0, x1, x2, fd.corner) * total;
  }
  V3<float> np, nv, nF;
  const float m = P4.w;
  integrate_point<float>(c.integration, c.dt, P, V, F, m, np, nv, nF);
  collide_point<float>(static_cast<const ObsFace*>(c.obstacle_faces), c.n_obstacle_faces, P, V, F, m, np, nv, c);
  pos_out[v] = make4<float>(np, m);
  vel_out[v] = make4<float>(nv, V4.w);
  const bool bad = !(finite3(np) && finite3(nv));
  if (__any_sync(__activemask(), bad) && bad && c.flags) atomicOr(c.flags, 1u);
}


// ---------------------------------------------------------------------------
// Tiled kernel.  A CTA owns a TW x TH tile of vertices.  It stages the tile
// plus a 2-vertex halo (binding struts reach 2 vertices) in shared memory,
// computes every strut and face touching the tile once, and each thread then
// gathers its vertex's terms from shared memory in the reference's order.
// Binding struts come after all triangle struts in strut order, so they are
// computed and summed in a second phase that reuses the same buffer; faces
// come after all struts and use it a third time.

template <int TW, int TH>
struct TileGeom {
  static constexpr int EW = TW + 4, EH = TH + 4;  // staged region, origin (r0-2, c0-2)
  // resident CTAs per SM the launch bounds ask for: 64 registers per thread
  // at TW * TH + 64 threads (32x4: 5, 32x8: 3, 32x12: 2 with 72 registers)
  static constexpr int MIN_CTAS = TH <= 4 ? 5 : (TH <= 8 ? 3 : 2);
};

template <int TW, int TH>
struct Interior {
  static constexpr int OW = TW + 2, OH = TH + 2;  // owner grid: rows r0-2.., cols c0-2..
  static constexpr int NO = OW * OH;
  static constexpr int QW = TW + 1, QH = TH + 1;  // quads: rows r0-1.., cols c0-1..
  static constexpr int NQ = QW * QH;
  // bytes after the staged pos/vel: 5 strut kinds x (float4 (u, s1) + float s2), 3 float4 per quad
  static constexpr int BYTES = 5 * NO * 20 + NQ * 48;
  static_assert((5 * NO * 20) % 16 == 0, "the quad results must start 16-byte aligned");
};

// Strut of the compact form: unit vector u and the spring/damper scalars
// s1 = k(|d| - L), s2 = c (dv . u); the forces are s1*u and s2*u, which a
// gathering thread forms itself (the same products, so the same bits).
__device__ __forceinline__ void strut_terms(float4 pa, float4 pb, float4 va, float4 vb, float k, float cd, float L,
                                            float4& su, float& s2) {
  const V3<float> d = xyz<float>(pb) - xyz<float>(pa);
  const float mag = magnitude(d);
  const V3<float> u = d * rcp_of_root(mag);  // 1 / mag, the IEEE bits
  const float s1 = k * (mag - L);
  s2 = cd * dot(xyz<float>(vb) - xyz<float>(va), u);
  su = make_float4(u.x, u.y, u.z, s1);
}
__device__ __forceinline__ void strut_compact(const float4* __restrict__ s_pos, const float4* __restrict__ s_vel,
                                              int ia, int ib, float k, float cd, float L, float4* __restrict__ su,
                                              float* __restrict__ s2) {
  float4 u;
  float d;
  strut_terms(s_pos[ia], s_pos[ib], s_vel[ia], s_vel[ib], k, cd, L, u, d);
  *su = u;
  *s2 = d;
}

__device__ __forceinline__ void add_compact(V3<float>& F, float4 su, float s2, int role) {
  const V3<float> u{su.x, su.y, su.z};
  if (role == 0) {
    F = F + su.w * u;
    F = F + s2 * u;
  } else {  // -1.0 * (s*u) == (-s)*u exactly
    F = F + (-su.w) * u;
    F = F + (-s2) * u;
  }
}

__device__ __forceinline__ void quad_to(const float4* __restrict__ s_pos, const float4* __restrict__ s_vel, int e00,
                                        int e01, int e10, int e11, V3<float> wind, float neg_cd, float neg_lift,
                                        float one,
                                        float4* __restrict__ qa, float4* __restrict__ qb, float4* __restrict__ qw) {
  float4 a, b;
  float2 wa, wb;
  // A = (i+1, i+C, i), B = (i+1, i+C+1, i+C) for quad origin i: lane 0 face A, lane 1 face B
  const V3<float> p00 = xyz<float>(s_pos[e00]), p01 = xyz<float>(s_pos[e01]), p10 = xyz<float>(s_pos[e10]),
                  p11 = xyz<float>(s_pos[e11]);
  const V3<float> u00 = xyz<float>(s_vel[e00]), u01 = xyz<float>(s_vel[e01]), u10 = xyz<float>(s_vel[e10]),
                  u11 = xyz<float>(s_vel[e11]);
  face_terms2(pk3(p01, p01), pk3(p10, p11), pk3(p00, p10), pk3(u01, u01), pk3(u10, u11), pk3(u00, u10),
              pk3(wind, wind), neg_cd, neg_lift, one, a, wa, b, wb);
  *qa = a;
  *qb = b;
  *qw = make_float4(wa.x, wa.y, wb.x, wb.y);
}

// One CTA = a TW x TH tile: TW*TH "main" threads (one per vertex) plus
// HALO helper threads that compute the tile's halo struts and faces while
// the main threads compute their own, so no thread does double work.
// Tiles split into an interior rectangle [bx0, bx1] x [by0, by1] (every
// neighbour of every tile vertex exists: fixed offsets, no checks) and the
// ring of boundary tiles around it, launched as two kernels.
struct TileSplit {
  int tx, ty;          // tiles per row / column
  int bx0, bx1, by0, by1;  // interior rectangle (empty when bx1 < bx0 or by1 < by0)
};

__host__ __device__ __forceinline__ void ring_tile(const TileSplit& t, int k, int& bx, int& by) {
  const bool has_interior = t.bx1 >= t.bx0 && t.by1 >= t.by0;
  if (!has_interior) {
    bx = k % t.tx;
    by = k / t.tx;
    return;
  }
  const int top = t.by0 * t.tx;
  if (k < top) {
    bx = k % t.tx;
    by = k / t.tx;
    return;
  }
  k -= top;
  const int bottom = (t.ty - 1 - t.by1) * t.tx;
  if (k < bottom) {
    bx = k % t.tx;
    by = t.by1 + 1 + k / t.tx;
    return;
  }
  k -= bottom;
  const int per_row = t.bx0 + (t.tx - 1 - t.bx1);
  by = t.by0 + k / per_row;
  const int j = k % per_row;
  bx = j < t.bx0 ? j : t.bx1 + 1 + (j - t.bx0);
}

// Tile of CTA b of the single-cloth kernel: the first n_ring CTAs take the
// ring tiles in ring_tile's order, the rest the interior rectangle row by
// row.  Returns whether the tile is an interior one.
__host__ __device__ __forceinline__ bool grid_tile(const TileSplit& t, int n_ring, int b, int& bx, int& by) {
  if (b < n_ring) {
    ring_tile(t, b, bx, by);
    return false;
  }
  const int k = b - n_ring, nbx = t.bx1 - t.bx0 + 1;
  bx = t.bx0 + k % nbx;
  by = t.by0 + k / nbx;
  return true;
}

// One tile of one cloth.  No early return: the batched kernel runs it in a
// loop, so every thread reaches the end of every tile.
template <int TW, int TH, int HALO, bool INTERIOR, bool TMA = false>
__device__ __forceinline__ void tile_step(int bx, int by, int R, int C, const float4* __restrict__ planes,
                                          const float4* __restrict__ pos, const float4* __restrict__ vel,
                                          const float4* __restrict__ force_in, float4* __restrict__ pos_out,
                                          float4* __restrict__ vel_out, const StepConsts& c, V3<float> wind,
                                          unsigned* flags, const CUtensorMap* map_pos = nullptr,
                                          const CUtensorMap* map_vel = nullptr, uint64_t* tma_bar = nullptr,
                                          uint32_t tma_phase = 0) {
  using G = TileGeom<TW, TH>;
  using I = Interior<TW, TH>;
  constexpr int NMAIN = TW * TH, NT = TW * TH + HALO;
  static_assert(HALO == 2 * TW && TW + 2 * TH + 1 <= 2 * TW && TW >= 32, "helper layout assumes 64 helpers");
  constexpr int EW = G::EW, OW = I::OW, NO = I::NO, QW = I::QW, NQ = I::NQ;
  extern __shared__ __align__(128) float4 s_dyn[];
  float4* s_pos = s_dyn;
  float4* s_vel = s_dyn + G::EH * G::EW;
  float4* s_su = s_dyn + 2 * G::EH * G::EW;                  // [5][NO] unit vector, s1
  float* s_s2 = reinterpret_cast<float*>(s_su + 5 * NO);     // [5][NO] s2
  float4* s_qa = reinterpret_cast<float4*>(s_s2 + 5 * NO);   // [NQ] face A: D, w0
  float4* s_qb = s_qa + NQ;                                  // [NQ] face B: D, w0
  float4* s_qw = s_qb + NQ;                                  // [NQ] A w1, A w2, B w1, B w2
  const int n = R * C;
  const int c0 = bx * TW, r0 = by * TH;
  const int tid = threadIdx.x;
  const float4* __restrict__ plane0 = planes;
  const float4* __restrict__ plane1 = planes + n;
  const float4* __restrict__ plane2 = planes + 2 * size_t(n);
  const float4* __restrict__ plane3 = planes + 3 * size_t(n);
  auto e = [](int rr, int ccl) { return (rr + 2) * EW + (ccl + 2); };  // tile-relative staged index
  auto o = [](int rr, int ccl) { return (rr + 2) * OW + (ccl + 2); };  // tile-relative owner index
  auto qi = [](int rr, int ccl) { return (rr + 1) * QW + (ccl + 1); };
  // does the strut of `kind` owned by tile-relative (rr, ccl) exist?
  auto has = [&](int kind, int rr, int ccl) { return INTERIOR || owned_exists(kind, r0 + rr, c0 + ccl, R, C); };

  const int lr = tid / TW, lc = tid % TW;
  const int r = r0 + lr, cc = c0 + lc;
  const bool vertex = tid < NMAIN && (INTERIOR || (r < R && cc < C));
  V3<float> F{c.force0[0], c.force0[1], c.force0[2]};

  // ---- stage positions/velocities; prefetch the strut constants this thread needs.
  // With tensor maps, one thread asks the TMA engine for the two (TH+4) x (TW+4)
  // boxes (rows r0-2.., columns c0-2..; outside the cloth they read zeros, which
  // no thread uses) while every thread loads its strut constants.
  // (tma_bar: an mbarrier the kernel initialised once; tma_phase: the parity
  // of its phase this tile completes)
  const bool tma = TMA && (tc::smem_u32(s_pos) & 127u) == 0;
  if (tma) {
    if (tid == 0) {
      tc::mbar_arrive_expect_tx(tma_bar, 2u * G::EH * G::EW * 16u);
      tc::tma_load_2d(s_pos, map_pos, 4 * (c0 - 2), r0 - 2, tma_bar);
      tc::tma_load_2d(s_vel, map_vel, 4 * (c0 - 2), r0 - 2, tma_bar);
    }
  } else {
    for (int i = tid; i < G::EH * G::EW; i += NT) {
      const int gr = r0 - 2 + i / G::EW, gc = c0 - 2 + i % G::EW;
      if (INTERIOR || (gr >= 0 && gr < R && gc >= 0 && gc < C)) {
        s_pos[i] = pos[gr * C + gc];
        s_vel[i] = vel[gr * C + gc];
      }
    }
  }
  const int h = tid - NMAIN;
  // Main threads: the five struts owned by their vertex and its quad.
  // Helper lanes: up to three strut jobs (kind, owner) and at most one quad,
  // laid out so a warp never runs two expensive branches one after another:
  //   h in [0, 32):  owner (-1, h): vertical, shear, vertical binding; quad (-1, h)
  //   h in [32, 64): vertical binding owned by (-2, h-32), plus
  //     h in [32, 40): horizontal and shear owned by (h-32, -1); quad (h-32, -1)
  //     h in [40, 48): horizontal bindings owned by (h-40, -2) and (h-40, -1)
  //     h == 48:       shear owned by (-1, -1); quad (-1, -1)
  float4 q0 = make_float4(0, 0, 0, 0), q1 = q0, q2 = q0, q3 = q0;
  int job_kind[3] = {-1, -1, -1}, job_r[3] = {0, 0, 0}, job_c[3] = {0, 0, 0};
  float job_k[3] = {0, 0, 0}, job_cd[3] = {0, 0, 0}, job_L[3] = {0, 0, 0};
  int quad_r = -3, quad_c = 0;
  if (tid < NMAIN) {
    if (vertex) {
      const int v = r * C + cc;
      q0 = __ldg(plane0 + v);
      q1 = __ldg(plane1 + v);
      q2 = __ldg(plane2 + v);
      q3 = __ldg(plane3 + v);
      if (force_in) F = xyz<float>(force_in[v]) + F;
    }
    quad_r = lr;
    quad_c = lc;
  } else {
    if (h < TW) {
      job_kind[0] = KV; job_r[0] = -1; job_c[0] = h;
      job_kind[1] = KS; job_r[1] = -1; job_c[1] = h;
      job_kind[2] = KBV; job_r[2] = -1; job_c[2] = h;
      quad_r = -1; quad_c = h;
    } else {
      job_kind[0] = KBV; job_r[0] = -2; job_c[0] = h - TW;
      if (h < TW + TH) {
        job_kind[1] = KH; job_r[1] = h - TW; job_c[1] = -1;
        job_kind[2] = KS; job_r[2] = h - TW; job_c[2] = -1;
        quad_r = h - TW; quad_c = -1;
      } else if (h < TW + 2 * TH) {
        job_kind[1] = KBH; job_r[1] = h - TW - TH; job_c[1] = -2;
        job_kind[2] = KBH; job_r[2] = h - TW - TH; job_c[2] = -1;
      } else if (h == TW + 2 * TH) {
        job_kind[1] = KS; job_r[1] = -1; job_c[1] = -1;
        quad_r = -1; quad_c = -1;
      }
    }
    const float* pl = reinterpret_cast<const float*>(planes);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      if (job_kind[j] < 0 || !has(job_kind[j], job_r[j], job_c[j])) {
        job_kind[j] = -1;
        continue;
      }
      const size_t v = size_t((r0 + job_r[j]) * C + c0 + job_c[j]);
      const int ik = param_index(job_kind[j], 0);
      job_k[j] = __ldg(pl + size_t(ik >> 2) * 4 * n + 4 * v + (ik & 3));
      job_cd[j] = __ldg(pl + size_t((ik + 1) >> 2) * 4 * n + 4 * v + ((ik + 1) & 3));
      job_L[j] = __ldg(pl + size_t((ik + 2) >> 2) * 4 * n + 4 * v + ((ik + 2) & 3));
    }
  }
  if (!INTERIOR && quad_r > -3 && !quad_exists(r0 + quad_r, c0 + quad_c, R, C)) quad_r = -3;
  __syncthreads();
  if (tma && !tc::mbar_wait(tma_bar, tma_phase) && flags) atomicOr(flags, 2u);  // bounded: a stuck copy is reported

  // ---- compute every strut and face of the tile once
  auto put = [&](int kind, int rr, int ccl, float k, float cd, float L) {
    int ia = e(rr, ccl), ib;
    switch (kind) {
      case KH: ib = ia + 1; break;
      case KV: ib = ia + EW; break;
      case KS: ib = ia + EW; ia += 1; break;
      case KBH: ib = ia + 2; break;
      default: ib = ia + 2 * EW; break;
    }
    strut_compact(s_pos, s_vel, ia, ib, k, cd, L, s_su + kind * NO + o(rr, ccl), s_s2 + kind * NO + o(rr, ccl));
  };
  if (tid < NMAIN) {
    // the five struts owned by this vertex: first the five strut vectors and
    // their lengths (independent chains the compiler can interleave), then
    // each strut's unit vector and scalars, stored where the strut exists
    // (every slot read lies inside the staged tile; a slot outside the cloth
    // is never stored)
    const int i = e(lr, lc);
    const int ia[5] = {i, i, i + 1, i, i}, ib[5] = {i + 1, i + EW, i + EW, i + 2, i + 2 * EW};
    const float kk[5] = {q0.x, q0.w, q1.z, q2.y, q3.x}, cc5[5] = {q0.y, q1.x, q1.w, q2.z, q3.y},
                LL[5] = {q0.z, q1.y, q2.x, q2.w, q3.z};
    V3<float> d[5];
    float mag[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) d[j] = xyz<float>(s_pos[ib[j]]) - xyz<float>(s_pos[ia[j]]);
#pragma unroll
    for (int j = 0; j < 5; ++j) mag[j] = magnitude(d[j]);
    const int oi = o(lr, lc);
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      const V3<float> u = d[j] * rcp_of_root(mag[j]);
      const float s1 = kk[j] * (mag[j] - LL[j]);
      const float s2 = cc5[j] * dot(xyz<float>(s_vel[ib[j]]) - xyz<float>(s_vel[ia[j]]), u);
      if (has(j, lr, lc)) {  // kinds KH, KV, KS, KBH, KBV = 0..4
        s_su[j * NO + oi] = make_float4(u.x, u.y, u.z, s1);
        s_s2[j * NO + oi] = s2;
      }
    }
  } else {
#pragma unroll
    for (int j = 0; j < 3; ++j)
      if (job_kind[j] >= 0) put(job_kind[j], job_r[j], job_c[j], job_k[j], job_cd[j], job_L[j]);
  }
  if (quad_r > -3)
    quad_to(s_pos, s_vel, e(quad_r, quad_c), e(quad_r, quad_c + 1), e(quad_r + 1, quad_c), e(quad_r + 1, quad_c + 1),
            wind, c.neg_drag, c.neg_lift, c.one, s_qa + qi(quad_r, quad_c), s_qb + qi(quad_r, quad_c),
            s_qw + qi(quad_r, quad_c));
  __syncthreads();
  if (vertex) {
    // ---- gather in the reference's summation order (grid_order.h)
    auto take = [&](int kind, int rr, int ccl, int role) {
      const int i = kind * NO + o(rr, ccl);
      add_compact(F, s_su[i], s_s2[i], role);
    };
    if (INTERIOR) {
      take(KS, lr - 1, lc, 1);   // SH_UP
      take(KV, lr - 1, lc, 1);   // VT_UP
      take(KS, lr, lc - 1, 0);   // SH_LEFT
      take(KH, lr, lc - 1, 1);   // HZ_LEFT
      take(KV, lr, lc, 0);       // VT_DOWN
      take(KH, lr, lc, 0);       // HZ_RIGHT
      take(KBV, lr - 2, lc, 1);  // BV_UP
      take(KBH, lr, lc - 2, 1);  // BH_LEFT
      take(KBH, lr, lc, 0);      // BH_RIGHT
      take(KBV, lr, lc, 0);      // BV_DOWN
    } else {
#pragma unroll  // every slot but the last column's permuted three folds to constants
      for (int j = 0; j < N_SLOTS; ++j) {
        const SlotDesc d = slot_desc(slot_at(j, r, cc, R, C));
        if (owned_exists(d.kind, r + d.dr, cc + d.dc, R, C)) take(d.kind, lr + d.dr, lc + d.dc, d.role);
      }
    }
#pragma unroll
    for (int sl = 0; sl < N_FACE_SLOTS; ++sl) {
      const FaceDesc fd = face_desc(sl);
      if (!INTERIOR && !quad_exists(r + fd.dr, cc + fd.dc, R, C)) continue;
      const int q = qi(lr + fd.dr, lc + fd.dc);
      const float4 D = fd.is_b ? s_qb[q] : s_qa[q];
      float w;
      if (fd.corner == 0) w = D.w;
      else if (fd.corner == 1) w = fd.is_b ? s_qw[q].z : s_qw[q].x;
      else w = fd.is_b ? s_qw[q].w : s_qw[q].y;
      F = F + w * V3<float>{D.x, D.y, D.z};
    }

    // ---- integrate, collide, write
    const int v = r * C + cc;
    const float4 P4 = s_pos[e(lr, lc)];
    const float4 V4 = s_vel[e(lr, lc)];
    if (V4.w != 0.0f) {  // pinned: update_points restores the old point
      pos_out[v] = P4;
      vel_out[v] = V4;
    } else {
      const V3<float> P = xyz<float>(P4), V = xyz<float>(V4);
      const float m = P4.w;
      V3<float> np, nv, nF;
      integrate_point<float>(c.integration, c.dt, P, V, F, m, np, nv, nF);
      collide_point<float>(static_cast<const ObsFace*>(c.obstacle_faces), c.n_obstacle_faces, P, V, F, m, np, nv, c);
      pos_out[v] = make4<float>(np, m);
      vel_out[v] = make4<float>(nv, V4.w);
      const bool bad = !(finite3(np) && finite3(nv));
      if (__any_sync(__activemask(), bad) && bad && flags) atomicOr(flags, 1u);
    }
  }
}

// One launch for all tiles: the boundary ring first (its tiles are slower
// and then overlap the interior ones instead of running as a lone wave).
template <int TW, int TH, int HALO, bool TMA>
__global__ void __launch_bounds__(TW * TH + HALO, TileGeom<TW, TH>::MIN_CTAS) k_step_grid_tiled(int R, int C, TileSplit split, int n_ring,
                                                                      const float4* __restrict__ planes,
                                                                      const float4* __restrict__ pos,
                                                                      const float4* __restrict__ vel,
                                                                      const float4* __restrict__ force_in,
                                                                      float4* __restrict__ pos_out,
                                                                      float4* __restrict__ vel_out, StepConsts c,
                                                                      const __grid_constant__ CUtensorMap map_pos,
                                                                      const __grid_constant__ CUtensorMap map_vel) {
  __shared__ uint64_t bar;
  const int b = blockIdx.x;
  const CUtensorMap* mp = &map_pos;
  const CUtensorMap* mv = &map_vel;
  if (TMA && threadIdx.x == 0) {  // the same thread issues the copies after this
    tc::mbar_init(&bar, 1);
    tc::mbar_fence_init();
  }
  int bx, by;
  if (!grid_tile(split, n_ring, b, bx, by))
    tile_step<TW, TH, HALO, false, TMA>(bx, by, R, C, planes, pos, vel, force_in, pos_out, vel_out, c,
                                        V3<float>{c.wind[0], c.wind[1], c.wind[2]}, c.flags, mp, mv, &bar, 0);
  else
    tile_step<TW, TH, HALO, true, TMA>(bx, by, R, C, planes, pos, vel, force_in, pos_out, vel_out, c,
                                       V3<float>{c.wind[0], c.wind[1], c.wind[2]}, c.flags, mp, mv, &bar, 0);
}

// Many cloths in one launch.  Work items {cloth, tile x, tile y, interior}
// come from a list packed on the host (largest cloths first, each cloth's
// boundary tiles before its interior ones); in persistent mode every CTA
// pulls items from a global counter until the list is exhausted.
template <int TW, int TH, int HALO, bool TMA>
__global__ void __launch_bounds__(TW * TH + HALO, TileGeom<TW, TH>::MIN_CTAS) k_step_batched(const ClothDesc* __restrict__ cloths,
                                                                   const int4* __restrict__ work, int n_work,
                                                                   int* __restrict__ counter, int parity,
                                                                   int persistent, StepConsts c,
                                                                   const CUtensorMap* __restrict__ maps,
                                                                   const int* __restrict__ n_work_dev) {
  __shared__ int s_item;
  // the current item's cloth descriptor, staged once per item: read from
  // shared memory where the tile uses it, instead of held in registers
  // (pointers and wind) across the whole tile
  __shared__ ClothDesc s_d;
  __shared__ int4 s_w;
  if (n_work_dev) n_work = *n_work_dev;  // a count made on the device (persistent mode)
  __shared__ uint64_t bar;
  uint32_t phase = 0;
  if (TMA && threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    tc::mbar_fence_init();
  }
  int item = blockIdx.x;
  // persistent mode: thread 0 claims the item after the current one while the
  // current tile runs (the claims of one CTA only grow, so when the current
  // item is past the end the claimed one is too, and no item is lost)
  int next = 0;
  if (persistent && threadIdx.x == 0) next = atomicAdd(counter, 1);
  while (true) {
    if (persistent) {
      if (threadIdx.x == 0) {
        s_item = next;
        next = atomicAdd(counter, 1);
      }
      __syncthreads();  // also: every thread has finished the previous tile
      item = s_item;
      __syncthreads();
    }
    if (item >= n_work) break;
    if (threadIdx.x == 0) {
      s_w = work[item];
      s_d = cloths[s_w.x];
    }
    __syncthreads();  // also: every thread has finished the previous tile
    const int4 w = s_w;
    const ClothDesc& d = s_d;
    if (d.skip) {  // masked out: uniform over the CTA
      __syncthreads();  // s_d is rewritten for the next item
      if (!persistent) break;
      continue;
    }
    const V3<float> wind{d.wind[0], d.wind[1], d.wind[2]};
    // maps: per cloth, {pos[0], vel[0], pos[1], vel[1]} (empty maps: thread staging)
    const CUtensorMap* mp = TMA ? maps + 4 * size_t(w.x) + 2 * parity : nullptr;
    const CUtensorMap* mv = TMA ? mp + 1 : nullptr;
    if (w.w)
      tile_step<TW, TH, HALO, true, TMA>(w.y, w.z, d.rows, d.cols, d.planes, d.pos[parity], d.vel[parity],
                                         d.force_in, d.pos[parity ^ 1], d.vel[parity ^ 1], c, wind, d.flags, mp, mv,
                                         &bar, phase);
    else
      tile_step<TW, TH, HALO, false, TMA>(w.y, w.z, d.rows, d.cols, d.planes, d.pos[parity], d.vel[parity],
                                          d.force_in, d.pos[parity ^ 1], d.vel[parity ^ 1], c, wind, d.flags, mp, mv,
                                          &bar, phase);
    phase ^= TMA ? 1u : 0u;
    if (!persistent) break;
  }
}

constexpr int kTileW = 32, kTileH = 8, kHalo = 64;  // the single-cloth kernel's tile; the batch's default

template <int TH>
size_t tiled_smem_bytes_t() {
  using G = TileGeom<kTileW, TH>;
  using I = Interior<kTileW, TH>;
  return 2 * sizeof(float4) * G::EH * G::EW + size_t(I::BYTES);
}

// Tensor map of one float4 state array of an R x C grid, seen as R rows of
// 4C floats, with the staging box of a 32 x th tile ((32+4) float4 x (th+4) rows).
bool encode_state_map(CUtensorMap* m, const float4* base, int R, int C, int th) {
  using Encode = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                              const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  static Encode encode = nullptr;
  static std::once_flag looked_up;  // the driver entry point is process-wide
  std::call_once(looked_up, [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      encode = reinterpret_cast<Encode>(fn);
    else
      cudaGetLastError();
  });
  if (!encode || (reinterpret_cast<uintptr_t>(base) & 15) != 0) return false;
  const cuuint64_t dims[2] = {4ull * cuuint64_t(C), cuuint64_t(R)};
  const cuuint64_t strides[1] = {16ull * cuuint64_t(C)};
  const cuuint32_t box[2] = {4u * (kTileW + 4), cuuint32_t(th + 4)};
  const cuuint32_t elem[2] = {1, 1};
  return encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float4*>(base), dims, strides, box, elem,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Ring / interior split of an R x C cloth's 32 x th tiles.  Interior tiles
// have every neighbour of every vertex inside the cloth:
// c0 >= 2, c0 + 32 <= C - 2, r0 >= 2, r0 + th <= R - 2.
TileSplit split_tiles(int rows, int cols, int th) {
  TileSplit t;
  t.tx = (cols + kTileW - 1) / kTileW;
  t.ty = (rows + th - 1) / th;
  t.bx0 = 1;
  t.bx1 = cols >= kTileW + 4 ? (cols - 2 - kTileW) / kTileW : 0;
  t.by0 = 1;
  t.by1 = rows >= th + 4 ? (rows - 2 - th) / th : 0;
  return t;
}

template <int TH>
cudaError_t prime_batched() {
  const int smem = int(tiled_smem_bytes_t<TH>());
  cudaError_t e = cudaFuncSetAttribute(k_step_batched<kTileW, TH, kHalo, true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_step_batched<kTileW, TH, kHalo, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem);
  return e;
}

template <int TH>
int batched_ctas_per_sm_t() {
  int n = 0;
  if (prime_batched<TH>() != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_step_batched<kTileW, TH, kHalo, true>, kTileW * TH + kHalo,
                                                    tiled_smem_bytes_t<TH>()) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return n > 0 ? n : 1;
}

template <int TH>
void launch_batched_t(int grid, const ClothDesc* cloths, const int4* work, int n_work, int* counter, int parity,
                      int mode, const StepConsts& c, cudaStream_t s, const CUtensorMap* m, const int* n_work_dev) {
  const size_t smem = tiled_smem_bytes_t<TH>();
  if (m)
    k_step_batched<kTileW, TH, kHalo, true><<<grid, kTileW * TH + kHalo, smem, s>>>(
        cloths, work, n_work, counter, parity, mode == 1, c, m, n_work_dev);
  else
    k_step_batched<kTileW, TH, kHalo, false><<<grid, kTileW * TH + kHalo, smem, s>>>(
        cloths, work, n_work, counter, parity, mode == 1, c, m, n_work_dev);
}

}  // namespace

bool batch_tile_height_ok(int th) { return th == 4 || th == 8 || th == 12; }

bool encode_cloth_maps(const ClothDesc& d, int th, void* out) {
  CUtensorMap* m = static_cast<CUtensorMap*>(out);
  if (!batch_tile_height_ok(th)) return false;
  for (int k = 0; k < 2; ++k)
    if (!encode_state_map(m + 2 * k, d.pos[k], d.rows, d.cols, th) ||
        !encode_state_map(m + 2 * k + 1, d.vel[k], d.rows, d.cols, th))
      return false;
  return true;
}

void batch_tiles(int cloth, int rows, int cols, int th, int* out4, int* n_ring, int* n_interior) {
  const TileSplit t = split_tiles(rows, cols, th);
  const bool has_interior = t.bx1 >= t.bx0 && t.by1 >= t.by0;
  const int ni = has_interior ? (t.bx1 - t.bx0 + 1) * (t.by1 - t.by0 + 1) : 0;
  const int nr = t.tx * t.ty - ni;
  *n_ring = nr;
  *n_interior = ni;
  if (!out4) return;
  int k = 0;
  for (int by = 0; by < t.ty; ++by)  // ring tiles first
    for (int bx = 0; bx < t.tx; ++bx) {
      const bool inner = has_interior && bx >= t.bx0 && bx <= t.bx1 && by >= t.by0 && by <= t.by1;
      if (inner) continue;
      out4[4 * k] = cloth; out4[4 * k + 1] = bx; out4[4 * k + 2] = by; out4[4 * k + 3] = 0;
      ++k;
    }
  for (int by = t.by0; has_interior && by <= t.by1; ++by)
    for (int bx = t.bx0; bx <= t.bx1; ++bx) {
      out4[4 * k] = cloth; out4[4 * k + 1] = bx; out4[4 * k + 2] = by; out4[4 * k + 3] = 1;
      ++k;
    }
}

int grid_tiles(int rows, int cols, int th, int* out3) {
  const TileSplit t = split_tiles(rows, cols, th);
  const bool has_interior = t.bx1 >= t.bx0 && t.by1 >= t.by0;
  const int n_interior = has_interior ? (t.bx1 - t.bx0 + 1) * (t.by1 - t.by0 + 1) : 0;
  const int n_ring = t.tx * t.ty - n_interior;
  for (int b = 0; out3 && b < n_ring + n_interior; ++b)  // blockIdx.x b of k_step_grid_tiled
    out3[3 * b + 2] = grid_tile(t, n_ring, b, out3[3 * b], out3[3 * b + 1]) ? 1 : 0;
  return n_ring + n_interior;
}

cudaError_t prime_step_kernels() {
  // the attribute is per function and per device: set once on each device used
  static PerDeviceOnce once;
  return once.run([] {
    const int smem = int(tiled_smem_bytes_t<kTileH>());
    cudaError_t e = cudaFuncSetAttribute(k_step_grid_tiled<kTileW, kTileH, kHalo, true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_step_grid_tiled<kTileW, kTileH, kHalo, false>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) e = prime_batched<4>();
    if (e == cudaSuccess) e = prime_batched<8>();
    if (e == cudaSuccess) e = prime_batched<12>();
    return e;
  });
}

int batched_ctas_per_sm(int th) {
  switch (th) {
    case 4: return batched_ctas_per_sm_t<4>();
    case 12: return batched_ctas_per_sm_t<12>();
    default: return batched_ctas_per_sm_t<8>();
  }
}

cudaError_t launch_step_batched(const ClothDesc* cloths, const int4* work, int n_work, int* counter, int parity,
                                int mode, int persistent_ctas, const StepConsts& c, cudaStream_t s, const void* maps,
                                const int* n_work_dev, int th) {
  if (n_work <= 0) return cudaSuccess;
  if (n_work_dev && mode != 1) return cudaErrorInvalidValue;  // a device count needs the persistent form
  if (!batch_tile_height_ok(th)) return cudaErrorInvalidValue;
  const cudaError_t ea = prime_step_kernels();
  if (ea != cudaSuccess) return ea;
  const int grid = mode == 1 ? (persistent_ctas < n_work ? persistent_ctas : n_work) : n_work;
  const CUtensorMap* m = static_cast<const CUtensorMap*>(maps);
  switch (th) {
    case 4: launch_batched_t<4>(grid, cloths, work, n_work, counter, parity, mode, c, s, m, n_work_dev); break;
    case 12: launch_batched_t<12>(grid, cloths, work, n_work, counter, parity, mode, c, s, m, n_work_dev); break;
    default: launch_batched_t<8>(grid, cloths, work, n_work, counter, parity, mode, c, s, m, n_work_dev); break;
  }
  return cudaGetLastError();
}

cudaError_t launch_step_grid(const GridTopo& g, const float4* pos, const float4* vel, const float4* force_in,
                             float4* pos_out, float4* vel_out, const StepConsts& c, cudaStream_t s) {
  const int n = g.rows * g.cols;
  if (n <= 0) return cudaSuccess;
  if (g.variant == 1) {
    k_step_grid_v1<<<(n + 255) / 256, 256, 0, s>>>(g.rows, g.cols, g.params, pos, vel, force_in, pos_out, vel_out,
                                                   c);
  } else {
    const TileSplit t = split_tiles(g.rows, g.cols, kTileH);
    const bool has_interior = t.bx1 >= t.bx0 && t.by1 >= t.by0;
    const int n_interior = has_interior ? (t.bx1 - t.bx0 + 1) * (t.by1 - t.by0 + 1) : 0;
    const int n_ring = t.tx * t.ty - n_interior;
    const size_t smem = tiled_smem_bytes_t<kTileH>();
    const cudaError_t ea = prime_step_kernels();
    if (ea != cudaSuccess) return ea;
    CUtensorMap map_pos, map_vel;
    std::memset(&map_pos, 0, sizeof(map_pos));
    std::memset(&map_vel, 0, sizeof(map_vel));
    const bool use_tma = encode_state_map(&map_pos, pos, g.rows, g.cols, kTileH) &&
                         encode_state_map(&map_vel, vel, g.rows, g.cols, kTileH);
    if (use_tma)
      k_step_grid_tiled<kTileW, kTileH, kHalo, true><<<n_ring + n_interior, kTileW * kTileH + kHalo, smem, s>>>(
          g.rows, g.cols, t, n_ring, g.params, pos, vel, force_in, pos_out, vel_out, c, map_pos, map_vel);
    else
      k_step_grid_tiled<kTileW, kTileH, kHalo, false><<<n_ring + n_interior, kTileW * kTileH + kHalo, smem, s>>>(
          g.rows, g.cols, t, n_ring, g.params, pos, vel, force_in, pos_out, vel_out, c, map_pos, map_vel);
  }
  return cudaGetLastError();
}

}  // namespace fgb
