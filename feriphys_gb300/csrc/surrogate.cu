// Kernels of the learned surrogate (surrogate.h).
//
// Tensor-core mapping (tcgen05, operands in shared memory in the blocked
// layout of tc05.cuh, accumulators in tensor memory):
//  * a tile is 128 vertices = the 128 rows (TMEM lanes) of one M = 128 MMA;
//    thread t of a 128-thread group owns row t: it writes that row's inputs
//    and reads that row's accumulators back (warp w reads lanes 32w..32w+31);
//  * inference (k_sur_step): z1 = X W1^T (K = 64), z2 = H1 W2^T (K = 128),
//    y = H2 W3^T (N = 16, 3 used), each followed by the bias + GELU epilogue
//    that writes the next layer's bf16 operand in place of the previous one;
//    the weights are loaded into shared memory once per CTA by one bulk copy
//    and shared by G groups that work on G tiles at once;
//  * training (k_train): the forward pass keeps H1, H2 and the GELU slopes in
//    shared memory; the backward pass runs dH2 = dY W3, dH1 = dZ2 W2 and the
//    weight gradients dW = dZ^T H as MMAs that read the same tiles in the
//    other orientation (MN-major), and the bias gradients as dZ^T * ones; the
//    weight and bias gradients accumulate in tensor memory over all tiles of
//    the CTA and are written out once.
#include <cuda_bf16.h>

#include "devmath.cuh"
#include "grid_order.h"
#include "per_device.h"
#include "physics.cuh"
#include "surrogate.h"
#include "tc05.cuh"

namespace fgb {
namespace sur {
namespace {

constexpr float kInvPi = 0.318309873342514038f;  // RN(1/pi)
constexpr float kGeluC = 0.797884560802865356f;  // sqrt(2/pi)
constexpr float kGeluA = 0.044715f;

__device__ __forceinline__ uint32_t pack_bf2(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&h);
}

__device__ __forceinline__ float2 unpack_bf2(uint32_t u) {
  __nv_bfloat162 h = *reinterpret_cast<__nv_bfloat162*>(&u);
  return __bfloat1622float2(h);
}

// GELU, tanh form: 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))), and its
// slope 0.5 (1 + t) + 0.5 x (1 - t^2) sqrt(2/pi) (1 + 3 * 0.044715 x^2), with
// the tanh argument as x (c + c a x^2) and explicit fused multiply-adds (this
// file is compiled with -fmad=false).  Evaluated on pairs of columns with the
// packed f32x2 operations (the same per-lane roundings as the scalar form).
constexpr float kGeluCA = kGeluC * kGeluA;

using tc::f32x2;

__device__ __forceinline__ f32x2 tanh2(f32x2 u) {
  const float2 v = tc::f2_unpack(u);
  return tc::f2_pack(tc::tanh_fast(v.x), tc::tanh_fast(v.y));
}

// GELU of the pair x, rounded to a bf16 pair.
__device__ __forceinline__ uint32_t gelu2_bf(f32x2 x) {
  const f32x2 u = tc::f2_mul(tc::f2_fma(tc::f2_splat(kGeluCA), tc::f2_mul(x, x), tc::f2_splat(kGeluC)), x);
  const f32x2 t = tanh2(u);
  const float2 h = tc::f2_unpack(tc::f2_mul(x, tc::f2_fma(tc::f2_splat(0.5f), t, tc::f2_splat(0.5f))));
  return pack_bf2(h.x, h.y);
}

// GELU and its slope of the pair x, each rounded to a bf16 pair.
__device__ __forceinline__ void gelu2_slope_bf(f32x2 x, uint32_t& g, uint32_t& dg) {
  const f32x2 x2 = tc::f2_mul(x, x);
  const f32x2 u = tc::f2_mul(tc::f2_fma(tc::f2_splat(kGeluCA), x2, tc::f2_splat(kGeluC)), x);
  const f32x2 t = tanh2(u);
  const f32x2 half1pt = tc::f2_fma(tc::f2_splat(0.5f), t, tc::f2_splat(0.5f));
  const float2 gv = tc::f2_unpack(tc::f2_mul(x, half1pt));
  const f32x2 neg_t = tc::f2_mul(t, tc::f2_splat(-1.0f));  // exact
  const f32x2 one_m_t2 = tc::f2_fma(neg_t, t, tc::f2_splat(1.0f));
  const f32x2 du = tc::f2_fma(tc::f2_splat(3.0f * kGeluCA), x2, tc::f2_splat(kGeluC));
  const f32x2 a = tc::f2_mul(tc::f2_mul(tc::f2_splat(0.5f), x), one_m_t2);
  const float2 dv = tc::f2_unpack(tc::f2_fma(a, du, half1pt));
  g = pack_bf2(gv.x, gv.y);
  dg = pack_bf2(dv.x, dv.y);
}

// Barrier of one group of `n` threads (id 0: the whole CTA).
__device__ __forceinline__ void group_sync(int id, int n = 128) {
  if (id == 0)
    __syncthreads();
  else
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}

// Generic-proxy writes and tensor-memory reads done by the group become
// ordered before the MMA that one thread of the group issues next.
__device__ __forceinline__ void sync_for_mma(int id, int n = 128) {
  tc::fence_before_sync();
  tc::fence_async_smem();
  group_sync(id, n);
  tc::fence_after_sync();
}

// Bounded wait on an MMA/copy barrier by a whole group; every thread of the
// group returns the same verdict.
__device__ __forceinline__ bool group_wait(uint64_t* bar, uint32_t& phase, int id, volatile int* fail_flag,
                                           int n = 128) {
  const bool ok = tc::mbar_wait(bar, phase);
  phase ^= 1u;
  if (!ok) *fail_flag = 1;
  group_sync(id, n);
  const bool all = *fail_flag == 0;
  tc::fence_after_sync();
  return all;
}

// ---- features --------------------------------------------------------------

__device__ __forceinline__ void vertex_features(const SurCloth& c, int parity, int r, int col, float (&f)[kFeat]) {
  const int R = c.rows, C = c.cols;
  const float4* __restrict__ P = c.pos[parity];
  const float4* __restrict__ Vl = c.vel[parity];
  const float4* __restrict__ P0 = c.rest;
  const int i = r * C + col;
  const float4 p = P[i], v = Vl[i], p0 = P0[i];
  const float ih = c.inv_h, s = c.sv;
  float3 q[8];
  bool has[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int dr = k < 3 ? -1 : (k < 5 ? 0 : 1);
    const int dc = (k == 0 || k == 3 || k == 5) ? -1 : ((k == 1 || k == 6) ? 0 : 1);
    const int rr = r + dr, cc = col + dc;
    has[k] = rr >= 0 && rr < R && cc >= 0 && cc < C;
    if (has[k]) {
      const int j = rr * C + cc;
      const float4 a = P[j], w = Vl[j], a0 = P0[j];
      q[k] = make_float3(a.x, a.y, a.z);
      f[3 * k + 0] = ((a.x - p.x) - (a0.x - p0.x)) * ih;
      f[3 * k + 1] = ((a.y - p.y) - (a0.y - p0.y)) * ih;
      f[3 * k + 2] = ((a.z - p.z) - (a0.z - p0.z)) * ih;
      f[24 + 3 * k + 0] = (w.x - v.x) * s;
      f[24 + 3 * k + 1] = (w.y - v.y) * s;
      f[24 + 3 * k + 2] = (w.z - v.z) * s;
    } else {
      q[k] = make_float3(p.x, p.y, p.z);
      f[3 * k + 0] = 0.0f;
      f[3 * k + 1] = 0.0f;
      f[3 * k + 2] = 0.0f;
      f[24 + 3 * k + 0] = 0.0f;
      f[24 + 3 * k + 1] = 0.0f;
      f[24 + 3 * k + 2] = 0.0f;
    }
  }
  f[48] = v.w != 0.0f ? 1.0f : 0.0f;
  f[49] = (c.wind[0] - v.x) * s;
  f[50] = (c.wind[1] - v.y) * s;
  f[51] = (c.wind[2] - v.z) * s;
  // normal from the row and column differences: (right - left) x (up - down)
  const float ax = q[4].x - q[3].x, ay = q[4].y - q[3].y, az = q[4].z - q[3].z;
  const float bx = q[6].x - q[1].x, by = q[6].y - q[1].y, bz = q[6].z - q[1].z;
  const float nx = ay * bz - az * by, ny = az * bx - ax * bz, nz = ax * by - ay * bx;
  const float len = sqrtf((nx * nx + ny * ny) + nz * nz);
  float ux = 0.0f, uy = 0.0f, uz = 1.0f;
  if (len > 0.0f && isfinite(len)) {
    const float il = 1.0f / len;
    ux = nx * il;
    uy = ny * il;
    uz = nz * il;
  }
  f[52] = acosf(fminf(fmaxf(uy, -1.0f), 1.0f)) * kInvPi;
  f[53] = atan2f(uz, ux) * kInvPi;
}

// The features of one row split over two threads: half 0 computes the
// neighbours 0..3 and the pin and wind features (columns 0-11, 24-35,
// 48-51), half 1 the neighbours 4..7 and the normal (columns 12-23, 36-47,
// 52-53; 54-63 are zero); each writes its columns standardised, as bf16, into
// the 64-wide tile.  Every feature is vertex_features' expression.
template <int HALF>
__device__ __forceinline__ void store_features_half(const SurCloth& c, int parity, int v, bool valid, const Norm& nm,
                                                    unsigned char* X, int row) {
  constexpr int NL = HALF == 0 ? 28 : 36;
  float f[NL];
#pragma unroll
  for (int i = 0; i < NL; ++i) f[i] = 0.0f;
  if (valid) {
    const int R = c.rows, C = c.cols, r = v / C, col = v % C;
    const float4* __restrict__ P = c.pos[parity];
    const float4* __restrict__ Vl = c.vel[parity];
    const float4* __restrict__ P0 = c.rest;
    const float4 p = P[v], w0 = Vl[v], p0 = P0[v];
    const float ih = c.inv_h, s = c.sv;
    float3 q[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int k = 4 * HALF + j;
      const int dr = k < 3 ? -1 : (k < 5 ? 0 : 1);
      const int dc = (k == 0 || k == 3 || k == 5) ? -1 : ((k == 1 || k == 6) ? 0 : 1);
      const int rr = r + dr, cc = col + dc;
      q[j] = make_float3(p.x, p.y, p.z);
      if (rr >= 0 && rr < R && cc >= 0 && cc < C) {
        const int i = rr * C + cc;
        const float4 a = P[i], w = Vl[i], a0 = P0[i];
        q[j] = make_float3(a.x, a.y, a.z);
        f[3 * j + 0] = ((a.x - p.x) - (a0.x - p0.x)) * ih;
        f[3 * j + 1] = ((a.y - p.y) - (a0.y - p0.y)) * ih;
        f[3 * j + 2] = ((a.z - p.z) - (a0.z - p0.z)) * ih;
        f[12 + 3 * j + 0] = (w.x - w0.x) * s;
        f[12 + 3 * j + 1] = (w.y - w0.y) * s;
        f[12 + 3 * j + 2] = (w.z - w0.z) * s;
      }
    }
    if (HALF == 0) {
      f[24] = w0.w != 0.0f ? 1.0f : 0.0f;
      f[25] = (c.wind[0] - w0.x) * s;
      f[26] = (c.wind[1] - w0.y) * s;
      f[27] = (c.wind[2] - w0.z) * s;
    } else {
      // neighbours 1 (up) and 3 (left) belong to the other half: load them here
      float3 q1 = make_float3(p.x, p.y, p.z), q3 = q1;
      if (r > 0) {
        const float4 a = P[v - C];
        q1 = make_float3(a.x, a.y, a.z);
      }
      if (col > 0) {
        const float4 a = P[v - 1];
        q3 = make_float3(a.x, a.y, a.z);
      }
      const float3 q4 = q[0], q6 = q[2];
      const float ax = q4.x - q3.x, ay = q4.y - q3.y, az = q4.z - q3.z;
      const float bx = q6.x - q1.x, by = q6.y - q1.y, bz = q6.z - q1.z;
      const float nx = ay * bz - az * by, ny = az * bx - ax * bz, nz = ax * by - ay * bx;
      const float len = sqrtf((nx * nx + ny * ny) + nz * nz);
      float ux = 0.0f, uy = 0.0f, uz = 1.0f;
      if (len > 0.0f && isfinite(len)) {
        const float il = 1.0f / len;
        ux = nx * il;
        uy = ny * il;
        uz = nz * il;
      }
      f[24] = acosf(fminf(fmaxf(uy, -1.0f), 1.0f)) * kInvPi;
      f[25] = atan2f(uz, ux) * kInvPi;
    }
  }
#pragma unroll
  for (int g4 = 0; g4 < NL / 4; ++g4) {
    const int li = 4 * g4;
    const int col = li < 12 ? 12 * HALF + li : (li < 24 ? 24 + 12 * HALF + (li - 12) : 48 + 4 * HALF + (li - 24));
    float x[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int k = col + e < kFeat ? col + e : 0;
      x[e] = (valid && col + e < kFeat) ? (f[li + e] - nm.in_mean[k]) * nm.in_inv_std[k] : 0.0f;
    }
    *reinterpret_cast<uint2*>(X + tc::blk_off(kIn, row, col)) = make_uint2(pack_bf2(x[0], x[1]), pack_bf2(x[2], x[3]));
  }
}

// Standardised features of row `lt` as bf16 into a 64-wide blocked tile.
__device__ __forceinline__ void store_input_row(unsigned char* X, int lt, const float (&f)[kFeat], bool valid,
                                                const Norm& nm) {
#pragma unroll
  for (int kc = 0; kc < kIn / 8; ++kc) {
    uint32_t q[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int k0 = kc * 8 + 2 * j, k1 = k0 + 1;
      const float a = (valid && k0 < kFeat) ? (f[k0 < kFeat ? k0 : 0] - nm.in_mean[k0 < kFeat ? k0 : 0]) *
                                                  nm.in_inv_std[k0 < kFeat ? k0 : 0]
                                            : 0.0f;
      const float b = (valid && k1 < kFeat) ? (f[k1 < kFeat ? k1 : 0] - nm.in_mean[k1 < kFeat ? k1 : 0]) *
                                                  nm.in_inv_std[k1 < kFeat ? k1 : 0]
                                            : 0.0f;
      q[j] = pack_bf2(a, b);
    }
    *reinterpret_cast<uint4*>(X + tc::blk_off(kIn, lt, kc * 8)) = make_uint4(q[0], q[1], q[2], q[3]);
  }
}

// ---- network stages --------------------------------------------------------

// z (TMEM lane = this thread's row, columns [c0, c1)) + bias -> GELU -> bf16
// row of the 128-wide tile H; with G != null also the GELU slope into G.
// BIAS = false: the accumulator already holds the bias (bias_to_tmem).
template <bool BIAS = true>
__device__ __forceinline__ void epilogue_gelu(uint32_t taddr, const float* __restrict__ bias, unsigned char* H,
                                              unsigned char* G, int lt, int c0 = 0, int c1 = kHid) {
  const f32x2* __restrict__ bias2 = reinterpret_cast<const f32x2*>(bias);
#pragma unroll 1
  for (int cb = c0; cb < c1; cb += 32) {
    float z[32];
    tc::tmem_ld32(taddr + cb, z);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      uint32_t uh[4], ug[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int a = 8 * q + 2 * j;
        const f32x2 zz = tc::f2_pack(z[a], z[a + 1]);
        const f32x2 x = BIAS ? tc::f2_add(zz, bias2[(cb + a) >> 1]) : zz;
        if (G)
          gelu2_slope_bf(x, uh[j], ug[j]);
        else
          uh[j] = gelu2_bf(x);
      }
      const uint32_t off = tc::blk_off(kHid, lt, cb + 8 * q);
      *reinterpret_cast<uint4*>(H + off) = make_uint4(uh[0], uh[1], uh[2], uh[3]);
      if (G) *reinterpret_cast<uint4*>(G + off) = make_uint4(ug[0], ug[1], ug[2], ug[3]);
    }
  }
}

// dZ = dH (TMEM) * slope (bf16 tile G), rounded to bf16, written over G.
__device__ __forceinline__ void epilogue_backward(uint32_t taddr, unsigned char* G, int lt, int c0 = 0,
                                                  int c1 = kHid) {
#pragma unroll 1
  for (int cb = c0; cb < c1; cb += 32) {
    float d[32];
    tc::tmem_ld32(taddr + cb, d);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint32_t off = tc::blk_off(kHid, lt, cb + 8 * q);
      const uint4 gq = *reinterpret_cast<const uint4*>(G + off);
      const uint32_t gw[4] = {gq.x, gq.y, gq.z, gq.w};
      uint32_t o[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float2 g = unpack_bf2(gw[j]);
        const float2 p = tc::f2_unpack(
            tc::f2_mul(tc::f2_pack(d[8 * q + 2 * j], d[8 * q + 2 * j + 1]), tc::f2_pack(g.x, g.y)));
        o[j] = pack_bf2(p.x, p.y);
      }
      *reinterpret_cast<uint4*>(G + off) = make_uint4(o[0], o[1], o[2], o[3]);
    }
  }
}

// The layer's bias as the initial value of this thread's accumulator row
// (TMEM lane = its row, columns [c0, c1)): the MMAs then accumulate onto it,
// so the epilogue has no bias to add.
__device__ __forceinline__ void bias_to_tmem(uint32_t taddr, const float* __restrict__ bias, int c0, int c1) {
#pragma unroll 1
  for (int cb = c0; cb < c1; cb += 32) {
    float v[32];
    const float4* b4 = reinterpret_cast<const float4*>(bias + cb);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const float4 q = b4[k];
      v[4 * k] = q.x;
      v[4 * k + 1] = q.y;
      v[4 * k + 2] = q.z;
      v[4 * k + 3] = q.w;
    }
    tc::tmem_st32(taddr + cb, v);
  }
}

// The three layers for the tile in `act` (inputs in the 64-wide layout on
// entry; the hidden activations overwrite it), run by a group of 128 * H
// threads: thread lt of the group owns row lt % 128 and the hidden columns
// [64 h, 64 h + 128 / H) with h = lt / 128.  The threads of h = 0 return their
// row of the 16 output columns with the bias added in y.
template <int H>
__device__ __forceinline__ bool mlp_tile(unsigned char* act, const unsigned char* wsm, uint32_t tmem,
                                         uint32_t lane_off, uint64_t* bar, uint32_t& phase, int lt, int bar_id,
                                         volatile int* fail_flag, float (&y)[16]) {
  constexpr int NT = 128 * H, NC = kHid / H;
  const int row = lt & 127, c0 = (lt >> 7) * NC;
  const uint32_t a_act = tc::smem_u32(act);
  const uint32_t a_w1 = tc::smem_u32(wsm + kBlobW1), a_w2 = tc::smem_u32(wsm + kBlobW2),
                 a_w3 = tc::smem_u32(wsm + kBlobW3);
  const float* b1 = reinterpret_cast<const float*>(wsm + kBlobB1);
  const float* b2 = reinterpret_cast<const float*>(wsm + kBlobB2);
  const float* b3 = reinterpret_cast<const float*>(wsm + kBlobB3);
  constexpr uint32_t id_hid = tc::idesc_bf16(128, kHid), id_out = tc::idesc_bf16(128, kOutPad);

  bias_to_tmem(tmem + lane_off, b1, c0, c0 + NC);
  sync_for_mma(bar_id, NT);
  if (lt == 0) {
#pragma unroll
    for (int s = 0; s < kIn / 16; ++s)
      tc::mma_bf16(tmem, tc::sdesc(a_act + 256 * s, 128, kIn * 16), tc::sdesc(a_w1 + 256 * s, 128, kIn * 16), id_hid,
                   true);
    tc::mma_commit(bar);
  }
  if (!group_wait(bar, phase, bar_id, fail_flag, NT)) return false;
  epilogue_gelu<false>(tmem + lane_off, b1, act, nullptr, row, c0, c0 + NC);

  bias_to_tmem(tmem + lane_off, b2, c0, c0 + NC);
  sync_for_mma(bar_id, NT);
  if (lt == 0) {
#pragma unroll
    for (int s = 0; s < kHid / 16; ++s)
      tc::mma_bf16(tmem, tc::sdesc(a_act + 256 * s, 128, kHid * 16), tc::sdesc(a_w2 + 256 * s, 128, kHid * 16),
                   id_hid, true);
    tc::mma_commit(bar);
  }
  if (!group_wait(bar, phase, bar_id, fail_flag, NT)) return false;
  epilogue_gelu<false>(tmem + lane_off, b2, act, nullptr, row, c0, c0 + NC);

  sync_for_mma(bar_id, NT);
  if (lt == 0) {
#pragma unroll
    for (int s = 0; s < kHid / 16; ++s)
      tc::mma_bf16(tmem, tc::sdesc(a_act + 256 * s, 128, kHid * 16), tc::sdesc(a_w3 + 256 * s, 128, kHid * 16),
                   id_out, s > 0);
    tc::mma_commit(bar);
  }
  if (!group_wait(bar, phase, bar_id, fail_flag, NT)) return false;
  if (lt < 128) {  // warp-uniform
    tc::tmem_ld16(tmem + lane_off, y);
#pragma unroll
    for (int j = 0; j < 16; ++j) y[j] += b3[j];
  }
  return true;
}

// ---- inference: the coarse step --------------------------------------------

// G groups of 128 * H threads; a group takes one 128-vertex tile at a time,
// H threads per vertex row (H = 2: each computes half of the row's features
// and half of its hidden columns, so twice the warps hide the latencies).
template <int G, int H>
__global__ void __launch_bounds__(128 * G * H, 1)
    k_sur_step(const SurCloth* __restrict__ cloths, const Tile* __restrict__ tiles, int n_tiles, int parity,
               const unsigned char* __restrict__ blob, const Norm norm, const StepConsts cst, int* err) {
  static_assert(H == 1 || H == 2, "one or two threads per row");
  constexpr int NT = 128 * H;
  constexpr uint32_t kCols = G == 1 ? 128 : (G == 2 ? 256 : 512);  // a power of two >= 128 G
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t bar_w;
  __shared__ uint64_t bar_g[G];
  __shared__ uint32_t tslot;
  __shared__ int gfail[G];
  const int tid = threadIdx.x, g = tid / NT, lt = tid % NT, row = lt & 127;
  if (tid < 32) {
    tc::tmem_alloc(&tslot, kCols);
    tc::tmem_relinquish();
    tc::fence_before_sync();
  }
  if (tid == 0) {
    tc::mbar_init(&bar_w, 1);
    for (int k = 0; k < G; ++k) tc::mbar_init(&bar_g[k], 1);
    tc::mbar_fence_init();
  }
  if (lt == 0) gfail[g] = 0;
  __syncthreads();
  tc::fence_after_sync();
  if (tid == 0) {
    tc::mbar_arrive_expect_tx(&bar_w, kBlobBytes);
    tc::bulk_g2s(smem, blob, kBlobBytes, &bar_w);
  }
  bool ok = __syncthreads_and(tc::mbar_wait(&bar_w, 0)) != 0;
  const uint32_t tmem = tslot + uint32_t(g * 128);
  const uint32_t lane_off = uint32_t((row >> 5) * 32) << 16;
  unsigned char* act = smem + kBlobSmem + g * 32768;
  const ObsFace* faces = static_cast<const ObsFace*>(cst.obstacle_faces);
  uint32_t phase = 0;
  for (int t = blockIdx.x * G + g; ok && t < n_tiles; t += gridDim.x * G) {
    const Tile w = tiles[t];
    const SurCloth& c = cloths[w.x];
    const int n = c.rows * c.cols;
    const int v = w.y + row;
    const bool valid = v < n;
    if (H == 1) {
      float f[kFeat];
      if (valid) vertex_features(c, parity, v / c.cols, v % c.cols, f);
      store_input_row(act, row, f, valid, norm);
    } else if (lt < 128) {  // warp-uniform
      store_features_half<0>(c, parity, v, valid, norm, act, row);
    } else {
      store_features_half<1>(c, parity, v, valid, norm, act, row);
    }
    float y[16];
    ok = mlp_tile<H>(act, smem, tmem, lane_off, &bar_g[g], phase, lt, 1 + g, &gfail[g], y);
    if (!ok) break;
    if (valid && lt < 128) {
      const float4 P = c.pos[parity][v], V = c.vel[parity][v];
      float4 PO = P, VO = V;
      if (V.w == 0.0f) {
        const V3<float> p{P.x, P.y, P.z}, vv{V.x, V.y, V.z};
        const float isv = c.inv_sv;
        const V3<float> dv{(y[0] * norm.out_std[0] + norm.out_mean[0]) * isv,
                           (y[1] * norm.out_std[1] + norm.out_mean[1]) * isv,
                           (y[2] * norm.out_std[2] + norm.out_mean[2]) * isv};
        V3<float> nv = vv + dv;
        V3<float> np = p + (vv + nv) * (0.5f * cst.dt);
        if (cst.n_obstacle_faces > 0) {
          const V3<float> oF = dv * (P.w / cst.dt);
          collide_point<float>(faces, cst.n_obstacle_faces, p, vv, oF, P.w, np, nv, cst);
        }
        if (!(finite3(np) && finite3(nv)) && c.flags) atomicOr(c.flags, 1u);
        PO = make_float4(np.x, np.y, np.z, P.w);
        VO = make_float4(nv.x, nv.y, nv.z, 0.0f);
      }
      c.pos[parity ^ 1][v] = PO;
      c.vel[parity ^ 1][v] = VO;
    }
    tc::fence_before_sync();
  }
  if (!ok && lt == 0) atomicOr(err, 1);
  __syncthreads();
  if (tid < 32) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tslot, kCols);
  }
}

// Network outputs for rows already standardised and packed (tests, tools).
__global__ void __launch_bounds__(128, 1)
    k_forward(const unsigned char* __restrict__ X, int n_tiles, const unsigned char* __restrict__ blob,
              float* __restrict__ Y, int* err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t bar_w, bar_x, bar_m;
  __shared__ uint32_t tslot;
  __shared__ int fail;
  const int lt = threadIdx.x;
  if (lt < 32) {
    tc::tmem_alloc(&tslot, 128);
    tc::tmem_relinquish();
    tc::fence_before_sync();
  }
  if (lt == 0) {
    tc::mbar_init(&bar_w, 1);
    tc::mbar_init(&bar_x, 1);
    tc::mbar_init(&bar_m, 1);
    tc::mbar_fence_init();
    fail = 0;
  }
  __syncthreads();
  tc::fence_after_sync();
  if (lt == 0) {
    tc::mbar_arrive_expect_tx(&bar_w, kBlobBytes);
    tc::bulk_g2s(smem, blob, kBlobBytes, &bar_w);
  }
  bool ok = __syncthreads_and(tc::mbar_wait(&bar_w, 0)) != 0;
  const uint32_t tmem = tslot, lane_off = uint32_t((lt >> 5) * 32) << 16;
  unsigned char* act = smem + kBlobSmem;
  uint32_t ph_x = 0, ph_m = 0;
  for (int t = blockIdx.x; ok && t < n_tiles; t += gridDim.x) {
    sync_for_mma(0);  // the previous tile's MMAs are complete; act may be overwritten
    if (lt == 0) {
      tc::mbar_arrive_expect_tx(&bar_x, 16384);
      tc::bulk_g2s(act, X + size_t(t) * 16384, 16384, &bar_x);
    }
    ok = group_wait(&bar_x, ph_x, 0, &fail);
    if (!ok) break;
    float y[16];
    ok = mlp_tile<1>(act, smem, tmem, lane_off, &bar_m, ph_m, lt, 0, &fail, y);
    if (!ok) break;
    reinterpret_cast<float4*>(Y)[size_t(t) * 128 + lt] = make_float4(y[0], y[1], y[2], 0.0f);
    tc::fence_before_sync();
  }
  if (!ok && lt == 0) atomicOr(err, 1);
  __syncthreads();
  if (lt < 32) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tslot, 128);
  }
}

// ---- training: fused forward + backward ------------------------------------

// Layout of a CTA's gradient partials: the parameter order, except that the
// W1 and W2 blocks are stored column by column (entry (o, i) at i * 128 + o),
// so that the 32 threads of a warp, which hold 32 consecutive rows o of one
// column i in tensor memory, write 128 consecutive bytes.  The reduction
// kernels walk the partials in this order and map back.
__device__ __forceinline__ int partial_of_param(int p) {
  if (p < kOffB1) return kOffW1 + ((p - kOffW1) % kIn) * kHid + (p - kOffW1) / kIn;
  if (p >= kOffW2 && p < kOffB2) return kOffW2 + ((p - kOffW2) % kHid) * kHid + (p - kOffW2) / kHid;
  return p;
}
__device__ __forceinline__ int param_of_partial(int q) {
  if (q < kOffB1) return kOffW1 + ((q - kOffW1) % kHid) * kIn + (q - kOffW1) / kHid;
  if (q >= kOffW2 && q < kOffB2) return kOffW2 + ((q - kOffW2) % kHid) * kHid + (q - kOffW2) / kHid;
  return q;
}

constexpr int kTrX = kBlobSmem;            // 128 x 64
constexpr int kTrH1 = kTrX + 16384;        // 128 x 128
constexpr int kTrH2 = kTrH1 + 32768;
constexpr int kTrG1 = kTrH2 + 32768;       // GELU slopes, then dZ1
constexpr int kTrG2 = kTrG1 + 32768;       // GELU slopes, then dZ2
constexpr int kTrDY = kTrG2 + 32768;       // 128 x 16
constexpr int kTrOnes = kTrDY + 4096;      // 16 x 128 of 1.0
constexpr int kTrSmem = kTrOnes + 4096;    // 210944 B
constexpr int kTrThreads = 256;            // two threads per row of a 128-row tile

// tensor-memory columns
constexpr uint32_t kCA = 0, kCB = 128, kCW2 = 256, kCW1 = 384, kCW3 = 448, kCB2 = 464, kCB1 = 480;

// Two threads per row: thread lt owns row lt % 128 and the hidden columns
// [64 h, 64 h + 64) with h = lt / 128 in every epilogue; the threads of h = 0
// form the loss and dY of their row.
__global__ void __launch_bounds__(kTrThreads, 1)
    k_train(const unsigned char* __restrict__ X, const float* __restrict__ T, int n_tiles,
            const unsigned char* __restrict__ blob, float* __restrict__ partials, float dscale, int* err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t bar_w, bar_x, bar_m;
  __shared__ uint32_t tslot;
  __shared__ int fail;
  __shared__ float red[4][4];
  __shared__ float acc[4];  // loss, db3[0..2] of this CTA
  const int lt = threadIdx.x, warp = lt >> 5, lane = lt & 31;
  const int row = lt & 127, half = lt >> 7, c0 = half * (kHid / 2), c1 = c0 + kHid / 2;
  if (warp == 0) {
    tc::tmem_alloc(&tslot, 512);
    tc::tmem_relinquish();
    tc::fence_before_sync();
  }
  if (lt == 0) {
    tc::mbar_init(&bar_w, 1);
    tc::mbar_init(&bar_x, 1);
    tc::mbar_init(&bar_m, 1);
    tc::mbar_fence_init();
    fail = 0;
  }
  if (lt < 4) acc[lt] = 0.0f;
  for (int e = lt; e < 16 * (kHid / 8); e += kTrThreads) {  // the ones tile (bf16 1.0 = 0x3F80)
    const int r = e / (kHid / 8), kc = e % (kHid / 8);
    *reinterpret_cast<uint4*>(smem + kTrOnes + tc::blk_off(kHid, r, kc * 8)) =
        make_uint4(0x3F803F80u, 0x3F803F80u, 0x3F803F80u, 0x3F803F80u);
  }
  __syncthreads();
  tc::fence_after_sync();
  if (lt == 0) {
    tc::mbar_arrive_expect_tx(&bar_w, kBlobBytes);
    tc::bulk_g2s(smem, blob, kBlobBytes, &bar_w);
  }
  bool ok = __syncthreads_and(tc::mbar_wait(&bar_w, 0)) != 0;
  const uint32_t tmem = tslot, lane_off = uint32_t((warp & 3) * 32) << 16;  // the row's TMEM lane quarter
  unsigned char* sX = smem + kTrX;
  unsigned char* sH1 = smem + kTrH1;
  unsigned char* sH2 = smem + kTrH2;
  unsigned char* sG1 = smem + kTrG1;
  unsigned char* sG2 = smem + kTrG2;
  unsigned char* sDY = smem + kTrDY;
  const uint32_t aX = tc::smem_u32(sX), aH1 = tc::smem_u32(sH1), aH2 = tc::smem_u32(sH2), aG1 = tc::smem_u32(sG1),
                 aG2 = tc::smem_u32(sG2), aDY = tc::smem_u32(sDY), aOn = tc::smem_u32(smem + kTrOnes);
  const uint32_t aW1 = tc::smem_u32(smem + kBlobW1), aW2 = tc::smem_u32(smem + kBlobW2),
                 aW3 = tc::smem_u32(smem + kBlobW3);
  const float* b1 = reinterpret_cast<const float*>(smem + kBlobB1);
  const float* b2 = reinterpret_cast<const float*>(smem + kBlobB2);
  const float* b3 = reinterpret_cast<const float*>(smem + kBlobB3);
  constexpr uint32_t KM_H = kHid * 16;  // row-group stride of a 128-wide tile
  uint32_t ph_x = 0, ph_m = 0;
  bool first = true;
  for (int t = blockIdx.x; ok && t < n_tiles; t += gridDim.x) {
    if (lt == 0) {
      tc::mbar_arrive_expect_tx(&bar_x, 16384);
      tc::bulk_g2s(sX, X + size_t(t) * 16384, 16384, &bar_x);
    }
    const float4 tg = reinterpret_cast<const float4*>(T)[size_t(t) * 128 + row];
    // the layer biases as the accumulators' starting values, as in inference
    bias_to_tmem(tmem + kCA + lane_off, b1, c0, c1);
    bias_to_tmem(tmem + kCB + lane_off, b2, c0, c1);
    tc::fence_before_sync();
    if (!(ok = group_wait(&bar_x, ph_x, 0, &fail))) break;
    // layer 1: z1 -> cols [0, 128)
    if (lt == 0) {
#pragma unroll
      for (int s = 0; s < kIn / 16; ++s)
        tc::mma_bf16(tmem + kCA, tc::sdesc(aX + 256 * s, 128, kIn * 16), tc::sdesc(aW1 + 256 * s, 128, kIn * 16),
                     tc::idesc_bf16(128, kHid), true);
      tc::mma_commit(&bar_m);
    }
    if (!(ok = group_wait(&bar_m, ph_m, 0, &fail))) break;
    epilogue_gelu<false>(tmem + kCA + lane_off, b1, sH1, sG1, row, c0, c1);
    sync_for_mma(0);
    // layer 2: z2 -> cols [128, 256)
    if (lt == 0) {
#pragma unroll
      for (int s = 0; s < kHid / 16; ++s)
        tc::mma_bf16(tmem + kCB, tc::sdesc(aH1 + 256 * s, 128, KM_H), tc::sdesc(aW2 + 256 * s, 128, KM_H),
                     tc::idesc_bf16(128, kHid), true);
      tc::mma_commit(&bar_m);
    }
    if (!(ok = group_wait(&bar_m, ph_m, 0, &fail))) break;
    epilogue_gelu<false>(tmem + kCB + lane_off, b2, sH2, sG2, row, c0, c1);
    sync_for_mma(0);
    // layer 3: y -> cols [0, 16)
    if (lt == 0) {
#pragma unroll
      for (int s = 0; s < kHid / 16; ++s)
        tc::mma_bf16(tmem + kCA, tc::sdesc(aH2 + 256 * s, 128, KM_H), tc::sdesc(aW3 + 256 * s, 128, KM_H),
                     tc::idesc_bf16(128, kOutPad), s > 0);
      tc::mma_commit(&bar_m);
    }
    if (!(ok = group_wait(&bar_m, ph_m, 0, &fail))) break;
    if (half == 0) {  // warp-uniform
      float y[16];
      tc::tmem_ld16(tmem + kCA + lane_off, y);
      const float r0 = (y[0] + b3[0]) - tg.x, r1 = (y[1] + b3[1]) - tg.y, r2 = (y[2] + b3[2]) - tg.z;
      float ls = (r0 * r0 + r1 * r1) + r2 * r2;
      const uint32_t q0 = pack_bf2(r0 * dscale, r1 * dscale), q1 = pack_bf2(r2 * dscale, 0.0f);
      *reinterpret_cast<uint4*>(sDY + tc::blk_off(16, row, 0)) = make_uint4(q0, q1, 0u, 0u);
      *reinterpret_cast<uint4*>(sDY + tc::blk_off(16, row, 8)) = make_uint4(0u, 0u, 0u, 0u);
      const float2 e0 = unpack_bf2(q0), e1 = unpack_bf2(q1);
      float s0 = e0.x, s1 = e0.y, s2 = e1.x;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        ls += __shfl_xor_sync(0xffffffffu, ls, o);
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
      }
      if (lane == 0) {
        red[warp][0] = ls;
        red[warp][1] = s0;
        red[warp][2] = s1;
        red[warp][3] = s2;
      }
    }
    sync_for_mma(0);
    if (lt < 4) acc[lt] += ((red[0][lt] + red[1][lt]) + red[2][lt]) + red[3][lt];
    // dW3^T (+)= H2^T dY -> cols [448, 464); dH2 = dY W3 -> cols [128, 256)
    if (lt == 0) {
#pragma unroll
      for (int s = 0; s < 8; ++s)
        tc::mma_bf16(tmem + kCW3, tc::sdesc(aH2 + 2 * KM_H * s, KM_H, 128), tc::sdesc(aDY + 512 * s, 256, 128),
                     tc::idesc_bf16(128, kOutPad, true, true), !(first && s == 0));
      tc::mma_bf16(tmem + kCB, tc::sdesc(aDY, 128, 256), tc::sdesc(aW3, KM_H, 128), tc::idesc_bf16(128, kHid, false, true),
                   0);
      tc::mma_commit(&bar_m);
    }
    if (!(ok = group_wait(&bar_m, ph_m, 0, &fail))) break;
    epilogue_backward(tmem + kCB + lane_off, sG2, row, c0, c1);
    sync_for_mma(0);
    // dW2 (+)= dZ2^T H1; db2 (+)= dZ2^T 1; dH1 = dZ2 W2 -> cols [0, 128)
    if (lt == 0) {
#pragma unroll
      for (int s = 0; s < 8; ++s)
        tc::mma_bf16(tmem + kCW2, tc::sdesc(aG2 + 2 * KM_H * s, KM_H, 128), tc::sdesc(aH1 + 2 * KM_H * s, KM_H, 128),
                     tc::idesc_bf16(128, kHid, true, true), !(first && s == 0));
#pragma unroll
      for (int s = 0; s < 8; ++s)
        tc::mma_bf16(tmem + kCB2, tc::sdesc(aG2 + 2 * KM_H * s, KM_H, 128), tc::sdesc(aOn + 256 * s, 128, KM_H),
                     tc::idesc_bf16(128, kOutPad, true, false), !(first && s == 0));
#pragma unroll
      for (int s = 0; s < 8; ++s)
        tc::mma_bf16(tmem + kCA, tc::sdesc(aG2 + 256 * s, 128, KM_H), tc::sdesc(aW2 + 2 * KM_H * s, KM_H, 128),
                     tc::idesc_bf16(128, kHid, false, true), s > 0);
      tc::mma_commit(&bar_m);
    }
    if (!(ok = group_wait(&bar_m, ph_m, 0, &fail))) break;
    epilogue_backward(tmem + kCA + lane_off, sG1, row, c0, c1);
    sync_for_mma(0);
    // dW1 (+)= dZ1^T X; db1 (+)= dZ1^T 1
    if (lt == 0) {
#pragma unroll
      for (int s = 0; s < 8; ++s)
        tc::mma_bf16(tmem + kCW1, tc::sdesc(aG1 + 2 * KM_H * s, KM_H, 128), tc::sdesc(aX + 2 * kIn * 16 * s, kIn * 16, 128),
                     tc::idesc_bf16(128, kIn, true, true), !(first && s == 0));
#pragma unroll
      for (int s = 0; s < 8; ++s)
        tc::mma_bf16(tmem + kCB1, tc::sdesc(aG1 + 2 * KM_H * s, KM_H, 128), tc::sdesc(aOn + 256 * s, 128, KM_H),
                     tc::idesc_bf16(128, kOutPad, true, false), !(first && s == 0));
      tc::mma_commit(&bar_m);
    }
    if (!(ok = group_wait(&bar_m, ph_m, 0, &fail))) break;
    first = false;
  }
  float* P = partials + size_t(blockIdx.x) * kPartialStride;
  if (ok && !first) {
    float v[32];
#pragma unroll 1
    for (int cb = half * (kIn / 2); cb < (half + 1) * (kIn / 2); cb += 32) {
      tc::tmem_ld32(tmem + kCW1 + lane_off + cb, v);
      for (int j = 0; j < 32; ++j) P[partial_of_param(kOffW1 + row * kIn + cb + j)] = v[j];
    }
#pragma unroll 1
    for (int cb = c0; cb < c1; cb += 32) {
      tc::tmem_ld32(tmem + kCW2 + lane_off + cb, v);
      for (int j = 0; j < 32; ++j) P[partial_of_param(kOffW2 + row * kHid + cb + j)] = v[j];
    }
    if (half == 0) {  // warp-uniform
      float u[16];
      tc::tmem_ld16(tmem + kCW3 + lane_off, u);
      for (int o = 0; o < kOutPad; ++o) P[kOffW3 + o * kHid + row] = o < kOut ? u[o] : 0.0f;
      tc::tmem_ld16(tmem + kCB1 + lane_off, u);
      P[kOffB1 + row] = u[0];
      tc::tmem_ld16(tmem + kCB2 + lane_off, u);
      P[kOffB2 + row] = u[0];
      if (lt < kOutPad) P[kOffB3 + lt] = (lt < kOut) ? acc[1 + lt] : 0.0f;
      if (lt == 0) P[kNumParams] = acc[0];
    }
  } else {
    for (int p = lt; p < kPartialStride; p += kTrThreads) P[p] = 0.0f;
  }
  if (!ok && lt == 0) atomicOr(err, 1);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tslot, 512);
  }
}

// ---- parameters ------------------------------------------------------------

__device__ __forceinline__ bool param_used(int p) {
  if (p < kOffB1) return (p - kOffW1) % kIn < kFeat;
  if (p >= kOffW3 && p < kOffB3) return (p - kOffW3) / kHid < kOut;
  if (p >= kOffB3) return p - kOffB3 < kOut;
  return true;
}

__device__ __forceinline__ void blob_store(unsigned char* blob, int p, float w) {
  if (p < kOffB1) {
    const int o = (p - kOffW1) / kIn, i = (p - kOffW1) % kIn;
    *reinterpret_cast<__nv_bfloat16*>(blob + kBlobW1 + tc::blk_off(kIn, o, i)) = __float2bfloat16_rn(w);
  } else if (p < kOffW2) {
    reinterpret_cast<float*>(blob + kBlobB1)[p - kOffB1] = w;
  } else if (p < kOffB2) {
    const int o = (p - kOffW2) / kHid, i = (p - kOffW2) % kHid;
    *reinterpret_cast<__nv_bfloat16*>(blob + kBlobW2 + tc::blk_off(kHid, o, i)) = __float2bfloat16_rn(w);
  } else if (p < kOffW3) {
    reinterpret_cast<float*>(blob + kBlobB2)[p - kOffB2] = w;
  } else if (p < kOffB3) {
    const int o = (p - kOffW3) / kHid, i = (p - kOffW3) % kHid;
    *reinterpret_cast<__nv_bfloat16*>(blob + kBlobW3 + tc::blk_off(kHid, o, i)) = __float2bfloat16_rn(w);
  } else {
    reinterpret_cast<float*>(blob + kBlobB3)[p - kOffB3] = w;
  }
}

__device__ __forceinline__ float loss_sum(const float* partials, int ctas) {
  float s = 0.0f;
  for (int c = 0; c < ctas; ++c) s += partials[size_t(c) * kPartialStride + kNumParams];
  return s;
}

// the gradient of parameter p = param_of_partial(q), summed over the CTAs in
// CTA order (the threads of a block read consecutive partials q)
__device__ __forceinline__ float grad_sum(const float* partials, int ctas, int q, int p) {
  float g = 0.0f;
  for (int c = 0; c < ctas; ++c) g += partials[size_t(c) * kPartialStride + q];
  return param_used(p) ? g : 0.0f;
}

__global__ void k_reduce_grad(const float* __restrict__ partials, int ctas, float inv_count, float* __restrict__ grad,
                              float* __restrict__ loss_out) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q == 0 && loss_out) loss_out[0] = loss_sum(partials, ctas) * inv_count;
  if (q >= kNumParams) return;
  const int p = param_of_partial(q);
  grad[p] = grad_sum(partials, ctas, q, p);
}

__global__ void k_adam(const float* __restrict__ partials, int ctas, float* __restrict__ master, float* __restrict__ m,
                       float* __restrict__ v, float lr, float beta1, float beta2, float eps, float c1, float c2,
                       unsigned char* __restrict__ blob, float* __restrict__ loss_out, float inv_count) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q == 0 && loss_out) loss_out[0] = loss_sum(partials, ctas) * inv_count;
  if (q >= kNumParams) return;
  const int p = param_of_partial(q);
  const float g = grad_sum(partials, ctas, q, p);
  const float mm = beta1 * m[p] + (1.0f - beta1) * g;
  const float vv = beta2 * v[p] + (1.0f - beta2) * (g * g);
  m[p] = mm;
  v[p] = vv;
  float w = master[p] - lr * (mm * c1) / (sqrtf(vv * c2) + eps);
  if (!param_used(p)) w = 0.0f;
  master[p] = w;
  blob_store(blob, p, w);
}

__global__ void k_pack_blob(const float* __restrict__ master, unsigned char* __restrict__ blob) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < kNumParams) blob_store(blob, p, param_used(p) ? master[p] : 0.0f);
}

// ---- dataset ---------------------------------------------------------------

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ULL;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebULL;
  x ^= x >> 31;
  return x;
}

__global__ void k_collect_features(const SurCloth* __restrict__ cloths, const Tile* __restrict__ tiles, int n_tiles,
                                   int parity, float* __restrict__ feat, float* __restrict__ tgt, long long cap) {
  const int t = blockIdx.x;
  if (t >= n_tiles) return;
  const Tile w = tiles[t];
  const SurCloth& c = cloths[w.x];
  const int v = w.y + threadIdx.x;
  if (v >= c.rows * c.cols) return;
  float f[kFeat];
  vertex_features(c, parity, v / c.cols, v % c.cols, f);
  const long long row = (c.vbase + v) % cap;
  float* o = feat + row * kRawStride;
#pragma unroll
  for (int k = 0; k < kRawStride; ++k) o[k] = k < kFeat ? f[k < kFeat ? k : 0] : 0.0f;
  const float4 vel = c.vel[parity][v];
  reinterpret_cast<float4*>(tgt)[row] = make_float4(vel.x, vel.y, vel.z, c.sv);
}

__global__ void k_collect_targets(const SurCloth* __restrict__ cloths, const Tile* __restrict__ tiles, int n_tiles,
                                  int parity, float* __restrict__ tgt, long long cap) {
  const int t = blockIdx.x;
  if (t >= n_tiles) return;
  const Tile w = tiles[t];
  const SurCloth& c = cloths[w.x];
  const int v = w.y + threadIdx.x;
  if (v >= c.rows * c.cols) return;
  const long long row = (c.vbase + v) % cap;
  const float4 old = reinterpret_cast<const float4*>(tgt)[row];
  const float4 nv = c.vel[parity][v];
  reinterpret_cast<float4*>(tgt)[row] =
      make_float4((nv.x - old.x) * old.w, (nv.y - old.y) * old.w, (nv.z - old.z) * old.w, 0.0f);
}

__global__ void k_features(const SurCloth* __restrict__ cloth, const Tile* __restrict__ tiles, int n_tiles,
                           int parity, float* __restrict__ out) {
  const int t = blockIdx.x;
  if (t >= n_tiles) return;
  const Tile w = tiles[t];
  const SurCloth& c = cloth[w.x];
  const int v = w.y + threadIdx.x;
  if (v >= c.rows * c.cols) return;
  float f[kFeat];
  vertex_features(c, parity, v / c.cols, v % c.cols, f);
#pragma unroll
  for (int k = 0; k < kFeat; ++k) out[size_t(v) * kFeat + k] = f[k];
}

__global__ void k_pack_batch(const float* __restrict__ feat, const float* __restrict__ tgt, long long count,
                             uint64_t seed, int n_rows, const Norm nm, unsigned char* __restrict__ X,
                             float* __restrict__ T) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n_rows) return;
  const long long row = (long long)(mix64(seed ^ (uint64_t(b) * 0x9E3779B97F4A7C15ULL)) % uint64_t(count));
  const float* f = feat + row * kRawStride;
  float x[kFeat];
#pragma unroll
  for (int k = 0; k < kFeat; ++k) x[k] = f[k];
  store_input_row(X + size_t(b >> 7) * 16384, b & 127, x, true, nm);
  const float4 t = reinterpret_cast<const float4*>(tgt)[row];
  reinterpret_cast<float4*>(T)[b] = make_float4((t.x - nm.out_mean[0]) / nm.out_std[0],
                                                (t.y - nm.out_mean[1]) / nm.out_std[1],
                                                (t.z - nm.out_mean[2]) / nm.out_std[2], 0.0f);
}

__global__ void k_pack_rows(const float* __restrict__ x, const float* __restrict__ t, int n, int n_pad,
                            unsigned char* __restrict__ X, float* __restrict__ T) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n_pad) return;
  const bool valid = b < n;
#pragma unroll
  for (int kc = 0; kc < kIn / 8; ++kc) {
    uint32_t q[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int k0 = kc * 8 + 2 * j, k1 = k0 + 1;
      const float a = (valid && k0 < kFeat) ? x[size_t(b) * kFeat + k0] : 0.0f;
      const float c = (valid && k1 < kFeat) ? x[size_t(b) * kFeat + k1] : 0.0f;
      q[j] = pack_bf2(a, c);
    }
    *reinterpret_cast<uint4*>(X + size_t(b >> 7) * 16384 + tc::blk_off(kIn, b & 127, kc * 8)) =
        make_uint4(q[0], q[1], q[2], q[3]);
  }
  if (T) {
    float4 o = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (valid && t) o = make_float4(t[size_t(b) * 3], t[size_t(b) * 3 + 1], t[size_t(b) * 3 + 2], 0.0f);
    reinterpret_cast<float4*>(T)[b] = o;
  }
}

// blockIdx.y = column (54 features, then 3 targets); per-block f64 sums.
__global__ void k_stats(const float* __restrict__ feat, const float* __restrict__ tgt, long long count,
                        double* __restrict__ partials) {
  __shared__ double sh[2][8];
  const int j = blockIdx.y;
  double s = 0.0, q = 0.0;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < count;
       r += (long long)gridDim.x * blockDim.x) {
    const double x = j < kFeat ? double(feat[r * kRawStride + j]) : double(tgt[r * 4 + (j - kFeat)]);
    s += x;
    q += x * x;
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    q += __shfl_xor_sync(0xffffffffu, q, o);
  }
  const int warp = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    sh[0][warp] = s;
    sh[1][warp] = q;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double S = 0.0, Q = 0.0;
    for (int w = 0; w < int(blockDim.x >> 5); ++w) {
      S += sh[0][w];
      Q += sh[1][w];
    }
    partials[(size_t(j) * gridDim.x + blockIdx.x) * 2] = S;
    partials[(size_t(j) * gridDim.x + blockIdx.x) * 2 + 1] = Q;
  }
}

// ---- checks ----------------------------------------------------------------

__global__ void __launch_bounds__(128) k_check(const SurCloth* __restrict__ cloths, const Tile* __restrict__ tiles,
                                               int n_tiles, int parity, float3 gf, float2* __restrict__ tile_out) {
  __shared__ float2 red[4];
  const int t = blockIdx.x;
  if (t >= n_tiles) return;
  const Tile w = tiles[t];
  const SurCloth& c = cloths[w.x];
  const int R = c.rows, C = c.cols, n = R * C;
  const int v = w.y + threadIdx.x;
  const float4* __restrict__ P = c.pos[parity];
  const float4* __restrict__ Vl = c.vel[parity];
  float E = 0.0f, S = 0.0f;
  if (v < n) {
    const int r = v / C, col = v % C;
    const float4 p = P[v], vel = Vl[v];
    // the vertex's owned-strut constants: one row of each of the four planes
    float prm[16];
    {
      const float4 q0 = c.planes[v], q1 = c.planes[size_t(n) + v], q2 = c.planes[2 * size_t(n) + v],
                   q3 = c.planes[3 * size_t(n) + v];
      const float4 q[4] = {q0, q1, q2, q3};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        prm[4 * j] = q[j].x;
        prm[4 * j + 1] = q[j].y;
        prm[4 * j + 2] = q[j].z;
        prm[4 * j + 3] = q[j].w;
      }
    }
    E = 0.5f * p.w * ((vel.x * vel.x + vel.y * vel.y) + vel.z * vel.z) - ((gf.x * p.x + gf.y * p.y) + gf.z * p.z);
#pragma unroll
    for (int kind = 0; kind < 5; ++kind) {
      if (!grid::owned_exists(kind, r, col, R, C)) continue;
      int a = v, b;
      switch (kind) {
        case grid::KH: b = v + 1; break;
        case grid::KV: b = v + C; break;
        case grid::KS: a = v + 1; b = v + C; break;
        case grid::KBH: b = v + 2; break;
        default: b = v + 2 * C; break;
      }
      const float4 pa = a == v ? p : P[a], pb = P[b];
      const float dx = pb.x - pa.x, dy = pb.y - pa.y, dz = pb.z - pa.z;
      const float d = sqrtf((dx * dx + dy * dy) + dz * dz);
      const float k = prm[grid::param_index(kind, 0)];
      const float L = prm[grid::param_index(kind, 2)];
      const float e = d - L;
      E += 0.5f * k * (e * e);
      S = fmaxf(S, fabsf(e / L));
    }
    if (!isfinite(E)) E = __int_as_float(0x7f800000);
    if (!(S == S)) S = __int_as_float(0x7f800000);
  }
  for (int o = 16; o > 0; o >>= 1) {
    E += __shfl_xor_sync(0xffffffffu, E, o);
    S = fmaxf(S, __shfl_xor_sync(0xffffffffu, S, o));
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = make_float2(E, S);
  __syncthreads();
  if (threadIdx.x == 0)
    tile_out[t] = make_float2(((red[0].x + red[1].x) + red[2].x) + red[3].x,
                              fmaxf(fmaxf(red[0].y, red[1].y), fmaxf(red[2].y, red[3].y)));
}

// One block per cloth: sums (and maxima) of its tiles' entries, strided by
// thread, then a fixed-order tree over the block (the same order on every
// run, whatever the number of tiles).
constexpr int kReduceBlock = 256;

__global__ void __launch_bounds__(kReduceBlock) k_check_reduce(const SurCloth* __restrict__ cloths,
                                                               const float2* __restrict__ tile_out,
                                                               float2* __restrict__ cloth_out) {
  __shared__ float2 sh[kReduceBlock];
  const int c = blockIdx.x;
  const SurCloth& cl = cloths[c];
  float E = 0.0f, S = 0.0f;
  for (int k = threadIdx.x; k < cl.ntiles; k += kReduceBlock) {
    const float2 e = tile_out[cl.tile0 + k];
    E += e.x;
    S = fmaxf(S, e.y);
  }
  sh[threadIdx.x] = make_float2(E, S);
  __syncthreads();
#pragma unroll
  for (int h = kReduceBlock / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      const float2 a = sh[threadIdx.x], b = sh[threadIdx.x + h];
      sh[threadIdx.x] = make_float2(a.x + b.x, fmaxf(a.y, b.y));
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) cloth_out[c] = sh[0];
}

__global__ void k_copy_unskipped(const ClothDesc* __restrict__ cloths, int from) {
  const ClothDesc& d = cloths[blockIdx.x];
  if (d.skip) return;
  const int n = d.rows * d.cols;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    d.pos[from ^ 1][i] = d.pos[from][i];
    d.vel[from ^ 1][i] = d.vel[from][i];
  }
}

// ---- device-side decisions of a checked rollout ------------------------------

// Per cloth: the rollout's energy/strain test of the state a coarse step
// produced (cloth_out) against the last accepted energy e_old and the margin
// growth * e_ref + abs, evaluated in double exactly as the host form does.
// Passing cloths accept their new energy; fail[c] is the verdict; n_fail
// counts this step's failures.
__global__ void k_decide(const float2* __restrict__ cloth_out, int n_cloths, float* __restrict__ e_old,
                         const double* __restrict__ e_ref, float growth, float abs_margin, float max_strain,
                         int* __restrict__ fail, int* __restrict__ n_fail) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_cloths) return;
  const float2 o = cloth_out[c];
  const double E0 = e_old[c], E1 = o.x, S1 = o.y;
  const double margin = double(growth) * e_ref[c] + double(abs_margin);
  const bool ok = isfinite(E1) && isfinite(S1) && (E1 <= E0 + margin) && (S1 <= double(max_strain));
  fail[c] = ok ? 0 : 1;
  if (ok)
    e_old[c] = o.x;
  else
    atomicAdd(n_fail, 1);
}

// One thread: the graph's fallback conditional from this step's failure
// count, which is also added to the call's running total.
__global__ void k_set_fallback(cudaGraphConditionalHandle h, const int* __restrict__ n_fail,
                               unsigned long long* __restrict__ total) {
  const int v = *n_fail;
  cudaGraphSetConditional(h, v > 0 ? 1u : 0u);
  *total += (unsigned long long)v;
}

// The batched fallback's cloth table (the batch's, with skip = !fail and no
// carried forces) and, for each failing cloth, where its work items go in the
// compacted list (an exclusive scan in batch order, so the compacted list
// keeps the full list's order); the item count goes to *n_out.  One block.
constexpr int kScanBlock = 1024;

__global__ void __launch_bounds__(kScanBlock) k_fallback_tables(const ClothDesc* __restrict__ desc,
                                                                const int* __restrict__ bmesh, int n_batch,
                                                                const int* __restrict__ fail,
                                                                const int* __restrict__ cnt,
                                                                ClothDesc* __restrict__ fdesc,
                                                                int* __restrict__ dst, int* __restrict__ n_out) {
  __shared__ int warp_sum[kScanBlock / 32];
  __shared__ int carry;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int b0 = 0; b0 < n_batch; b0 += kScanBlock) {
    const int b = b0 + threadIdx.x;
    int m = 0;
    if (b < n_batch) {
      const int f = fail[bmesh[b]];
      ClothDesc d = desc[b];
      d.skip = f ? 0 : 1;
      d.force_in = nullptr;
      fdesc[b] = d;
      m = f ? cnt[b] : 0;
    }
    int x = m;  // inclusive scan within the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_sum[wid] = x;
    __syncthreads();
    if (wid == 0) {
      int w = warp_sum[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      warp_sum[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    const int before = carry + (wid > 0 ? warp_sum[wid - 1] : 0) + x - m;
    if (b < n_batch) dst[b] = before;
    __syncthreads();
    if (threadIdx.x == kScanBlock - 1) carry = before + m;
    __syncthreads();
  }
  if (threadIdx.x == 0) *n_out = carry;
}

// One block per cloth of the batch: a failing cloth's work items
// [off, off + cnt) of the full list, copied to [dst, dst + cnt).
__global__ void k_fallback_items(const int* __restrict__ bmesh, const int* __restrict__ fail,
                                 const int* __restrict__ off, const int* __restrict__ cnt,
                                 const int* __restrict__ dst, const int4* __restrict__ work,
                                 int4* __restrict__ fwork) {
  const int b = blockIdx.x;
  if (!fail[bmesh[b]]) return;
  const int o = off[b], n = cnt[b], d = dst[b];
  for (int i = threadIdx.x; i < n; i += blockDim.x) fwork[d + i] = work[o + i];
}

// After a fallback: the re-checked energy of every cloth that fell back
// becomes its accepted energy.
__global__ void k_accept(const float2* __restrict__ cloth_out, int n_cloths, const int* __restrict__ fail,
                         float* __restrict__ e_old) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n_cloths && fail[c]) e_old[c] = cloth_out[c].x;
}

// SMs of the current device (asked every time: a process may use several devices).
int sm_count() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return sms > 0 ? sms : 1;
}

template <int G, int H>
cudaError_t sur_step_attr() {
  // the attribute is per function and per device: set once on each device used
  static PerDeviceOnce once;
  return once.run(
      [] { return cudaFuncSetAttribute(k_sur_step<G, H>, cudaFuncAttributeMaxDynamicSharedMemorySize, kBlobSmem + G * 32768); });
}

template <int G, int H>
cudaError_t sur_step_g(const SurCloth* cloths, const Tile* tiles, int n_tiles, int parity, const void* blob,
                       const Norm& norm, const StepConsts& consts, int ctas, int* err, cudaStream_t s) {
  const int smem = kBlobSmem + G * 32768;
  const cudaError_t e = sur_step_attr<G, H>();
  if (e != cudaSuccess) return e;
  int grid = (n_tiles + G - 1) / G;
  const int cap = ctas > 0 ? ctas : sm_count();
  if (grid > cap) grid = cap;
  if (grid < 1) return cudaSuccess;
  k_sur_step<G, H><<<grid, 128 * G * H, smem, s>>>(cloths, tiles, n_tiles, parity,
                                                   static_cast<const unsigned char*>(blob), norm, consts, err);
  return cudaGetLastError();
}

}  // namespace

// Threads per vertex row in k_sur_step.
constexpr int kRowThreads = 2;

int sur_step_max_ctas(int) { return sm_count(); }

cudaError_t prime_sur_step(int groups) {
  switch (groups) {
    case 1: return sur_step_attr<1, kRowThreads>();
    case 2: return sur_step_attr<2, kRowThreads>();
    case 3: return sur_step_attr<3, kRowThreads>();
    default: return sur_step_attr<4, kRowThreads>();
  }
}



cudaError_t launch_sur_step(const SurCloth* cloths, const Tile* tiles, int n_tiles, int parity, const void* blob,
                            const Norm& norm, const StepConsts& consts, int groups, int ctas, int* err,
                            cudaStream_t s) {
  if (n_tiles <= 0) return cudaSuccess;
  switch (groups) {
    case 1: return sur_step_g<1, kRowThreads>(cloths, tiles, n_tiles, parity, blob, norm, consts, ctas, err, s);
    case 2: return sur_step_g<2, kRowThreads>(cloths, tiles, n_tiles, parity, blob, norm, consts, ctas, err, s);
    case 3: return sur_step_g<3, kRowThreads>(cloths, tiles, n_tiles, parity, blob, norm, consts, ctas, err, s);
    default: return sur_step_g<4, kRowThreads>(cloths, tiles, n_tiles, parity, blob, norm, consts, ctas, err, s);
  }
}

cudaError_t launch_forward(const void* X, int n_rows, const void* blob, float* Y, int* err, cudaStream_t s) {
  const int n_tiles = n_rows / kTile;
  if (n_tiles <= 0) return cudaSuccess;
  const int smem = kBlobSmem + 32768;
  cudaError_t e = cudaFuncSetAttribute(k_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  const int grid = n_tiles < sm_count() ? n_tiles : sm_count();
  k_forward<<<grid, 128, smem, s>>>(static_cast<const unsigned char*>(X), n_tiles,
                                    static_cast<const unsigned char*>(blob), Y, err);
  return cudaGetLastError();
}

int train_ctas(int n_rows) {
  const int n_tiles = n_rows / kTile;
  return n_tiles < sm_count() ? n_tiles : sm_count();
}

cudaError_t launch_train(const void* X, const float* T, int n_rows, const void* blob, float* partials, int ctas,
                         int* err, cudaStream_t s) {
  const int n_tiles = n_rows / kTile;
  if (n_tiles <= 0 || ctas <= 0) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(k_train, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrSmem);
  if (e != cudaSuccess) return e;
  const float dscale = 2.0f / (3.0f * float(n_rows));
  k_train<<<ctas, kTrThreads, kTrSmem, s>>>(static_cast<const unsigned char*>(X), T, n_tiles,
                                     static_cast<const unsigned char*>(blob), partials, dscale, err);
  return cudaGetLastError();
}

cudaError_t launch_reduce_grad(const float* partials, int ctas, float inv_count, float* grad, float* loss_out,
                               cudaStream_t s) {
  k_reduce_grad<<<(kNumParams + 255) / 256, 256, 0, s>>>(partials, ctas, inv_count, grad, loss_out);
  return cudaGetLastError();
}

cudaError_t launch_adam(const float* partials, int ctas, float* master, float* m, float* v, float lr, float beta1,
                        float beta2, float eps, float c1, float c2, void* blob, float* loss_out, float inv_count,
                        cudaStream_t s) {
  k_adam<<<(kNumParams + 255) / 256, 256, 0, s>>>(partials, ctas, master, m, v, lr, beta1, beta2, eps, c1, c2,
                                                  static_cast<unsigned char*>(blob), loss_out, inv_count);
  return cudaGetLastError();
}

cudaError_t launch_pack_blob(const float* master, void* blob, cudaStream_t s) {
  k_pack_blob<<<(kNumParams + 255) / 256, 256, 0, s>>>(master, static_cast<unsigned char*>(blob));
  return cudaGetLastError();
}

cudaError_t launch_collect_features(const SurCloth* cloths, const Tile* tiles, int n_tiles, int parity, float* feat,
                                    float* tgt, long long cap, cudaStream_t s) {
  if (n_tiles <= 0) return cudaSuccess;
  k_collect_features<<<n_tiles, kTile, 0, s>>>(cloths, tiles, n_tiles, parity, feat, tgt, cap);
  return cudaGetLastError();
}

cudaError_t launch_collect_targets(const SurCloth* cloths, const Tile* tiles, int n_tiles, int parity, float* tgt,
                                   long long cap, cudaStream_t s) {
  if (n_tiles <= 0) return cudaSuccess;
  k_collect_targets<<<n_tiles, kTile, 0, s>>>(cloths, tiles, n_tiles, parity, tgt, cap);
  return cudaGetLastError();
}

cudaError_t launch_features(const SurCloth* cloth, const Tile* tiles, int n_tiles, int parity, float* out,
                            cudaStream_t s) {
  if (n_tiles <= 0) return cudaSuccess;
  k_features<<<n_tiles, kTile, 0, s>>>(cloth, tiles, n_tiles, parity, out);
  return cudaGetLastError();
}

cudaError_t launch_pack_batch(const float* feat, const float* tgt, long long count, uint64_t seed, int n_rows,
                              const Norm& norm, void* X, float* T, cudaStream_t s) {
  if (n_rows <= 0 || count <= 0) return cudaErrorInvalidValue;
  k_pack_batch<<<(n_rows + 127) / 128, 128, 0, s>>>(feat, tgt, count, seed, n_rows, norm,
                                                    static_cast<unsigned char*>(X), T);
  return cudaGetLastError();
}

cudaError_t launch_pack_rows(const float* x, const float* t, int n, int n_pad, void* X, float* T, cudaStream_t s) {
  if (n_pad <= 0) return cudaSuccess;
  k_pack_rows<<<(n_pad + 127) / 128, 128, 0, s>>>(x, t, n, n_pad, static_cast<unsigned char*>(X), T);
  return cudaGetLastError();
}

cudaError_t launch_stats(const float* feat, const float* tgt, long long count, double* partials, int blocks,
                         cudaStream_t s) {
  k_stats<<<dim3(blocks, kFeat + kOut), 256, 0, s>>>(feat, tgt, count, partials);
  return cudaGetLastError();
}

cudaError_t launch_check(const SurCloth* cloths, const Tile* tiles, int n_tiles, int n_cloths, int parity,
                         float3 gforce, float2* tile_out, float2* cloth_out, cudaStream_t s) {
  if (n_tiles <= 0) return cudaSuccess;
  k_check<<<n_tiles, kTile, 0, s>>>(cloths, tiles, n_tiles, parity, gforce, tile_out);
  if (n_cloths > 0) k_check_reduce<<<n_cloths, kReduceBlock, 0, s>>>(cloths, tile_out, cloth_out);
  return cudaGetLastError();
}

cudaError_t launch_decide(const float2* cloth_out, int n_cloths, float* e_old, const double* e_ref, float growth,
                          float abs_margin, float max_strain, int* fail, int* n_fail, cudaStream_t s) {
  if (n_cloths <= 0) return cudaSuccess;
  k_decide<<<(n_cloths + 255) / 256, 256, 0, s>>>(cloth_out, n_cloths, e_old, e_ref, growth, abs_margin, max_strain,
                                                  fail, n_fail);
  return cudaGetLastError();
}

cudaError_t launch_set_fallback(cudaGraphConditionalHandle h, const int* n_fail, unsigned long long* total,
                                cudaStream_t s) {
  k_set_fallback<<<1, 1, 0, s>>>(h, n_fail, total);
  return cudaGetLastError();
}

cudaError_t launch_fallback_tables(const ClothDesc* desc, const int* bmesh, int n_batch, const int* fail,
                                   const int* off, const int* cnt, const int4* work, ClothDesc* fdesc, int* dst,
                                   int4* fwork, int* n_out, cudaStream_t s) {
  if (n_batch <= 0) return cudaSuccess;
  k_fallback_tables<<<1, kScanBlock, 0, s>>>(desc, bmesh, n_batch, fail, cnt, fdesc, dst, n_out);
  k_fallback_items<<<n_batch, 128, 0, s>>>(bmesh, fail, off, cnt, dst, work, fwork);
  return cudaGetLastError();
}

cudaError_t launch_accept(const float2* cloth_out, int n_cloths, const int* fail, float* e_old, cudaStream_t s) {
  if (n_cloths <= 0) return cudaSuccess;
  k_accept<<<(n_cloths + 255) / 256, 256, 0, s>>>(cloth_out, n_cloths, fail, e_old);
  return cudaGetLastError();
}

cudaError_t launch_copy_unskipped(const ClothDesc* cloths, int n_cloths, int from, cudaStream_t s) {
  if (n_cloths <= 0) return cudaSuccess;
  k_copy_unskipped<<<n_cloths, 256, 0, s>>>(cloths, from);
  return cudaGetLastError();
}

}  // namespace sur
}  // namespace fgb
