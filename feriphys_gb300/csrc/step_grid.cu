// Grid-stencil step for meshes with Cloth::new's topology (cloth.rs:20-113).
//
// The neighbourhood of every vertex is implicit in (row, col): no index
// lists are read.  Strut constants live in 4 float4 planes indexed by the
// owning vertex (grid_order.h).  The force terms are summed in the exact
// order of the reference's scatter loops (strut ids ascending, then face ids
// ascending -- checked on the host against the real ids before this kernel is
// chosen), so the result is bit-identical to the general gather.
#include "grid_order.h"
#include "kernels.h"
#include "physics.cuh"

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

}  // namespace

cudaError_t launch_step_grid(const GridTopo& g, const float4* pos, const float4* vel, const float4* force_in,
                             float4* pos_out, float4* vel_out, const StepConsts& c, cudaStream_t s) {
  const int n = g.rows * g.cols;
  if (n <= 0) return cudaSuccess;
  k_step_grid_v1<<<(n + 255) / 256, 256, 0, s>>>(g.rows, g.cols, g.params, pos, vel, force_in, pos_out, vel_out, c);
  return cudaGetLastError();
}

}  // namespace fgb
