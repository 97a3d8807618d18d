// Learned surrogate of the cloth step (an extension with no counterpart in
// the reference): a per-vertex MLP 54 -> 128 -> 128 -> 3 (GELU, bf16
// weights, f32 accumulation on the tensor cores) that predicts the velocity
// change of a grid-cloth vertex over one coarse step of `ratio` fine steps.
//
// Inputs of vertex (r, c) of a Cloth::new grid with rest spacing h, coarse
// step T = ratio * dt, s = T / h (in this order; a missing neighbour gives
// zeros; p0 are the positions the mesh was built from, so the first block is
// the stencil's deformation from its rest shape):
//   0..23   ((p_nb - p) - (p0_nb - p0)) / h   for the 8 neighbours (dr, dc) =
//           (-1,-1) (-1,0) (-1,1) (0,-1) (0,1) (1,-1) (1,0) (1,1)
//   24..47  (v_nb - v) * s        same order
//   48      pinned (1 or 0)
//   49..51  (wind - v) * s
//   52, 53  acos(n_y) / pi, atan2(n_z, n_x) / pi of the unit normal
//           n = (p_right - p_left) x (p_up - p_down) (one-sided at the edges;
//           (0, 0, 1) when degenerate)
// Output: (v(t + T) - v(t)) * s, i.e. the velocity change in spacings per
// coarse step.  Inputs and outputs are standardised by per-feature mean and
// standard deviation taken from the training data.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.h"
#include "step_consts.h"

namespace fgb {
namespace sur {

constexpr int kFeat = 54;     // network inputs
constexpr int kIn = 64;       // padded input width (a multiple of the MMA K)
constexpr int kHid = 128;     // hidden width
constexpr int kOut = 3;       // outputs
constexpr int kOutPad = 16;   // padded output width (the smallest MMA N)
constexpr int kRawStride = 64;  // floats per raw feature row in the dataset ring
constexpr int kTile = 128;    // vertices (rows) per tensor-core tile

// Padded f32 parameter vector: master weights, Adam moments and gradients.
constexpr int kOffW1 = 0;                          // [128][64]
constexpr int kOffB1 = kOffW1 + kHid * kIn;        // [128]
constexpr int kOffW2 = kOffB1 + kHid;              // [128][128]
constexpr int kOffB2 = kOffW2 + kHid * kHid;       // [128]
constexpr int kOffW3 = kOffB2 + kHid;              // [16][128]
constexpr int kOffB3 = kOffW3 + kOutPad * kHid;    // [16]
constexpr int kNumParams = kOffB3 + kOutPad;       // 26896
constexpr int kPartialStride = kNumParams + 16;    // per-CTA gradient partials, then the loss sum
// Unpadded parameter count of the public flat layout:
// W1[128][54], b1[128], W2[128][128], b2[128], W3[3][128], b3[3].
constexpr int kNumParamsFlat = kHid * kFeat + kHid + kHid * kHid + kHid + kOut * kHid + kOut;  // 23939

// Network blob (one bulk copy into shared memory): bf16 weights in the
// blocked layout of tc05.cuh, rows = outputs, then f32 biases.
constexpr int kBlobW1 = 0;                             // 128 x 64 bf16   16384 B
constexpr int kBlobW2 = kBlobW1 + kHid * kIn * 2;      // 128 x 128 bf16  32768 B
constexpr int kBlobW3 = kBlobW2 + kHid * kHid * 2;     // 16 x 128 bf16    4096 B
constexpr int kBlobB1 = kBlobW3 + kOutPad * kHid * 2;  // 128 f32
constexpr int kBlobB2 = kBlobB1 + kHid * 4;            // 128 f32
constexpr int kBlobB3 = kBlobB2 + kHid * 4;            // 16 f32
constexpr int kBlobBytes = kBlobB3 + kOutPad * 4;      // 54336
constexpr int kBlobSmem = 55296;                       // blob region in shared memory (1 KB multiple)

struct Norm {
  float in_mean[kFeat];
  float in_inv_std[kFeat];
  float out_mean[kOut];
  float out_std[kOut];
};

// One grid cloth as the surrogate kernels see it.
// Buffers [parity] are read and [parity ^ 1] written by a coarse step.
struct SurCloth {
  float4* pos[2];
  float4* vel[2];
  const float4* planes;  // owned-strut constants (grid_order.h), for the checks
  const float4* rest;    // positions the mesh was built from (x, y, z, 0)
  unsigned* flags;       // bit 0: a vertex went non-finite
  int rows, cols;
  int tile0, ntiles;     // this cloth's tiles in the work list
  long long vbase;       // first dataset row of this cloth's vertices (collection)
  float inv_h;           // 1 / rest spacing
  float sv;              // T / h
  float inv_sv;          // h / T
  float wind[3];
};

// Work list entry: {cloth, first vertex of the 128-vertex tile}.
using Tile = int2;

// Coarse step of every listed tile: features, MLP on the tensor cores,
// v' = v + dv, p' = p + (v + v') T / 2 (the mean velocity over the step), collision response against the obstacles
// (consts: dt = T), pinned vertices unchanged.  groups = 128-thread groups per
// CTA (2 or 4), ctas = persistent CTAs (0: one per tile group).
cudaError_t launch_sur_step(const SurCloth* cloths, const Tile* tiles, int n_tiles, int parity, const void* blob,
                            const Norm& norm, const StepConsts& consts, int groups, int ctas, int* err,
                            cudaStream_t s);
int sur_step_max_ctas(int groups);

// Network outputs (standardised units, bias included) for standardised
// inputs X (bf16, blocked layout, n_rows a multiple of 128): Y[n][4].
cudaError_t launch_forward(const void* X, int n_rows, const void* blob, float* Y, int* err, cudaStream_t s);

// Fused forward + backward of the mean squared error over n_rows rows (a
// multiple of 128): per-CTA gradient partials [ctas][kPartialStride] (the
// loss sum at kNumParams).  ctas <= min(#SMs, n_rows / 128).
cudaError_t launch_train(const void* X, const float* T, int n_rows, const void* blob, float* partials, int ctas,
                         int* err, cudaStream_t s);
int train_ctas(int n_rows);

// Sum of the partials in CTA order; then either only the gradient (grad !=
// null) or an Adam step of the master weights (m, v moments; c1, c2 the bias
// corrections 1/(1-beta^t)) followed by the blob refresh.  loss_out[0] =
// mean squared error of the batch.
cudaError_t launch_reduce_grad(const float* partials, int ctas, float inv_count, float* grad, float* loss_out,
                               cudaStream_t s);
cudaError_t launch_adam(const float* partials, int ctas, float* master, float* m, float* v, float lr, float beta1,
                        float beta2, float eps, float c1, float c2, void* blob, float* loss_out, float inv_count,
                        cudaStream_t s);
// master (padded f32) -> blob.
cudaError_t launch_pack_blob(const float* master, void* blob, cudaStream_t s);

// Raw features of every listed vertex into ring rows (vbase + v) % cap and
// the vertex's velocity and s into the target slot; targets then become
// (v_new - v_old) * s.
cudaError_t launch_collect_features(const SurCloth* cloths, const Tile* tiles, int n_tiles, int parity, float* feat,
                                    float* tgt, long long cap, cudaStream_t s);
cudaError_t launch_collect_targets(const SurCloth* cloths, const Tile* tiles, int n_tiles, int parity, float* tgt,
                                   long long cap, cudaStream_t s);
// Raw features of one cloth into out[n][54] (row-major f32).
cudaError_t launch_features(const SurCloth* cloth, const Tile* tiles, int n_tiles, int parity, float* out,
                            cudaStream_t s);

// Training batch: n_rows rows drawn from the first `count` ring rows (seeded
// hash), standardised, X as bf16 blocked, T[n][4] f32.
cudaError_t launch_pack_batch(const float* feat, const float* tgt, long long count, uint64_t seed, int n_rows,
                              const Norm& norm, void* X, float* T, cudaStream_t s);
// Standardised host rows (x[n][54], t[n][3] or null) -> X blocked, T[n][4];
// rows n..n_pad-1 are zero.
cudaError_t launch_pack_rows(const float* x, const float* t, int n, int n_pad, void* X, float* T, cudaStream_t s);

// Per-feature sums and sums of squares over ring rows [0, count):
// out[0..53] sum x, [54..107] sum x^2, [108..110] sum t, [111..113] sum t^2
// (f64, per-block partials summed on the host in block order).
cudaError_t launch_stats(const float* feat, const float* tgt, long long count, double* partials, int blocks,
                         cudaStream_t s);

// Energy and maximum strain of each cloth's state in buffers [parity]:
// E = sum (m |v|^2 / 2 - g . p) + sum over struts k (|d| - L)^2 / 2,
// strain = max |(|d| - L) / L|; g is the gravity force of a point.  One entry
// per tile (warp-shuffle sums), then one per cloth (a block sums the cloth's
// tiles in a fixed order): cloth_out[c] = {E, strain}.
cudaError_t launch_check(const SurCloth* cloths, const Tile* tiles, int n_tiles, int n_cloths, int parity,
                         float3 gforce, float2* tile_out, float2* cloth_out, cudaStream_t s);

// For every cloth of a batched-step table whose skip flag is 0: copy its
// state from buffers [from] to [from ^ 1] (the fine-step fallback restores
// the pre-step state before stepping from it).
cudaError_t launch_copy_unskipped(const ClothDesc* cloths, int n_cloths, int from, cudaStream_t s);

// Device-side decisions of a checked rollout (no host round trip per coarse
// step).  launch_decide: per cloth, the energy/strain test of cloth_out
// against e_old and the margin growth * e_ref + abs (in double, as the host
// form), fail[c] = verdict, e_old[c] = E for passing cloths, n_fail += the
// failures.  launch_set_fallback: one thread sets the graph conditional h to
// (*n_fail > 0) and adds *n_fail to *total.  launch_fallback_tables: the
// batched fallback's cloth table (skip = !fail[bmesh[b]], no forces) and the
// failing cloths' work items (cloth b owns items [off[b], off[b] + cnt[b])
// of `work`) compacted in list order into fwork, their count in *n_out
// (dst: n_batch ints of scratch).  launch_accept: e_old[c] = cloth_out[c].x
// for every failing cloth.
cudaError_t launch_decide(const float2* cloth_out, int n_cloths, float* e_old, const double* e_ref, float growth,
                          float abs_margin, float max_strain, int* fail, int* n_fail, cudaStream_t s);
cudaError_t launch_set_fallback(cudaGraphConditionalHandle h, const int* n_fail, unsigned long long* total,
                                cudaStream_t s);
cudaError_t launch_fallback_tables(const ClothDesc* desc, const int* bmesh, int n_batch, const int* fail,
                                   const int* off, const int* cnt, const int4* work, ClothDesc* fdesc, int* dst,
                                   int4* fwork, int* n_out, cudaStream_t s);
cudaError_t launch_accept(const float2* cloth_out, int n_cloths, const int* fail, float* e_old, cudaStream_t s);

// Sets the launch attributes of the coarse-step kernels (call before a
// stream capture that launches them).
cudaError_t prime_sur_step(int groups);

}  // namespace sur
}  // namespace fgb
