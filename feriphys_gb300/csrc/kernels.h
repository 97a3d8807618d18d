// Host-visible launch wrappers of the device kernels (no CUDA types beyond
// cudaStream_t/cudaError_t in the signatures).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "step_consts.h"

namespace fgb {

// CSR incidence lists of the general gather (see step_general.cu).
struct GeneralTopo {
  const int* strut_off;
  const int2* strut_inc;
  const float4* strut_kcl;
  const int* face_off;
  const int* face_inc;
  const int4* face_vtx;
  // the compact form (mesh_build.h: CompactTopo): form 1 with 32-bit strut
  // words, 2 with 16-bit ones; form 0 reads the lists above instead
  int form = 0;
  const int* own_off = nullptr;
  const float* sk = nullptr;
  const float* sc = nullptr;
  const float* sl = nullptr;
  const uint32_t* strut_word = nullptr;
  const uint16_t* strut_word16 = nullptr;
  const uint16_t* face_word = nullptr;
};

// Grid (Cloth::new topology) description for the stencil kernel (see
// step_grid.cu).  params holds 4 planes of n float4 (owned-strut constants).
struct GridTopo {
  int rows, cols;
  const float4* params;
  int variant;  // 0: shared-memory tiles, 1: one thread per vertex reading global memory
};

template <class T>
cudaError_t launch_step_general(int n, const void* pos, const void* vel, const void* force_in, void* pos_out,
                                void* vel_out, const GeneralTopo& t, const StepConsts& c, cudaStream_t s);
template <class T>
cudaError_t launch_accumulate(int n, const void* pos, const void* vel, void* force, const GeneralTopo& t,
                              const StepConsts& c, cudaStream_t s);
template <class T>
cudaError_t launch_integrate(int n, int integration, float h, const void* pos, const void* vel, const void* force,
                             void* spos, void* svel, void* sforce, cudaStream_t s);
template <class T>
cudaError_t launch_update(int n, void* pos, void* vel, void* force, const void* spos, const void* svel,
                          const void* sforce, const StepConsts& c, cudaStream_t s);
template <class T>
cudaError_t launch_zero4(int n, void* a, cudaStream_t s);

cudaError_t launch_step_grid(const GridTopo& g, const float4* pos, const float4* vel, const float4* force_in,
                             float4* pos_out, float4* vel_out, const StepConsts& c, cudaStream_t s);

// One cloth of a batch (Cloth::new topology); buffers [parity] are read and
// [parity ^ 1] written by a step.
struct ClothDesc {
  const float4* planes;
  float4* pos[2];
  float4* vel[2];
  const float4* force_in;  // accumulated force carried into the step, or null
  unsigned* flags;         // non-finite flag of this cloth
  int rows, cols;
  float wind[3];
  int skip;  // nonzero: the batched step leaves this cloth untouched (masked fallback steps)
};

// Batch tiles are 32 wide and kDefaultTileH (or another height the
// autotuner picks, batch_tile_height_ok) tall.
constexpr int kDefaultTileH = 8;
constexpr int kBatchTileHeights[3] = {4, 8, 12};
bool batch_tile_height_ok(int th);

// Tiles of one cloth for the batch work list: {cloth, tile x, tile y, interior}.
void batch_tiles(int cloth, int rows, int cols, int th, int* out4 /* may be null */, int* n_ring, int* n_interior);

// The single-cloth tiled kernel's grid: the CTA count for an R x C cloth and
// 32 x th tiles, and (out3 non-null) each CTA's {tile x, tile y, interior}
// in blockIdx order, by the kernel's own mapping.
int grid_tiles(int rows, int cols, int th, int* out3 /* may be null */);

// mode 0: one CTA per work item; mode 1: persistent CTAs pulling items from
// *counter (reset to 0 by the caller before the launch).
// maps: null, or per cloth 4 tensor maps {pos[0], vel[0], pos[1], vel[1]}
// (encode_cloth_maps) for TMA staging of the tiles.  n_work_dev: null, or the
// item count in device memory (mode 1 only; n_work is then its upper bound,
// which sizes the grid).
// th: the tile height the work list and the maps were made for.
cudaError_t launch_step_batched(const ClothDesc* cloths, const int4* work, int n_work, int* counter, int parity,
                                int mode, int persistent_ctas, const StepConsts& c, cudaStream_t s,
                                const void* maps = nullptr, const int* n_work_dev = nullptr,
                                int th = kDefaultTileH);
// Sets the launch attributes of the tiled and batched step kernels (done by
// their launchers on first use; call it before a stream capture).
cudaError_t prime_step_kernels();
// Size of one cloth's tensor maps (4 x 128 bytes) and their encoding; false
// when the driver's encoder is unavailable or an address is misaligned.
constexpr size_t kClothMapBytes = 4 * 128;
bool encode_cloth_maps(const ClothDesc& d, int th, void* out /* kClothMapBytes, 64-byte aligned */);
int batched_ctas_per_sm(int th = kDefaultTileH);

}  // namespace fgb
