// Internal: the C ABI's handle types and the helpers shared by the C ABI
// translation units (capi.cu, capi_surrogate.cu).  Not part of the public
// interface.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "feriphys_gb300.h"
#include "kernels.h"
#include "mesh_build.h"
#include "devmath.cuh"
#include "step_consts.h"

using fgb::MeshTopo;

// A library-created stream shared by every mesh that issues work on it (all
// meshes of a batched simulation share one); destroyed with its last user.
struct StreamOwner {
  cudaStream_t s = nullptr;
  ~StreamOwner() {
    if (s) cudaStreamDestroy(s);
  }
};

struct fgb_obstacle {
  uint64_t n_vertices = 0;
  uint64_t n_edges = 0;
  std::vector<fgb::ObsFace> faces;  // device layout, computed on the host
};

struct fgb_mesh {
  MeshTopo topo;
  int device = 0;
  int path_req = 0;      // 0 auto, 1 general, 2 grid
  int grid_variant = 0;  // 0 tiled grid kernel, 1 per-vertex grid kernel
  bool plain_csr = false;  // general gather over the plain CSR even when the compact lists exist
  int precision = 32;    // 32 or 64
  int active_path = 0;   // 1 general, 2 grid (valid after topology upload)
  cudaStream_t stream = nullptr;      // the stream all work of this mesh is issued on
  std::shared_ptr<StreamOwner> own;   // library stream (possibly shared with a batch)
  bool external_stream = false;
  float wind[3] = {0, 0, 0};          // per-mesh wind (extension), used when has_wind
  bool has_wind = false;
  float rest_spacing = 0.0f;          // mean horizontal neighbour distance at construction (0: not yet computed)

  // host copy of the state while the device does not hold it (as_state layout)
  std::vector<float> host_pts;
  bool state_on_device = false;
  bool topo_dirty = true;
  bool pins_dirty = true;
  bool csr_ready = false;

  // device state
  void* pos[2] = {nullptr, nullptr};
  void* vel[2] = {nullptr, nullptr};
  int cur = 0;
  void* force = nullptr;
  bool has_force = false;  // force buffer holds the points' accumulated force
  void* spos = nullptr;
  void* svel = nullptr;
  void* sforce = nullptr;
  bool staged = false;
  float* d_io = nullptr;  // as_state staging (10 floats per point; doubles for f64 readback)
  size_t d_io_bytes = 0;
  uint8_t* d_pinned = nullptr;
  unsigned* d_flags = nullptr;

  // general topology
  int* d_strut_off = nullptr;
  int2* d_strut_inc = nullptr;
  float4* d_strut_kcl = nullptr;
  int* d_face_off = nullptr;
  int* d_face_inc = nullptr;
  int4* d_face_vtx = nullptr;
  // its compact form (null when the mesh does not fit it)
  int* d_own_off = nullptr;
  float* d_sk = nullptr;
  float* d_sc = nullptr;
  float* d_sl = nullptr;
  uint32_t* d_strut_word = nullptr;
  uint16_t* d_strut_word16 = nullptr;
  uint16_t* d_face_word = nullptr;
  int compact_form = 0;  // 0 none, 1 32-bit strut words, 2 16-bit strut words
  // grid topology
  float4* d_grid = nullptr;
  float4* d_rest = nullptr;  // construction positions (x, y, z, 0), uploaded for the surrogate's inputs

  size_t elem() const { return precision == 64 ? sizeof(fgb::Dbl4) : sizeof(float4); }
};

struct fgb_sim {
  std::vector<fgb_mesh*> meshes;
  std::vector<fgb_obstacle*> obstacles;
  fgb_config cfg;
  std::vector<fgb::ObsFace> faces;  // flattened obstacle faces (uploaded at the first step)
  fgb::ObsFace* d_faces = nullptr;
  int n_faces = 0;
  bool faces_uploaded = false;
  bool broadphase = true;
  fgb::ObsAccel accel{};  // device broad phase (pointers into d_accel)
  int* d_accel = nullptr;
  // batched stepping of grid meshes (two or more): one kernel per step
  std::vector<fgb_mesh*> batch;           // grid meshes, largest first
  std::vector<fgb::ClothDesc> desc;       // host copy of the device table
  fgb::ClothDesc* d_desc = nullptr;
  size_t d_desc_cap = 0;
  int4* d_work = nullptr;
  int n_work = 0;
  std::vector<int> work_host;             // host copy of the work list (4 ints per item)
  unsigned char* d_maps = nullptr;        // per batch cloth: 4 tensor maps for TMA staging (null: thread staging)
  size_t d_maps_cap = 0;
  int* d_counter = nullptr;
  int parity = 0;
  int mode = -1, ctas = 0;                // launch form chosen by the tuner
  int forced_mode = -1;                   // fgb_sim_set_batch_mode (-1: tuner)
  int tile_h = fgb::kDefaultTileH;        // tile height (rows) chosen by the tuner
  int forced_tile_h = 0;                  // fgb_sim_set_batch_tile (0: tuner)
  int built_tile_h = -1;                  // tile height of the uploaded work list and maps
  bool graphs = true;
  std::map<std::pair<uint64_t, int>, cudaGraphExec_t> graph_cache;
  fgb_config graph_cfg;
  std::shared_ptr<StreamOwner> stream;    // shared with the batch's meshes
  cudaStream_t ext_stream = nullptr;      // caller's stream (fgb_sim_set_stream), if any
};

namespace fgb {
namespace detail {

// Records the message for fgb_last_error and returns code.
int fail(int code, const std::string& msg);
// Device state, pins and topology of a mesh ready for a step.
int ensure_device(fgb_mesh* m);
// Obstacle faces and broad phase uploaded, every mesh ready.
int ensure_sim(fgb_sim* s);
// Step constants for a configuration (dt as given).
StepConsts make_consts(const fgb_config& cfg, const ObsFace* faces, int n_faces, unsigned* flags,
                       const ObsAccel* accel);
// The stream the simulation's batched work runs on (its meshes' stream).
cudaStream_t sim_stream(fgb_sim* s);

}  // namespace detail
}  // namespace fgb
