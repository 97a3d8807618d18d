// C ABI implementation (include/feriphys_gb300.h): handles, device memory,
// streams and kernel launches.  Host-side construction lives in
// mesh_build.cpp; the kernels in step_general.cu / step_grid.cu / state_io.cu.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <set>
#include <string>
#include <utility>
#include <vector>

#include <sys/stat.h>

#include "feriphys_gb300.h"
#include "handles.h"
#include "per_device.h"
#include "kernels.h"
#include "mesh_build.h"
#include "obstacle_accel.h"
#include "physics.cuh"
#include "state_io.h"

namespace {
thread_local std::string g_err;
}  // namespace

int fgb::detail::fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

using fgb::detail::fail;

namespace {

#define FGB_CUDA(call)                                                                              \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess) return fail(FGB_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define FGB_CHECK_RC(expr)   \
  do {                       \
    int rc_ = (expr);        \
    if (rc_ != FGB_OK) return rc_; \
  } while (0)

template <class P>
void dfree(P*& p) {
  if (p) cudaFree(reinterpret_cast<void*>(p));
  p = nullptr;
}

template <class P>
cudaError_t dalloc(P*& p, size_t bytes) {
  dfree(p);
  if (bytes == 0) bytes = 16;
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, bytes);
  p = static_cast<P*>(q);
  return e;
}

bool finite_nonneg(float x) { return std::isfinite(x) && x >= 0.0f; }

}  // namespace

namespace {

void init_host_state(fgb_mesh* m) {
  const uint32_t n = m->topo.n;
  m->host_pts.assign(10 * size_t(n), 0.0f);
  for (uint32_t i = 0; i < n; ++i) {
    float* p = &m->host_pts[10 * size_t(i)];
    p[0] = m->topo.mass_per_vert;
    p[1] = m->topo.pos[3 * size_t(i)];
    p[2] = m->topo.pos[3 * size_t(i) + 1];
    p[3] = m->topo.pos[3 * size_t(i) + 2];
  }
  m->state_on_device = false;
}

int ensure_stream(fgb_mesh* m) {
  if (!m->own) {
    m->own = std::make_shared<StreamOwner>();
    FGB_CUDA(cudaStreamCreateWithFlags(&m->own->s, cudaStreamNonBlocking));
  }
  if (!m->external_stream) m->stream = m->own->s;
  return FGB_OK;
}

// Device address of a pinned (page-locked, mapped) host buffer, or null for
// pageable memory, which is staged through a device buffer instead.
template <class P>
P* mapped_host(P* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
  return static_cast<P*>(a.devicePointer);
}

int ensure_io(fgb_mesh* m, size_t bytes) {
  if (m->d_io_bytes < bytes || !m->d_io) {
    m->d_io_bytes = 0;  // a failed allocation leaves no buffer and no capacity
    FGB_CUDA(dalloc(m->d_io, bytes));
    m->d_io_bytes = bytes;
  }
  return FGB_OK;
}

void free_state(fgb_mesh* m) {
  for (int i = 0; i < 2; ++i) {
    dfree(m->pos[i]);
    dfree(m->vel[i]);
  }
  dfree(m->force);
  dfree(m->spos);
  dfree(m->svel);
  dfree(m->sforce);
  m->has_force = false;
  m->staged = false;
}

void free_topology(fgb_mesh* m) {
  dfree(m->d_strut_off);
  dfree(m->d_strut_inc);
  dfree(m->d_strut_kcl);
  dfree(m->d_face_off);
  dfree(m->d_face_inc);
  dfree(m->d_face_vtx);
  dfree(m->d_own_off);
  dfree(m->d_sk);
  dfree(m->d_sc);
  dfree(m->d_sl);
  dfree(m->d_strut_word);
  dfree(m->d_strut_word16);
  dfree(m->d_face_word);
  m->compact_form = 0;
  dfree(m->d_grid);
  dfree(m->d_rest);
  m->csr_ready = false;
}

// Device state -> host_pts (as_state layout, f32).
int download_state(fgb_mesh* m) {
  if (!m->state_on_device) return FGB_OK;
  const int n = int(m->topo.n);
  FGB_CHECK_RC(ensure_io(m, 10 * sizeof(float) * size_t(n)));
  const void* F = m->has_force ? m->force : nullptr;
  if (m->precision == 64)
    FGB_CUDA((fgb::launch_pack_f32<double>(n, m->pos[m->cur], m->vel[m->cur], F, m->d_io, m->stream)));
  else
    FGB_CUDA((fgb::launch_pack_f32<float>(n, m->pos[m->cur], m->vel[m->cur], F, m->d_io, m->stream)));
  m->host_pts.resize(10 * size_t(n));
  FGB_CUDA(cudaMemcpyAsync(m->host_pts.data(), m->d_io, 10 * sizeof(float) * size_t(n), cudaMemcpyDeviceToHost,
                           m->stream));
  FGB_CUDA(cudaStreamSynchronize(m->stream));
  return FGB_OK;
}

int upload_pins(fgb_mesh* m) {
  const uint32_t n = m->topo.n;
  std::vector<uint8_t> pinned(n, 0);
  for (uint32_t p : m->topo.pins) pinned[p] = 1;
  FGB_CUDA(dalloc(m->d_pinned, n));
  FGB_CUDA(cudaMemcpy(m->d_pinned, pinned.data(), n, cudaMemcpyHostToDevice));
  m->pins_dirty = false;
  return FGB_OK;
}

int alloc_state(fgb_mesh* m) {
  const size_t bytes = m->elem() * size_t(m->topo.n);
  for (int i = 0; i < 2; ++i) {
    if (!m->pos[i]) FGB_CUDA(dalloc(m->pos[i], bytes));
    if (!m->vel[i]) FGB_CUDA(dalloc(m->vel[i], bytes));
  }
  if (!m->d_flags) {
    FGB_CUDA(dalloc(m->d_flags, sizeof(unsigned)));
    FGB_CUDA(cudaMemsetAsync(m->d_flags, 0, sizeof(unsigned), m->stream));
  }
  return FGB_OK;
}

int ensure_force(fgb_mesh* m) {
  if (!m->force) FGB_CUDA(dalloc(m->force, m->elem() * size_t(m->topo.n)));
  if (!m->has_force) {
    FGB_CUDA(cudaMemsetAsync(m->force, 0, m->elem() * size_t(m->topo.n), m->stream));
    m->has_force = true;
  }
  return FGB_OK;
}

// host_pts -> device (pos/vel, and force when any accumulated force is set).
int upload_state(fgb_mesh* m) {
  const int n = int(m->topo.n);
  FGB_CHECK_RC(alloc_state(m));
  bool any_force = false;
  for (int i = 0; i < n && !any_force; ++i) {
    const float* p = &m->host_pts[10 * size_t(i)];
    any_force = p[7] != 0.0f || p[8] != 0.0f || p[9] != 0.0f || std::signbit(p[7]) || std::signbit(p[8]) ||
                std::signbit(p[9]);
  }
  FGB_CHECK_RC(ensure_io(m, 10 * sizeof(float) * size_t(n)));
  FGB_CUDA(cudaMemcpyAsync(m->d_io, m->host_pts.data(), 10 * sizeof(float) * size_t(n), cudaMemcpyHostToDevice,
                           m->stream));
  void* F = nullptr;
  if (any_force) {
    if (!m->force) FGB_CUDA(dalloc(m->force, m->elem() * size_t(n)));
    F = m->force;
  }
  m->cur = 0;
  if (m->precision == 64)
    FGB_CUDA((fgb::launch_unpack<double>(n, m->d_io, m->d_pinned, m->pos[0], m->vel[0], F, m->stream)));
  else
    FGB_CUDA((fgb::launch_unpack<float>(n, m->d_io, m->d_pinned, m->pos[0], m->vel[0], F, m->stream)));
  FGB_CUDA(cudaStreamSynchronize(m->stream));
  m->has_force = any_force;
  m->staged = false;
  m->state_on_device = true;
  return FGB_OK;
}

int ensure_csr(fgb_mesh* m) {
  if (m->csr_ready) return FGB_OK;
  fgb::CsrTopo t;
  std::string err;
  FGB_CHECK_RC(fgb::build_csr(m->topo, t, err) ? fail(FGB_EINVAL, err) : FGB_OK);
  FGB_CUDA(dalloc(m->d_strut_off, t.strut_off.size() * sizeof(int)));
  FGB_CUDA(dalloc(m->d_strut_inc, t.strut_inc.size() * sizeof(int)));
  FGB_CUDA(dalloc(m->d_strut_kcl, t.strut_kcl.size() * sizeof(float)));
  FGB_CUDA(dalloc(m->d_face_off, t.face_off.size() * sizeof(int)));
  FGB_CUDA(dalloc(m->d_face_inc, t.face_inc.size() * sizeof(int)));
  FGB_CUDA(dalloc(m->d_face_vtx, t.face_vtx.size() * sizeof(int)));
  FGB_CUDA(cudaMemcpy(m->d_strut_off, t.strut_off.data(), t.strut_off.size() * sizeof(int), cudaMemcpyHostToDevice));
  FGB_CUDA(cudaMemcpy(m->d_strut_inc, t.strut_inc.data(), t.strut_inc.size() * sizeof(int), cudaMemcpyHostToDevice));
  FGB_CUDA(cudaMemcpy(m->d_strut_kcl, t.strut_kcl.data(), t.strut_kcl.size() * sizeof(float),
                      cudaMemcpyHostToDevice));
  FGB_CUDA(cudaMemcpy(m->d_face_off, t.face_off.data(), t.face_off.size() * sizeof(int), cudaMemcpyHostToDevice));
  FGB_CUDA(cudaMemcpy(m->d_face_inc, t.face_inc.data(), t.face_inc.size() * sizeof(int), cudaMemcpyHostToDevice));
  FGB_CUDA(cudaMemcpy(m->d_face_vtx, t.face_vtx.data(), t.face_vtx.size() * sizeof(int), cudaMemcpyHostToDevice));
  fgb::CompactTopo ct;
  if (fgb::build_compact(m->topo, t, ct)) {
    auto up = [&](auto*& d, const auto& v) -> cudaError_t {
      const size_t bytes = v.size() * sizeof(v[0]);
      cudaError_t e = dalloc(d, bytes);
      if (e == cudaSuccess && bytes) e = cudaMemcpy(d, v.data(), bytes, cudaMemcpyHostToDevice);
      return e;
    };
    FGB_CUDA(up(m->d_own_off, ct.own_off));
    FGB_CUDA(up(m->d_sk, ct.sk));
    FGB_CUDA(up(m->d_sc, ct.sc));
    FGB_CUDA(up(m->d_sl, ct.sl));
    FGB_CUDA(ct.strut_word16.size() || ct.strut_word.empty() ? up(m->d_strut_word16, ct.strut_word16)
                                                              : up(m->d_strut_word, ct.strut_word));
    FGB_CUDA(up(m->d_face_word, ct.face_word));
    m->compact_form = ct.strut_word.empty() ? 2 : 1;
  }
  m->csr_ready = true;
  return FGB_OK;
}

// The general gather's topology: the compact lists when the mesh has them
// (and the caller has not asked for the plain CSR), else the plain CSR.
fgb::GeneralTopo general_topo(const fgb_mesh* m) {
  fgb::GeneralTopo t{m->d_strut_off, m->d_strut_inc, m->d_strut_kcl, m->d_face_off, m->d_face_inc, m->d_face_vtx};
  if (m->compact_form && !m->plain_csr) {
    t.form = m->compact_form;
    t.own_off = m->d_own_off;
    t.sk = m->d_sk;
    t.sc = m->d_sc;
    t.sl = m->d_sl;
    t.strut_word = m->d_strut_word;
    t.strut_word16 = m->d_strut_word16;
    t.face_word = m->d_face_word;
  }
  return t;
}

// Path choice (host only): 2 = grid kernel, 1 = general gather.
int decide_path(fgb_mesh* m, int* path) {
  const bool grid_ok = m->precision == 32 && m->topo.rows > 0 && fgb::grid_layout_ok(m->topo);
  if (m->path_req == 2 && !grid_ok)
    return fail(FGB_ESTATE, "grid path requested but the mesh is not a Cloth::new grid (or precision is f64)");
  *path = (m->path_req == 1 || !grid_ok) ? 1 : 2;
  return FGB_OK;
}

// Topology upload.
int ensure_topology(fgb_mesh* m) {
  if (!m->topo_dirty) return FGB_OK;
  free_topology(m);
  FGB_CHECK_RC(decide_path(m, &m->active_path));
  if (m->active_path == 2) {
    std::vector<float> planes;
    fgb::build_grid_params(m->topo, planes);
    FGB_CUDA(dalloc(m->d_grid, planes.size() * sizeof(float)));
    FGB_CUDA(cudaMemcpy(m->d_grid, planes.data(), planes.size() * sizeof(float), cudaMemcpyHostToDevice));
  } else {
    FGB_CHECK_RC(ensure_csr(m));
  }
  m->topo_dirty = false;
  return FGB_OK;
}

int ensure_device(fgb_mesh* m) {
  FGB_CUDA(cudaSetDevice(m->device));
  FGB_CHECK_RC(ensure_stream(m));
  if (m->pins_dirty) {
    if (m->state_on_device) {
      FGB_CHECK_RC(download_state(m));
      m->state_on_device = false;
    }
    FGB_CHECK_RC(upload_pins(m));
  }
  FGB_CHECK_RC(ensure_topology(m));
  if (!m->state_on_device) FGB_CHECK_RC(upload_state(m));
  return FGB_OK;
}

fgb::StepConsts make_consts(const fgb_config& cfg, const fgb::ObsFace* faces, int n_faces, unsigned* flags,
                            const fgb::ObsAccel* accel = nullptr) {
  fgb::StepConsts c;
  std::memset(&c, 0, sizeof(c));
  if (accel) c.accel = *accel;
  c.integration = cfg.integration;
  c.dt = cfg.dt;
  c.dt_duration = fgb::duration_roundtrip(cfg.dt);
  for (int i = 0; i < 3; ++i) {
    c.force0[i] = 0.0f + cfg.gravity[i];
    c.wind[i] = cfg.wind[i];
  }
  c.neg_drag = -1.0f * cfg.drag_coefficient;
  c.neg_lift = -1.0f * cfg.lift_coefficient;
  c.restitution = cfg.coefficient_of_restitution;
  c.friction = cfg.coefficient_of_friction;
  c.one = 1.0f;
  c.n_obstacle_faces = n_faces;
  c.obstacle_faces = faces;
  c.flags = flags;
  return c;
}

int check_config(const fgb_config* cfg) {
  if (!cfg) return fail(FGB_EINVAL, "null config");
  if (cfg->integration != FGB_EULER && cfg->integration != FGB_RK4) return fail(FGB_EINVAL, "bad integration");
  // Duration::from_secs_f32 panics on negative, NaN or overflowing input.
  if (!finite_nonneg(cfg->dt) || cfg->dt > 1.0e9f) return fail(FGB_EINVAL, "dt must be finite, >= 0 and < 1e9 s");
  return FGB_OK;
}

// One fused Simulation::step of one mesh.
int step_mesh(fgb_mesh* m, const fgb::StepConsts& c) {
  const int n = int(m->topo.n);
  const int nxt = m->cur ^ 1;
  const void* F = m->has_force ? m->force : nullptr;
  if (m->active_path == 2) {
    fgb::GridTopo g{int(m->topo.rows), int(m->topo.cols), m->d_grid, m->grid_variant};
    FGB_CUDA(fgb::launch_step_grid(g, static_cast<const float4*>(m->pos[m->cur]),
                                   static_cast<const float4*>(m->vel[m->cur]), static_cast<const float4*>(F),
                                   static_cast<float4*>(m->pos[nxt]), static_cast<float4*>(m->vel[nxt]), c,
                                   m->stream));
  } else {
    const fgb::GeneralTopo t = general_topo(m);
    if (m->precision == 64)
      FGB_CUDA(fgb::launch_step_general<double>(n, m->pos[m->cur], m->vel[m->cur], F, m->pos[nxt], m->vel[nxt], t,
                                                c, m->stream));
    else
      FGB_CUDA(fgb::launch_step_general<float>(n, m->pos[m->cur], m->vel[m->cur], F, m->pos[nxt], m->vel[nxt], t,
                                               c, m->stream));
  }
  m->cur = nxt;
  m->has_force = false;  // clear_forces
  m->staged = false;
  return FGB_OK;
}

cudaStream_t batch_stream(const fgb_sim* s) { return s->ext_stream ? s->ext_stream : s->stream->s; }

void drop_graphs(fgb_sim* s) {
  for (auto& kv : s->graph_cache) cudaGraphExecDestroy(kv.second);
  s->graph_cache.clear();
}

// Grid meshes stepped together (two or more): largest first, one shared
// stream, buffers aligned to the simulation's parity, descriptor table and
// work list uploaded when they change.
int prepare_batch(fgb_sim* s) {
  std::vector<fgb_mesh*> grid;
  for (fgb_mesh* m : s->meshes)
    if (m->active_path == 2 && m->grid_variant == 0 && m->precision == 32) grid.push_back(m);
  if (grid.size() < 2) {
    s->batch.clear();
    return FGB_OK;
  }
  std::stable_sort(grid.begin(), grid.end(), [](const fgb_mesh* a, const fgb_mesh* b) { return a->topo.n > b->topo.n; });
  if (!s->stream) s->stream = grid[0]->own;
  const cudaStream_t bs = batch_stream(s);
  for (fgb_mesh* m : grid) {
    if (m->stream != bs) {
      if (m->stream) FGB_CUDA(cudaStreamSynchronize(m->stream));
      if (s->ext_stream) {
        m->external_stream = true;
      } else {
        m->own = s->stream;
        m->external_stream = false;
      }
      m->stream = bs;
    }
    if (m->cur != s->parity) {
      std::swap(m->pos[0], m->pos[1]);
      std::swap(m->vel[0], m->vel[1]);
      m->cur = s->parity;
    }
  }
  const bool membership = grid != s->batch;
  const bool reshape = s->built_tile_h != s->tile_h;
  std::vector<fgb::ClothDesc> desc(grid.size());
  for (size_t i = 0; i < grid.size(); ++i) {
    fgb_mesh* m = grid[i];
    fgb::ClothDesc& d = desc[i];
    std::memset(&d, 0, sizeof(d));
    d.planes = m->d_grid;
    for (int k = 0; k < 2; ++k) {
      d.pos[k] = static_cast<float4*>(m->pos[k]);
      d.vel[k] = static_cast<float4*>(m->vel[k]);
    }
    d.force_in = m->has_force ? static_cast<const float4*>(m->force) : nullptr;
    d.flags = m->d_flags;
    d.rows = int(m->topo.rows);
    d.cols = int(m->topo.cols);
    for (int k = 0; k < 3; ++k) d.wind[k] = m->has_wind ? m->wind[k] : s->cfg.wind[k];
  }
  if (membership || reshape) {  // the work list of s->tile_h-row tiles
    std::vector<int> work;
    for (size_t i = 0; i < grid.size(); ++i) {
      int nr, ni;
      fgb::batch_tiles(int(i), int(grid[i]->topo.rows), int(grid[i]->topo.cols), s->tile_h, nullptr, &nr, &ni);
      const size_t at = work.size();
      work.resize(at + 4 * size_t(nr + ni));
      fgb::batch_tiles(int(i), int(grid[i]->topo.rows), int(grid[i]->topo.cols), s->tile_h, work.data() + at, &nr,
                       &ni);
    }
    drop_graphs(s);  // before the buffers the graphs launch on are replaced
    s->n_work = 0;
    FGB_CUDA(dalloc(s->d_work, work.size() * sizeof(int)));
    FGB_CUDA(cudaMemcpy(s->d_work, work.data(), work.size() * sizeof(int), cudaMemcpyHostToDevice));
    s->n_work = int(work.size() / 4);
    s->work_host = work;
    if (!s->d_counter) FGB_CUDA(dalloc(s->d_counter, sizeof(int)));
    if (membership) s->mode = -1;
  }
  if (membership || reshape || desc.size() != s->desc.size() ||
      std::memcmp(desc.data(), s->desc.data(), desc.size() * sizeof(fgb::ClothDesc)) != 0) {
    if (s->d_desc_cap < desc.size() || !s->d_desc) {
      drop_graphs(s);
      s->d_desc_cap = 0;
      FGB_CUDA(dalloc(s->d_desc, desc.size() * sizeof(fgb::ClothDesc)));
      s->d_desc_cap = desc.size();
    }
    FGB_CUDA(cudaMemcpyAsync(s->d_desc, desc.data(), desc.size() * sizeof(fgb::ClothDesc), cudaMemcpyHostToDevice,
                             bs));
    // TMA staging maps for every cloth's buffers (all or none)
    std::vector<unsigned char> maps(desc.size() * fgb::kClothMapBytes + 64);
    unsigned char* mp = maps.data() + ((64 - (reinterpret_cast<uintptr_t>(maps.data()) & 63)) & 63);
    bool maps_ok = true;
    for (size_t i = 0; i < desc.size() && maps_ok; ++i)
      maps_ok = fgb::encode_cloth_maps(desc[i], s->tile_h, mp + i * fgb::kClothMapBytes);
    if (maps_ok) {
      if (s->d_maps_cap < desc.size() || !s->d_maps) {
        drop_graphs(s);
        s->d_maps_cap = 0;
        FGB_CUDA(dalloc(s->d_maps, desc.size() * fgb::kClothMapBytes));
        s->d_maps_cap = desc.size();
      }
      FGB_CUDA(cudaMemcpyAsync(s->d_maps, mp, desc.size() * fgb::kClothMapBytes, cudaMemcpyHostToDevice, bs));
    } else {
      dfree(s->d_maps);
      s->d_maps_cap = 0;
      drop_graphs(s);
    }
    FGB_CUDA(cudaStreamSynchronize(bs));
    s->desc = std::move(desc);
  }
  s->built_tile_h = s->tile_h;
  s->batch = std::move(grid);
  return FGB_OK;
}

int batch_launch(fgb_sim* s, int parity, int mode, int ctas) {
  cudaStream_t st = batch_stream(s);
  FGB_CUDA(cudaMemsetAsync(s->d_counter, 0, sizeof(int), st));
  FGB_CUDA(fgb::launch_step_batched(s->d_desc, s->d_work, s->n_work, s->d_counter, parity, mode, ctas,
                                    make_consts(s->cfg, s->d_faces, s->n_faces, nullptr, &s->accel), st, s->d_maps,
                                    nullptr, s->tile_h));
  return FGB_OK;
}

// Autotuner: times every tile height (32 x 4, 32 x 8, 32 x 12 vertex tiles,
// each with its own block size) and launch form (one CTA per tile, or
// persistent CTAs at the occupancy the tile allows) on this batch -- launches
// that read the current buffers and write the other ones, so the state is
// untouched -- and caches the winner per GPU and batch in a text file
// ($FGB_AUTOTUNE_CACHE, default ~/.cache/feriphys_gb300/autotune.txt).
std::string tune_cache_path() {
  if (const char* p = std::getenv("FGB_AUTOTUNE_CACHE")) return p;
  const char* home = std::getenv("HOME");
  return std::string(home ? home : "/tmp") + "/.cache/feriphys_gb300/autotune.txt";
}

int use_launch_form(fgb_sim* s, int tile_h, int mode, int sms) {
  if (s->tile_h != tile_h) {
    s->tile_h = tile_h;
    FGB_CHECK_RC(prepare_batch(s));  // work list and maps for this tile height
  }
  s->mode = mode;
  s->ctas = fgb::batched_ctas_per_sm(tile_h) * sms;
  return FGB_OK;
}

int tune_batch(fgb_sim* s) {
  int dev = 0;
  FGB_CUDA(cudaGetDevice(&dev));
  cudaDeviceProp prop;
  FGB_CUDA(cudaGetDeviceProperties(&prop, dev));
  const int sms = prop.multiProcessorCount;
  std::vector<int> heights, modes;
  if (s->forced_tile_h > 0) heights.push_back(s->forced_tile_h);
  else heights.assign(std::begin(fgb::kBatchTileHeights), std::end(fgb::kBatchTileHeights));
  if (s->forced_mode >= 0) modes.push_back(s->forced_mode);
  else modes = {0, 1};
  if (heights.size() == 1 && modes.size() == 1) return use_launch_form(s, heights[0], modes[0], sms);
  size_t verts = 0;
  for (const fgb_mesh* m : s->batch) verts += m->topo.n;
  int vb = 0, cb = 0;
  while ((size_t(1) << vb) < verts) ++vb;
  while ((size_t(1) << cb) < s->batch.size()) ++cb;
  char key[512];
  std::snprintf(key, sizeof(key), "batched %s sms=%d cloths=2^%d vertices=2^%d heights=%zu modes=%zu", prop.name, sms,
                cb, vb, heights.size(), modes.size());
  for (char* c = key; *c; ++c)
    if (*c == '\n') *c = ' ';
  const std::string path = tune_cache_path();
  if (FILE* f = std::fopen(path.c_str(), "r")) {
    char line[600];
    int mode = -1, th = 0;
    while (std::fgets(line, sizeof(line), f)) {
      int m = -1, t = 0;
      const char* sep = std::strstr(line, " -> ");
      if (!sep || std::string(line, sep - line) != key) continue;
      if (std::sscanf(sep + 4, "mode=%d tile_h=%d", &m, &t) == 2 && (m == 0 || m == 1) &&
          fgb::batch_tile_height_ok(t) && std::find(heights.begin(), heights.end(), t) != heights.end() &&
          std::find(modes.begin(), modes.end(), m) != modes.end()) {
        mode = m;
        th = t;
      }
    }
    std::fclose(f);
    if (mode >= 0) return use_launch_form(s, th, mode, sms);
  }
  float best = 1e30f;
  int best_mode = modes[0], best_h = heights[0];
  cudaEvent_t a, b;
  FGB_CUDA(cudaEventCreate(&a));
  if (const cudaError_t e = cudaEventCreate(&b); e != cudaSuccess) {
    cudaEventDestroy(a);
    return fail(FGB_ECUDA, std::string("cudaEventCreate: ") + cudaGetErrorString(e));
  }
  int rc = FGB_OK;
  for (int th : heights) {
    for (int mode : modes) {
      if ((rc = use_launch_form(s, th, mode, sms)) != FGB_OK) break;
      if ((rc = batch_launch(s, s->parity, mode, s->ctas)) != FGB_OK) break;  // warm-up
      cudaEventRecord(a, batch_stream(s));
      for (int r = 0; r < 5 && rc == FGB_OK; ++r) rc = batch_launch(s, s->parity, mode, s->ctas);
      cudaEventRecord(b, batch_stream(s));
      float ms = 0.0f;
      cudaError_t e = cudaEventSynchronize(b);
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
      if (rc == FGB_OK && e != cudaSuccess) rc = fail(FGB_ECUDA, cudaGetErrorString(e));
      if (rc != FGB_OK) break;
      if (ms < best) {
        best = ms;
        best_mode = mode;
        best_h = th;
      }
    }
    if (rc != FGB_OK) break;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc != FGB_OK) return rc;
  FGB_CHECK_RC(use_launch_form(s, best_h, best_mode, sms));
  const std::string dir = path.substr(0, path.rfind('/'));
  // create the cache directory (best effort) and append the result
  for (size_t i = 1; i <= dir.size(); ++i)
    if (i == dir.size() || dir[i] == '/') {
      const std::string sub = dir.substr(0, i);
      mkdir(sub.c_str(), 0755);
    }
  if (FILE* f = std::fopen(path.c_str(), "a")) {
    std::fprintf(f, "%s -> mode=%d tile_h=%d ctas_per_sm=%d time_ms=%.4f\n", key, best_mode, best_h,
                 s->ctas / sms, best / 5.0f);
    std::fclose(f);
  }
  return FGB_OK;
}

int batched_steps(fgb_sim* s, uint64_t n) {
  cudaStream_t st = batch_stream(s);
  if (n == 0) return FGB_OK;
  bool forces = false;
  for (fgb_mesh* m : s->batch) forces = forces || m->has_force;
  if (forces) {  // the first step carries accumulated forces: run it directly
    if (s->mode < 0) FGB_CHECK_RC(tune_batch(s));
    FGB_CHECK_RC(batch_launch(s, s->parity, s->mode, s->ctas));
    s->parity ^= 1;
    for (fgb_mesh* m : s->batch) {
      m->cur = s->parity;
      m->has_force = false;
      m->staged = false;
    }
    FGB_CHECK_RC(prepare_batch(s));
    --n;
    if (n == 0) return FGB_OK;
  }
  if (s->mode < 0) FGB_CHECK_RC(tune_batch(s));
  if (std::memcmp(&s->graph_cfg, &s->cfg, sizeof(fgb_config)) != 0) {
    drop_graphs(s);
    s->graph_cfg = s->cfg;
  }
  if (s->graphs && n >= 2) {
    const auto key = std::make_pair(uint64_t(n), s->parity | (s->accel.enabled << 1));
    auto it = s->graph_cache.find(key);
    if (it == s->graph_cache.end()) {
      cudaGraph_t g;
      FGB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      int rc = FGB_OK;
      for (uint64_t k = 0; k < n && rc == FGB_OK; ++k) rc = batch_launch(s, s->parity ^ int(k & 1), s->mode, s->ctas);
      const cudaError_t e = cudaStreamEndCapture(st, &g);
      if (rc != FGB_OK) return rc;
      FGB_CUDA(e);
      cudaGraphExec_t exec;
      const cudaError_t ei = cudaGraphInstantiate(&exec, g, 0);
      cudaGraphDestroy(g);
      FGB_CUDA(ei);
      it = s->graph_cache.emplace(key, exec).first;
    }
    FGB_CUDA(cudaGraphLaunch(it->second, st));
  } else {
    for (uint64_t k = 0; k < n; ++k) FGB_CHECK_RC(batch_launch(s, s->parity ^ int(k & 1), s->mode, s->ctas));
  }
  s->parity ^= int(n & 1);
  for (fgb_mesh* m : s->batch) {
    m->cur = s->parity;
    m->has_force = false;
    m->staged = false;
  }
  return FGB_OK;
}

int make_obstacle_faces(fgb_obstacle* const* obs, uint64_t nobs, std::vector<fgb::ObsFace>& out) {
  out.clear();
  for (uint64_t i = 0; i < nobs; ++i) {
    if (!obs[i]) return fail(FGB_EINVAL, "null obstacle");
    out.insert(out.end(), obs[i]->faces.begin(), obs[i]->faces.end());
  }
  if (out.size() > 0x7fffffffull) return fail(FGB_EINVAL, "too many obstacle faces");
  return FGB_OK;
}

}  // namespace

namespace {

// Obstacle faces and their broad phase on the device (once per simulation).
int upload_faces(fgb_sim* s) {
  if (!s->faces_uploaded) {
    if (!s->faces.empty()) {
      FGB_CUDA(dalloc(s->d_faces, s->faces.size() * sizeof(fgb::ObsFace)));
      FGB_CUDA(cudaMemcpy(s->d_faces, s->faces.data(), s->faces.size() * sizeof(fgb::ObsFace),
                          cudaMemcpyHostToDevice));
      std::vector<int> first, count;
      int base = 0;
      for (fgb_obstacle* o : s->obstacles) {
        first.push_back(base);
        count.push_back(int(o->faces.size()));
        base += int(o->faces.size());
      }
      fgb::AccelHost a;
      fgb::build_obstacle_accel(s->faces, first, count, a);
      const size_t n_off = a.cell_off.size(), n_cf = a.cell_faces.size(), n_al = a.always.size();
      const size_t n_grid_ints = a.grids.size() * sizeof(fgb::ObsGrid3) / sizeof(int);
      FGB_CUDA(dalloc(s->d_accel, (n_off + n_cf + n_al + n_grid_ints + 4) * sizeof(int)));
      FGB_CUDA(cudaMemcpy(s->d_accel, a.cell_off.data(), n_off * sizeof(int), cudaMemcpyHostToDevice));
      FGB_CUDA(cudaMemcpy(s->d_accel + n_off, a.cell_faces.data(), n_cf * sizeof(int), cudaMemcpyHostToDevice));
      FGB_CUDA(cudaMemcpy(s->d_accel + n_off + n_cf, a.always.data(), n_al * sizeof(int), cudaMemcpyHostToDevice));
      // grid descriptors last, 16-byte aligned
      const size_t gofs = (n_off + n_cf + n_al + 3) & ~size_t(3);
      FGB_CUDA(cudaMemcpy(s->d_accel + gofs, a.grids.data(), a.grids.size() * sizeof(fgb::ObsGrid3),
                          cudaMemcpyHostToDevice));
      s->accel.cell_off = s->d_accel;
      s->accel.cell_faces = s->d_accel + n_off;
      s->accel.always = s->d_accel + n_off + n_cf;
      s->accel.grids = reinterpret_cast<const fgb::ObsGrid3*>(s->d_accel + gofs);
      s->accel.n_grids = int(a.grids.size());
    }
    s->faces_uploaded = true;
  }
  s->accel.enabled = (s->broadphase && s->d_accel) ? 1 : 0;
  return FGB_OK;
}

}  // namespace

extern "C" {

const char* fgb_last_error(void) { return g_err.c_str(); }

int fgb_config_default(fgb_config* out) {
  if (!out) return fail(FGB_EINVAL, "null out");
  std::memset(out, 0, sizeof(*out));
  out->integration = FGB_RK4;
  out->dt = fgb::duration_roundtrip(0.001f);  // Duration::from_millis(1).as_secs_f32()
  out->gravity[1] = -10.0f;
  out->lift_coefficient = 1.0f;
  out->drag_coefficient = 1.0f;
  out->coefficient_of_restitution = 0.95f;
  out->coefficient_of_friction = 0.3f;
  return FGB_OK;
}

static int finish_new_mesh(MeshTopo&& topo, fgb_mesh** out) {
  fgb_mesh* m = new (std::nothrow) fgb_mesh();
  if (!m) return fail(FGB_ENOMEM, "out of host memory");
  m->topo = std::move(topo);
  cudaGetDevice(&m->device);
  init_host_state(m);
  *out = m;
  return FGB_OK;
}

int fgb_mesh_new(const float* positions, uint64_t n_vertices, const uint32_t* indices, uint64_t n_indices,
                 float mass, float default_stiffness, float default_damping, const fgb_spring_override* overrides,
                 uint64_t n_overrides, fgb_mesh** out) {
  if (!out) return fail(FGB_EINVAL, "null out");
  *out = nullptr;
  std::vector<fgb::Override> ov(n_overrides);
  for (uint64_t i = 0; i < n_overrides; ++i)
    ov[i] = fgb::Override{overrides[i].a, overrides[i].b, overrides[i].stiffness, overrides[i].damping};
  MeshTopo topo;
  std::string err;
  try {
    const int rc = fgb::build_springy(positions, n_vertices, indices, n_indices, mass, default_stiffness,
                                      default_damping, ov.data(), n_overrides, topo, err);
    if (rc) return fail(rc, err);
  } catch (const std::bad_alloc&) {
    return fail(FGB_ENOMEM, "out of host memory");
  }
  return finish_new_mesh(std::move(topo), out);
}

int fgb_mesh_new_device(const float* positions, uint64_t n_vertices, const uint32_t* indices, uint64_t n_indices,
                        float mass, float default_stiffness, float default_damping,
                        const fgb_spring_override* overrides, uint64_t n_overrides, fgb_mesh** out) {
  if (!out) return fail(FGB_EINVAL, "null out");
  *out = nullptr;
  std::vector<fgb::Override> ov(n_overrides);
  for (uint64_t i = 0; i < n_overrides; ++i)
    ov[i] = fgb::Override{overrides[i].a, overrides[i].b, overrides[i].stiffness, overrides[i].damping};
  MeshTopo topo;
  std::string err;
  try {
    const int rc = fgb::build_springy_device(positions, n_vertices, indices, n_indices, mass, default_stiffness,
                                             default_damping, ov.data(), n_overrides, topo, err);
    if (rc) return fail(rc, err);
  } catch (const std::bad_alloc&) {
    return fail(FGB_ENOMEM, "out of host memory");
  }
  return finish_new_mesh(std::move(topo), out);
}

int fgb_cloth_new(uint64_t rows, uint64_t cols, float spacing, const float position[3], float point_mass,
                  float tensile_stiffness, float tensile_damping, float shear_stiffness, float shear_damping,
                  float binding_stiffness, float binding_damping, const uint32_t* pinned, uint64_t n_pinned,
                  fgb_mesh** out) {
  if (!out) return fail(FGB_EINVAL, "null out");
  *out = nullptr;
  MeshTopo topo;
  std::string err;
  try {
    const int rc = fgb::build_cloth(rows, cols, spacing, position, point_mass, tensile_stiffness, tensile_damping,
                                    shear_stiffness, shear_damping, binding_stiffness, binding_damping, pinned,
                                    n_pinned, topo, err);
    if (rc) return fail(rc, err);
  } catch (const std::bad_alloc&) {
    return fail(FGB_ENOMEM, "out of host memory");
  }
  return finish_new_mesh(std::move(topo), out);
}

int fgb_mesh_add_strut(fgb_mesh* m, uint32_t a, uint32_t b, float stiffness, float damping) {
  return fgb_mesh_add_struts(m, &a, &b, &stiffness, &damping, 1);
}

int fgb_mesh_add_struts(fgb_mesh* m, const uint32_t* a, const uint32_t* b, const float* stiffness,
                        const float* damping, uint64_t n) {
  if (!m) return fail(FGB_EINVAL, "null mesh");
  if (n && (!a || !b || !stiffness || !damping)) return fail(FGB_EINVAL, "null buffer");
  // The rest length uses the points' current positions (springy_mesh.rs:407-408).
  FGB_CHECK_RC(download_state(m));
  std::string err;
  for (uint64_t i = 0; i < n; ++i) {
    const int rc = fgb::add_strut(m->topo, a[i], b[i], stiffness[i], damping[i], m->host_pts.data() + 1, 10, err);
    if (rc) {
      m->state_on_device = false;
      m->topo_dirty = true;
      return fail(rc, err);
    }
  }
  m->state_on_device = false;  // host_pts is current; re-upload with the new topology
  m->topo_dirty = true;
  return FGB_OK;
}

int fgb_mesh_add_pin(fgb_mesh* m, uint32_t index) { return fgb_mesh_add_pins(m, &index, 1); }

int fgb_mesh_add_pins(fgb_mesh* m, const uint32_t* index, uint64_t n) {
  if (!m) return fail(FGB_EINVAL, "null mesh");
  if (n && !index) return fail(FGB_EINVAL, "null buffer");
  for (uint64_t i = 0; i < n; ++i)
    if (index[i] >= m->topo.n) return fail(FGB_EINDEX, "pin index out of range");
  m->topo.pins.insert(m->topo.pins.end(), index, index + n);
  m->pins_dirty = true;
  return FGB_OK;
}

int fgb_mesh_counts(const fgb_mesh* m, uint64_t out[4]) {
  if (!m || !out) return fail(FGB_EINVAL, "null argument");
  out[0] = m->topo.n;
  out[1] = m->topo.sa.size();
  out[2] = m->topo.fv.size() / 3;
  out[3] = m->topo.pins.size();
  return FGB_OK;
}

int fgb_mesh_get_struts(const fgb_mesh* m, float* kcl, uint32_t* ab) {
  if (!m) return fail(FGB_EINVAL, "null mesh");
  const size_t S = m->topo.sa.size();
  for (size_t s = 0; s < S; ++s) {
    if (kcl) {
      kcl[3 * s] = m->topo.sk[s];
      kcl[3 * s + 1] = m->topo.sc[s];
      kcl[3 * s + 2] = m->topo.sl[s];
    }
    if (ab) {
      ab[2 * s] = m->topo.sa[s];
      ab[2 * s + 1] = m->topo.sb[s];
    }
  }
  return FGB_OK;
}

int fgb_mesh_set_strut_params(fgb_mesh* m, const float* stiffness, const float* damping) {
  if (!m || !stiffness || !damping) return fail(FGB_EINVAL, "null argument");
  std::copy(stiffness, stiffness + m->topo.sk.size(), m->topo.sk.begin());
  std::copy(damping, damping + m->topo.sc.size(), m->topo.sc.begin());
  m->topo_dirty = true;
  return FGB_OK;
}

int fgb_mesh_get_points(fgb_mesh* m, float* out) {
  if (!m || !out) return fail(FGB_EINVAL, "null argument");
  const size_t n = m->topo.n;
  if (!m->state_on_device) {
    std::memcpy(out, m->host_pts.data(), 10 * sizeof(float) * n);
    return FGB_OK;
  }
  FGB_CUDA(cudaSetDevice(m->device));
  const void* F = m->has_force ? m->force : nullptr;
  if (float* direct = mapped_host(out)) {
    // pinned host rows: the conversion kernel writes them across the host link itself
    if (m->precision == 64)
      FGB_CUDA((fgb::launch_pack_f32<double>(int(n), m->pos[m->cur], m->vel[m->cur], F, direct, m->stream)));
    else
      FGB_CUDA((fgb::launch_pack_f32<float>(int(n), m->pos[m->cur], m->vel[m->cur], F, direct, m->stream)));
    FGB_CUDA(cudaStreamSynchronize(m->stream));
    return FGB_OK;
  }
  FGB_CHECK_RC(ensure_io(m, 10 * sizeof(float) * n));
  if (m->precision == 64)
    FGB_CUDA((fgb::launch_pack_f32<double>(int(n), m->pos[m->cur], m->vel[m->cur], F, m->d_io, m->stream)));
  else
    FGB_CUDA((fgb::launch_pack_f32<float>(int(n), m->pos[m->cur], m->vel[m->cur], F, m->d_io, m->stream)));
  FGB_CUDA(cudaMemcpyAsync(out, m->d_io, 10 * sizeof(float) * n, cudaMemcpyDeviceToHost, m->stream));
  FGB_CUDA(cudaStreamSynchronize(m->stream));
  return FGB_OK;
}

int fgb_mesh_get_points_f64(fgb_mesh* m, double* out) {
  if (!m || !out) return fail(FGB_EINVAL, "null argument");
  const size_t n = m->topo.n;
  if (!m->state_on_device) {
    for (size_t i = 0; i < 10 * n; ++i) out[i] = double(m->host_pts[i]);
    return FGB_OK;
  }
  FGB_CUDA(cudaSetDevice(m->device));
  FGB_CHECK_RC(ensure_io(m, 10 * sizeof(double) * n));
  const void* F = m->has_force ? m->force : nullptr;
  double* d = reinterpret_cast<double*>(m->d_io);
  if (m->precision == 64)
    FGB_CUDA((fgb::launch_pack_f64<double>(int(n), m->pos[m->cur], m->vel[m->cur], F, d, m->stream)));
  else
    FGB_CUDA((fgb::launch_pack_f64<float>(int(n), m->pos[m->cur], m->vel[m->cur], F, d, m->stream)));
  FGB_CUDA(cudaMemcpyAsync(out, d, 10 * sizeof(double) * n, cudaMemcpyDeviceToHost, m->stream));
  FGB_CUDA(cudaStreamSynchronize(m->stream));
  return FGB_OK;
}

int fgb_mesh_set_points(fgb_mesh* m, const float* in) {
  if (!m || !in) return fail(FGB_EINVAL, "null argument");
  const size_t n = m->topo.n;
  if (!m->state_on_device || m->pins_dirty || m->topo_dirty) {
    m->host_pts.assign(in, in + 10 * n);
    m->state_on_device = false;
    return FGB_OK;
  }
  // Device-resident: DMA the raw points and convert on the device; the
  // accumulated forces go to the force buffer (read once by the next step).
  FGB_CUDA(cudaSetDevice(m->device));
  if (!m->force) FGB_CUDA(dalloc(m->force, m->elem() * n));
  const float* rows = mapped_host(in);  // pinned host rows are read across the host link by the kernel itself
  if (!rows) {
    FGB_CHECK_RC(ensure_io(m, 10 * sizeof(float) * n));
    FGB_CUDA(cudaMemcpyAsync(m->d_io, in, 10 * sizeof(float) * n, cudaMemcpyHostToDevice, m->stream));
    rows = m->d_io;
  }
  if (m->precision == 64)
    FGB_CUDA((fgb::launch_unpack<double>(int(n), rows, m->d_pinned, m->pos[m->cur], m->vel[m->cur], m->force,
                                         m->stream)));
  else
    FGB_CUDA((fgb::launch_unpack<float>(int(n), rows, m->d_pinned, m->pos[m->cur], m->vel[m->cur], m->force,
                                        m->stream)));
  FGB_CUDA(cudaStreamSynchronize(m->stream));
  m->has_force = true;
  m->staged = false;
  return FGB_OK;
}

int fgb_mesh_get_positions(fgb_mesh* m, float* out) {
  if (!m || !out) return fail(FGB_EINVAL, "null argument");
  const size_t n = m->topo.n;
  if (!m->state_on_device) {
    for (size_t i = 0; i < n; ++i)
      for (int k = 0; k < 3; ++k) out[3 * i + k] = m->host_pts[10 * i + 1 + k];
    return FGB_OK;
  }
  FGB_CUDA(cudaSetDevice(m->device));
  if (float* direct = mapped_host(out)) {
    // pinned host rows: the kernel writes them across the host link itself
    if (m->precision == 64)
      FGB_CUDA(fgb::launch_positions<double>(int(n), m->pos[m->cur], direct, m->stream));
    else
      FGB_CUDA(fgb::launch_positions<float>(int(n), m->pos[m->cur], direct, m->stream));
    FGB_CUDA(cudaStreamSynchronize(m->stream));
    return FGB_OK;
  }
  FGB_CHECK_RC(ensure_io(m, 3 * sizeof(float) * n));
  if (m->precision == 64)
    FGB_CUDA(fgb::launch_positions<double>(int(n), m->pos[m->cur], m->d_io, m->stream));
  else
    FGB_CUDA(fgb::launch_positions<float>(int(n), m->pos[m->cur], m->d_io, m->stream));
  FGB_CUDA(cudaMemcpyAsync(out, m->d_io, 3 * sizeof(float) * n, cudaMemcpyDeviceToHost, m->stream));
  FGB_CUDA(cudaStreamSynchronize(m->stream));
  return FGB_OK;
}

int fgb_mesh_get_vertices(fgb_mesh* m, float* positions, uint32_t* indices) {
  if (!m) return fail(FGB_EINVAL, "null mesh");
  if (positions) FGB_CHECK_RC(fgb_mesh_get_positions(m, positions));
  if (indices) std::memcpy(indices, m->topo.fv.data(), m->topo.fv.size() * sizeof(uint32_t));
  return FGB_OK;
}

int fgb_mesh_export_vertices(fgb_mesh* m, void* device_out, const float* color, void* stream) {
  if (!m || !device_out) return fail(FGB_EINVAL, "null argument");
  FGB_CHECK_RC(ensure_device(m));
  FGB_CHECK_RC(ensure_csr(m));
  const cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : m->stream;
  if (st != m->stream) FGB_CUDA(cudaStreamSynchronize(m->stream));
  const float r = color ? color[0] : 1.0f, g = color ? color[1] : 1.0f, b = color ? color[2] : 1.0f;
  const int n = int(m->topo.n);
  if (m->precision == 64)
    FGB_CUDA(fgb::launch_render_vertices<double>(n, m->pos[m->cur], m->d_face_off, m->d_face_inc, m->d_face_vtx, r, g,
                                                 b, static_cast<float*>(device_out), st));
  else
    FGB_CUDA(fgb::launch_render_vertices<float>(n, m->pos[m->cur], m->d_face_off, m->d_face_inc, m->d_face_vtx, r, g,
                                                b, static_cast<float*>(device_out), st));
  return FGB_OK;
}

int fgb_mesh_export_indices(fgb_mesh* m, void* device_out, void* stream) {
  if (!m || !device_out) return fail(FGB_EINVAL, "null argument");
  FGB_CHECK_RC(ensure_device(m));
  const cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : m->stream;
  FGB_CUDA(cudaMemcpyAsync(device_out, m->topo.fv.data(), m->topo.fv.size() * sizeof(uint32_t),
                           cudaMemcpyHostToDevice, st));
  FGB_CUDA(cudaStreamSynchronize(st));
  return FGB_OK;
}

int fgb_mesh_set_path(fgb_mesh* m, int path) {
  if (!m || path < 0 || path > 4) return fail(FGB_EINVAL, "path must be 0, 1, 2, 3 or 4");
  m->path_req = path == 3 ? 2 : (path == 4 ? 1 : path);
  m->grid_variant = path == 3 ? 1 : 0;
  m->plain_csr = path == 4;
  m->topo_dirty = true;
  return FGB_OK;
}

int fgb_mesh_get_path(fgb_mesh* m, int* path) {
  if (!m || !path) return fail(FGB_EINVAL, "null argument");
  if (!m->topo_dirty) {
    *path = m->active_path;
    return FGB_OK;
  }
  return decide_path(m, path);
}

int fgb_mesh_set_precision(fgb_mesh* m, int bits) {
  if (!m || (bits != 32 && bits != 64)) return fail(FGB_EINVAL, "precision must be 32 or 64");
  if (bits == m->precision) return FGB_OK;
  FGB_CHECK_RC(download_state(m));
  m->state_on_device = false;
  free_state(m);
  m->precision = bits;
  m->topo_dirty = true;
  return FGB_OK;
}

int fgb_mesh_accumulate_forces(fgb_mesh* m, const fgb_config* cfg) {
  if (!m) return fail(FGB_EINVAL, "null mesh");
  FGB_CHECK_RC(check_config(cfg));
  FGB_CHECK_RC(ensure_device(m));
  FGB_CHECK_RC(ensure_csr(m));
  FGB_CHECK_RC(ensure_force(m));
  const fgb::StepConsts c = make_consts(*cfg, nullptr, 0, m->d_flags);
  const fgb::GeneralTopo t = general_topo(m);
  if (m->precision == 64)
    FGB_CUDA(fgb::launch_accumulate<double>(int(m->topo.n), m->pos[m->cur], m->vel[m->cur], m->force, t, c, m->stream));
  else
    FGB_CUDA(fgb::launch_accumulate<float>(int(m->topo.n), m->pos[m->cur], m->vel[m->cur], m->force, t, c, m->stream));
  return FGB_OK;
}

int fgb_mesh_integrate(fgb_mesh* m, int32_t integration, float dt) {
  if (!m) return fail(FGB_EINVAL, "null mesh");
  if (integration != FGB_EULER && integration != FGB_RK4) return fail(FGB_EINVAL, "bad integration");
  FGB_CHECK_RC(ensure_device(m));
  FGB_CHECK_RC(ensure_force(m));
  const size_t bytes = m->elem() * size_t(m->topo.n);
  if (!m->spos) FGB_CUDA(dalloc(m->spos, bytes));
  if (!m->svel) FGB_CUDA(dalloc(m->svel, bytes));
  if (!m->sforce) FGB_CUDA(dalloc(m->sforce, bytes));
  if (m->precision == 64)
    FGB_CUDA(fgb::launch_integrate<double>(int(m->topo.n), integration, dt, m->pos[m->cur], m->vel[m->cur], m->force,
                                           m->spos, m->svel, m->sforce, m->stream));
  else
    FGB_CUDA(fgb::launch_integrate<float>(int(m->topo.n), integration, dt, m->pos[m->cur], m->vel[m->cur], m->force,
                                          m->spos, m->svel, m->sforce, m->stream));
  m->staged = true;
  return FGB_OK;
}

int fgb_mesh_update_points(fgb_mesh* m, fgb_obstacle* const* obstacles, uint64_t n_obstacles, const fgb_config* cfg) {
  if (!m) return fail(FGB_EINVAL, "null mesh");
  FGB_CHECK_RC(check_config(cfg));
  if (!m->staged) return fail(FGB_ESTATE, "update_points needs staged points: call fgb_mesh_integrate first");
  if (n_obstacles && !obstacles) return fail(FGB_EINVAL, "null obstacle list");
  std::vector<fgb::ObsFace> faces;
  FGB_CHECK_RC(make_obstacle_faces(obstacles, n_obstacles, faces));
  fgb::ObsFace* d_faces = nullptr;
  FGB_CUDA(dalloc(d_faces, faces.size() * sizeof(fgb::ObsFace)));
  FGB_CUDA(cudaMemcpy(d_faces, faces.data(), faces.size() * sizeof(fgb::ObsFace), cudaMemcpyHostToDevice));
  const fgb::StepConsts c = make_consts(*cfg, d_faces, int(faces.size()), m->d_flags);
  cudaError_t e;
  if (m->precision == 64)
    e = fgb::launch_update<double>(int(m->topo.n), m->pos[m->cur], m->vel[m->cur], m->force, m->spos, m->svel,
                                   m->sforce, c, m->stream);
  else
    e = fgb::launch_update<float>(int(m->topo.n), m->pos[m->cur], m->vel[m->cur], m->force, m->spos, m->svel,
                                  m->sforce, c, m->stream);
  const cudaError_t s = cudaStreamSynchronize(m->stream);
  dfree(d_faces);
  FGB_CUDA(e);
  FGB_CUDA(s);
  m->staged = false;
  return FGB_OK;
}

int fgb_mesh_clear_forces(fgb_mesh* m) {
  if (!m) return fail(FGB_EINVAL, "null mesh");
  if (!m->state_on_device) {
    for (size_t i = 0; i < m->topo.n; ++i)
      for (int k = 7; k < 10; ++k) m->host_pts[10 * i + k] = 0.0f;
    return FGB_OK;
  }
  m->has_force = false;  // a missing force buffer reads as zero
  return FGB_OK;
}

int fgb_mesh_synchronize(fgb_mesh* m) {
  if (!m) return fail(FGB_EINVAL, "null mesh");
  if (m->stream) FGB_CUDA(cudaStreamSynchronize(m->stream));
  return FGB_OK;
}

int fgb_mesh_destroy(fgb_mesh* m) {
  if (!m) return FGB_OK;
  cudaSetDevice(m->device);
  if (m->stream) cudaStreamSynchronize(m->stream);
  free_state(m);
  free_topology(m);
  dfree(m->d_io);
  dfree(m->d_pinned);
  dfree(m->d_flags);
  m->own.reset();
  delete m;
  return FGB_OK;
}

int fgb_collidable_new(const float* positions, uint64_t n_vertices, const uint32_t* indices, uint64_t n_indices,
                       fgb_obstacle** out) {
  if (!out) return fail(FGB_EINVAL, "null out");
  *out = nullptr;
  if ((n_vertices && !positions) || (n_indices && !indices)) return fail(FGB_EINVAL, "null buffer");
  const uint64_t nt = n_indices / 3;
  std::set<std::pair<uint32_t, uint32_t>> edges;
  std::vector<fgb::ObsFace> faces;
  faces.reserve(nt);
  for (uint64_t t = 0; t < nt; ++t) {
    const uint32_t i[3] = {indices[3 * t], indices[3 * t + 1], indices[3 * t + 2]};
    for (int k = 0; k < 3; ++k)
      if (i[k] >= n_vertices) return fail(FGB_EINDEX, "collidable mesh index out of range");
    if (i[0] == i[1] || i[1] == i[2] || i[2] == i[0])
      return fail(FGB_EINVAL, "collidable mesh triangle repeats a vertex");
    for (int k = 0; k < 3; ++k) edges.insert({std::min(i[k], i[(k + 1) % 3]), std::max(i[k], i[(k + 1) % 3])});
    const float* p0 = positions + 3 * size_t(i[0]);
    const float* p1 = positions + 3 * size_t(i[1]);
    const float* p2 = positions + 3 * size_t(i[2]);
    // Face::normal, collidable_mesh.rs:41-43: (v1 - v0).cross(v2 - v0).normalize()
    const float ax = p1[0] - p0[0], ay = p1[1] - p0[1], az = p1[2] - p0[2];
    const float bx = p2[0] - p0[0], by = p2[1] - p0[1], bz = p2[2] - p0[2];
    const float cx = ay * bz - az * by, cy = az * bx - ax * bz, cz = ax * by - ay * bx;
    const float inv = 1.0f / std::sqrt(cx * cx + cy * cy + cz * cz);
    const float nx = cx * inv, ny = cy * inv, nz = cz * inv;
    // projection axis of collidable_mesh.rs:133-154 (signed comparisons)
    int axis = 2;
    if (nx >= ny && nx >= nz) axis = 0;
    else if (ny >= nx && ny >= nz) axis = 1;
    fgb::ObsFace f;
    float axis_bits;
    std::memcpy(&axis_bits, &axis, 4);
    f.v0 = make_float4(p0[0], p0[1], p0[2], axis_bits);
    f.v1 = make_float4(p1[0], p1[1], p1[2], 0.0f);
    f.v2 = make_float4(p2[0], p2[1], p2[2], 0.0f);
    f.n = make_float4(nx, ny, nz, 0.0f);
    faces.push_back(f);
  }
  fgb_obstacle* o = new (std::nothrow) fgb_obstacle();
  if (!o) return fail(FGB_ENOMEM, "out of host memory");
  o->n_vertices = n_vertices;
  o->n_edges = edges.size();
  o->faces = std::move(faces);
  *out = o;
  return FGB_OK;
}

int fgb_collidable_counts(const fgb_obstacle* o, uint64_t out[3]) {
  if (!o || !out) return fail(FGB_EINVAL, "null argument");
  out[0] = o->n_vertices;
  out[1] = o->n_edges;
  out[2] = o->faces.size();
  return FGB_OK;
}

int fgb_collidable_destroy(fgb_obstacle* o) {
  delete o;
  return FGB_OK;
}

int fgb_sim_new(fgb_mesh* const* meshes, uint64_t n_meshes, fgb_obstacle* const* obstacles, uint64_t n_obstacles,
                fgb_sim** out) {
  if (!out) return fail(FGB_EINVAL, "null out");
  *out = nullptr;
  if ((n_meshes && !meshes) || (n_obstacles && !obstacles)) return fail(FGB_EINVAL, "null list");
  std::vector<fgb::ObsFace> faces;
  FGB_CHECK_RC(make_obstacle_faces(obstacles, n_obstacles, faces));
  for (uint64_t i = 0; i < n_meshes; ++i)
    if (!meshes[i]) return fail(FGB_EINVAL, "null mesh");
  // the reference's Simulation owns its meshes (a Vec<SpringyMesh>), so none
  // appears twice; a repeated handle would be stepped twice per step by the
  // one-mesh path and once by the batched one
  {
    std::set<const fgb_mesh*> seen;
    for (uint64_t i = 0; i < n_meshes; ++i)
      if (!seen.insert(meshes[i]).second)
        return fail(FGB_EINVAL, "mesh " + std::to_string(i) + " appears twice in the simulation's mesh list");
  }
  // one simulation steps its meshes with one kernel per step on one device:
  // meshes created on different devices cannot share it
  for (uint64_t i = 1; i < n_meshes; ++i)
    if (meshes[i]->device != meshes[0]->device)
      return fail(FGB_EINVAL, "meshes of one simulation must be on one device (mesh " + std::to_string(i) +
                                  " is on device " + std::to_string(meshes[i]->device) + ", mesh 0 on device " +
                                  std::to_string(meshes[0]->device) + ")");
  fgb_sim* s = new (std::nothrow) fgb_sim();
  if (!s) return fail(FGB_ENOMEM, "out of host memory");
  s->meshes.assign(meshes, meshes + n_meshes);
  s->obstacles.assign(obstacles, obstacles + n_obstacles);
  fgb_config_default(&s->cfg);
  s->n_faces = int(faces.size());
  s->faces = std::move(faces);
  *out = s;
  return FGB_OK;
}

int fgb_sim_set_config(fgb_sim* s, const fgb_config* cfg) {
  if (!s) return fail(FGB_EINVAL, "null sim");
  FGB_CHECK_RC(check_config(cfg));
  s->cfg = *cfg;
  return FGB_OK;
}

int fgb_sim_get_config(const fgb_sim* s, fgb_config* out) {
  if (!s || !out) return fail(FGB_EINVAL, "null argument");
  *out = s->cfg;
  return FGB_OK;
}

int fgb_sim_step(fgb_sim* s, uint64_t n_steps) {
  if (!s) return fail(FGB_EINVAL, "null sim");
  FGB_CHECK_RC(upload_faces(s));
  for (fgb_mesh* m : s->meshes) FGB_CHECK_RC(ensure_device(m));
  FGB_CHECK_RC(prepare_batch(s));
  if (!s->batch.empty()) FGB_CHECK_RC(batched_steps(s, n_steps));
  std::set<fgb_mesh*> in_batch(s->batch.begin(), s->batch.end());
  for (uint64_t k = 0; k < n_steps; ++k)
    for (fgb_mesh* m : s->meshes)
      if (!in_batch.count(m))
        FGB_CHECK_RC(step_mesh(m, make_consts(s->cfg, s->d_faces, s->n_faces, m->d_flags, &s->accel)));
  return FGB_OK;
}

int fgb_mesh_set_wind(fgb_mesh* m, const float* wind) {
  if (!m) return fail(FGB_EINVAL, "null mesh");
  if (wind) {
    for (int k = 0; k < 3; ++k) m->wind[k] = wind[k];
    m->has_wind = true;
  } else {
    m->has_wind = false;
  }
  return FGB_OK;
}

int fgb_sim_set_batch_mode(fgb_sim* s, int mode) {
  if (!s || mode < -1 || mode > 1) return fail(FGB_EINVAL, "mode must be -1, 0 or 1");
  s->forced_mode = mode;
  s->mode = -1;
  drop_graphs(s);
  return FGB_OK;
}

int fgb_sim_set_graphs(fgb_sim* s, int enabled) {
  if (!s) return fail(FGB_EINVAL, "null sim");
  s->graphs = enabled != 0;
  return FGB_OK;
}

int fgb_sim_set_batch_tile(fgb_sim* s, int tile_rows) {
  if (!s || !(tile_rows == 0 || fgb::batch_tile_height_ok(tile_rows)))
    return fail(FGB_EINVAL, "tile_rows must be 0 (autotuner), 4, 8 or 12");
  s->forced_tile_h = tile_rows;
  s->mode = -1;
  drop_graphs(s);
  return FGB_OK;
}

int fgb_sim_batch_info(const fgb_sim* s, int64_t out[5]) {
  if (!s || !out) return fail(FGB_EINVAL, "null argument");
  out[0] = int64_t(s->batch.size());
  out[1] = s->n_work;
  out[2] = s->mode;
  out[3] = s->ctas;
  out[4] = s->tile_h;
  return FGB_OK;
}

int fgb_sim_set_collision_broadphase(fgb_sim* s, int enabled) {
  if (!s) return fail(FGB_EINVAL, "null sim");
  s->broadphase = enabled != 0;
  return FGB_OK;
}

int fgb_sim_set_stream(fgb_sim* s, void* stream) {
  if (!s) return fail(FGB_EINVAL, "null sim");
  s->ext_stream = static_cast<cudaStream_t>(stream);
  for (fgb_mesh* m : s->meshes) {
    if (m->stream) FGB_CUDA(cudaStreamSynchronize(m->stream));
    m->external_stream = stream != nullptr;
    m->stream = stream ? static_cast<cudaStream_t>(stream) : (m->own ? m->own->s : nullptr);
  }
  return FGB_OK;
}

int fgb_sim_get_timestep(const fgb_sim* s, double* seconds) {
  if (!s || !seconds) return fail(FGB_EINVAL, "null argument");
  *seconds = fgb::duration_seconds_f64(s->cfg.dt);
  return FGB_OK;
}

int fgb_sim_synchronize(fgb_sim* s, int* nonfinite) {
  if (!s) return fail(FGB_EINVAL, "null sim");
  int bad = 0;
  unsigned all = 0;
  for (fgb_mesh* m : s->meshes) {
    if (m->stream) FGB_CUDA(cudaStreamSynchronize(m->stream));
    if (m->d_flags) {
      unsigned f = 0;
      FGB_CUDA(cudaMemcpy(&f, m->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost));
      if (f) {
        bad = bad || (f & 1u);
        all |= f;
        FGB_CUDA(cudaMemsetAsync(m->d_flags, 0, sizeof(unsigned), m->stream));
        FGB_CUDA(cudaStreamSynchronize(m->stream));
      }
    }
  }
  if (nonfinite) *nonfinite = bad;
  if (all & 2u) return fail(FGB_ECHECK, "a tile's staging copy did not complete in time");
  return FGB_OK;
}

int fgb_sim_destroy(fgb_sim* s) {
  if (!s) return FGB_OK;
  // The meshes may already be destroyed: touch none of them.  cudaFree waits
  // for in-flight work that reads the obstacle faces.
  dfree(s->d_faces);
  dfree(s->d_accel);
  for (auto& kv : s->graph_cache) cudaGraphExecDestroy(kv.second);
  dfree(s->d_desc);
  dfree(s->d_work);
  dfree(s->d_counter);
  dfree(s->d_maps);
  delete s;
  return FGB_OK;
}

}  // extern "C"

int fgb::detail::ensure_device(fgb_mesh* m) { return ::ensure_device(m); }

fgb::StepConsts fgb::detail::make_consts(const fgb_config& cfg, const fgb::ObsFace* faces, int n_faces,
                                         unsigned* flags, const fgb::ObsAccel* accel) {
  return ::make_consts(cfg, faces, n_faces, flags, accel);
}

int fgb::detail::ensure_sim(fgb_sim* s) {
  FGB_CHECK_RC(upload_faces(s));
  for (fgb_mesh* m : s->meshes) FGB_CHECK_RC(::ensure_device(m));
  return prepare_batch(s);
}

cudaStream_t fgb::detail::sim_stream(fgb_sim* s) {
  if (!s->batch.empty()) return batch_stream(s);
  return s->meshes.empty() ? nullptr : s->meshes[0]->stream;
}

// ===================================================== allocation-free step ===
//
// Some hosts cannot let a library allocate device memory once they are
// running: game engines and renderers that hand out all GPU memory through
// their own allocators and forbid plugin allocations inside the frame loop,
// and real-time loops that cannot afford cudaMalloc/cudaFree (both can
// synchronise the whole device).  fgb_sim_step_static advances a prepared
// simulation with the batched persistent kernel while keeping that kernel's
// scratch -- its work counter, the cloth descriptor table and the tile list --
// in the fixed array below instead of memory allocated for the simulation.

namespace {

// Stated maximum: 4 MiB per GPU, held by every GPU that loads the library.
constexpr size_t kStaticScratchBytes = size_t(4) << 20;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_static_mutex;
unsigned char* g_static_ptr[kMaxDevices] = {};

// Device address of g_static_scratch on the current device (looked up once
// per device, with that device current).
int static_scratch(unsigned char** out) {
  int dev = 0;
  FGB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(FGB_EINVAL, "device index beyond the supported range");
  std::lock_guard<std::mutex> lock(g_static_mutex);
  if (!g_static_ptr[dev]) {
    void* p = nullptr;
    FGB_CUDA(cudaGetSymbolAddress(&p, g_static_scratch));
    g_static_ptr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_static_ptr[dev];
  return FGB_OK;
}

}  // namespace

extern "C" int fgb_sim_step_static(fgb_sim* s, uint64_t n_steps, void* stream) {
  if (!s) return fail(FGB_EINVAL, "null sim");
  if (s->meshes.empty()) return FGB_OK;
  for (fgb_mesh* m : s->meshes)
    if (m->topo.rows == 0 || m->path_req == 1 || m->grid_variant != 0 || m->precision != 32)
      return fail(FGB_EINVAL, "the allocation-free step handles Cloth::new grid meshes on the f32 grid path only");
  // descriptor table and tile list, largest cloths first (as the batched step)
  std::vector<fgb_mesh*> order(s->meshes.begin(), s->meshes.end());
  std::stable_sort(order.begin(), order.end(), [](const fgb_mesh* a, const fgb_mesh* b) { return a->topo.n > b->topo.n; });
  size_t n_work = 0;
  for (size_t i = 0; i < order.size(); ++i) {
    int nr, ni;
    fgb::batch_tiles(int(i), int(order[i]->topo.rows), int(order[i]->topo.cols), fgb::kDefaultTileH, nullptr, &nr,
                     &ni);
    n_work += size_t(nr + ni);
  }
  const size_t desc_off = 256;
  const size_t work_off = (desc_off + order.size() * sizeof(fgb::ClothDesc) + 255) & ~size_t(255);
  const size_t need = work_off + n_work * sizeof(int4);
  if (need > kStaticScratchBytes)
    return fail(FGB_EINVAL, "this batch needs " + std::to_string(need) + " bytes of scratch; the allocation-free step "
                            "holds at most " + std::to_string(kStaticScratchBytes) +
                            " (" + std::to_string(sizeof(fgb::ClothDesc)) + " bytes per cloth plus 16 bytes per 32x8 tile)");
  // Everything the step reads must already be on the device: this call
  // uploads no topology, state or obstacles (that would allocate).
  if (!s->faces_uploaded)
    return fail(FGB_ESTATE, "simulation not prepared: call fgb_sim_step(sim, 0) once during set-up");
  for (fgb_mesh* m : s->meshes) {
    if (!m->state_on_device || m->topo_dirty || m->pins_dirty || m->staged || m->active_path != 2)
      return fail(FGB_ESTATE, "mesh not prepared: call fgb_sim_step(sim, 0) once during set-up (and after any "
                              "topology, pin or precision change)");
  }
  const fgb::DeviceGuard keep_device;  // the caller's current device is restored on every return
  FGB_CUDA(cudaSetDevice(s->meshes[0]->device));
  unsigned char* scratch = nullptr;
  FGB_CHECK_RC(static_scratch(&scratch));
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : s->meshes[0]->stream;

  std::vector<int> work(4 * n_work);
  for (size_t i = 0, at = 0; i < order.size(); ++i) {
    int nr, ni;
    fgb::batch_tiles(int(i), int(order[i]->topo.rows), int(order[i]->topo.cols), fgb::kDefaultTileH,
                     work.data() + 4 * at, &nr, &ni);
    at += size_t(nr + ni);
  }
  for (fgb_mesh* m : order) {  // all cloths read buffer [0] at the first step
    if (m->stream != st) FGB_CUDA(cudaStreamSynchronize(m->stream));
    if (m->cur != 0) {
      std::swap(m->pos[0], m->pos[1]);
      std::swap(m->vel[0], m->vel[1]);
      m->cur = 0;
    }
  }
  std::vector<fgb::ClothDesc> desc(order.size());
  for (size_t i = 0; i < order.size(); ++i) {
    fgb_mesh* m = order[i];
    fgb::ClothDesc& d = desc[i];
    std::memset(&d, 0, sizeof(d));
    d.planes = m->d_grid;
    for (int k = 0; k < 2; ++k) {
      d.pos[k] = static_cast<float4*>(m->pos[k]);
      d.vel[k] = static_cast<float4*>(m->vel[k]);
    }
    d.force_in = m->has_force ? static_cast<const float4*>(m->force) : nullptr;
    d.flags = m->d_flags;
    d.rows = int(m->topo.rows);
    d.cols = int(m->topo.cols);
    for (int k = 0; k < 3; ++k) d.wind[k] = m->has_wind ? m->wind[k] : s->cfg.wind[k];
  }
  fgb::ClothDesc* d_desc = reinterpret_cast<fgb::ClothDesc*>(scratch + desc_off);
  int4* d_work = reinterpret_cast<int4*>(scratch + work_off);
  int* d_counter = reinterpret_cast<int*>(scratch);
  FGB_CUDA(cudaMemcpyAsync(d_desc, desc.data(), desc.size() * sizeof(fgb::ClothDesc), cudaMemcpyHostToDevice, st));
  FGB_CUDA(cudaMemcpyAsync(d_work, work.data(), work.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  int dev = 0, sms = 0;
  FGB_CUDA(cudaGetDevice(&dev));
  FGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int ctas = fgb::batched_ctas_per_sm() * sms;
  s->accel.enabled = (s->broadphase && s->d_accel) ? 1 : 0;
  for (uint64_t k = 0; k < n_steps; ++k) {
    // the counter keeps the previous call's value: clear it before every launch
    FGB_CUDA(cudaMemsetAsync(d_counter, 0, sizeof(int), st));
    FGB_CUDA(fgb::launch_step_batched(d_desc, d_work, int(n_work), d_counter, int(k & 1), 1, ctas,
                                      make_consts(s->cfg, s->d_faces, s->n_faces, nullptr, &s->accel), st));
    if (k == 0 && n_steps > 1) {  // carried forces apply to the first step only
      bool forces = false;
      for (const fgb::ClothDesc& d : desc) forces = forces || d.force_in;
      if (forces) {
        for (fgb::ClothDesc& d : desc) d.force_in = nullptr;
        FGB_CUDA(cudaMemcpyAsync(d_desc, desc.data(), desc.size() * sizeof(fgb::ClothDesc), cudaMemcpyHostToDevice,
                                 st));
      }
    }
  }
  FGB_CUDA(cudaStreamSynchronize(st));  // the host tables above are released on return
  for (fgb_mesh* m : order) {
    m->cur = int(n_steps & 1);
    m->has_force = m->has_force && n_steps == 0;
    m->staged = false;
  }
  // The regular batched step keeps its work list, launch form and graphs: its
  // next call finds m->cur != s->parity where the buffers were swapped,
  // swaps them back and re-uploads the cloth table (prepare_batch).
  return FGB_OK;
}
