// C ABI of the learned surrogate (include/feriphys_gb300.h, "Learned
// surrogate"): parameter handling, dataset ring, training loop, and the
// coarse rollout with the energy/strain checks and the fine-step fallback.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "feriphys_gb300.h"
#include "handles.h"
#include "kernels.h"
#include "surrogate.h"

using fgb::detail::fail;
namespace S = fgb::sur;

#define FGB_CUDA(call)                                                                              \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess) return fail(FGB_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define FGB_CHECK_RC(expr)         \
  do {                             \
    int rc_ = (expr);              \
    if (rc_ != FGB_OK) return rc_; \
  } while (0)

namespace {

template <class P>
void dfree(P*& p) {
  if (p) cudaFree(reinterpret_cast<void*>(p));
  p = nullptr;
}

template <class P>
cudaError_t dgrow(P*& p, size_t& cap, size_t need, size_t elem) {
  if (need <= cap && p) return cudaSuccess;
  dfree(p);
  void* q = nullptr;
  const size_t n = std::max<size_t>(need, 1);
  cudaError_t e = cudaMalloc(&q, n * elem);
  p = static_cast<P*>(q);
  cap = e == cudaSuccess ? n : 0;
  return e;
}

}  // namespace

struct fgb_surrogate {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<float> master;  // padded host copy, valid unless host_stale
  bool host_stale = false;
  float* d_master = nullptr;
  float* d_m = nullptr;
  float* d_v = nullptr;
  void* d_blob = nullptr;
  S::Norm norm;
  uint64_t adam_t = 0;
  // dataset ring
  float* d_feat = nullptr;
  float* d_tgt = nullptr;
  long long cap = 0, count = 0, head = 0;
  // scratch
  unsigned char* d_X = nullptr;
  size_t X_cap = 0;  // bytes
  float* d_T = nullptr;
  size_t T_cap = 0;  // floats
  float* d_xin = nullptr;
  size_t xin_cap = 0;
  float* d_tin = nullptr;
  size_t tin_cap = 0;
  float* d_partials = nullptr;
  size_t partials_cap = 0;
  float* d_loss = nullptr;
  size_t loss_cap = 0;
  float* d_grad = nullptr;
  size_t grad_cap = 0;
  double* d_stats = nullptr;
  size_t stats_cap = 0;
  int* d_err = nullptr;
  // coarse-step tables
  S::SurCloth* d_cloths = nullptr;
  size_t cloths_cap = 0;
  S::Tile* d_tiles = nullptr;
  size_t tiles_cap = 0;
  float2* d_tile_chk = nullptr;
  size_t tile_chk_cap = 0;
  float2* d_cloth_chk = nullptr;
  size_t cloth_chk_cap = 0;
  float* d_out = nullptr;
  size_t out_cap = 0;
  fgb::ClothDesc* d_fdesc = nullptr;  // batched fine-step fallback table (batch order, skip flags)
  size_t fdesc_cap = 0;
  int4* d_fwork = nullptr;            // work items of the failing cloths only
  size_t fwork_cap = 0;
  int* d_fcounter = nullptr;
  int groups = 4;
  // checked rollout decided on the device (per cloth: accepted energy, margin
  // scale, verdict; per batch cloth: work-list range, mesh index, compacted
  // position; counters: this step's failures, fallback items, running total)
  float* d_e_old = nullptr;
  size_t e_old_cap = 0;
  double* d_e_ref = nullptr;
  size_t e_ref_cap = 0;
  int* d_fail = nullptr;
  size_t fail_cap = 0;
  int* d_bidx = nullptr;  // 4 x n_batch: off, cnt, mesh, dst
  size_t bidx_cap = 0;
  int* d_counts = nullptr;  // [0] failures this step, [1] fallback items
  unsigned long long* d_total = nullptr;
  cudaStream_t side = nullptr;  // captures the fallback body
};

namespace {

constexpr int kFlat = S::kNumParamsFlat;

// Public flat layout <-> padded device layout.
void flat_to_padded(const float* in, std::vector<float>& P) {
  P.assign(S::kNumParams, 0.0f);
  const float* q = in;
  for (int o = 0; o < S::kHid; ++o)
    for (int i = 0; i < S::kFeat; ++i) P[S::kOffW1 + o * S::kIn + i] = *q++;
  for (int o = 0; o < S::kHid; ++o) P[S::kOffB1 + o] = *q++;
  for (int o = 0; o < S::kHid; ++o)
    for (int i = 0; i < S::kHid; ++i) P[S::kOffW2 + o * S::kHid + i] = *q++;
  for (int o = 0; o < S::kHid; ++o) P[S::kOffB2 + o] = *q++;
  for (int o = 0; o < S::kOut; ++o)
    for (int i = 0; i < S::kHid; ++i) P[S::kOffW3 + o * S::kHid + i] = *q++;
  for (int o = 0; o < S::kOut; ++o) P[S::kOffB3 + o] = *q++;
}

void padded_to_flat(const float* P, float* out) {
  float* q = out;
  for (int o = 0; o < S::kHid; ++o)
    for (int i = 0; i < S::kFeat; ++i) *q++ = P[S::kOffW1 + o * S::kIn + i];
  for (int o = 0; o < S::kHid; ++o) *q++ = P[S::kOffB1 + o];
  for (int o = 0; o < S::kHid; ++o)
    for (int i = 0; i < S::kHid; ++i) *q++ = P[S::kOffW2 + o * S::kHid + i];
  for (int o = 0; o < S::kHid; ++o) *q++ = P[S::kOffB2 + o];
  for (int o = 0; o < S::kOut; ++o)
    for (int i = 0; i < S::kHid; ++i) *q++ = P[S::kOffW3 + o * S::kHid + i];
  for (int o = 0; o < S::kOut; ++o) *q++ = P[S::kOffB3 + o];
}

// Uniform in [-a, a) from a 64-bit generator (splitmix64), identical on
// every host.
struct Rng {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  }
  float uniform(float a) { return a * (2.0f * float(next() >> 40) * (1.0f / 16777216.0f) - 1.0f); }
};

int upload_master(fgb_surrogate* g, bool reset_adam) {
  FGB_CUDA(cudaMemcpyAsync(g->d_master, g->master.data(), S::kNumParams * sizeof(float), cudaMemcpyHostToDevice,
                           g->stream));
  if (reset_adam) {
    FGB_CUDA(cudaMemsetAsync(g->d_m, 0, S::kNumParams * sizeof(float), g->stream));
    FGB_CUDA(cudaMemsetAsync(g->d_v, 0, S::kNumParams * sizeof(float), g->stream));
    g->adam_t = 0;
  }
  FGB_CUDA(S::launch_pack_blob(g->d_master, g->d_blob, g->stream));
  FGB_CUDA(cudaStreamSynchronize(g->stream));
  g->host_stale = false;
  return FGB_OK;
}

int sync_host_master(fgb_surrogate* g) {
  if (!g->host_stale) return FGB_OK;
  FGB_CUDA(cudaMemcpyAsync(g->master.data(), g->d_master, S::kNumParams * sizeof(float), cudaMemcpyDeviceToHost,
                           g->stream));
  FGB_CUDA(cudaStreamSynchronize(g->stream));
  g->host_stale = false;
  return FGB_OK;
}

int check_err(fgb_surrogate* g, cudaStream_t st) {
  int e = 0;
  FGB_CUDA(cudaMemcpyAsync(&e, g->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
  FGB_CUDA(cudaStreamSynchronize(st));
  if (e) {
    FGB_CUDA(cudaMemsetAsync(g->d_err, 0, sizeof(int), st));
    return fail(FGB_ECHECK, "a tensor-core kernel gave up waiting for its copies or MMAs");
  }
  return FGB_OK;
}

// Standardised host rows -> packed bf16 tiles (and targets) on the device.
int stage_rows(fgb_surrogate* g, const float* x, const float* t, uint64_t n, uint64_t n_pad) {
  FGB_CUDA(dgrow(g->d_xin, g->xin_cap, size_t(n) * S::kFeat, sizeof(float)));
  FGB_CUDA(cudaMemcpyAsync(g->d_xin, x, size_t(n) * S::kFeat * sizeof(float), cudaMemcpyHostToDevice, g->stream));
  const float* dt = nullptr;
  if (t) {
    FGB_CUDA(dgrow(g->d_tin, g->tin_cap, size_t(n) * 3, sizeof(float)));
    FGB_CUDA(cudaMemcpyAsync(g->d_tin, t, size_t(n) * 3 * sizeof(float), cudaMemcpyHostToDevice, g->stream));
    dt = g->d_tin;
  }
  FGB_CUDA(dgrow(g->d_X, g->X_cap, size_t(n_pad) * S::kIn * 2, 1));
  FGB_CUDA(dgrow(g->d_T, g->T_cap, size_t(n_pad) * 4, sizeof(float)));
  FGB_CUDA(S::launch_pack_rows(g->d_xin, dt, int(n), int(n_pad), g->d_X, g->d_T, g->stream));
  return FGB_OK;
}

int ensure_train_scratch(fgb_surrogate* g, int ctas, size_t n_losses) {
  FGB_CUDA(dgrow(g->d_partials, g->partials_cap, size_t(ctas) * S::kPartialStride, sizeof(float)));
  FGB_CUDA(dgrow(g->d_loss, g->loss_cap, std::max<size_t>(n_losses, 1), sizeof(float)));
  return FGB_OK;
}

// One Adam step on the rows staged in d_X/d_T.
int adam_step(fgb_surrogate* g, uint64_t n_rows, float lr, float* d_loss_slot) {
  const int ctas = S::train_ctas(int(n_rows));
  FGB_CUDA(S::launch_train(g->d_X, g->d_T, int(n_rows), g->d_blob, g->d_partials, ctas, g->d_err, g->stream));
  g->adam_t += 1;
  const double t = double(g->adam_t);
  const float c1 = float(1.0 / (1.0 - std::pow(0.9, t)));
  const float c2 = float(1.0 / (1.0 - std::pow(0.999, t)));
  FGB_CUDA(S::launch_adam(g->d_partials, ctas, g->d_master, g->d_m, g->d_v, lr, 0.9f, 0.999f, 1e-8f, c1, c2,
                          g->d_blob, d_loss_slot, 1.0f / (3.0f * float(n_rows)), g->stream));
  g->host_stale = true;
  return FGB_OK;
}

// Rest spacing of a grid: the mean distance of horizontal neighbours at
// construction (vertical ones in a single column), in f64, rounded to f32.
float mesh_spacing(fgb_mesh* m) {
  if (m->rest_spacing > 0.0f) return m->rest_spacing;
  const int R = int(m->topo.rows), C = int(m->topo.cols);
  const float* p = m->topo.pos.data();
  const int step = C >= 2 ? 1 : C;
  double sum = 0.0;
  long long cnt = 0;
  for (int r = 0; r < R; ++r)
    for (int c = 0; c < C; ++c) {
      const long long i = (long long)r * C + c, j = i + step;
      if ((C >= 2 && c + 1 >= C) || (C < 2 && r + 1 >= R)) continue;
      const double dx = double(p[3 * j]) - p[3 * i], dy = double(p[3 * j + 1]) - p[3 * i + 1],
                   dz = double(p[3 * j + 2]) - p[3 * i + 2];
      sum += std::sqrt(dx * dx + dy * dy + dz * dz);
      ++cnt;
    }
  const double h = cnt ? sum / double(cnt) : 1.0;
  m->rest_spacing = h > 0.0 ? float(h) : 1.0f;
  return m->rest_spacing;
}

// The positions the mesh was built from, on the device (x, y, z, 0).
int ensure_rest(fgb_mesh* m) {
  if (m->d_rest) return FGB_OK;
  const size_t n = m->topo.n;
  std::vector<float4> h(n);
  for (size_t i = 0; i < n; ++i)
    h[i] = make_float4(m->topo.pos[3 * i], m->topo.pos[3 * i + 1], m->topo.pos[3 * i + 2], 0.0f);
  FGB_CUDA(cudaMalloc(&m->d_rest, std::max<size_t>(n, 1) * sizeof(float4)));
  FGB_CUDA(cudaMemcpy(m->d_rest, h.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
  return FGB_OK;
}

S::SurCloth make_cloth(fgb_mesh* m, float T, const float wind[3], long long vbase) {
  S::SurCloth c;
  std::memset(&c, 0, sizeof(c));
  for (int k = 0; k < 2; ++k) {
    c.pos[k] = static_cast<float4*>(m->pos[k]);
    c.vel[k] = static_cast<float4*>(m->vel[k]);
  }
  c.planes = m->d_grid;
  c.rest = m->d_rest;
  c.flags = m->d_flags;
  c.rows = int(m->topo.rows);
  c.cols = int(m->topo.cols);
  const float h = mesh_spacing(m);
  c.inv_h = 1.0f / h;
  c.sv = T / h;
  c.inv_sv = h / T;
  for (int k = 0; k < 3; ++k) c.wind[k] = wind[k];
  c.vbase = vbase;
  return c;
}

void add_tiles(int cloth, S::SurCloth& c, std::vector<S::Tile>& tiles) {
  const int n = c.rows * c.cols;
  c.tile0 = int(tiles.size());
  c.ntiles = (n + S::kTile - 1) / S::kTile;
  for (int k = 0; k < c.ntiles; ++k) tiles.push_back(make_int2(cloth, k * S::kTile));
}

int upload_tables(fgb_surrogate* g, const std::vector<S::SurCloth>& cl, const std::vector<S::Tile>& tiles,
                  cudaStream_t st) {
  FGB_CUDA(dgrow(g->d_cloths, g->cloths_cap, cl.size(), sizeof(S::SurCloth)));
  FGB_CUDA(dgrow(g->d_tiles, g->tiles_cap, tiles.size(), sizeof(S::Tile)));
  FGB_CUDA(cudaMemcpyAsync(g->d_cloths, cl.data(), cl.size() * sizeof(S::SurCloth), cudaMemcpyHostToDevice, st));
  FGB_CUDA(cudaMemcpyAsync(g->d_tiles, tiles.data(), tiles.size() * sizeof(S::Tile), cudaMemcpyHostToDevice, st));
  FGB_CUDA(cudaStreamSynchronize(st));
  return FGB_OK;
}

// Every mesh must be a Cloth::new grid on the f32 grid path, on one stream.
int check_grid_sim(fgb_sim* s) {
  if (s->meshes.empty()) return fail(FGB_EINVAL, "the simulation has no meshes");
  for (fgb_mesh* m : s->meshes)
    if (m->active_path != 2 || m->precision != 32 || m->topo.rows == 0)
      return fail(FGB_EINVAL, "the surrogate needs Cloth::new grid meshes on the f32 grid path");
  if (s->meshes.size() > 1 && s->batch.size() != s->meshes.size())
    return fail(FGB_EINVAL, "the surrogate needs every mesh in the batched grid path (tiled grid variant)");
  return FGB_OK;
}

// Puts every mesh's current state in buffers [s->parity].
void align_parity(fgb_sim* s) {
  for (fgb_mesh* m : s->meshes) {
    if (m->cur != s->parity) {
      std::swap(m->pos[0], m->pos[1]);
      std::swap(m->vel[0], m->vel[1]);
      m->cur = s->parity;
    }
  }
}

void mesh_wind(const fgb_sim* s, const fgb_mesh* m, float w[3]) {
  for (int k = 0; k < 3; ++k) w[k] = m->has_wind ? m->wind[k] : s->cfg.wind[k];
}

int build_sim_tables(fgb_surrogate* g, fgb_sim* s, float T, long long vbase0, std::vector<S::SurCloth>& cl,
                     std::vector<S::Tile>& tiles, cudaStream_t st) {
  cl.clear();
  tiles.clear();
  long long vb = vbase0;
  for (fgb_mesh* m : s->meshes) FGB_CHECK_RC(ensure_rest(m));
  for (size_t i = 0; i < s->meshes.size(); ++i) {
    float w[3];
    mesh_wind(s, s->meshes[i], w);
    cl.push_back(make_cloth(s->meshes[i], T, w, vb));
    add_tiles(int(i), cl.back(), tiles);
    vb += (long long)s->meshes[i]->topo.n;
  }
  return upload_tables(g, cl, tiles, st);
}

int run_check(fgb_surrogate* g, fgb_sim* s, int n_tiles, int parity, std::vector<float2>& out, cudaStream_t st) {
  const int nc = int(s->meshes.size());
  FGB_CUDA(dgrow(g->d_tile_chk, g->tile_chk_cap, size_t(n_tiles), sizeof(float2)));
  FGB_CUDA(dgrow(g->d_cloth_chk, g->cloth_chk_cap, size_t(nc), sizeof(float2)));
  const float3 gf = make_float3(s->cfg.gravity[0], s->cfg.gravity[1], s->cfg.gravity[2]);
  FGB_CUDA(S::launch_check(g->d_cloths, g->d_tiles, n_tiles, nc, parity, gf, g->d_tile_chk, g->d_cloth_chk, st));
  out.resize(nc);
  FGB_CUDA(cudaMemcpyAsync(out.data(), g->d_cloth_chk, nc * sizeof(float2), cudaMemcpyDeviceToHost, st));
  FGB_CUDA(cudaStreamSynchronize(st));
  return FGB_OK;
}

// `ratio` fine steps of the meshes in `failing` (indices into s->meshes),
// starting from buffers [par] and ending in [par ^ 1], the other meshes
// untouched.  Single meshes step with the grid kernel; a batch with one
// masked launch of the batched kernel per fine step.
int fine_fallback(fgb_surrogate* g, fgb_sim* s, const std::vector<int>& failing, int par, uint32_t ratio,
                  cudaStream_t st) {
  const fgb::StepConsts fc = fgb::detail::make_consts(s->cfg, s->d_faces, s->n_faces, nullptr, &s->accel);
  if (s->batch.empty()) {
    for (int c : failing) {
      fgb_mesh* m = s->meshes[c];
      const fgb::GridTopo gt{int(m->topo.rows), int(m->topo.cols), m->d_grid, 0};
      fgb::StepConsts mc = fc;
      mc.flags = m->d_flags;
      int a = par;
      for (uint32_t j = 0; j < ratio; ++j, a ^= 1)
        FGB_CUDA(fgb::launch_step_grid(gt, static_cast<const float4*>(m->pos[a]), static_cast<const float4*>(m->vel[a]),
                                       nullptr, static_cast<float4*>(m->pos[a ^ 1]), static_cast<float4*>(m->vel[a ^ 1]),
                                       mc, st));
      if (a != (par ^ 1)) {
        const size_t bytes = size_t(m->topo.n) * sizeof(float4);
        FGB_CUDA(cudaMemcpyAsync(m->pos[par ^ 1], m->pos[a], bytes, cudaMemcpyDeviceToDevice, st));
        FGB_CUDA(cudaMemcpyAsync(m->vel[par ^ 1], m->vel[a], bytes, cudaMemcpyDeviceToDevice, st));
      }
    }
    return FGB_OK;
  }
  std::vector<char> fail_mesh(s->meshes.size(), 0);
  for (int c : failing) fail_mesh[c] = 1;
  std::vector<fgb::ClothDesc> d = s->desc;
  std::vector<char> fail_batch(s->batch.size(), 0);
  for (size_t b = 0; b < s->batch.size(); ++b) {
    const size_t mi = size_t(std::find(s->meshes.begin(), s->meshes.end(), s->batch[b]) - s->meshes.begin());
    fail_batch[b] = (mi < fail_mesh.size() && fail_mesh[mi]) ? 1 : 0;
    d[b].skip = fail_batch[b] ? 0 : 1;
    d[b].force_in = nullptr;
  }
  // the failing cloths' work items, in the list's order (largest cloths and boundary tiles first)
  std::vector<int> fw;
  for (size_t i = 0; i + 3 < s->work_host.size(); i += 4)
    if (fail_batch[size_t(s->work_host[i])]) fw.insert(fw.end(), s->work_host.begin() + i, s->work_host.begin() + i + 4);
  const int n_fw = int(fw.size() / 4);
  FGB_CUDA(dgrow(g->d_fdesc, g->fdesc_cap, d.size(), sizeof(fgb::ClothDesc)));
  FGB_CUDA(dgrow(g->d_fwork, g->fwork_cap, std::max<size_t>(fw.size() / 4, 1), sizeof(int4)));
  if (!g->d_fcounter) FGB_CUDA(cudaMalloc(&g->d_fcounter, sizeof(int)));
  FGB_CUDA(cudaMemcpyAsync(g->d_fdesc, d.data(), d.size() * sizeof(fgb::ClothDesc), cudaMemcpyHostToDevice, st));
  if (n_fw) FGB_CUDA(cudaMemcpyAsync(g->d_fwork, fw.data(), fw.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  int from = par;
  if ((ratio & 1u) == 0) {
    FGB_CUDA(S::launch_copy_unskipped(g->d_fdesc, int(d.size()), par, st));
    from = par ^ 1;
  }
  int ctas = s->ctas;
  if (s->mode != 1 || ctas <= 0) {
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    ctas = fgb::batched_ctas_per_sm(s->tile_h) * sms;
  }
  ctas = std::max(1, std::min(ctas, n_fw));
  for (uint32_t j = 0; j < ratio && n_fw > 0; ++j) {
    FGB_CUDA(cudaMemsetAsync(g->d_fcounter, 0, sizeof(int), st));
    FGB_CUDA(fgb::launch_step_batched(g->d_fdesc, g->d_fwork, n_fw, g->d_fcounter, from ^ int(j & 1u), 1, ctas, fc,
                                      st, s->d_maps, nullptr, s->tile_h));
  }
  FGB_CUDA(cudaStreamSynchronize(st));  // the host table must outlive its upload
  return FGB_OK;
}

// ---- checked rollout decided on the device ---------------------------------

constexpr int kHostDecides = 1;  // not an error: run the host-decided loop instead

// Inputs of the graph-built rollout that stay fixed for one call.
struct Rollout {
  uint32_t ratio = 1;
  int n_tiles = 0, n_cloths = 0, n_batch = 0, ctas = 1;
  fgb::StepConsts coarse, fine;
  float3 gforce;
  float growth = 0.0f, abs_margin = 0.0f, max_strain = 0.0f;
};

// The fallback of the cloths that failed this step (the body of the graph's
// conditional): the same fine steps as fine_fallback, with the failing set
// and the compacted work list made on the device, then a re-check whose
// energies the failing cloths accept.  Launched on `bs` while it captures.
int capture_fallback(fgb_surrogate* g, fgb_sim* s, const Rollout& ro, int par, cudaStream_t bs) {
  if (s->batch.empty()) {
    fgb_mesh* m = s->meshes[0];
    const fgb::GridTopo gt{int(m->topo.rows), int(m->topo.cols), m->d_grid, 0};
    fgb::StepConsts mc = ro.fine;
    mc.flags = m->d_flags;
    int a = par;
    for (uint32_t j = 0; j < ro.ratio; ++j, a ^= 1)
      FGB_CUDA(fgb::launch_step_grid(gt, static_cast<const float4*>(m->pos[a]), static_cast<const float4*>(m->vel[a]),
                                     nullptr, static_cast<float4*>(m->pos[a ^ 1]), static_cast<float4*>(m->vel[a ^ 1]),
                                     mc, bs));
    if (a != (par ^ 1)) {
      const size_t bytes = size_t(m->topo.n) * sizeof(float4);
      FGB_CUDA(cudaMemcpyAsync(m->pos[par ^ 1], m->pos[a], bytes, cudaMemcpyDeviceToDevice, bs));
      FGB_CUDA(cudaMemcpyAsync(m->vel[par ^ 1], m->vel[a], bytes, cudaMemcpyDeviceToDevice, bs));
    }
  } else {
    const int nb = ro.n_batch;
    int* off = g->d_bidx;
    int* cnt = off + nb;
    int* mesh = cnt + nb;
    int* dst = mesh + nb;
    FGB_CUDA(S::launch_fallback_tables(s->d_desc, mesh, nb, g->d_fail, off, cnt, s->d_work, g->d_fdesc, dst,
                                       g->d_fwork, g->d_counts + 1, bs));
    int from = par;
    if ((ro.ratio & 1u) == 0) {
      FGB_CUDA(S::launch_copy_unskipped(g->d_fdesc, nb, par, bs));
      from = par ^ 1;
    }
    for (uint32_t j = 0; j < ro.ratio; ++j) {
      FGB_CUDA(cudaMemsetAsync(g->d_fcounter, 0, sizeof(int), bs));
      FGB_CUDA(fgb::launch_step_batched(g->d_fdesc, g->d_fwork, s->n_work, g->d_fcounter, from ^ int(j & 1u), 1,
                                        ro.ctas, ro.fine, bs, s->d_maps, g->d_counts + 1, s->tile_h));
    }
  }
  FGB_CUDA(S::launch_check(g->d_cloths, g->d_tiles, ro.n_tiles, ro.n_cloths, par ^ 1, ro.gforce, g->d_tile_chk,
                           g->d_cloth_chk, bs));
  FGB_CUDA(S::launch_accept(g->d_cloth_chk, ro.n_cloths, g->d_fail, g->d_e_old, bs));
  return FGB_OK;
}

// One coarse step from buffers [par] as a graph: surrogate step, check,
// verdicts, and the fallback body under an IF conditional the verdict
// kernel sets.
int capture_checked_step(fgb_surrogate* g, fgb_sim* s, const Rollout& ro, int par, cudaStream_t st,
                         cudaGraphExec_t* out) {
  FGB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  int rc = FGB_OK;
  cudaError_t e = cudaSuccess;
  do {
    if ((e = cudaMemsetAsync(g->d_counts, 0, sizeof(int), st)) != cudaSuccess) break;
    if ((e = S::launch_sur_step(g->d_cloths, g->d_tiles, ro.n_tiles, par, g->d_blob, g->norm, ro.coarse, g->groups, 0,
                                g->d_err, st)) != cudaSuccess)
      break;
    if ((e = S::launch_check(g->d_cloths, g->d_tiles, ro.n_tiles, ro.n_cloths, par ^ 1, ro.gforce, g->d_tile_chk,
                             g->d_cloth_chk, st)) != cudaSuccess)
      break;
    if ((e = S::launch_decide(g->d_cloth_chk, ro.n_cloths, g->d_e_old, g->d_e_ref, ro.growth, ro.abs_margin,
                              ro.max_strain, g->d_fail, g->d_counts, st)) != cudaSuccess)
      break;
    cudaStreamCaptureStatus cs;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    if ((e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &cg, nullptr, nullptr, nullptr)) != cudaSuccess) break;
    cudaGraphConditionalHandle h;
    if ((e = cudaGraphConditionalHandleCreate(&h, cg, 0, cudaGraphCondAssignDefault)) != cudaSuccess) break;
    if ((e = S::launch_set_fallback(h, g->d_counts, g->d_total, st)) != cudaSuccess) break;
    if ((e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &cg, &deps, nullptr, &nd)) != cudaSuccess) break;
    cudaGraphNodeParams cp{};  // every member zero
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeIf;
    cp.conditional.size = 1;
    cudaGraphNode_t cn;
    if ((e = cudaGraphAddNode(&cn, cg, deps, nullptr, nd, &cp)) != cudaSuccess) break;
    if ((e = cudaStreamUpdateCaptureDependencies(st, &cn, nullptr, 1, cudaStreamSetCaptureDependencies)) !=
        cudaSuccess)
      break;
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    if ((e = cudaStreamBeginCaptureToGraph(g->side, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) !=
        cudaSuccess)
      break;
    rc = capture_fallback(g, s, ro, par, g->side);
    cudaGraph_t body_out = nullptr;
    const cudaError_t eb = cudaStreamEndCapture(g->side, &body_out);
    if (rc == FGB_OK && eb != cudaSuccess) e = eb;
  } while (false);
  cudaGraph_t graph = nullptr;
  const cudaError_t ee = cudaStreamEndCapture(st, &graph);
  if (rc == FGB_OK && e == cudaSuccess) e = ee;
  if (rc != FGB_OK || e != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    return rc != FGB_OK ? rc : fail(FGB_ECUDA, cudaGetErrorString(e));
  }
  e = cudaGraphInstantiate(out, graph, 0);
  cudaGraphDestroy(graph);
  FGB_CUDA(e);
  return FGB_OK;
}

// The checked rollout with every decision on the device: one graph launch
// per coarse step and one host wait at the end.  Decisions, fallbacks and
// states equal the host-decided loop's (the same kernels; the verdict is the
// same double-precision test).  Returns kHostDecides before touching the
// state when the graph cannot be built (the caller then decides on the host).
int rollout_on_device(fgb_surrogate* g, fgb_sim* s, uint32_t ratio, uint64_t n_coarse,
                      const fgb_surrogate_check* chk, int n_tiles, const fgb::StepConsts& cst,
                      const std::vector<float2>& e_old, const std::vector<double>& e_ref, cudaStream_t st,
                      uint64_t* n_fallbacks) {
  Rollout ro;
  ro.ratio = ratio;
  ro.n_tiles = n_tiles;
  ro.n_cloths = int(s->meshes.size());
  ro.n_batch = int(s->batch.size());
  ro.coarse = cst;
  ro.fine = fgb::detail::make_consts(s->cfg, s->d_faces, s->n_faces, nullptr, &s->accel);
  ro.gforce = make_float3(s->cfg.gravity[0], s->cfg.gravity[1], s->cfg.gravity[2]);
  ro.growth = chk->energy_growth;
  ro.abs_margin = chk->energy_abs;
  ro.max_strain = chk->max_strain;
  const int nc = ro.n_cloths, nb = ro.n_batch;
  if (nb == 0 && nc != 1) return kHostDecides;
  std::vector<int> bidx;
  if (nb > 0) {
    // each batch cloth's work items are one contiguous range of the list
    bidx.assign(4 * size_t(nb), 0);
    std::vector<char> seen(nb, 0);
    int prev = -1;
    for (size_t i = 0; i + 3 < s->work_host.size(); i += 4) {
      const int b = s->work_host[i];
      if (b < 0 || b >= nb) return kHostDecides;
      if (b != prev) {
        if (seen[b]) return kHostDecides;
        seen[b] = 1;
        bidx[b] = int(i / 4);
        prev = b;
      }
      ++bidx[nb + b];
    }
    for (int b = 0; b < nb; ++b) {
      const size_t mi = size_t(std::find(s->meshes.begin(), s->meshes.end(), s->batch[b]) - s->meshes.begin());
      if (mi >= s->meshes.size()) return kHostDecides;
      bidx[2 * nb + b] = int(mi);
    }
    int ctas = s->ctas;
    if (s->mode != 1 || ctas <= 0) {
      int dev = 0, sms = 1;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      ctas = fgb::batched_ctas_per_sm(s->tile_h) * sms;
    }
    ro.ctas = std::max(1, std::min(ctas, s->n_work));
    FGB_CUDA(dgrow(g->d_bidx, g->bidx_cap, bidx.size(), sizeof(int)));
    FGB_CUDA(dgrow(g->d_fdesc, g->fdesc_cap, size_t(nb), sizeof(fgb::ClothDesc)));
    FGB_CUDA(dgrow(g->d_fwork, g->fwork_cap, size_t(std::max(s->n_work, 1)), sizeof(int4)));
    if (!g->d_fcounter) FGB_CUDA(cudaMalloc(&g->d_fcounter, sizeof(int)));
  }
  FGB_CUDA(dgrow(g->d_e_old, g->e_old_cap, size_t(nc), sizeof(float)));
  FGB_CUDA(dgrow(g->d_e_ref, g->e_ref_cap, size_t(nc), sizeof(double)));
  FGB_CUDA(dgrow(g->d_fail, g->fail_cap, size_t(nc), sizeof(int)));
  if (!g->d_counts) FGB_CUDA(cudaMalloc(&g->d_counts, 2 * sizeof(int)));
  if (!g->d_total) FGB_CUDA(cudaMalloc(&g->d_total, sizeof(unsigned long long)));
  if (!g->side) FGB_CUDA(cudaStreamCreateWithFlags(&g->side, cudaStreamNonBlocking));
  std::vector<float> e0(nc);
  for (int c = 0; c < nc; ++c) e0[c] = e_old[c].x;
  FGB_CUDA(cudaMemcpyAsync(g->d_e_old, e0.data(), nc * sizeof(float), cudaMemcpyHostToDevice, st));
  FGB_CUDA(cudaMemcpyAsync(g->d_e_ref, e_ref.data(), nc * sizeof(double), cudaMemcpyHostToDevice, st));
  if (nb > 0)
    FGB_CUDA(cudaMemcpyAsync(g->d_bidx, bidx.data(), bidx.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  FGB_CUDA(cudaMemsetAsync(g->d_total, 0, sizeof(unsigned long long), st));
  FGB_CUDA(cudaStreamSynchronize(st));  // the host tables must outlive their upload
  FGB_CUDA(S::prime_sur_step(g->groups));
  FGB_CUDA(fgb::prime_step_kernels());

  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  const int p0 = s->parity;
  int rc = capture_checked_step(g, s, ro, p0, st, &exec[p0]);
  if (rc == FGB_OK && n_coarse > 1) rc = capture_checked_step(g, s, ro, p0 ^ 1, st, &exec[p0 ^ 1]);
  if (rc != FGB_OK) {
    for (cudaGraphExec_t x : exec)
      if (x) cudaGraphExecDestroy(x);
    cudaGetLastError();
    return kHostDecides;
  }
  cudaError_t e = cudaSuccess;
  for (uint64_t k = 0; k < n_coarse && e == cudaSuccess; ++k) {
    e = cudaGraphLaunch(exec[s->parity], st);
    if (e != cudaSuccess) break;
    s->parity ^= 1;
    for (fgb_mesh* m : s->meshes) {
      m->cur = s->parity;
      m->has_force = false;
      m->staged = false;
    }
  }
  unsigned long long total = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&total, g->d_total, sizeof(total), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  for (cudaGraphExec_t x : exec)
    if (x) cudaGraphExecDestroy(x);
  FGB_CUDA(e);
  if (n_fallbacks) *n_fallbacks = total;
  return FGB_OK;
}

}  // namespace

extern "C" {

int fgb_surrogate_new(uint64_t seed, fgb_surrogate** out) {
  if (!out) return fail(FGB_EINVAL, "null output");
  *out = nullptr;
  fgb_surrogate* g = new (std::nothrow) fgb_surrogate();
  if (!g) return fail(FGB_ENOMEM, "out of host memory");
  int rc = FGB_OK;
  do {
    if (cudaGetDevice(&g->device) != cudaSuccess) {
      rc = fail(FGB_ECUDA, "no CUDA device");
      break;
    }
    if (cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&g->d_master, S::kNumParams * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&g->d_m, S::kNumParams * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&g->d_v, S::kNumParams * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&g->d_blob, S::kBlobBytes) != cudaSuccess || cudaMalloc(&g->d_err, sizeof(int)) != cudaSuccess ||
        cudaMemset(g->d_err, 0, sizeof(int)) != cudaSuccess || cudaMemset(g->d_blob, 0, S::kBlobBytes) != cudaSuccess) {
      rc = fail(FGB_ECUDA, "device allocation failed");
      break;
    }
    std::vector<float> flat(kFlat, 0.0f);
    Rng r{seed};
    float* q = flat.data();
    const float a1 = std::sqrt(6.0f / float(S::kFeat + S::kHid)), a2 = std::sqrt(6.0f / float(2 * S::kHid)),
                a3 = std::sqrt(6.0f / float(S::kHid + S::kOut));
    for (int i = 0; i < S::kHid * S::kFeat; ++i) *q++ = r.uniform(a1);
    q += S::kHid;
    for (int i = 0; i < S::kHid * S::kHid; ++i) *q++ = r.uniform(a2);
    q += S::kHid;
    for (int i = 0; i < S::kOut * S::kHid; ++i) *q++ = r.uniform(a3);
    flat_to_padded(flat.data(), g->master);
    for (int k = 0; k < S::kFeat; ++k) {
      g->norm.in_mean[k] = 0.0f;
      g->norm.in_inv_std[k] = 1.0f;
    }
    for (int k = 0; k < S::kOut; ++k) {
      g->norm.out_mean[k] = 0.0f;
      g->norm.out_std[k] = 1.0f;
    }
    rc = upload_master(g, true);
  } while (false);
  if (rc != FGB_OK) {
    fgb_surrogate_destroy(g);
    return rc;
  }
  *out = g;
  return FGB_OK;
}

int fgb_surrogate_destroy(fgb_surrogate* g) {
  if (!g) return FGB_OK;
  cudaSetDevice(g->device);
  if (g->stream) cudaStreamSynchronize(g->stream);
  dfree(g->d_master);
  dfree(g->d_m);
  dfree(g->d_v);
  dfree(g->d_blob);
  dfree(g->d_feat);
  dfree(g->d_tgt);
  dfree(g->d_X);
  dfree(g->d_T);
  dfree(g->d_xin);
  dfree(g->d_tin);
  dfree(g->d_partials);
  dfree(g->d_loss);
  dfree(g->d_grad);
  dfree(g->d_stats);
  dfree(g->d_err);
  dfree(g->d_cloths);
  dfree(g->d_tiles);
  dfree(g->d_tile_chk);
  dfree(g->d_cloth_chk);
  dfree(g->d_out);
  dfree(g->d_fdesc);
  dfree(g->d_fwork);
  dfree(g->d_fcounter);
  dfree(g->d_e_old);
  dfree(g->d_e_ref);
  dfree(g->d_fail);
  dfree(g->d_bidx);
  dfree(g->d_counts);
  dfree(g->d_total);
  if (g->side) cudaStreamDestroy(g->side);
  if (g->stream) cudaStreamDestroy(g->stream);
  delete g;
  return FGB_OK;
}

int fgb_surrogate_get_params(fgb_surrogate* g, float* out) {
  if (!g || !out) return fail(FGB_EINVAL, "null argument");
  FGB_CHECK_RC(sync_host_master(g));
  padded_to_flat(g->master.data(), out);
  return FGB_OK;
}

int fgb_surrogate_set_params(fgb_surrogate* g, const float* in) {
  if (!g || !in) return fail(FGB_EINVAL, "null argument");
  for (int i = 0; i < kFlat; ++i)
    if (!std::isfinite(in[i])) return fail(FGB_EINVAL, "non-finite parameter");
  flat_to_padded(in, g->master);
  return upload_master(g, true);
}

int fgb_surrogate_set_normalization(fgb_surrogate* g, const float* in_mean, const float* in_std,
                                    const float* out_mean, const float* out_std) {
  if (!g || !in_mean || !in_std || !out_mean || !out_std) return fail(FGB_EINVAL, "null argument");
  for (int k = 0; k < S::kFeat; ++k)
    if (!(in_std[k] > 0.0f) || !std::isfinite(in_std[k]) || !std::isfinite(in_mean[k]))
      return fail(FGB_EINVAL, "input standard deviations must be finite and positive");
  for (int k = 0; k < S::kOut; ++k)
    if (!(out_std[k] > 0.0f) || !std::isfinite(out_std[k]) || !std::isfinite(out_mean[k]))
      return fail(FGB_EINVAL, "output standard deviations must be finite and positive");
  for (int k = 0; k < S::kFeat; ++k) {
    g->norm.in_mean[k] = in_mean[k];
    g->norm.in_inv_std[k] = 1.0f / in_std[k];
  }
  for (int k = 0; k < S::kOut; ++k) {
    g->norm.out_mean[k] = out_mean[k];
    g->norm.out_std[k] = out_std[k];
  }
  return FGB_OK;
}

int fgb_surrogate_get_normalization(const fgb_surrogate* g, float* in_mean, float* in_std, float* out_mean,
                                    float* out_std) {
  if (!g) return fail(FGB_EINVAL, "null surrogate");
  for (int k = 0; k < S::kFeat; ++k) {
    if (in_mean) in_mean[k] = g->norm.in_mean[k];
    if (in_std) in_std[k] = 1.0f / g->norm.in_inv_std[k];
  }
  for (int k = 0; k < S::kOut; ++k) {
    if (out_mean) out_mean[k] = g->norm.out_mean[k];
    if (out_std) out_std[k] = g->norm.out_std[k];
  }
  return FGB_OK;
}

int fgb_surrogate_features(fgb_surrogate* g, fgb_mesh* m, float coarse_dt, const float* wind, float* out) {
  if (!g || !m || !out) return fail(FGB_EINVAL, "null argument");
  if (!(coarse_dt > 0.0f) || !std::isfinite(coarse_dt)) return fail(FGB_EINVAL, "coarse_dt must be positive");
  FGB_CHECK_RC(fgb::detail::ensure_device(m));
  if (m->active_path != 2 || m->precision != 32) return fail(FGB_EINVAL, "features need a grid mesh (f32 grid path)");
  FGB_CHECK_RC(ensure_rest(m));
  float w[3] = {0.0f, 0.0f, 0.0f};
  for (int k = 0; k < 3; ++k) w[k] = wind ? wind[k] : (m->has_wind ? m->wind[k] : 0.0f);
  std::vector<S::SurCloth> cl{make_cloth(m, coarse_dt, w, 0)};
  std::vector<S::Tile> tiles;
  add_tiles(0, cl[0], tiles);
  FGB_CHECK_RC(upload_tables(g, cl, tiles, m->stream));
  const size_t n = m->topo.n;
  FGB_CUDA(dgrow(g->d_out, g->out_cap, n * S::kFeat, sizeof(float)));
  FGB_CUDA(S::launch_features(g->d_cloths, g->d_tiles, int(tiles.size()), m->cur, g->d_out, m->stream));
  FGB_CUDA(cudaMemcpyAsync(out, g->d_out, n * S::kFeat * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
  FGB_CUDA(cudaStreamSynchronize(m->stream));
  return FGB_OK;
}

int fgb_surrogate_forward(fgb_surrogate* g, const float* x, uint64_t n, float* y) {
  if (!g || (n && (!x || !y))) return fail(FGB_EINVAL, "null argument");
  if (n == 0) return FGB_OK;
  if (n > (1ull << 30)) return fail(FGB_EINVAL, "too many rows");
  const uint64_t n_pad = (n + S::kTile - 1) / S::kTile * S::kTile;
  FGB_CHECK_RC(stage_rows(g, x, nullptr, n, n_pad));
  FGB_CUDA(S::launch_forward(g->d_X, int(n_pad), g->d_blob, g->d_T, g->d_err, g->stream));
  std::vector<float> Y(n_pad * 4);
  FGB_CUDA(cudaMemcpyAsync(Y.data(), g->d_T, n_pad * 4 * sizeof(float), cudaMemcpyDeviceToHost, g->stream));
  FGB_CHECK_RC(check_err(g, g->stream));
  for (uint64_t i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) y[3 * i + k] = Y[4 * i + k];
  return FGB_OK;
}

int fgb_surrogate_gradients(fgb_surrogate* g, const float* x, const float* t, uint64_t n, float* grad, float* loss) {
  if (!g || !x || !t || !grad) return fail(FGB_EINVAL, "null argument");
  if (n == 0 || n % S::kTile || n > (1ull << 30)) return fail(FGB_EINVAL, "n must be a positive multiple of 128");
  FGB_CHECK_RC(stage_rows(g, x, t, n, n));
  const int ctas = S::train_ctas(int(n));
  FGB_CHECK_RC(ensure_train_scratch(g, ctas, 1));
  FGB_CUDA(dgrow(g->d_grad, g->grad_cap, S::kNumParams, sizeof(float)));
  FGB_CUDA(S::launch_train(g->d_X, g->d_T, int(n), g->d_blob, g->d_partials, ctas, g->d_err, g->stream));
  FGB_CUDA(S::launch_reduce_grad(g->d_partials, ctas, 1.0f / (3.0f * float(n)), g->d_grad, g->d_loss, g->stream));
  std::vector<float> P(S::kNumParams);
  float l = 0.0f;
  FGB_CUDA(cudaMemcpyAsync(P.data(), g->d_grad, S::kNumParams * sizeof(float), cudaMemcpyDeviceToHost, g->stream));
  FGB_CUDA(cudaMemcpyAsync(&l, g->d_loss, sizeof(float), cudaMemcpyDeviceToHost, g->stream));
  FGB_CHECK_RC(check_err(g, g->stream));
  padded_to_flat(P.data(), grad);
  if (loss) *loss = l;
  return FGB_OK;
}

int fgb_surrogate_train_batch(fgb_surrogate* g, const float* x, const float* t, uint64_t n, float lr, float* loss) {
  if (!g || !x || !t) return fail(FGB_EINVAL, "null argument");
  if (n == 0 || n % S::kTile || n > (1ull << 30)) return fail(FGB_EINVAL, "n must be a positive multiple of 128");
  if (!(lr >= 0.0f) || !std::isfinite(lr)) return fail(FGB_EINVAL, "bad learning rate");
  FGB_CHECK_RC(stage_rows(g, x, t, n, n));
  FGB_CHECK_RC(ensure_train_scratch(g, S::train_ctas(int(n)), 1));
  FGB_CHECK_RC(adam_step(g, n, lr, g->d_loss));
  float l = 0.0f;
  FGB_CUDA(cudaMemcpyAsync(&l, g->d_loss, sizeof(float), cudaMemcpyDeviceToHost, g->stream));
  FGB_CHECK_RC(check_err(g, g->stream));
  if (loss) *loss = l;
  return FGB_OK;
}

int fgb_surrogate_dataset_reserve(fgb_surrogate* g, uint64_t capacity_rows) {
  if (!g || capacity_rows == 0 || capacity_rows > (1ull << 34)) return fail(FGB_EINVAL, "bad capacity");
  FGB_CUDA(cudaStreamSynchronize(g->stream));
  dfree(g->d_feat);
  dfree(g->d_tgt);
  g->cap = g->count = g->head = 0;
  FGB_CUDA(cudaMalloc(&g->d_feat, capacity_rows * S::kRawStride * sizeof(float)));
  FGB_CUDA(cudaMalloc(&g->d_tgt, capacity_rows * 4 * sizeof(float)));
  g->cap = (long long)capacity_rows;
  return FGB_OK;
}

int fgb_surrogate_collect(fgb_surrogate* g, fgb_sim* s, uint32_t ratio, uint64_t n_coarse) {
  if (!g || !s) return fail(FGB_EINVAL, "null argument");
  if (ratio == 0) return fail(FGB_EINVAL, "ratio must be >= 1");
  if (g->cap == 0) return fail(FGB_ESTATE, "call fgb_surrogate_dataset_reserve first");
  FGB_CHECK_RC(fgb::detail::ensure_sim(s));
  FGB_CHECK_RC(check_grid_sim(s));
  const float T = float(ratio) * s->cfg.dt;
  if (!(T > 0.0f)) return fail(FGB_EINVAL, "dt must be positive");
  long long total = 0;
  for (fgb_mesh* m : s->meshes) total += (long long)m->topo.n;
  if (total > g->cap) return fail(FGB_EINVAL, "the dataset ring is smaller than one snapshot of the simulation");
  std::vector<S::SurCloth> cl;
  std::vector<S::Tile> tiles;
  for (uint64_t k = 0; k < n_coarse; ++k) {
    cudaStream_t st = fgb::detail::sim_stream(s);
    align_parity(s);
    FGB_CHECK_RC(build_sim_tables(g, s, T, g->head, cl, tiles, st));
    FGB_CUDA(S::launch_collect_features(g->d_cloths, g->d_tiles, int(tiles.size()), s->parity, g->d_feat, g->d_tgt,
                                        g->cap, st));
    FGB_CUDA(cudaStreamSynchronize(st));
    FGB_CHECK_RC(fgb_sim_step(s, ratio));
    st = fgb::detail::sim_stream(s);
    align_parity(s);
    FGB_CHECK_RC(build_sim_tables(g, s, T, g->head, cl, tiles, st));
    FGB_CUDA(S::launch_collect_targets(g->d_cloths, g->d_tiles, int(tiles.size()), s->parity, g->d_tgt, g->cap, st));
    FGB_CUDA(cudaStreamSynchronize(st));
    g->head = (g->head + total) % g->cap;
    g->count = std::min(g->cap, g->count + total);
  }
  return FGB_OK;
}

int fgb_surrogate_dataset_info(const fgb_surrogate* g, uint64_t out[2]) {
  if (!g || !out) return fail(FGB_EINVAL, "null argument");
  out[0] = uint64_t(g->count);
  out[1] = uint64_t(g->cap);
  return FGB_OK;
}

int fgb_surrogate_dataset_get(fgb_surrogate* g, uint64_t first, uint64_t n, float* feat, float* tgt) {
  if (!g) return fail(FGB_EINVAL, "null surrogate");
  const uint64_t count = uint64_t(g->count);
  if (first > count || n > count - first) return fail(FGB_EINDEX, "rows beyond the dataset");
  if (n == 0) return FGB_OK;
  std::vector<float> F(n * S::kRawStride), Tt(n * 4);
  FGB_CUDA(cudaMemcpy(F.data(), g->d_feat + first * S::kRawStride, F.size() * sizeof(float), cudaMemcpyDeviceToHost));
  FGB_CUDA(cudaMemcpy(Tt.data(), g->d_tgt + first * 4, Tt.size() * sizeof(float), cudaMemcpyDeviceToHost));
  for (uint64_t i = 0; i < n; ++i) {
    if (feat)
      for (int k = 0; k < S::kFeat; ++k) feat[i * S::kFeat + k] = F[i * S::kRawStride + k];
    if (tgt)
      for (int k = 0; k < 3; ++k) tgt[i * 3 + k] = Tt[i * 4 + k];
  }
  return FGB_OK;
}

int fgb_surrogate_fit_normalization(fgb_surrogate* g) {
  if (!g) return fail(FGB_EINVAL, "null surrogate");
  if (g->count == 0) return fail(FGB_ESTATE, "the dataset is empty");
  constexpr int kBlocks = 64, kCols = S::kFeat + S::kOut;
  FGB_CUDA(dgrow(g->d_stats, g->stats_cap, size_t(kCols) * kBlocks * 2, sizeof(double)));
  FGB_CUDA(S::launch_stats(g->d_feat, g->d_tgt, g->count, g->d_stats, kBlocks, g->stream));
  std::vector<double> P(size_t(kCols) * kBlocks * 2);
  FGB_CUDA(cudaMemcpyAsync(P.data(), g->d_stats, P.size() * sizeof(double), cudaMemcpyDeviceToHost, g->stream));
  FGB_CUDA(cudaStreamSynchronize(g->stream));
  float mean[kCols], sd[kCols];
  for (int j = 0; j < kCols; ++j) {
    double s = 0.0, q = 0.0;
    for (int b = 0; b < kBlocks; ++b) {
      s += P[(size_t(j) * kBlocks + b) * 2];
      q += P[(size_t(j) * kBlocks + b) * 2 + 1];
    }
    const double m = s / double(g->count);
    const double var = std::max(0.0, q / double(g->count) - m * m);
    const double d = std::sqrt(var);
    mean[j] = float(m);
    sd[j] = d < 1e-6 ? 1.0f : float(d);
  }
  return fgb_surrogate_set_normalization(g, mean, sd, mean + S::kFeat, sd + S::kFeat);
}

int fgb_surrogate_train(fgb_surrogate* g, uint64_t n_steps, uint64_t batch, float lr, uint64_t seed, float* losses) {
  if (!g) return fail(FGB_EINVAL, "null surrogate");
  if (batch == 0 || batch % S::kTile || batch > (1ull << 28)) return fail(FGB_EINVAL, "batch must be a positive multiple of 128");
  if (!(lr >= 0.0f) || !std::isfinite(lr)) return fail(FGB_EINVAL, "bad learning rate");
  if (g->count == 0) return fail(FGB_ESTATE, "the dataset is empty");
  if (n_steps == 0) return FGB_OK;
  FGB_CUDA(dgrow(g->d_X, g->X_cap, size_t(batch) * S::kIn * 2, 1));
  FGB_CUDA(dgrow(g->d_T, g->T_cap, size_t(batch) * 4, sizeof(float)));
  FGB_CHECK_RC(ensure_train_scratch(g, S::train_ctas(int(batch)), size_t(n_steps)));
  for (uint64_t k = 0; k < n_steps; ++k) {
    const uint64_t bseed = seed * 0x2545F4914F6CDD1DULL + k * 0x9E3779B97F4A7C15ULL;
    FGB_CUDA(S::launch_pack_batch(g->d_feat, g->d_tgt, g->count, bseed, int(batch), g->norm, g->d_X, g->d_T,
                                  g->stream));
    FGB_CHECK_RC(adam_step(g, batch, lr, g->d_loss + k));
  }
  if (losses)
    FGB_CUDA(cudaMemcpyAsync(losses, g->d_loss, n_steps * sizeof(float), cudaMemcpyDeviceToHost, g->stream));
  return check_err(g, g->stream);
}

int fgb_sim_step_surrogate(fgb_sim* s, fgb_surrogate* g, uint32_t ratio, uint64_t n_coarse,
                           const fgb_surrogate_check* chk, uint64_t* n_fallbacks) {
  if (!s || !g) return fail(FGB_EINVAL, "null argument");
  if (ratio == 0) return fail(FGB_EINVAL, "ratio must be >= 1");
  if (n_fallbacks) *n_fallbacks = 0;
  FGB_CHECK_RC(fgb::detail::ensure_sim(s));
  FGB_CHECK_RC(check_grid_sim(s));
  const float T = float(ratio) * s->cfg.dt;
  if (!(T > 0.0f)) return fail(FGB_EINVAL, "dt must be positive");
  if (n_coarse == 0) return FGB_OK;
  cudaStream_t st = fgb::detail::sim_stream(s);
  FGB_CUDA(cudaStreamSynchronize(g->stream));  // training writes to the blob are done
  align_parity(s);
  std::vector<S::SurCloth> cl;
  std::vector<S::Tile> tiles;
  FGB_CHECK_RC(build_sim_tables(g, s, T, 0, cl, tiles, st));
  const int n_tiles = int(tiles.size());
  fgb_config cc = s->cfg;
  cc.dt = T;
  const fgb::StepConsts cst = fgb::detail::make_consts(cc, s->d_faces, s->n_faces, nullptr, &s->accel);
  const bool checks = chk && chk->enabled;
  std::vector<float2> e_old, e_new;
  std::vector<double> e_ref(s->meshes.size());
  {
    const double gmag = std::sqrt(double(s->cfg.gravity[0]) * s->cfg.gravity[0] +
                                  double(s->cfg.gravity[1]) * s->cfg.gravity[1] +
                                  double(s->cfg.gravity[2]) * s->cfg.gravity[2]);
    for (size_t c = 0; c < s->meshes.size(); ++c)
      e_ref[c] = double(s->meshes[c]->topo.n) * gmag * double(mesh_spacing(s->meshes[c]));
  }
  if (checks) {
    FGB_CHECK_RC(run_check(g, s, n_tiles, s->parity, e_old, st));
    // the margin's scale is fixed for the whole call, so the allowed growth is
    // linear in the number of coarse steps, never compounding
    for (size_t c = 0; c < s->meshes.size(); ++c) e_ref[c] += std::fabs(double(e_old[c].x));
  }
  if (checks && s->graphs) {
    const int rd = rollout_on_device(g, s, ratio, n_coarse, chk, n_tiles, cst, e_old, e_ref, st, n_fallbacks);
    if (rd != kHostDecides) return rd == FGB_OK ? check_err(g, st) : rd;
  }
  uint64_t fallbacks = 0;
  std::vector<int> failing;
  for (uint64_t k = 0; k < n_coarse; ++k) {
    const int par = s->parity;
    FGB_CUDA(S::launch_sur_step(g->d_cloths, g->d_tiles, n_tiles, par, g->d_blob, g->norm, cst, g->groups, 0,
                                g->d_err, st));
    if (checks) {
      FGB_CHECK_RC(run_check(g, s, n_tiles, par ^ 1, e_new, st));
      failing.clear();
      for (size_t c = 0; c < s->meshes.size(); ++c) {
        const double E0 = e_old[c].x, E1 = e_new[c].x, S1 = e_new[c].y;
        const double margin = double(chk->energy_growth) * e_ref[c] + double(chk->energy_abs);
        const bool ok = std::isfinite(E1) && std::isfinite(S1) && (E1 <= E0 + margin) &&
                        (S1 <= double(chk->max_strain));
        if (!ok) failing.push_back(int(c));
      }
      if (!failing.empty()) {
        fallbacks += failing.size();
        FGB_CHECK_RC(fine_fallback(g, s, failing, par, ratio, st));
        FGB_CHECK_RC(run_check(g, s, n_tiles, par ^ 1, e_new, st));
      }
      e_old.swap(e_new);
    }
    s->parity ^= 1;
    for (fgb_mesh* m : s->meshes) {
      m->cur = s->parity;
      m->has_force = false;
      m->staged = false;
    }
  }
  if (n_fallbacks) *n_fallbacks = fallbacks;
  return check_err(g, st);
}

int fgb_sim_energy(fgb_sim* s, float* out) {
  if (!s || !out) return fail(FGB_EINVAL, "null argument");
  FGB_CHECK_RC(fgb::detail::ensure_sim(s));
  FGB_CHECK_RC(check_grid_sim(s));
  cudaStream_t st = fgb::detail::sim_stream(s);
  align_parity(s);
  fgb_surrogate tmp;  // tables only
  std::vector<S::SurCloth> cl;
  std::vector<S::Tile> tiles;
  int rc = build_sim_tables(&tmp, s, s->cfg.dt > 0.0f ? s->cfg.dt : 1.0f, 0, cl, tiles, st);
  std::vector<float2> e;
  if (rc == FGB_OK) rc = run_check(&tmp, s, int(tiles.size()), s->parity, e, st);
  dfree(tmp.d_cloths);
  dfree(tmp.d_tiles);
  dfree(tmp.d_tile_chk);
  dfree(tmp.d_cloth_chk);
  if (rc != FGB_OK) return rc;
  for (size_t c = 0; c < e.size(); ++c) {
    out[2 * c] = e[c].x;
    out[2 * c + 1] = e[c].y;
  }
  return FGB_OK;
}

}  // extern "C"
