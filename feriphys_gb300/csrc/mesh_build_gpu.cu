// SpringyMesh::new's strut de-duplication on the GPU (springy_mesh.rs:284-345)
// for meshes of millions of vertices.
//
// The reference walks the triangles in order and inserts each edge
// (v0,v1), (v1,v2), (v2,v0) into a hash map; a new key becomes the next
// strut.  Here every edge occurrence e = 3t + j gets the key
// (min(a, b) << kb | max(a, b)), 2^kb >= #vertices; a stable radix sort of (key, e) groups equal
// keys with their occurrences in ascending e, so a group's first entry is the
// occurrence that created the strut.  Flagging those occurrences in e order
// and taking an exclusive scan numbers the struts exactly in creation order.
// A manifold edge has at most two occurrences, so a group's second entry finds
// its strut id one position back; a third occurrence is the reference's
// "more than two adjacent faces" panic, reported at the smallest such e, i.e.
// at the same face and edge where the sequential loop stops.  Rest lengths and
// the 1/L scaling use the same f32 expressions as the host build, so every
// output value is bit-identical to it.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "feriphys_gb300.h"
#include "mesh_build.h"

namespace fgb {
namespace {

__host__ __device__ __forceinline__ unsigned long long edge_key(uint32_t a, uint32_t b, int kb) {
  return a <= b ? (static_cast<unsigned long long>(a) << kb) | b : (static_cast<unsigned long long>(b) << kb) | a;
}

__global__ void k_edge_keys(const uint32_t* __restrict__ idx, long long n_occ, int kb,
                            unsigned long long* __restrict__ keys, int* __restrict__ occ) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n_occ;
       e += (long long)gridDim.x * blockDim.x) {
    const long long t = e / 3;
    const int j = int(e - 3 * t);
    const uint32_t a = idx[3 * t + j], b = idx[3 * t + (j == 2 ? 0 : j + 1)];
    keys[e] = edge_key(a, b, kb);
    occ[e] = int(e);
  }
}

// first[e] = 1 when occurrence e creates its strut; *third = the smallest
// occurrence that is an edge's third (or later).
__global__ void k_heads(const unsigned long long* __restrict__ skeys, const int* __restrict__ socc, long long n,
                        int* __restrict__ first, int* __restrict__ third) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    if (i == 0 || skeys[i] != skeys[i - 1]) first[socc[i]] = 1;
    if (i >= 2 && skeys[i] == skeys[i - 2]) atomicMin(third, socc[i]);
  }
}

__device__ __forceinline__ float rest_length(const float* __restrict__ pos, uint32_t a, uint32_t b) {
  const float dx = pos[3 * size_t(a)] - pos[3 * size_t(b)];
  const float dy = pos[3 * size_t(a) + 1] - pos[3 * size_t(b) + 1];
  const float dz = pos[3 * size_t(a) + 2] - pos[3 * size_t(b) + 2];
  return sqrtf(dx * dx + dy * dy + dz * dz);
}

// Per strut (at its group's first sorted entry): ends, constants, rest length;
// per occurrence: the face's strut id.
__global__ void k_struts(const unsigned long long* __restrict__ skeys, const int* __restrict__ socc, long long n,
                         int kb, const int* __restrict__ sid, const float* __restrict__ pos,
                         const unsigned long long* __restrict__ ov_keys, const float2* __restrict__ ov_kc, int n_ov,
                         float k, float c, uint32_t* __restrict__ sa, uint32_t* __restrict__ sb,
                         float* __restrict__ sk, float* __restrict__ sc, float* __restrict__ sl,
                         uint32_t* __restrict__ fs) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const bool head = i == 0 || skeys[i] != skeys[i - 1];
    const int e = socc[i];
    const int s = head ? sid[e] : sid[socc[i - 1]];
    fs[e] = uint32_t(s);
    if (!head) continue;
    const unsigned long long key = skeys[i];
    const uint32_t a = uint32_t(key >> kb), b = uint32_t(key & ((1ull << kb) - 1));
    float kk = k, cc = c;
    int lo = 0, hi = n_ov;  // overrides sorted by key, one entry per key
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (ov_keys[mid] < key) lo = mid + 1;
      else hi = mid;
    }
    if (lo < n_ov && ov_keys[lo] == key) {
      kk = ov_kc[lo].x;
      cc = ov_kc[lo].y;
    }
    const float L = rest_length(pos, a, b);
    sa[s] = a;
    sb[s] = b;
    sk[s] = 1.0f / L * kk;
    sc[s] = 1.0f / L * cc;
    sl[s] = L;
  }
}

struct DevBuf {
  void* p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  cudaError_t alloc(size_t bytes) { return cudaMalloc(&p, bytes ? bytes : 16); }
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

int cuda_fail(cudaError_t e, const char* what, std::string& err) {
  err = std::string(what) + ": " + cudaGetErrorString(e);
  return FGB_ECUDA;
}

#define MB_CUDA(call)                                      \
  do {                                                     \
    cudaError_t e_ = (call);                               \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call, err); \
  } while (0)

}  // namespace

int build_springy_device(const float* pos, uint64_t nv, const uint32_t* idx, uint64_t ni, float mass, float k,
                         float c, const Override* ov, uint64_t nov, MeshTopo& m, std::string& err) {
  if (nv > 0x7fffffffull) {
    err = "too many vertices (limit 2^31-1)";
    return FGB_EINVAL;
  }
  if ((nv && !pos) || (ni && !idx) || (nov && !ov)) {
    err = "null buffer with a non-zero size";
    return FGB_EINVAL;
  }
  const uint64_t nt = ni / 3;  // itertools::tuples drops a trailing remainder
  if (3 * nt > 0x7fffffffull) {
    err = "too many triangles for the device build (limit (2^31-1)/3)";
    return FGB_EINVAL;
  }
  for (uint64_t i = 0; i < 3 * nt; ++i)
    if (idx[i] >= nv) {
      err = "triangle index " + std::to_string(idx[i]) + " out of range for " + std::to_string(nv) + " vertices";
      return FGB_EINDEX;
    }
  m = MeshTopo();
  m.n = uint32_t(nv);
  m.pos.assign(pos, pos + 3 * nv);
  m.mass_per_vert = mass / float(nv);  // springy_mesh.rs:277
  m.fv.assign(idx, idx + 3 * nt);
  m.fs.assign(3 * nt, 0u);
  const long long n_occ = (long long)(3 * nt);
  if (n_occ > 0) {
    int kb = 1;
    while (kb < 32 && (1ull << kb) < nv) ++kb;
    // overrides: one entry per key, the last given wins (FxHashMap::insert);
    // keys of pairs outside the mesh can never match a strut
    std::vector<std::pair<unsigned long long, size_t>> okeys;
    for (uint64_t i = 0; i < nov; ++i)
      if (ov[i].a < nv && ov[i].b < nv) okeys.push_back({edge_key(ov[i].a, ov[i].b, kb), size_t(i)});
    std::stable_sort(okeys.begin(), okeys.end(),
                     [](const std::pair<unsigned long long, size_t>& x, const std::pair<unsigned long long, size_t>& y) {
                       return x.first < y.first;
                     });
    std::vector<unsigned long long> ok;
    std::vector<float2> okc;
    for (size_t i = 0; i < okeys.size(); ++i) {
      if (i + 1 < okeys.size() && okeys[i + 1].first == okeys[i].first) continue;
      ok.push_back(okeys[i].first);
      okc.push_back(make_float2(ov[okeys[i].second].k, ov[okeys[i].second].c));
    }
    DevBuf d_idx, d_pos, d_keys, d_occ, d_skeys, d_socc, d_first, d_sid, d_third, d_ok, d_okc, d_tmp;
    MB_CUDA(d_idx.alloc(size_t(n_occ) * sizeof(uint32_t)));
    MB_CUDA(d_pos.alloc(3 * nv * sizeof(float)));
    MB_CUDA(d_keys.alloc(size_t(n_occ) * 8));
    MB_CUDA(d_skeys.alloc(size_t(n_occ) * 8));
    MB_CUDA(d_occ.alloc(size_t(n_occ) * 4));
    MB_CUDA(d_socc.alloc(size_t(n_occ) * 4));
    MB_CUDA(d_first.alloc(size_t(n_occ) * 4));
    MB_CUDA(d_sid.alloc(size_t(n_occ) * 4));
    MB_CUDA(d_third.alloc(4));
    MB_CUDA(d_ok.alloc(ok.size() * 8));
    MB_CUDA(d_okc.alloc(okc.size() * sizeof(float2)));
    MB_CUDA(cudaMemcpy(d_idx.p, idx, size_t(n_occ) * 4, cudaMemcpyHostToDevice));
    MB_CUDA(cudaMemcpy(d_pos.p, pos, 3 * nv * sizeof(float), cudaMemcpyHostToDevice));
    if (!ok.empty()) {
      MB_CUDA(cudaMemcpy(d_ok.p, ok.data(), ok.size() * 8, cudaMemcpyHostToDevice));
      MB_CUDA(cudaMemcpy(d_okc.p, okc.data(), okc.size() * sizeof(float2), cudaMemcpyHostToDevice));
    }
    MB_CUDA(cudaMemset(d_first.p, 0, size_t(n_occ) * 4));
    const int big = 0x7fffffff;
    MB_CUDA(cudaMemcpy(d_third.p, &big, 4, cudaMemcpyHostToDevice));
    const int threads = 256;
    const int blocks = int(std::min<long long>((n_occ + threads - 1) / threads, 65536));
    k_edge_keys<<<blocks, threads>>>(d_idx.as<uint32_t>(), n_occ, kb, d_keys.as<unsigned long long>(),
                                     d_occ.as<int>());
    MB_CUDA(cudaGetLastError());
    const int end_bit = 2 * kb;
    size_t tmp_sort = 0, tmp_scan = 0;
    MB_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_sort, d_keys.as<unsigned long long>(),
                                            d_skeys.as<unsigned long long>(), d_occ.as<int>(), d_socc.as<int>(),
                                            n_occ, 0, end_bit));
    MB_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp_scan, d_first.as<int>(), d_sid.as<int>(), n_occ));
    MB_CUDA(d_tmp.alloc(std::max(tmp_sort, tmp_scan)));
    size_t tmp_bytes = std::max(tmp_sort, tmp_scan);
    MB_CUDA(cub::DeviceRadixSort::SortPairs(d_tmp.p, tmp_bytes, d_keys.as<unsigned long long>(),
                                            d_skeys.as<unsigned long long>(), d_occ.as<int>(), d_socc.as<int>(),
                                            n_occ, 0, end_bit));
    k_heads<<<blocks, threads>>>(d_skeys.as<unsigned long long>(), d_socc.as<int>(), n_occ, d_first.as<int>(),
                                 d_third.as<int>());
    MB_CUDA(cudaGetLastError());
    tmp_bytes = std::max(tmp_sort, tmp_scan);
    MB_CUDA(cub::DeviceScan::ExclusiveSum(d_tmp.p, tmp_bytes, d_first.as<int>(), d_sid.as<int>(), n_occ));
    int third = big, last_sid = 0, last_first = 0;
    MB_CUDA(cudaMemcpy(&third, d_third.p, 4, cudaMemcpyDeviceToHost));
    if (third != big) {
      const uint64_t t = uint64_t(third) / 3;
      const int j = third % 3;
      const uint32_t a = idx[3 * t + j], b = idx[3 * t + (j == 2 ? 0 : j + 1)];
      err = "A strut shouldn't have more than two adjacent faces! (edge " + std::to_string(std::min(a, b)) + "-" +
            std::to_string(std::max(a, b)) + ")";
      return FGB_ENONMANIFOLD;
    }
    MB_CUDA(cudaMemcpy(&last_sid, d_sid.as<int>() + (n_occ - 1), 4, cudaMemcpyDeviceToHost));
    MB_CUDA(cudaMemcpy(&last_first, d_first.as<int>() + (n_occ - 1), 4, cudaMemcpyDeviceToHost));
    const size_t U = size_t(last_sid) + size_t(last_first);
    DevBuf d_sa, d_sb, d_sk, d_sc, d_sl, d_fs;
    MB_CUDA(d_sa.alloc(U * 4));
    MB_CUDA(d_sb.alloc(U * 4));
    MB_CUDA(d_sk.alloc(U * 4));
    MB_CUDA(d_sc.alloc(U * 4));
    MB_CUDA(d_sl.alloc(U * 4));
    MB_CUDA(d_fs.alloc(size_t(n_occ) * 4));
    k_struts<<<blocks, threads>>>(d_skeys.as<unsigned long long>(), d_socc.as<int>(), n_occ, kb, d_sid.as<int>(),
                                  d_pos.as<float>(), d_ok.as<unsigned long long>(), d_okc.as<float2>(), int(ok.size()),
                                  k, c, d_sa.as<uint32_t>(), d_sb.as<uint32_t>(), d_sk.as<float>(), d_sc.as<float>(),
                                  d_sl.as<float>(), d_fs.as<uint32_t>());
    MB_CUDA(cudaGetLastError());
    m.sa.resize(U);
    m.sb.resize(U);
    m.sk.resize(U);
    m.sc.resize(U);
    m.sl.resize(U);
    MB_CUDA(cudaMemcpy(m.sa.data(), d_sa.p, U * 4, cudaMemcpyDeviceToHost));
    MB_CUDA(cudaMemcpy(m.sb.data(), d_sb.p, U * 4, cudaMemcpyDeviceToHost));
    MB_CUDA(cudaMemcpy(m.sk.data(), d_sk.p, U * 4, cudaMemcpyDeviceToHost));
    MB_CUDA(cudaMemcpy(m.sc.data(), d_sc.p, U * 4, cudaMemcpyDeviceToHost));
    MB_CUDA(cudaMemcpy(m.sl.data(), d_sl.p, U * 4, cudaMemcpyDeviceToHost));
    MB_CUDA(cudaMemcpy(m.fs.data(), d_fs.p, size_t(n_occ) * 4, cudaMemcpyDeviceToHost));
  }
  m.tri_struts = m.sa.size();
  uint32_t R, C;
  if (detect_cloth_pattern(idx, nt, m.n, R, C)) {
    m.rows = R;
    m.cols = C;
  }
  return FGB_OK;
}

}  // namespace fgb
