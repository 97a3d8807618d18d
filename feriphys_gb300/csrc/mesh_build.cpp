// Host-side mesh construction (see mesh_build.h).  Compiled with
// -ffp-contract=off: rest lengths and scaled constants must round exactly as
// the reference's f32 arithmetic does.
#include "mesh_build.h"

#include <cmath>
#include <cstring>

#include "feriphys_gb300.h"

namespace fgb {

namespace {

// Open-addressing map from an unordered vertex pair to a 32-bit value.
class PairMap {
 public:
  explicit PairMap(size_t expected) {
    size_t cap = 16;
    while (cap < 2 * expected + 16) cap <<= 1;
    keys_.assign(cap, kEmpty);
    vals_.resize(cap);
    mask_ = cap - 1;
  }
  static uint64_t key(uint32_t a, uint32_t b) {
    return a <= b ? (uint64_t(a) << 32) | b : (uint64_t(b) << 32) | a;
  }
  // Inserts (key, v) if absent; returns the slot's value pointer and whether
  // it was inserted.
  uint32_t* emplace(uint64_t k, uint32_t v, bool& inserted) {
    size_t h = mix(k) & mask_;
    while (true) {
      if (keys_[h] == kEmpty) {
        keys_[h] = k;
        vals_[h] = v;
        inserted = true;
        return &vals_[h];
      }
      if (keys_[h] == k) {
        inserted = false;
        return &vals_[h];
      }
      h = (h + 1) & mask_;
    }
  }
  const uint32_t* find(uint64_t k) const {
    size_t h = mix(k) & mask_;
    while (true) {
      if (keys_[h] == kEmpty) return nullptr;
      if (keys_[h] == k) return &vals_[h];
      h = (h + 1) & mask_;
    }
  }

 private:
  static constexpr uint64_t kEmpty = ~uint64_t(0);
  static uint64_t mix(uint64_t k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdULL;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ULL;
    k ^= k >> 33;
    return k;
  }
  std::vector<uint64_t> keys_;
  std::vector<uint32_t> vals_;
  size_t mask_;
};

inline float length_between(const float* pos, uint32_t a, uint32_t b, size_t stride = 3) {
  // (points[a].position - points[b].position).magnitude()
  const float* pa = pos + stride * a;
  const float* pb = pos + stride * b;
  const float dx = pa[0] - pb[0];
  const float dy = pa[1] - pb[1];
  const float dz = pa[2] - pb[2];
  return std::sqrt(dx * dx + dy * dy + dz * dz);
}

bool cloth_pattern(const uint32_t* idx, uint64_t nt, uint32_t n, uint32_t& R, uint32_t& C) {
  if (nt == 0) return false;
  const uint32_t cols = idx[1];  // first triangle (1, C, 0)
  if (cols < 2 || n % cols != 0) return false;
  const uint32_t rows = n / cols;
  if (rows < 2) return false;
  if (uint64_t(nt) != 2ull * (rows - 1) * (cols - 1)) return false;
  uint64_t t = 0;
  for (uint32_t r = 0; r + 1 < rows; ++r)
    for (uint32_t c = 0; c + 1 < cols; ++c, ++t) {
      const uint32_t i = r * cols + c;
      if (idx[3 * t] != i + 1 || idx[3 * t + 1] != i + cols || idx[3 * t + 2] != i) return false;
    }
  for (uint32_t r = 1; r < rows; ++r)
    for (uint32_t c = 0; c + 1 < cols; ++c, ++t) {
      const uint32_t i = r * cols + c;
      if (idx[3 * t] != i - cols + 1 || idx[3 * t + 1] != i + 1 || idx[3 * t + 2] != i) return false;
    }
  R = rows;
  C = cols;
  return true;
}

}  // namespace

namespace {

// Whole nanoseconds of Duration::from_secs_f32(x): x rounded to the nearest
// nanosecond, ties to even (Rust >= 1.63).  x finite and >= 0.
void duration_parts(float x, uint64_t& secs, uint32_t& nanos) {
  secs = 0;
  nanos = 0;
  uint32_t bits;
  std::memcpy(&bits, &x, 4);
  const int biased = int((bits >> 23) & 0xffu);
  const uint32_t frac = bits & 0x7fffffu;
  if (biased == 0 && frac == 0) return;
  const uint64_t m = biased == 0 ? frac : (frac | 0x800000u);
  const int e2 = biased == 0 ? -149 : biased - 150;  // x = m * 2^e2
  const unsigned __int128 prod = (unsigned __int128)m * 1000000000u;
  unsigned __int128 ns;
  if (e2 >= 0) {
    ns = prod << e2;
  } else {
    const int s = -e2;
    if (s >= 120) return;
    const unsigned __int128 one = 1;
    ns = prod >> s;
    const unsigned __int128 rem = prod & ((one << s) - 1);
    const unsigned __int128 half = one << (s - 1);
    if (rem > half || (rem == half && (ns & 1))) ns += 1;
  }
  secs = uint64_t(ns / 1000000000u);
  nanos = uint32_t(ns % 1000000000u);
}

}  // namespace

bool detect_cloth_pattern(const uint32_t* idx, uint64_t nt, uint32_t n, uint32_t& R, uint32_t& C) {
  return cloth_pattern(idx, nt, n, R, C);
}

float duration_roundtrip(float x) {
  uint64_t secs;
  uint32_t nanos;
  duration_parts(x, secs, nanos);
  return float(secs) + float(nanos) / 1000000000.0f;  // as_secs_f32
}

double duration_seconds_f64(float x) {
  uint64_t secs;
  uint32_t nanos;
  duration_parts(x, secs, nanos);
  return double(secs) + double(nanos) / 1e9;  // as_secs_f64
}

int build_springy(const float* pos, uint64_t nv, const uint32_t* idx, uint64_t ni, float mass, float k, float c,
                  const Override* ov, uint64_t nov, MeshTopo& m, std::string& err) {
  if (nv > 0x7fffffffull) {
    err = "too many vertices (limit 2^31-1)";
    return FGB_EINVAL;
  }
  if ((nv && !pos) || (ni && !idx) || (nov && !ov)) {
    err = "null buffer with a non-zero size";
    return FGB_EINVAL;
  }
  m = MeshTopo();
  m.n = uint32_t(nv);
  m.pos.assign(pos, pos + 3 * nv);
  m.mass_per_vert = mass / float(nv);  // springy_mesh.rs:277
  const uint64_t nt = ni / 3;          // itertools::tuples drops a trailing remainder
  for (uint64_t i = 0; i < 3 * nt; ++i)
    if (idx[i] >= nv) {
      err = "triangle index " + std::to_string(idx[i]) + " out of range for " + std::to_string(nv) + " vertices";
      return FGB_EINDEX;
    }
  PairMap overrides(nov);
  std::vector<Override> ovs(ov, ov + nov);
  for (uint64_t i = 0; i < nov; ++i) {
    bool ins;
    uint32_t* slot = overrides.emplace(PairMap::key(ov[i].a, ov[i].b), uint32_t(i), ins);
    if (!ins) *slot = uint32_t(i);  // FxHashMap::insert keeps the last value
  }
  PairMap struts(3 * nt);
  m.sa.reserve(2 * nt + 16);
  m.sb.reserve(2 * nt + 16);
  m.sk.reserve(2 * nt + 16);
  m.sc.reserve(2 * nt + 16);
  m.sl.reserve(2 * nt + 16);
  auto add = [&](uint32_t i1, uint32_t i2) {
    const uint64_t key = PairMap::key(i1, i2);
    bool ins;
    struts.emplace(key, uint32_t(m.sa.size()), ins);
    if (!ins) return;
    const uint32_t a = uint32_t(key >> 32), b = uint32_t(key & 0xffffffffu);
    float kk = k, cc = c;
    if (nov) {
      const uint32_t* o = overrides.find(key);
      if (o) {
        kk = ovs[*o].k;
        cc = ovs[*o].c;
      }
    }
    const float L = length_between(pos, a, b);
    m.sa.push_back(a);
    m.sb.push_back(b);
    m.sk.push_back(scaled(kk, L));
    m.sc.push_back(scaled(cc, L));
    m.sl.push_back(L);
  };
  for (uint64_t t = 0; t < nt; ++t) {
    add(idx[3 * t], idx[3 * t + 1]);
    add(idx[3 * t + 1], idx[3 * t + 2]);
    add(idx[3 * t + 2], idx[3 * t]);
  }
  m.tri_struts = m.sa.size();
  m.fv.assign(idx, idx + 3 * nt);
  m.fs.resize(3 * nt);
  std::vector<uint8_t> nfaces(m.sa.size(), 0);
  for (uint64_t t = 0; t < nt; ++t) {
    const uint32_t v[3] = {idx[3 * t], idx[3 * t + 1], idx[3 * t + 2]};
    for (int e = 0; e < 3; ++e) {
      const uint32_t s = *struts.find(PairMap::key(v[e], v[(e + 1) % 3]));
      m.fs[3 * t + e] = s;
      if (++nfaces[s] > 2) {
        err = "A strut shouldn't have more than two adjacent faces! (edge " + std::to_string(m.sa[s]) + "-" +
              std::to_string(m.sb[s]) + ")";
        return FGB_ENONMANIFOLD;
      }
    }
  }
  uint32_t R, C;
  if (cloth_pattern(idx, nt, m.n, R, C)) {
    m.rows = R;
    m.cols = C;
  }
  return FGB_OK;
}

int add_strut(MeshTopo& m, uint32_t a, uint32_t b, float k, float c, const float* cur_pos, size_t stride,
              std::string& err) {
  if (a >= m.n || b >= m.n) {
    err = "strut vertex out of range";
    return FGB_EINDEX;
  }
  const float L = length_between(cur_pos, a, b, stride);
  m.sa.push_back(a);
  m.sb.push_back(b);
  m.sk.push_back(scaled(k, L));
  m.sc.push_back(scaled(c, L));
  m.sl.push_back(L);
  return FGB_OK;
}

int build_cloth(uint64_t rows, uint64_t cols, float spacing, const float position[3], float point_mass, float tk,
                float tc, float sk, float sc, float bk, float bc, const uint32_t* pins, uint64_t npins,
                MeshTopo& m, std::string& err) {
  if (rows < 2 || cols < 2) {
    err = "Cloth::new needs rows >= 2 and cols >= 2";
    return FGB_EINVAL;
  }
  if (rows > 0x7fffffffull || cols > 0x7fffffffull || rows * cols > 0x7fffffffull) {  // no 64-bit wrap
    err = "cloth too large";
    return FGB_EINVAL;
  }
  if (!position || (npins && !pins)) {
    err = "null buffer";
    return FGB_EINVAL;
  }
  const uint64_t n = rows * cols;
  std::vector<float> pos(3 * n);
  const float cx = float(cols) / 2.0f * spacing, cy = float(rows) / 2.0f * spacing;  // cloth.rs:45-54
  for (uint64_t r = 0; r < rows; ++r)
    for (uint64_t c = 0; c < cols; ++c) {
      const uint64_t i = r * cols + c;
      pos[3 * i] = (float(c) * spacing - cx) + position[0];
      pos[3 * i + 1] = (float(r) * spacing - cy) + position[1];
      pos[3 * i + 2] = (0.0f - 0.0f) + position[2];
    }
  std::vector<uint32_t> idx;
  idx.reserve(6 * (rows - 1) * (cols - 1));
  std::vector<Override> shear;
  shear.reserve((rows - 1) * (cols - 1));
  for (uint64_t r = 0; r + 1 < rows; ++r)
    for (uint64_t c = 0; c + 1 < cols; ++c) {
      const uint32_t i = uint32_t(r * cols + c);
      idx.push_back(i + 1);
      idx.push_back(i + uint32_t(cols));
      idx.push_back(i);
      shear.push_back(Override{i + uint32_t(cols), i + 1, sk, sc});
    }
  for (uint64_t r = 1; r < rows; ++r)
    for (uint64_t c = 0; c + 1 < cols; ++c) {
      const uint32_t i = uint32_t(r * cols + c);
      idx.push_back(i - uint32_t(cols) + 1);
      idx.push_back(i + 1);
      idx.push_back(i);
    }
  int rc = build_springy(pos.data(), n, idx.data(), idx.size(), point_mass * float(rows) * float(cols), tk, tc,
                         shear.data(), shear.size(), m, err);
  if (rc) return rc;
  for (uint64_t p = 0; p < npins; ++p) {
    if (pins[p] >= n) {
      err = "pin index out of range";
      return FGB_EINDEX;
    }
    m.pins.push_back(pins[p]);
  }
  for (uint64_t r = 0; r + 2 < rows; ++r)
    for (uint64_t c = 0; c + 2 < cols; ++c) {
      const uint32_t i = uint32_t(r * cols + c);
      add_strut(m, i, i + 2, bk, bc, pos.data(), 3, err);
      add_strut(m, i, i + 2 * uint32_t(cols), bk, bc, pos.data(), 3, err);
    }
  return FGB_OK;
}

int build_csr(const MeshTopo& m, CsrTopo& t, std::string& err) {
  const uint32_t n = m.n;
  const size_t S = m.sa.size(), F = m.fv.size() / 3;
  if (2 * S > 0x7fffffffull || F > 0x1fffffffull || S > 0x3fffffffull) {
    err = "mesh too large for 32-bit incidence lists";
    return FGB_EINVAL;
  }
  t.strut_off.assign(n + 1, 0);
  for (size_t s = 0; s < S; ++s) {
    t.strut_off[m.sa[s] + 1]++;
    t.strut_off[m.sb[s] + 1]++;
  }
  for (uint32_t v = 0; v < n; ++v) t.strut_off[v + 1] += t.strut_off[v];
  t.strut_inc.assign(2 * size_t(t.strut_off[n]), 0);
  std::vector<int> fill(t.strut_off.begin(), t.strut_off.end() - 1);
  for (size_t s = 0; s < S; ++s) {  // strut order => each list ascends by strut id
    const int a = int(m.sa[s]), b = int(m.sb[s]);
    int e = fill[a]++;
    t.strut_inc[2 * e] = b;
    t.strut_inc[2 * e + 1] = int(s << 1);
    e = fill[b]++;
    t.strut_inc[2 * e] = a;
    t.strut_inc[2 * e + 1] = int((s << 1) | 1);
  }
  t.strut_kcl.resize(4 * S);
  for (size_t s = 0; s < S; ++s) {
    t.strut_kcl[4 * s] = m.sk[s];
    t.strut_kcl[4 * s + 1] = m.sc[s];
    t.strut_kcl[4 * s + 2] = m.sl[s];
    t.strut_kcl[4 * s + 3] = 0.0f;
  }
  t.face_off.assign(n + 1, 0);
  for (size_t f = 0; f < F; ++f)
    for (int k = 0; k < 3; ++k) t.face_off[m.fv[3 * f + k] + 1]++;
  for (uint32_t v = 0; v < n; ++v) t.face_off[v + 1] += t.face_off[v];
  t.face_inc.assign(size_t(t.face_off[n]), 0);
  std::vector<int> ffill(t.face_off.begin(), t.face_off.end() - 1);
  for (size_t f = 0; f < F; ++f)  // face order, then corner order
    for (int k = 0; k < 3; ++k) t.face_inc[ffill[m.fv[3 * f + k]]++] = int((f << 2) | size_t(k));
  t.face_vtx.resize(4 * F);
  for (size_t f = 0; f < F; ++f) {
    t.face_vtx[4 * f] = int(m.fv[3 * f]);
    t.face_vtx[4 * f + 1] = int(m.fv[3 * f + 1]);
    t.face_vtx[4 * f + 2] = int(m.fv[3 * f + 2]);
    t.face_vtx[4 * f + 3] = 0;
  }
  return FGB_OK;
}

bool build_compact(const MeshTopo& m, const CsrTopo& t, CompactTopo& out) {
  out = CompactTopo{};
  const uint32_t n = m.n;
  const size_t S = m.sa.size(), F = m.fv.size() / 3;
  std::vector<int> own_off(size_t(n) + 1, 0);
  for (size_t s = 0; s < S; ++s) own_off[m.sa[s] + 1]++;
  for (uint32_t v = 0; v < n; ++v) {
    if (own_off[v + 1] > 32) return false;  // rank must fit 5 bits
    own_off[v + 1] += own_off[v];
  }
  std::vector<int> fill(own_off.begin(), own_off.end() - 1);
  std::vector<uint32_t> rank(S);
  std::vector<float> sk(S), sc(S), sl(S);
  for (size_t s = 0; s < S; ++s) {  // strut order => each owner range ascends by strut id
    const uint32_t a = m.sa[s];
    const int i = fill[a]++;
    rank[s] = uint32_t(i - own_off[a]);
    sk[i] = m.sk[s];
    sc[i] = m.sc[s];
    sl[i] = m.sl[s];
  }
  const int64_t kLim = int64_t(1) << 25;
  const size_t E = t.strut_inc.size() / 2;
  std::vector<uint32_t> sw(E);
  bool fits16 = true;
  for (uint32_t v = 0; v < n; ++v) {
    if (t.strut_off[v + 1] - t.strut_off[v] > 127) return false;  // face positions must fit 7 bits
    for (int e = t.strut_off[v]; e < t.strut_off[v + 1]; ++e) {
      const int64_t off = int64_t(t.strut_inc[2 * e]) - int64_t(v);
      if (off <= -kLim || off >= kLim) return false;
      const uint32_t s = uint32_t(t.strut_inc[2 * e + 1]) >> 1, role = uint32_t(t.strut_inc[2 * e + 1]) & 1u;
      sw[e] = (uint32_t(int32_t(off)) << 6) | (rank[s] << 1) | role;
      fits16 = fits16 && (role ? off >= -2048 && off < 2048 && rank[s] < 8 : off >= -16384 && off < 16384);
    }
  }
  std::vector<uint16_t> sw16;
  if (fits16) {
    sw16.resize(E);
    for (size_t e = 0; e < E; ++e) {
      const int32_t off = int32_t(sw[e]) >> 6;
      sw16[e] = (sw[e] & 1u) ? uint16_t((uint32_t(off) << 4) | (((sw[e] >> 1) & 7u) << 1) | 1u)
                             : uint16_t(uint32_t(off) << 1);
    }
    sw.clear();
  }
  std::vector<uint16_t> fw(t.face_inc.size());
  for (uint32_t v = 0; v < n; ++v) {
    const int sb = t.strut_off[v], se = t.strut_off[v + 1];
    auto pos_of = [&](uint32_t u) -> int {  // first position of neighbour u in v's strut list
      for (int e = sb; e < se; ++e)
        if (uint32_t(t.strut_inc[2 * e]) == u) return e - sb;
      return -1;
    };
    for (int e = t.face_off[v]; e < t.face_off[v + 1]; ++e) {
      const size_t f = size_t(uint32_t(t.face_inc[e]) >> 2);
      const int corner = t.face_inc[e] & 3;
      if (f >= F) return false;
      const uint32_t* fv = &m.fv[3 * f];
      const uint32_t u1 = corner == 0 ? fv[1] : fv[0], u2 = corner == 2 ? fv[1] : fv[2];
      const int i1 = pos_of(u1), i2 = pos_of(u2);
      if (i1 < 0 || i2 < 0) return false;
      fw[e] = uint16_t(uint32_t(corner) | (uint32_t(i1) << 2) | (uint32_t(i2) << 9));
    }
  }
  out.own_off = std::move(own_off);
  out.sk = std::move(sk);
  out.sc = std::move(sc);
  out.sl = std::move(sl);
  out.strut_word = std::move(sw);
  out.strut_word16 = std::move(sw16);
  out.face_word = std::move(fw);
  return true;
}

namespace {

// Strut id of the strut in `slot` of vertex (r, c), or -1 when absent, found
// through the (already built) CSR of the vertex.
long grid_owned_strut(const MeshTopo& m, const PairMap& pm, int kind, int r, int c) {
  const int R = int(m.rows), C = int(m.cols);
  if (!grid::owned_exists(kind, r, c, R, C)) return -1;
  const uint32_t o = uint32_t(r * C + c);
  uint32_t a, b;
  switch (kind) {
    case grid::KH: a = o; b = o + 1; break;
    case grid::KV: a = o; b = o + uint32_t(C); break;
    case grid::KS: a = o + 1; b = o + uint32_t(C); break;
    case grid::KBH: a = o; b = o + 2; break;
    default: a = o; b = o + 2 * uint32_t(C); break;
  }
  const uint32_t* s = pm.find(PairMap::key(a, b));
  if (!s) return -2;  // expected but missing: not a grid
  // orientation must match the owned layout (first vertex = a)
  if (m.sa[*s] != a || m.sb[*s] != b) return -2;
  return long(*s);
}

}  // namespace

bool grid_layout_ok(const MeshTopo& m) {
  if (m.rows < 2 || m.cols < 2) return false;
  const uint64_t R = m.rows, C = m.cols;
  const size_t nbind = size_t(2 * (R >= 2 ? R - 2 : 0) * (C >= 2 ? C - 2 : 0));
  if (m.sa.size() != m.tri_struts + nbind) return false;
  size_t s = m.tri_struts;
  for (uint64_t r = 0; r + 2 < R; ++r)
    for (uint64_t c = 0; c + 2 < C; ++c) {
      const uint32_t i = uint32_t(r * C + c);
      if (m.sa[s] != i || m.sb[s] != i + 2) return false;
      ++s;
      if (m.sa[s] != i || m.sb[s] != i + 2 * uint32_t(C)) return false;
      ++s;
    }
  // Map every strut key once; then check, per vertex, that the slot order
  // visits strictly ascending strut ids and covers all incident struts.
  PairMap pm(m.sa.size());
  for (size_t k = 0; k < m.sa.size(); ++k) {
    bool ins;
    pm.emplace(PairMap::key(m.sa[k], m.sb[k]), uint32_t(k), ins);
    if (!ins) return false;  // duplicate strut: not the builder's layout
  }
  std::vector<uint8_t> degree(m.n, 0);
  for (size_t k = 0; k < m.sa.size(); ++k) {
    degree[m.sa[k]]++;
    degree[m.sb[k]]++;
  }
  for (int r = 0; r < int(R); ++r)
    for (int c = 0; c < int(C); ++c) {
      long prev = -1;
      int count = 0;
      for (int j = 0; j < grid::N_SLOTS; ++j) {
        const grid::SlotDesc d = grid::slot_desc(grid::slot_at(j, r, c, int(R), int(C)));
        const long sid = grid_owned_strut(m, pm, d.kind, r + d.dr, c + d.dc);
        if (sid == -2) return false;
        if (sid < 0) continue;
        if (sid <= prev) return false;
        prev = sid;
        ++count;
      }
      if (count != degree[uint32_t(r) * C + uint32_t(c)]) return false;
    }
  return true;
}

void build_grid_params(const MeshTopo& m, std::vector<float>& planes) {
  const uint32_t n = m.n, C = m.cols;
  planes.assign(16 * size_t(n), 0.0f);
  for (size_t s = 0; s < m.sa.size(); ++s) {
    const uint32_t a = m.sa[s], b = m.sb[s];
    int kind;
    uint32_t owner;
    if (s >= m.tri_struts) {
      kind = (b - a == 2) ? grid::KBH : grid::KBV;
      owner = a;
    } else if (b - a == C) {
      kind = grid::KV;
      owner = a;
    } else if (b - a == 1 && (a % C) != C - 1) {
      kind = grid::KH;
      owner = a;
    } else {
      kind = grid::KS;  // (i+1, i+C) owned by quad origin i
      owner = a - 1;
    }
    const float vals[3] = {m.sk[s], m.sc[s], m.sl[s]};
    for (int f = 0; f < 3; ++f) {
      const int slot = grid::param_index(kind, f);  // 0..14
      planes[size_t(slot / 4) * 4 * n + 4 * size_t(owner) + size_t(slot % 4)] = vals[f];
    }
  }
}

}  // namespace fgb
