// The general gather's compact incidence lists, in their 16-bit and 32-bit
// strut word forms, decode to exactly the plain CSR lists (white-box: calls
// the library's internal mesh builders; no GPU).
// For every vertex: each strut word gives the CSR entry's other vertex and
// role, and its owner-order constants are the strut's (k, c, L); each face
// word gives the face's corner and its vertices in face order.  Meshes that
// do not fit the compact form are refused.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "mesh_build.h"

namespace {

int failures = 0;
#define EXPECT(cond)                                                   \
  do {                                                                 \
    if (!(cond)) {                                                     \
      std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond);    \
      ++failures;                                                      \
    }                                                                  \
  } while (0)

// other-vertex offset, rank and role of strut word e, from whichever form was built
void word(const fgb::CompactTopo& c, int e, int& off, int& rank, int& role) {
  if (!c.strut_word16.empty()) {
    const uint32_t w = c.strut_word16[e];
    role = int(w & 1u);
    off = int(int16_t(uint16_t(w))) >> (role ? 4 : 1);
    rank = int((w >> 1) & 7u);
  } else {
    const uint32_t w = c.strut_word[e];
    off = int32_t(w) >> 6;
    rank = int((w >> 1) & 31u);
    role = int(w & 1u);
  }
}

// 0: refused, 1: 32-bit strut words, 2: 16-bit strut words (decoded and checked)
int check_decodes(const fgb::MeshTopo& m) {
  fgb::CsrTopo t;
  std::string err;
  if (fgb::build_csr(m, t, err) != 0) return 0;
  fgb::CompactTopo c;
  if (!fgb::build_compact(m, t, c)) return 0;
  const int n = int(m.n);
  const int form = c.strut_word16.empty() ? 1 : 2;
  EXPECT(c.own_off.size() == size_t(n) + 1 && c.own_off[n] == int(m.sa.size()));
  EXPECT((form == 2 ? c.strut_word16.size() : c.strut_word.size()) * 2 == t.strut_inc.size());
  EXPECT((form == 2 ? c.strut_word.size() : c.strut_word16.size()) == 0);
  EXPECT(c.face_word.size() == t.face_inc.size());
  for (int v = 0; v < n; ++v) {
    int own = c.own_off[v];
    const int sb = t.strut_off[v];
    for (int e = sb; e < t.strut_off[v + 1]; ++e) {
      int off, rank, role;
      word(c, e, off, rank, role);
      const int o = v + off;
      const int i = role ? c.own_off[o] + rank : own++;
      const int s = t.strut_inc[2 * e + 1] >> 1;
      EXPECT(o == t.strut_inc[2 * e]);
      EXPECT(role == (t.strut_inc[2 * e + 1] & 1));
      EXPECT(i >= c.own_off[role ? o : v] && i < c.own_off[(role ? o : v) + 1]);
      EXPECT(c.sk[i] == t.strut_kcl[4 * s] && c.sc[i] == t.strut_kcl[4 * s + 1] && c.sl[i] == t.strut_kcl[4 * s + 2]);
    }
    EXPECT(own == c.own_off[v + 1]);  // every owned strut taken once
    for (int e = t.face_off[v]; e < t.face_off[v + 1]; ++e) {
      const uint32_t h = c.face_word[e];
      const int corner = int(h & 3u);
      int o1, o2, rk, rl;
      word(c, sb + int((h >> 2) & 127u), o1, rk, rl);
      word(c, sb + int(h >> 9), o2, rk, rl);
      const int u1 = v + o1, u2 = v + o2;
      const int got[3] = {corner == 0 ? v : u1, corner == 0 ? u1 : (corner == 1 ? v : u2), corner == 2 ? v : u2};
      const int f = t.face_inc[e] >> 2;
      EXPECT(corner == (t.face_inc[e] & 3));
      for (int k = 0; k < 3; ++k) EXPECT(got[k] == t.face_vtx[4 * f + k]);
    }
  }
  return form;
}

}  // namespace

int main() {
  std::string err;
  {  // Cloth::new grids, with and without pins, square and ragged
    const float origin[3] = {0.5f, 1.0f, -0.25f};
    // rows, cols, the form expected: 16-bit words while a binding strut's
    // backward offset (two rows) stays within -2048
    const uint64_t shapes[][3] = {{2, 2, 2}, {3, 7, 2}, {16, 16, 2}, {33, 17, 2}, {64, 100, 2}, {5, 1024, 2},
                                  {5, 1025, 1}};
    for (const auto& sh : shapes) {
      fgb::MeshTopo m;
      const uint32_t pins[2] = {0, uint32_t(sh[1] - 1)};
      EXPECT(fgb::build_cloth(sh[0], sh[1], 0.05f, origin, 0.01f, 800.0f, 2.0f, 400.0f, 1.0f, 200.0f, 0.5f, pins, 2,
                              m, err) == 0);
      EXPECT(check_decodes(m) == int(sh[2]));
    }
  }
  {  // a strip whose triangles join vertex i to i + 3000: offsets beyond 16-bit words
    const uint32_t half = 3000;
    std::vector<float> pos(3 * 2 * half);
    for (uint32_t i = 0; i < 2 * half; ++i) {
      pos[3 * i] = float(i % half) * 0.01f;
      pos[3 * i + 1] = i < half ? 0.0f : 0.01f;
    }
    std::vector<uint32_t> idx;
    for (uint32_t i = 0; i + 1 < half; ++i) idx.insert(idx.end(), {i, i + 1, i + half, i + 1, i + half + 1, i + half});
    fgb::MeshTopo m;
    EXPECT(fgb::build_springy(pos.data(), 2 * half, idx.data(), idx.size(), 0.1f, 500.0f, 1.0f, nullptr, 0, m,
                              err) == 0);
    EXPECT(check_decodes(m) == 1);
  }
  {  // SpringyMesh::new of a random triangle soup over a small vertex set
    std::srand(7);
    const uint32_t nv = 200;
    std::vector<float> pos(3 * nv);
    for (auto& p : pos) p = float(std::rand() % 1000) * 0.001f;
    std::vector<uint32_t> idx;
    while (idx.size() < 3 * 300) {
      const uint32_t a = std::rand() % nv, b = std::rand() % nv, c = std::rand() % nv;
      if (a == b || b == c || a == c) continue;
      idx.insert(idx.end(), {a, b, c});
    }
    fgb::MeshTopo m;
    EXPECT(fgb::build_springy(pos.data(), nv, idx.data(), idx.size(), 0.1f, 500.0f, 1.0f, nullptr, 0, m, err) == 0);
    EXPECT(check_decodes(m) != 0);
  }
  {  // a fan whose centre is the first vertex of 40 struts: refused
    const uint32_t spokes = 40;
    std::vector<float> pos(3 * (spokes + 2), 0.0f);
    for (uint32_t i = 1; i < spokes + 2; ++i) {
      pos[3 * i] = float(i);
      pos[3 * i + 1] = float(i % 3);
    }
    std::vector<uint32_t> idx;
    for (uint32_t i = 1; i <= spokes; ++i) idx.insert(idx.end(), {0u, i, i + 1});
    fgb::MeshTopo m;
    EXPECT(fgb::build_springy(pos.data(), spokes + 2, idx.data(), idx.size(), 0.1f, 500.0f, 1.0f, nullptr, 0, m,
                              err) == 0);
    fgb::CsrTopo t;
    EXPECT(fgb::build_csr(m, t, err) == 0);
    fgb::CompactTopo c;
    EXPECT(!fgb::build_compact(m, t, c));
    EXPECT(c.strut_word.empty());
  }
  if (failures) return 1;
  std::printf("ok\n");
  return 0;
}
