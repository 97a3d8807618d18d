// The tile lists of the grid kernels cover every tile of a cloth exactly
// once, and every tile they run in the interior form (no bounds checks) has
// all neighbours of all its vertices inside the cloth (white-box: calls the
// library's host forms of the lists; no GPU).
//  * grid_tiles: the single-cloth kernel's blockIdx -> tile mapping, ring
//    tiles first;
//  * batch_tiles: the batched kernel's work items, ring tiles first.
// A vertex's struts and faces reach two vertices in each direction (binding
// struts), so an interior 32 x th tile at (r0, c0) needs r0 >= 2, c0 >= 2,
// r0 + th + 2 <= R and c0 + 32 + 2 <= C.
#include <cstdio>
#include <vector>

#include "kernels.h"

namespace {

int failures = 0;
#define EXPECT(cond, R, C, th)                                                                    \
  do {                                                                                            \
    if (!(cond)) {                                                                                \
      if (failures < 20) std::printf("FAILED %s:%d (R=%d C=%d th=%d): %s\n", __FILE__, __LINE__, \
                                     R, C, th, #cond);                                            \
      ++failures;                                                                                 \
    }                                                                                             \
  } while (0)

constexpr int kTileW = 32;

bool interior_ok(int R, int C, int th, int bx, int by) {
  const int r0 = by * th, c0 = bx * kTileW;
  return r0 >= 2 && c0 >= 2 && r0 + th + 2 <= R && c0 + kTileW + 2 <= C;
}

// each (bx, by) of the tx x ty tiles listed once; interior ones valid; ring first
void check_list(int R, int C, int th, const std::vector<int>& bx, const std::vector<int>& by,
                const std::vector<int>& inner) {
  const int tx = (C + kTileW - 1) / kTileW, ty = (R + th - 1) / th;
  EXPECT(int(bx.size()) == tx * ty, R, C, th);
  std::vector<int> seen(size_t(tx) * ty, 0);
  bool in_interior = false;
  for (size_t i = 0; i < bx.size(); ++i) {
    const bool ok = bx[i] >= 0 && bx[i] < tx && by[i] >= 0 && by[i] < ty;
    EXPECT(ok, R, C, th);
    if (!ok) continue;
    ++seen[size_t(by[i]) * tx + bx[i]];
    if (inner[i]) EXPECT(interior_ok(R, C, th, bx[i], by[i]), R, C, th);
    EXPECT(!(in_interior && !inner[i]), R, C, th);  // no ring tile after an interior one
    in_interior = in_interior || inner[i];
  }
  for (int v : seen) EXPECT(v == 1, R, C, th);
}

}  // namespace

int main() {
  std::vector<int> sizes;
  for (int n = 1; n <= 140; ++n) sizes.push_back(n);
  for (int n : {255, 256, 257, 511, 1023, 1024, 1025, 2047, 2048}) sizes.push_back(n);
  long interior_tiles = 0;
  for (int th : {4, 8, 12})
    for (int R : sizes)
      for (int C : sizes) {
        const int n = fgb::grid_tiles(R, C, th, nullptr);
        std::vector<int> g(3 * size_t(n));
        EXPECT(fgb::grid_tiles(R, C, th, g.data()) == n, R, C, th);
        std::vector<int> bx(n), by(n), inner(n);
        for (int i = 0; i < n; ++i) {
          bx[i] = g[3 * i];
          by[i] = g[3 * i + 1];
          inner[i] = g[3 * i + 2];
          interior_tiles += inner[i];
        }
        check_list(R, C, th, bx, by, inner);

        int nr = 0, ni = 0;
        fgb::batch_tiles(7, R, C, th, nullptr, &nr, &ni);
        std::vector<int> w(4 * size_t(nr + ni));
        fgb::batch_tiles(7, R, C, th, w.data(), &nr, &ni);
        EXPECT(nr + ni == n, R, C, th);
        std::vector<int> wx(nr + ni), wy(nr + ni), wi(nr + ni);
        int n_inner = 0;
        for (int i = 0; i < nr + ni; ++i) {
          EXPECT(w[4 * i] == 7, R, C, th);
          wx[i] = w[4 * i + 1];
          wy[i] = w[4 * i + 2];
          wi[i] = w[4 * i + 3];
          n_inner += wi[i];
        }
        EXPECT(n_inner == ni, R, C, th);
        check_list(R, C, th, wx, wy, wi);
      }
  // the interior form is used wherever a large cloth has room for it
  if (interior_tiles == 0) ++failures;
  {
    const int n = fgb::grid_tiles(1024, 1024, 8, nullptr);
    std::vector<int> g(3 * size_t(n));
    fgb::grid_tiles(1024, 1024, 8, g.data());
    int ni = 0;
    for (int i = 0; i < n; ++i) ni += g[3 * i + 2];
    EXPECT(n == 32 * 128 && ni == 30 * 126, 1024, 1024, 8);
  }
  if (failures) {
    std::printf("%d failures\n", failures);
    return 1;
  }
  std::printf("ok\n");
  return 0;
}
