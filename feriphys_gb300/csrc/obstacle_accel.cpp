// Host builder of the obstacle broad phase (see obstacle_accel.h).
#include "obstacle_accel.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace fgb {

namespace {

struct Box {
  double lo[3], hi[3];
};

float round_down(double x) {
  float f = float(x);
  return double(f) > x ? std::nextafter(f, -INFINITY) : f;
}
float round_up(double x) {
  float f = float(x);
  return double(f) < x ? std::nextafter(f, INFINITY) : f;
}

// 3D acceptance region of a face, or false when it cannot be bounded.
// `query_extent` is the largest query box a cell accepts (its slack x 2).
bool face_region(const ObsFace& F, double query_extent, Box& b) {
  int axis;
  std::memcpy(&axis, &F.v0.w, 4);
  if (axis < 0 || axis > 2) return false;
  const float* q[3] = {&F.v0.x, &F.v1.x, &F.v2.x};
  const float* n = &F.n.x;
  double maxabs = 0.0, lo[3], hi[3];
  for (int d = 0; d < 3; ++d) {
    lo[d] = INFINITY;
    hi[d] = -INFINITY;
    if (!std::isfinite(n[d])) return false;
  }
  for (int k = 0; k < 3; ++k)
    for (int d = 0; d < 3; ++d) {
      if (!std::isfinite(q[k][d])) return false;
      maxabs = std::max(maxabs, std::fabs(double(q[k][d])));
      lo[d] = std::min(lo[d], double(q[k][d]));
      hi[d] = std::max(hi[d], double(q[k][d]));
    }
  const double na = std::fabs(double(n[axis]));
  if (!(na >= 1e-4)) return false;
  const int iu = axis == 0 ? 1 : 0, iw = axis == 2 ? 1 : 2;
  double u[3], w[3], len[3], diam2 = 0.0;
  for (int k = 0; k < 3; ++k) {
    u[k] = q[k][iu];
    w[k] = q[k][iw];
  }
  const double area2 = std::fabs((u[1] - u[0]) * (w[2] - w[0]) - (w[1] - w[0]) * (u[2] - u[0]));
  for (int k = 0; k < 3; ++k) {
    len[k] = std::hypot(u[(k + 1) % 3] - u[k], w[(k + 1) % 3] - w[k]);
    diam2 = std::max(diam2, len[k]);
  }
  if (!(area2 > 0.0)) return false;
  const double s0 = area2 / (len[0] * len[2]), s1 = area2 / (len[0] * len[1]), s2 = area2 / (len[1] * len[2]);
  const double smin = std::min(s0, std::min(s1, s2));
  if (!(smin >= 1e-5)) return false;
  // Projected margin: a sign test errs only within ~6 ulps x |p - vertex| of
  // an edge line, i.e. ~6u * size / sin(min angle / 2) outside the triangle;
  // R is >10x that, plus floors relative to size and position.
  const double sin_half = std::sqrt(0.5 * (1.0 - std::sqrt(std::max(0.0, 1.0 - smin * smin))));
  const double R = 4e-6 * diam2 / std::max(sin_half, 1e-12) + 1e-3 * diam2 + 1e-5 * maxabs + 1e-30;
  // Plane margin: distance errors are a few ulps of |p - v0| (bounded by the
  // face size, the accepted query extent and the coordinates); >100x that.
  double diam3 = 0.0;
  for (int d = 0; d < 3; ++d) diam3 = std::max(diam3, hi[d] - lo[d]);
  const double tau = 1e-5 * (diam3 + query_extent + R) + 1e-5 * maxabs + 1e-30;
  const double nu = std::fabs(double(n[iu])), nw = std::fabs(double(n[iw]));
  for (int d = 0; d < 3; ++d) {
    const double g = d == axis ? (R * (nu + nw) + tau) / na + tau : R;
    b.lo[d] = lo[d] - g;
    b.hi[d] = hi[d] + g;
  }
  return true;
}

}  // namespace

void build_obstacle_accel(const std::vector<ObsFace>& faces, const std::vector<int>& first_face,
                          const std::vector<int>& n_faces, AccelHost& out) {
  out = AccelHost();
  const int kMaxCells = 64;
  for (size_t k = 0; k < first_face.size(); ++k) {
    const int fb = first_face[k], nf = n_faces[k];
    if (nf <= 0) continue;
    ObsGrid3 g;
    std::memset(&g, 0, sizeof(g));
    g.face_base = fb;
    g.n_faces = nf;
    // Cells a quarter of the typical face; query boxes up to 5% of a face
    // (a few steps' travel of a cloth vertex) fit one cell grown by the slack.
    std::vector<double> diam;
    for (int f = fb; f < fb + nf; ++f) {
      const ObsFace& F = faces[f];
      double d = 0.0;
      const float* q[3] = {&F.v0.x, &F.v1.x, &F.v2.x};
      for (int a = 0; a < 3; ++a)
        for (int b = a + 1; b < 3; ++b)
          d = std::max(d, std::sqrt(double(q[a][0] - q[b][0]) * (q[a][0] - q[b][0]) +
                                    double(q[a][1] - q[b][1]) * (q[a][1] - q[b][1]) +
                                    double(q[a][2] - q[b][2]) * (q[a][2] - q[b][2])));
      if (std::isfinite(d)) diam.push_back(d);
    }
    double med = 0.0;
    if (!diam.empty()) {
      std::nth_element(diam.begin(), diam.begin() + diam.size() / 2, diam.end());
      med = diam[diam.size() / 2];
    }
    const double query_extent = std::max(0.05 * med, 1e-6);
    std::vector<Box> reg(nf);
    std::vector<char> ok(nf, 0);
    Box u;
    for (int d = 0; d < 3; ++d) {
      u.lo[d] = INFINITY;
      u.hi[d] = -INFINITY;
    }
    g.always_base = int(out.always.size());
    for (int i = 0; i < nf; ++i) {
      ok[i] = face_region(faces[fb + i], query_extent, reg[i]);
      if (!ok[i]) {
        out.always.push_back(fb + i);
        continue;
      }
      for (int d = 0; d < 3; ++d) {
        u.lo[d] = std::min(u.lo[d], reg[i].lo[d]);
        u.hi[d] = std::max(u.hi[d], reg[i].hi[d]);
      }
    }
    g.n_always = int(out.always.size()) - g.always_base;
    g.off_base = int(out.cell_off.size());
    if (u.lo[0] <= u.hi[0]) {
      const double target = std::max(0.25 * med, 1e-9);
      double cell[3], margin = 0.0;
      for (int d = 0; d < 3; ++d) {
        const double span = std::max(u.hi[d] - u.lo[d], 1e-9);
        g.n[d] = std::max(1, std::min(kMaxCells, int(std::ceil(span / target))));
        cell[d] = span / g.n[d];
        margin = std::max(margin, 0.5 * cell[d]);
      }
      margin = std::max(std::min(margin, query_extent), 0.5 * query_extent);
      // a face is listed in every cell its region meets grown by `margin`; a
      // query must fit its cell grown by margin/2 (float rounding of the
      // device's cell bounds is far below margin/2)
      std::vector<std::vector<int>> cells(size_t(g.n[0]) * g.n[1] * g.n[2]);
      for (int i = 0; i < nf; ++i) {
        if (!ok[i]) continue;
        int c0[3], c1[3];
        for (int d = 0; d < 3; ++d) {
          c0[d] = std::max(0, int(std::floor((reg[i].lo[d] - margin - u.lo[d]) / cell[d])));
          c1[d] = std::min(g.n[d] - 1, int(std::floor((reg[i].hi[d] + margin - u.lo[d]) / cell[d])));
        }
        for (int x = c0[0]; x <= c1[0]; ++x)
          for (int y = c0[1]; y <= c1[1]; ++y)
            for (int z = c0[2]; z <= c1[2]; ++z) cells[(size_t(x) * g.n[1] + y) * g.n[2] + z].push_back(fb + i);
      }
      for (const auto& c : cells) {
        out.cell_off.push_back(int(out.cell_faces.size()));
        out.cell_faces.insert(out.cell_faces.end(), c.begin(), c.end());
      }
      out.cell_off.push_back(int(out.cell_faces.size()));
      for (int d = 0; d < 3; ++d) {
        g.lo[d] = round_down(u.lo[d]);
        g.hi[d] = round_up(u.hi[d]);
        g.cell[d] = float(cell[d]);
        g.inv[d] = float(1.0 / cell[d]);
      }
      g.slack = float(0.5 * margin);
    }
    out.grids.push_back(g);
  }
}

}  // namespace fgb
