// Exact broad phase for the first-hit vertex/obstacle-face search
// (collidable_mesh.rs:107-169).
//
// The reference accepts face f for a point moving from `old` to `new` when
// (1) the computed plane distances d_old, d_new differ in sign and (2) the
// computed crossing point cp = old + (dt*f)*((new-old)/dt),
// f = d_old/(d_old - d_new), projected onto the coordinate plane that drops
// the face's axis a (chosen by signed normal comparisons, lines 133-154),
// passes three cross-product sign tests against the projected triangle.
// Three bounds confine every accepted cp:
//  * f lies in [0, 1], so cp lies in the segment's box up to a few ulps;
//  * writing d = D + e with D the exact distance and |e| <= err (a few ulps
//    of |p - v0|), D(cp) = -eps*d_old - (1-f)*e_old - f*e_new, so cp lies
//    within err + 2u*|d_old| (+ the box slack) of the face's plane;
//  * a sign test can only err within a few ulps (times size / sin of the
//    smallest projected angle) of an edge line, so the projection of an
//    accepted cp lies in the projected triangle grown by a margin R.
// Together: cp lies in the face's 3D box grown by R along the two projected
// axes and by (R*(|n_u| + |n_w|) + tau) / |n_a| along a.  The face can only
// be hit when the segment's box (grown by its slack) meets that region.
// Each obstacle gets a 3D grid of its faces' regions; a query uses the
// cell holding its box (or, when the box does not fit one cell grown by the
// slack, tests every face of that obstacle).  Faces whose region cannot be
// bounded (degenerate projection, tiny |n_a|, non-finite data) are tested
// for every query.  Obstacles are visited in order and candidates in
// ascending face index, so the first hit is the reference's first hit.
#pragma once

#include <stdint.h>

#include <vector>

#include "step_consts.h"

namespace fgb {

struct AccelHost {
  std::vector<ObsGrid3> grids;  // one per obstacle with faces, in obstacle order
  std::vector<int> cell_off;    // all grids' cells, concatenated (+1 sentinel per grid)
  std::vector<int> cell_faces;  // ascending face ids per cell
  std::vector<int> always;      // per grid: faces every query must test (ascending)
};

// faces: flattened obstacle faces; first_face[k], n_faces[k]: obstacle k's range.
void build_obstacle_accel(const std::vector<ObsFace>& faces, const std::vector<int>& first_face,
                          const std::vector<int>& n_faces, AccelHost& out);

}  // namespace fgb
