// Step constants shared by the host launcher and every kernel (POD, passed by
// value as a kernel argument).
#pragma once

#include <stdint.h>
#include <vector_types.h>

namespace fgb {

// One obstacle face as stored on the device: v0 (w = drop axis 0/1/2 as
// float bits), v1, v2, unit normal (computed on the host exactly as
// collidable_mesh.rs:41-43 does).
struct ObsFace {
  float4 v0, v1, v2, n;
};

// Broad-phase grid of one obstacle (see obstacle_accel.h): a uniform 3D grid
// over the union of its faces' acceptance regions; each cell lists, in
// ascending order, the faces whose region meets the cell grown by 2*slack.
struct ObsGrid3 {
  float lo[3], hi[3];  // union of the faces' regions (outward-rounded)
  float cell[3];       // cell size
  float inv[3];        // 1 / cell size
  float slack;         // a query box must fit its cell grown by this
  int n[3];            // cells per axis (0: no bounded face)
  int off_base;        // first entry of this grid in cell_off
  int face_base, n_faces;     // the obstacle's faces in the flattened order
  int always_base, n_always;  // faces tested for every query (in `always`)
};

struct ObsAccel {
  int enabled;
  int n_grids;
  const ObsGrid3* grids;
  const int* cell_off;
  const int* cell_faces;
  const int* always;
};

struct StepConsts {
  int integration;     // 0 Euler, 1 Rk4 (state.rs:4-8)
  float dt;            // config.dt (springy/config.rs:11)
  float dt_duration;   // Duration::from_secs_f32(dt).as_secs_f32() (collidable_mesh.rs:114,129)
  float force0[3];     // 0 + config.gravity: the first term of every point's force
  float wind[3];
  float neg_drag;      // -1.0 * config.drag_coefficient (springy_mesh.rs:638)
  float neg_lift;      // -1.0 * config.lift_coefficient (springy_mesh.rs:639-640)
  float restitution;
  float friction;
  int n_obstacle_faces;
  const void* obstacle_faces;  // ObsFace[n_obstacle_faces], flattened obstacle order
  unsigned* flags;             // bit 0: a stepped vertex went non-finite; bit 1: a staging copy timed out
  ObsAccel accel;              // broad phase over obstacle_faces (enabled = 0: test all faces)
  float one;                   // 1.0f, set by the host: a unit multiplier the device compiler cannot see as 1
                               // (face_pair.cuh uses it to keep packed sums of products unfused)
};

}  // namespace fgb
