// Step constants shared by the host launcher and every kernel (POD, passed by
// value as a kernel argument).
#pragma once

#include <stdint.h>

namespace fgb {

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
  unsigned* flags;             // bit 0: a stepped vertex went non-finite
};

}  // namespace fgb
