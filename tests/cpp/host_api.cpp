// The C++ mirror of the reference's springy API (include/feriphys_gb300.hpp)
// driven like the reference's own unit tests, on the host only (mesh
// construction, points, vertices, errors, Simulation set-up and Config): no
// step runs here, so no GPU is needed.  Prints "ok" and returns 0 when every
// check holds.
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "feriphys_gb300.hpp"

namespace fg = feriphys_gb300;

static int failures = 0;
#define EXPECT(cond)                                                   \
  do {                                                                 \
    if (!(cond)) {                                                     \
      std::fprintf(stderr, "%s:%d: failed: %s\n", __FILE__, __LINE__, #cond); \
      ++failures;                                                      \
    }                                                                  \
  } while (0)

template <class F>
static int thrown_code(F&& f) {
  try {
    f();
  } catch (const fg::Error& e) {
    return e.code();
  }
  return 0;
}

int main() {
  // springy_mesh.rs:721-757 (ctor_triangle): mass split evenly, k and c scaled by 1/L
  {
    fg::SpringyMesh mesh({{0, 0, 0}, {2, 0, 0}, {0, 1, 0}}, {0, 1, 2}, 1.0f, 2.0f, 3.0f);
    EXPECT(mesh.num_points() == 3 && mesh.num_struts() == 3 && mesh.num_faces() == 1);
    const std::vector<fg::Point> pts = mesh.get_points();
    EXPECT(pts[0].mass == 1.0f / 3.0f);
    EXPECT(pts[1].position.x == 2.0f && pts[1].velocity.x == 0.0f && pts[1].accumulated_force.y == 0.0f);
    const auto verts = mesh.get_vertices();
    EXPECT(verts.first.size() == 3 && verts.second.size() == 3 && verts.second[2] == 2);
  }
  // springy/config.rs:20-32 (Config::default)
  {
    const fg::Config c = fg::Config::default_config();
    EXPECT(c.integration == fg::Integration::Rk4 && c.dt == 0.001f);
    EXPECT(c.gravity.y == -10.0f && c.lift_coefficient == 1.0f && c.drag_coefficient == 1.0f);
    EXPECT(c.coefficient_of_restitution == 0.95f && c.coefficient_of_friction == 0.3f);
  }
  // cloth.rs:20-113: a 4 x 3 cloth with two pins
  fg::Cloth cloth(4, 3, 0.5f, {0, 0, 0}, 0.01f, 5.0f, 0.1f, 2.0f, 0.1f, 1.0f, 0.1f, {9, 11});
  EXPECT(cloth.mesh.num_points() == 12 && cloth.mesh.num_struts() == 27 && cloth.mesh.num_faces() == 12);
  {
    const auto verts = cloth.mesh.get_vertices();
    EXPECT(verts.first.size() == 12 && verts.second.size() == 36);
    const std::vector<fg::Point> pts = cloth.mesh.get_points();
    EXPECT(pts[4].mass == 0.01f);
    // grid position (col * s, row * s, 0) - (cols / 2 * s, rows / 2 * s, 0) + position, with the
    // halves in f32 (cloth.rs:36-55): point 4 is row 1, col 1
    EXPECT(pts[4].position.x == 1 * 0.5f - 1.5f * 0.5f && pts[4].position.y == 1 * 0.5f - 2.0f * 0.5f);
  }
  // panics of the reference: a pin out of range, an edge with three faces,
  // an obstacle triangle that repeats a vertex
  EXPECT(thrown_code([&] { cloth.mesh.add_pin(12); }) == FGB_EINDEX);
  EXPECT(thrown_code([] {
           fg::SpringyMesh m({{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 1}}, {0, 1, 2, 0, 1, 3, 0, 1, 4},
                             1.0f, 1.0f, 1.0f);
         }) == FGB_ENONMANIFOLD);
  EXPECT(thrown_code([] { fg::CollidableMesh o({{0, 0, 0}, {1, 0, 0}, {0, 1, 0}}, {0, 0, 1}); }) == FGB_EINVAL);
  // add_strut appends in order
  cloth.mesh.add_strut({0, 11}, 3.0f, 0.2f);
  EXPECT(cloth.mesh.num_struts() == 28);
  // Simulation::new, get_timestep, sync_sim_config_from_ui, get_meshes, get_obstacles
  std::vector<fg::SpringyMesh> meshes;
  meshes.push_back(std::move(cloth.mesh));
  std::vector<fg::CollidableMesh> obstacles;
  obstacles.emplace_back(std::vector<fg::Vector3>{{-3, -1.5f, 3}, {3, -1.5f, 3}, {3, -1.5f, -3}, {-3, -1.5f, -3}},
                         std::vector<std::size_t>{0, 1, 2, 0, 2, 3});
  fg::Simulation sim(std::move(meshes), std::move(obstacles));
  EXPECT(sim.get_timestep().count() == 0.001);
  fg::Config c = fg::Config::default_config();
  c.integration = fg::Integration::Euler;
  c.dt = 1.0f / 600.0f;
  c.wind = {2.0f, 0.0f, 1.0f};
  sim.sync_sim_config_from_ui(c);
  EXPECT(sim.get_timestep().count() == 0.001666667);  // Duration keeps whole nanoseconds
  const fg::Config back = sim.get_config();
  EXPECT(back.integration == fg::Integration::Euler && back.dt == c.dt && back.wind.z == 1.0f);
  EXPECT(sim.get_meshes().size() == 1 && sim.get_meshes()[0].num_points() == 12);
  EXPECT(sim.get_obstacles().size() == 1 && sim.get_obstacles()[0].counts()[2] == 2);
  if (failures) return 1;
  std::printf("ok\n");
  return 0;
}
