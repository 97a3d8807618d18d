// feriphys_gb300 -- C++ mirror of the reference's springy-simulation API over
// the C ABI (feriphys_gb300.h).  Header only, C++17.
//
// The reference (jalberse/feriphys) is Rust; its demos drive the cloth step
// through these types and methods, which keep their names and argument
// meaning here:
//   Cloth::new                 springy/cloth.rs:20-113          -> Cloth(...)
//   SpringyMesh::new           springy/springy_mesh.rs:267-401  -> SpringyMesh(...)
//   SpringyMesh::add_strut     springy_mesh.rs:403-413
//   SpringyMesh::add_pin       springy_mesh.rs:415-417
//   SpringyMesh::get_points    springy_mesh.rs:419-421  (Point = Stateful layout, 242-255)
//   SpringyMesh::get_vertices  springy_mesh.rs:500-513
//   accumulate_forces / clear_forces  springy_mesh.rs:515-525, 656-660
//   CollidableMesh::new        collidable_mesh.rs:57-97         -> CollidableMesh(...)
//   Simulation::new / step / get_timestep / get_meshes / get_obstacles /
//   sync_sim_config_from_ui    springy/simulation.rs:17-77      -> Simulation(...)
//   Config, Config::default    springy/config.rs:9-33
// Where the reference panics (bad index, non-manifold edge, degenerate
// obstacle triangle) these throw feriphys_gb300::Error carrying the C ABI's
// status code and message.  Simulation::step queues the fused GPU step and
// returns the timestep like the reference's; reading points waits for it.
#ifndef FERIPHYS_GB300_HPP
#define FERIPHYS_GB300_HPP

#include <chrono>
#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "feriphys_gb300.h"

namespace feriphys_gb300 {

// cgmath::Vector3<f32>
struct Vector3 {
  float x = 0.0f, y = 0.0f, z = 0.0f;
};

// One point in the Stateful layout [mass, position, velocity, accumulated_force].
struct Point {
  float mass = 0.0f;
  Vector3 position, velocity, accumulated_force;
};
static_assert(sizeof(Point) == 10 * sizeof(float), "Point must be the 10-float Stateful layout");

// The reference panics where this is thrown.
class Error : public std::runtime_error {
 public:
  Error(int code, const std::string& message) : std::runtime_error(message), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

inline void check(int rc) {
  if (rc != FGB_OK) throw Error(rc, fgb_last_error());
}

// state.rs:4-8
enum class Integration : int32_t { Euler = FGB_EULER, Rk4 = FGB_RK4 };

// springy/config.rs:9-33.  gravity is a force added to every point
// (springy_mesh.rs:194-196).
struct Config {
  Integration integration = Integration::Rk4;
  float dt = 0.001f;
  Vector3 gravity{0.0f, -10.0f, 0.0f};
  Vector3 wind{0.0f, 0.0f, 0.0f};
  float lift_coefficient = 1.0f;
  float drag_coefficient = 1.0f;
  float coefficient_of_restitution = 0.95f;
  float coefficient_of_friction = 0.3f;

  // Config::default(), from the library.
  static Config default_config() {
    fgb_config c;
    check(fgb_config_default(&c));
    return from_c(c);
  }
  fgb_config to_c() const {
    fgb_config c;
    c.integration = static_cast<int32_t>(integration);
    c.dt = dt;
    c.gravity[0] = gravity.x; c.gravity[1] = gravity.y; c.gravity[2] = gravity.z;
    c.wind[0] = wind.x; c.wind[1] = wind.y; c.wind[2] = wind.z;
    c.lift_coefficient = lift_coefficient;
    c.drag_coefficient = drag_coefficient;
    c.coefficient_of_restitution = coefficient_of_restitution;
    c.coefficient_of_friction = coefficient_of_friction;
    return c;
  }
  static Config from_c(const fgb_config& c) {
    Config o;
    o.integration = static_cast<Integration>(c.integration);
    o.dt = c.dt;
    o.gravity = {c.gravity[0], c.gravity[1], c.gravity[2]};
    o.wind = {c.wind[0], c.wind[1], c.wind[2]};
    o.lift_coefficient = c.lift_coefficient;
    o.drag_coefficient = c.drag_coefficient;
    o.coefficient_of_restitution = c.coefficient_of_restitution;
    o.coefficient_of_friction = c.coefficient_of_friction;
    return o;
  }
};

namespace detail {
inline uint32_t index32(std::size_t i) {
  if (i > 0xffffffffu) throw Error(FGB_EINDEX, "vertex index does not fit the library's 32-bit indices");
  return static_cast<uint32_t>(i);
}
inline std::vector<float> flatten(const std::vector<Vector3>& v) {
  std::vector<float> out;
  out.reserve(3 * v.size());
  for (const Vector3& p : v) {
    out.push_back(p.x);
    out.push_back(p.y);
    out.push_back(p.z);
  }
  return out;
}
inline std::vector<uint32_t> indices32(const std::vector<std::size_t>& v) {
  std::vector<uint32_t> out;
  out.reserve(v.size());
  for (std::size_t i : v) out.push_back(index32(i));
  return out;
}
}  // namespace detail

// A per-edge stiffness/damping override of SpringyMesh::new (StrutKey ->
// SpringConfig, springy_mesh.rs:38-42, 96-107).
struct StrutOverride {
  std::pair<std::size_t, std::size_t> vertex_indices;
  float stiffness = 0.0f, damping = 0.0f;
};

class SpringyMesh {
 public:
  // SpringyMesh::new: mass is the total mass, split evenly over the points.
  SpringyMesh(const std::vector<Vector3>& vertex_positions, const std::vector<std::size_t>& vertex_indices,
              float mass, float default_stiffness, float default_damping,
              const std::vector<StrutOverride>& strut_overrides = {}) {
    const std::vector<float> pos = detail::flatten(vertex_positions);
    const std::vector<uint32_t> idx = detail::indices32(vertex_indices);
    std::vector<fgb_spring_override> ov;
    for (const StrutOverride& o : strut_overrides)
      ov.push_back({detail::index32(o.vertex_indices.first), detail::index32(o.vertex_indices.second), o.stiffness,
                    o.damping});
    check(fgb_mesh_new(pos.data(), vertex_positions.size(), idx.data(), idx.size(), mass, default_stiffness,
                       default_damping, ov.empty() ? nullptr : ov.data(), ov.size(), &h_));
  }
  explicit SpringyMesh(fgb_mesh* adopted) : h_(adopted) {}
  SpringyMesh(SpringyMesh&& o) noexcept : h_(std::exchange(o.h_, nullptr)) {}
  SpringyMesh& operator=(SpringyMesh&& o) noexcept {
    if (this != &o) {
      reset();
      h_ = std::exchange(o.h_, nullptr);
    }
    return *this;
  }
  SpringyMesh(const SpringyMesh&) = delete;
  SpringyMesh& operator=(const SpringyMesh&) = delete;
  ~SpringyMesh() { reset(); }

  void add_strut(std::pair<std::size_t, std::size_t> vertex_indices, float stiffness, float damping) {
    check(fgb_mesh_add_strut(h_, detail::index32(vertex_indices.first), detail::index32(vertex_indices.second),
                             stiffness, damping));
  }
  void add_pin(std::size_t pin_index) { check(fgb_mesh_add_pin(h_, detail::index32(pin_index))); }

  std::size_t num_points() const { return counts()[0]; }
  std::size_t num_struts() const { return counts()[1]; }
  std::size_t num_faces() const { return counts()[2]; }

  // get_points: a copy of the points (waits for queued steps).
  std::vector<Point> get_points() const {
    std::vector<Point> out(num_points());
    check(fgb_mesh_get_points(h_, reinterpret_cast<float*>(out.data())));
    return out;
  }
  // Stateful::from_state_vector applied to every point.
  void set_points(const std::vector<Point>& points) {
    if (points.size() != num_points()) throw Error(FGB_EINVAL, "expected one Point per mesh point");
    check(fgb_mesh_set_points(h_, reinterpret_cast<const float*>(points.data())));
  }
  // get_vertices: positions and the triangle index list.
  std::pair<std::vector<Vector3>, std::vector<std::size_t>> get_vertices() const {
    std::vector<Vector3> pos(num_points());
    std::vector<uint32_t> idx(3 * num_faces());
    check(fgb_mesh_get_vertices(h_, reinterpret_cast<float*>(pos.data()), idx.data()));
    return {std::move(pos), std::vector<std::size_t>(idx.begin(), idx.end())};
  }
  // The phase hooks of Simulation::step (the Simulation runs them fused).
  void accumulate_forces(const Config& config) {
    const fgb_config c = config.to_c();
    check(fgb_mesh_accumulate_forces(h_, &c));
  }
  void clear_forces() { check(fgb_mesh_clear_forces(h_)); }

  fgb_mesh* handle() const { return h_; }

 private:
  std::vector<uint64_t> counts() const {
    std::vector<uint64_t> c(4);
    check(fgb_mesh_counts(h_, c.data()));
    return c;
  }
  void reset() {
    if (h_) fgb_mesh_destroy(h_);
    h_ = nullptr;
  }
  fgb_mesh* h_ = nullptr;
};
static_assert(sizeof(Vector3) == 3 * sizeof(float), "Vector3 must be three packed floats");

// Cloth::new: a rows x cols grid of point_mass points, spacing apart, its
// triangles, the shear overrides, the pins and the binding struts.
struct Cloth {
  SpringyMesh mesh;

  Cloth(std::size_t rows, std::size_t cols, float spacing, Vector3 position, float point_mass,
        float tensile_stiffness, float tensile_damping, float shear_stiffness, float shear_damping,
        float binding_spring_stiffness, float binding_spring_damping, const std::vector<std::size_t>& pinned_vertices)
      : mesh(build(rows, cols, spacing, position, point_mass, tensile_stiffness, tensile_damping, shear_stiffness,
                   shear_damping, binding_spring_stiffness, binding_spring_damping, pinned_vertices)) {}

 private:
  static SpringyMesh build(std::size_t rows, std::size_t cols, float spacing, Vector3 position, float point_mass,
                           float tk, float tc, float sk, float sc, float bk, float bc,
                           const std::vector<std::size_t>& pinned) {
    const float p[3] = {position.x, position.y, position.z};
    const std::vector<uint32_t> pins = detail::indices32(pinned);
    fgb_mesh* h = nullptr;
    check(fgb_cloth_new(rows, cols, spacing, p, point_mass, tk, tc, sk, sc, bk, bc,
                        pins.empty() ? nullptr : pins.data(), pins.size(), &h));
    return SpringyMesh(h);
  }
};

class CollidableMesh {
 public:
  // CollidableMesh::new: a triangle soup; a triangle that repeats a vertex throws.
  CollidableMesh(const std::vector<Vector3>& positions, const std::vector<std::size_t>& indices) {
    const std::vector<float> pos = detail::flatten(positions);
    const std::vector<uint32_t> idx = detail::indices32(indices);
    check(fgb_collidable_new(pos.data(), positions.size(), idx.data(), idx.size(), &h_));
  }
  CollidableMesh(CollidableMesh&& o) noexcept : h_(std::exchange(o.h_, nullptr)) {}
  CollidableMesh& operator=(CollidableMesh&& o) noexcept {
    if (this != &o) {
      if (h_) fgb_collidable_destroy(h_);
      h_ = std::exchange(o.h_, nullptr);
    }
    return *this;
  }
  CollidableMesh(const CollidableMesh&) = delete;
  CollidableMesh& operator=(const CollidableMesh&) = delete;
  ~CollidableMesh() {
    if (h_) fgb_collidable_destroy(h_);
  }
  // (vertices, edges, faces)
  std::vector<uint64_t> counts() const {
    std::vector<uint64_t> c(3);
    check(fgb_collidable_counts(h_, c.data()));
    return c;
  }
  fgb_obstacle* handle() const { return h_; }

 private:
  fgb_obstacle* h_ = nullptr;
};

class Simulation {
 public:
  // Simulation::new: owns its meshes and obstacles; starts from Config::default().
  Simulation(std::vector<SpringyMesh> meshes, std::vector<CollidableMesh> obstacles)
      : meshes_(std::move(meshes)), obstacles_(std::move(obstacles)) {
    std::vector<fgb_mesh*> m;
    std::vector<fgb_obstacle*> o;
    for (const SpringyMesh& x : meshes_) m.push_back(x.handle());
    for (const CollidableMesh& x : obstacles_) o.push_back(x.handle());
    check(fgb_sim_new(m.empty() ? nullptr : m.data(), m.size(), o.empty() ? nullptr : o.data(), o.size(), &h_));
  }
  Simulation(Simulation&& o) noexcept
      : meshes_(std::move(o.meshes_)), obstacles_(std::move(o.obstacles_)), h_(std::exchange(o.h_, nullptr)) {}
  Simulation(const Simulation&) = delete;
  Simulation& operator=(const Simulation&) = delete;
  Simulation& operator=(Simulation&&) = delete;
  ~Simulation() {
    if (h_) fgb_sim_destroy(h_);
  }

  // Simulation::step: one step of every mesh; returns the timestep.
  std::chrono::duration<double> step() {
    check(fgb_sim_step(h_, 1));
    return get_timestep();
  }
  // The timestep as the reference's Duration holds it (whole nanoseconds).
  std::chrono::duration<double> get_timestep() const {
    double s = 0.0;
    check(fgb_sim_get_timestep(h_, &s));
    return std::chrono::duration<double>(s);
  }
  // get_meshes: waits for the queued steps first.
  std::vector<SpringyMesh>& get_meshes() {
    check(fgb_sim_synchronize(h_, nullptr));
    return meshes_;
  }
  const std::vector<CollidableMesh>& get_obstacles() const { return obstacles_; }
  // sync_sim_config_from_ui, headless: the eight Config fields.
  void sync_sim_config_from_ui(const Config& config) {
    const fgb_config c = config.to_c();
    check(fgb_sim_set_config(h_, &c));
  }
  Config get_config() const {
    fgb_config c;
    check(fgb_sim_get_config(h_, &c));
    return Config::from_c(c);
  }
  fgb_sim* handle() const { return h_; }

 private:
  std::vector<SpringyMesh> meshes_;
  std::vector<CollidableMesh> obstacles_;
  fgb_sim* h_ = nullptr;
};

}  // namespace feriphys_gb300

#endif  // FERIPHYS_GB300_HPP
