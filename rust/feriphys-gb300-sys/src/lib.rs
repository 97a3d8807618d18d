//! Raw bindings to `libferiphys_gb300`, the GB300 (sm_103a) cloth step behind
//! the C ABI of `include/feriphys_gb300.h`.
//!
//! Every item mirrors one declaration of that header, in its order, with the
//! same names, argument order and meaning.  Status codes are `c_int`: 0 is
//! success, a negative value one of the `FGB_E*` constants below, with the
//! message in `fgb_last_error()`.  The safe wrappers with the reference's
//! method names (`SpringyMesh`, `Cloth`, `Simulation`) live in the
//! `feriphys-gb300` crate next to this one.
//!
//! The declarations replace these reference items (paths inside
//! jalberse/feriphys):
//! * `fgb_mesh_new` -- `SpringyMesh::new` (src/simulation/springy/springy_mesh.rs:267-401)
//! * `fgb_cloth_new` -- `Cloth::new` (src/simulation/springy/cloth.rs:20-113)
//! * `fgb_mesh_add_strut` / `fgb_mesh_add_pin` -- springy_mesh.rs:403-417
//! * `fgb_mesh_get_points` / `fgb_mesh_set_points` -- `get_points` (springy_mesh.rs:419-421) in the
//!   `Stateful` layout (springy_mesh.rs:199-256)
//! * `fgb_mesh_get_vertices` -- springy_mesh.rs:500-513
//! * `fgb_mesh_accumulate_forces` / `fgb_mesh_integrate` / `fgb_mesh_update_points` /
//!   `fgb_mesh_clear_forces` -- the phases of `Simulation::step` (src/simulation/springy/simulation.rs:27-45)
//! * `fgb_collidable_new` -- `CollidableMesh::new` (src/simulation/collidable_mesh.rs:57-97)
//! * `fgb_sim_new` / `fgb_sim_step` / `fgb_sim_get_timestep` / `fgb_sim_set_config` --
//!   `Simulation::new`, `step`, `get_timestep`, `sync_sim_config_from_ui` (simulation.rs:17-77)
//! * `FgbConfig` -- `Config` (src/simulation/springy/config.rs:9-33)
//!
//! The remaining entry points are extensions with no reference counterpart
//! (batching, streams, the FP64 rerun, the GPU mesh build, the render export,
//! the allocation-free step and the learned surrogate).
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_int, c_void};

pub const FGB_OK: c_int = 0;
/// bad argument (null pointer, bad size, bad dt)
pub const FGB_EINVAL: c_int = -1;
/// vertex index out of range
pub const FGB_EINDEX: c_int = -2;
/// an edge has more than two faces (springy_mesh.rs:339)
pub const FGB_ENONMANIFOLD: c_int = -3;
/// CUDA runtime error (the message has the CUDA text)
pub const FGB_ECUDA: c_int = -4;
/// call not valid in the handle's current state
pub const FGB_ESTATE: c_int = -5;
/// host or device allocation failed
pub const FGB_ENOMEM: c_int = -6;
/// a device-side check failed (see the message)
pub const FGB_ECHECK: c_int = -7;

/// state.rs:4-8
pub const FGB_EULER: i32 = 0;
pub const FGB_RK4: i32 = 1;

/// springy/config.rs:9-18.  `gravity` is a force added to every point
/// (springy_mesh.rs:194-196); drag and lift have no air density
/// (springy_mesh.rs:636-646).
#[repr(C)]
#[derive(Clone, Copy, Debug, Default, PartialEq)]
pub struct FgbConfig {
    pub integration: i32,
    pub dt: f32,
    pub gravity: [f32; 3],
    pub wind: [f32; 3],
    pub lift_coefficient: f32,
    pub drag_coefficient: f32,
    pub coefficient_of_restitution: f32,
    pub coefficient_of_friction: f32,
}

/// StrutKey + SpringConfig (springy_mesh.rs:38-42, 96-107): per-edge override
/// of the default stiffness and damping used by `SpringyMesh::new`.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default, PartialEq)]
pub struct FgbSpringOverride {
    pub a: u32,
    pub b: u32,
    pub stiffness: f32,
    pub damping: f32,
}

/// Per-cloth energy and strain check of the learned surrogate's coarse steps.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default, PartialEq)]
pub struct FgbSurrogateCheck {
    pub enabled: i32,
    pub energy_growth: f32,
    pub energy_abs: f32,
    pub max_strain: f32,
}

/// Opaque handles (owned by the library; destroy with the matching call).
#[repr(C)]
pub struct FgbMesh {
    _private: [u8; 0],
}
#[repr(C)]
pub struct FgbObstacle {
    _private: [u8; 0],
}
#[repr(C)]
pub struct FgbSim {
    _private: [u8; 0],
}
#[repr(C)]
pub struct FgbSurrogate {
    _private: [u8; 0],
}

extern "C" {
    // ---- errors and configuration
    pub fn fgb_last_error() -> *const c_char;
    pub fn fgb_config_default(out: *mut FgbConfig) -> c_int;

    // ---- SpringyMesh / Cloth construction
    pub fn fgb_mesh_new(positions: *const f32, n_vertices: u64, indices: *const u32, n_indices: u64, mass: f32,
                        default_stiffness: f32, default_damping: f32, overrides: *const FgbSpringOverride,
                        n_overrides: u64, out: *mut *mut FgbMesh) -> c_int;
    pub fn fgb_mesh_new_device(positions: *const f32, n_vertices: u64, indices: *const u32, n_indices: u64,
                               mass: f32, default_stiffness: f32, default_damping: f32,
                               overrides: *const FgbSpringOverride, n_overrides: u64,
                               out: *mut *mut FgbMesh) -> c_int;
    pub fn fgb_cloth_new(rows: u64, cols: u64, spacing: f32, position: *const f32, point_mass: f32,
                         tensile_stiffness: f32, tensile_damping: f32, shear_stiffness: f32, shear_damping: f32,
                         binding_stiffness: f32, binding_damping: f32, pinned: *const u32, n_pinned: u64,
                         out: *mut *mut FgbMesh) -> c_int;
    pub fn fgb_mesh_add_strut(m: *mut FgbMesh, a: u32, b: u32, stiffness: f32, damping: f32) -> c_int;
    pub fn fgb_mesh_add_pin(m: *mut FgbMesh, index: u32) -> c_int;
    pub fn fgb_mesh_add_struts(m: *mut FgbMesh, a: *const u32, b: *const u32, stiffness: *const f32,
                               damping: *const f32, n: u64) -> c_int;
    pub fn fgb_mesh_add_pins(m: *mut FgbMesh, index: *const u32, n: u64) -> c_int;
    pub fn fgb_mesh_counts(m: *const FgbMesh, out: *mut u64) -> c_int;
    pub fn fgb_mesh_get_struts(m: *const FgbMesh, kcl: *mut f32, ab: *mut u32) -> c_int;
    pub fn fgb_mesh_set_strut_params(m: *mut FgbMesh, stiffness: *const f32, damping: *const f32) -> c_int;

    // ---- state in and out
    pub fn fgb_mesh_get_points(m: *mut FgbMesh, out: *mut f32) -> c_int;
    pub fn fgb_mesh_set_points(m: *mut FgbMesh, input: *const f32) -> c_int;
    pub fn fgb_mesh_get_positions(m: *mut FgbMesh, out: *mut f32) -> c_int;
    pub fn fgb_mesh_get_points_f64(m: *mut FgbMesh, out: *mut f64) -> c_int;
    pub fn fgb_mesh_get_vertices(m: *mut FgbMesh, positions: *mut f32, indices: *mut u32) -> c_int;
    pub fn fgb_mesh_export_vertices(m: *mut FgbMesh, device_out: *mut c_void, color: *const f32,
                                    stream: *mut c_void) -> c_int;
    pub fn fgb_mesh_export_indices(m: *mut FgbMesh, device_out: *mut c_void, stream: *mut c_void) -> c_int;

    // ---- kernel choice and precision
    pub fn fgb_mesh_set_path(m: *mut FgbMesh, path: c_int) -> c_int;
    pub fn fgb_mesh_get_path(m: *mut FgbMesh, path: *mut c_int) -> c_int;
    pub fn fgb_mesh_set_precision(m: *mut FgbMesh, bits: c_int) -> c_int;

    // ---- the phases of Simulation::step
    pub fn fgb_mesh_accumulate_forces(m: *mut FgbMesh, cfg: *const FgbConfig) -> c_int;
    pub fn fgb_mesh_integrate(m: *mut FgbMesh, integration: i32, dt: f32) -> c_int;
    pub fn fgb_mesh_update_points(m: *mut FgbMesh, obstacles: *const *mut FgbObstacle, n_obstacles: u64,
                                  cfg: *const FgbConfig) -> c_int;
    pub fn fgb_mesh_clear_forces(m: *mut FgbMesh) -> c_int;
    pub fn fgb_mesh_synchronize(m: *mut FgbMesh) -> c_int;
    pub fn fgb_mesh_destroy(m: *mut FgbMesh) -> c_int;

    // ---- CollidableMesh
    pub fn fgb_collidable_new(positions: *const f32, n_vertices: u64, indices: *const u32, n_indices: u64,
                              out: *mut *mut FgbObstacle) -> c_int;
    pub fn fgb_collidable_counts(o: *const FgbObstacle, out: *mut u64) -> c_int;
    pub fn fgb_collidable_destroy(o: *mut FgbObstacle) -> c_int;

    // ---- Simulation
    pub fn fgb_sim_new(meshes: *const *mut FgbMesh, n_meshes: u64, obstacles: *const *mut FgbObstacle,
                       n_obstacles: u64, out: *mut *mut FgbSim) -> c_int;
    pub fn fgb_sim_set_config(s: *mut FgbSim, cfg: *const FgbConfig) -> c_int;
    pub fn fgb_sim_get_config(s: *const FgbSim, out: *mut FgbConfig) -> c_int;
    pub fn fgb_sim_step(s: *mut FgbSim, n_steps: u64) -> c_int;
    pub fn fgb_mesh_set_wind(m: *mut FgbMesh, wind: *const f32) -> c_int;
    pub fn fgb_sim_set_graphs(s: *mut FgbSim, enabled: c_int) -> c_int;
    pub fn fgb_sim_set_batch_mode(s: *mut FgbSim, mode: c_int) -> c_int;
    pub fn fgb_sim_set_batch_tile(s: *mut FgbSim, tile_rows: c_int) -> c_int;
    pub fn fgb_sim_batch_info(s: *const FgbSim, out: *mut i64) -> c_int;
    pub fn fgb_sim_set_collision_broadphase(s: *mut FgbSim, enabled: c_int) -> c_int;
    pub fn fgb_sim_set_stream(s: *mut FgbSim, stream: *mut c_void) -> c_int;
    pub fn fgb_sim_step_static(s: *mut FgbSim, n_steps: u64, stream: *mut c_void) -> c_int;
    pub fn fgb_sim_get_timestep(s: *const FgbSim, seconds: *mut f64) -> c_int;
    pub fn fgb_sim_synchronize(s: *mut FgbSim, nonfinite: *mut c_int) -> c_int;
    pub fn fgb_sim_destroy(s: *mut FgbSim) -> c_int;

    // ---- the learned surrogate
    pub fn fgb_surrogate_new(seed: u64, out: *mut *mut FgbSurrogate) -> c_int;
    pub fn fgb_surrogate_destroy(g: *mut FgbSurrogate) -> c_int;
    pub fn fgb_surrogate_get_params(g: *mut FgbSurrogate, out: *mut f32) -> c_int;
    pub fn fgb_surrogate_set_params(g: *mut FgbSurrogate, input: *const f32) -> c_int;
    pub fn fgb_surrogate_set_normalization(g: *mut FgbSurrogate, in_mean: *const f32, in_std: *const f32,
                                           out_mean: *const f32, out_std: *const f32) -> c_int;
    pub fn fgb_surrogate_get_normalization(g: *const FgbSurrogate, in_mean: *mut f32, in_std: *mut f32,
                                           out_mean: *mut f32, out_std: *mut f32) -> c_int;
    pub fn fgb_surrogate_features(g: *mut FgbSurrogate, m: *mut FgbMesh, coarse_dt: f32, wind: *const f32,
                                  out: *mut f32) -> c_int;
    pub fn fgb_surrogate_forward(g: *mut FgbSurrogate, x: *const f32, n: u64, y: *mut f32) -> c_int;
    pub fn fgb_surrogate_gradients(g: *mut FgbSurrogate, x: *const f32, t: *const f32, n: u64, grad: *mut f32,
                                   loss: *mut f32) -> c_int;
    pub fn fgb_surrogate_train_batch(g: *mut FgbSurrogate, x: *const f32, t: *const f32, n: u64, lr: f32,
                                     loss: *mut f32) -> c_int;
    pub fn fgb_surrogate_dataset_reserve(g: *mut FgbSurrogate, capacity_rows: u64) -> c_int;
    pub fn fgb_surrogate_collect(g: *mut FgbSurrogate, s: *mut FgbSim, ratio: u32, n_coarse: u64) -> c_int;
    pub fn fgb_surrogate_dataset_info(g: *const FgbSurrogate, out: *mut u64) -> c_int;
    pub fn fgb_surrogate_dataset_get(g: *mut FgbSurrogate, first: u64, n: u64, feat: *mut f32,
                                     tgt: *mut f32) -> c_int;
    pub fn fgb_surrogate_fit_normalization(g: *mut FgbSurrogate) -> c_int;
    pub fn fgb_surrogate_train(g: *mut FgbSurrogate, n_steps: u64, batch: u64, lr: f32, seed: u64,
                               losses: *mut f32) -> c_int;
    pub fn fgb_sim_step_surrogate(s: *mut FgbSim, g: *mut FgbSurrogate, ratio: u32, n_coarse: u64,
                                  chk: *const FgbSurrogateCheck, n_fallbacks: *mut u64) -> c_int;
    pub fn fgb_sim_energy(s: *mut FgbSim, out: *mut f32) -> c_int;
}
