//! GPU-backed drop-ins for the springy cloth types of jalberse/feriphys.
//!
//! `SpringyMesh`, `Cloth`, `CollidableMesh`, `Simulation` and `Config` keep
//! the reference's constructors and method names (paths inside the reference
//! project):
//! * `SpringyMesh::new`, `add_strut`, `add_pin`, `get_points`, `get_vertices`
//!   -- src/simulation/springy/springy_mesh.rs:267-513
//! * `Cloth::new` -- src/simulation/springy/cloth.rs:20-113
//! * `CollidableMesh::new` -- src/simulation/collidable_mesh.rs:57-97
//! * `Simulation::new`, `step`, `get_timestep`, `get_meshes`, `get_obstacles`,
//!   `sync_sim_config_from_ui` -- src/simulation/springy/simulation.rs:17-77
//! * `Config` and its defaults -- src/simulation/springy/config.rs:9-33
//!
//! so a demo loop such as src/demos/cloth.rs:107-138 keeps its shape with the
//! GPU step underneath.  Where the reference panics (a non-manifold edge,
//! springy_mesh.rs:339; an index out of range) these types panic too, with
//! the library's message.  Vectors are `cgmath` 0.18's, as in the reference.
use std::ffi::CStr;
use std::os::raw::c_int;
use std::time::Duration;

use cgmath::Vector3;
use feriphys_gb300_sys as sys;

fn check(rc: c_int) {
    if rc != sys::FGB_OK {
        let msg = unsafe { CStr::from_ptr(sys::fgb_last_error()) }.to_string_lossy().into_owned();
        panic!("feriphys_gb300 error {rc}: {msg}");
    }
}

/// state.rs:4-8
#[derive(Clone, Copy, Debug, PartialEq, Eq)]
pub enum Integration {
    Euler,
    Rk4,
}

/// springy/config.rs:9-18.  `gravity` is the force added to every point
/// (springy_mesh.rs:194-196).
#[derive(Clone, Copy, Debug, PartialEq)]
pub struct Config {
    pub integration: Integration,
    pub dt: f32,
    pub gravity: Vector3<f32>,
    pub wind: Vector3<f32>,
    pub lift_coefficient: f32,
    pub drag_coefficient: f32,
    pub coefficient_of_restitution: f32,
    pub coefficient_of_friction: f32,
}

impl Default for Config {
    /// springy/config.rs:21-33, as the library states them (`fgb_config_default`).
    fn default() -> Self {
        let mut c = sys::FgbConfig::default();
        check(unsafe { sys::fgb_config_default(&mut c) });
        Config::from_raw(&c)
    }
}

impl Config {
    fn from_raw(c: &sys::FgbConfig) -> Self {
        Config {
            integration: if c.integration == sys::FGB_EULER { Integration::Euler } else { Integration::Rk4 },
            dt: c.dt,
            gravity: Vector3::new(c.gravity[0], c.gravity[1], c.gravity[2]),
            wind: Vector3::new(c.wind[0], c.wind[1], c.wind[2]),
            lift_coefficient: c.lift_coefficient,
            drag_coefficient: c.drag_coefficient,
            coefficient_of_restitution: c.coefficient_of_restitution,
            coefficient_of_friction: c.coefficient_of_friction,
        }
    }

    fn to_raw(&self) -> sys::FgbConfig {
        sys::FgbConfig {
            integration: match self.integration {
                Integration::Euler => sys::FGB_EULER,
                Integration::Rk4 => sys::FGB_RK4,
            },
            dt: self.dt,
            gravity: [self.gravity.x, self.gravity.y, self.gravity.z],
            wind: [self.wind.x, self.wind.y, self.wind.z],
            lift_coefficient: self.lift_coefficient,
            drag_coefficient: self.drag_coefficient,
            coefficient_of_restitution: self.coefficient_of_restitution,
            coefficient_of_friction: self.coefficient_of_friction,
        }
    }
}

/// springy_mesh.rs:176-182: one point of the mesh, as `get_points` returns it.
#[derive(Clone, Copy, Debug, PartialEq)]
pub struct Point {
    pub mass: f32,
    pub position: Vector3<f32>,
    pub velocity: Vector3<f32>,
    pub accumulated_force: Vector3<f32>,
}

/// A SpringyMesh whose state lives on the GPU.
pub struct SpringyMesh(*mut sys::FgbMesh);

impl SpringyMesh {
    /// springy_mesh.rs:267-401.  `strut_overrides` maps an edge (either
    /// vertex order) to its nominal (stiffness, damping).  Torsional springs
    /// are not supported: their force is not applied by the reference either
    /// (springy_mesh.rs:518-519).
    pub fn new(vertex_positions: Vec<Vector3<f32>>, vertex_indices: Vec<usize>, mass: f32, default_stiffness: f32,
               default_damping: f32, strut_overrides: &Option<Vec<((usize, usize), (f32, f32))>>) -> Self {
        Self::build(vertex_positions, vertex_indices, mass, default_stiffness, default_damping, strut_overrides,
                    false)
    }

    /// The same mesh as `new`, bit for bit, with the strut de-duplication run
    /// on the GPU (large meshes).
    pub fn new_on_device(vertex_positions: Vec<Vector3<f32>>, vertex_indices: Vec<usize>, mass: f32,
                         default_stiffness: f32, default_damping: f32,
                         strut_overrides: &Option<Vec<((usize, usize), (f32, f32))>>) -> Self {
        Self::build(vertex_positions, vertex_indices, mass, default_stiffness, default_damping, strut_overrides,
                    true)
    }

    fn build(vertex_positions: Vec<Vector3<f32>>, vertex_indices: Vec<usize>, mass: f32, default_stiffness: f32,
             default_damping: f32, strut_overrides: &Option<Vec<((usize, usize), (f32, f32))>>,
             on_device: bool) -> Self {
        let pos: Vec<f32> = vertex_positions.iter().flat_map(|v| [v.x, v.y, v.z]).collect();
        let idx: Vec<u32> = vertex_indices.iter().map(|&i| u32::try_from(i).expect("vertex index")).collect();
        let ov: Vec<sys::FgbSpringOverride> = strut_overrides
            .iter()
            .flatten()
            .map(|&((a, b), (k, c))| sys::FgbSpringOverride { a: a as u32, b: b as u32, stiffness: k, damping: c })
            .collect();
        let mut m = std::ptr::null_mut();
        let f = if on_device { sys::fgb_mesh_new_device } else { sys::fgb_mesh_new };
        check(unsafe {
            f(pos.as_ptr(), vertex_positions.len() as u64, idx.as_ptr(), idx.len() as u64, mass, default_stiffness,
              default_damping, ov.as_ptr(), ov.len() as u64, &mut m)
        });
        SpringyMesh(m)
    }

    /// springy_mesh.rs:403-413
    pub fn add_strut(&mut self, vertex_indices: (usize, usize), stiffness: f32, damping: f32) {
        check(unsafe {
            sys::fgb_mesh_add_strut(self.0, vertex_indices.0 as u32, vertex_indices.1 as u32, stiffness, damping)
        });
    }

    /// springy_mesh.rs:415-417
    pub fn add_pin(&mut self, pin_index: usize) {
        check(unsafe { sys::fgb_mesh_add_pin(self.0, pin_index as u32) });
    }

    fn counts(&self) -> [u64; 4] {
        let mut c = [0u64; 4];
        check(unsafe { sys::fgb_mesh_counts(self.0, c.as_mut_ptr()) });
        c
    }

    /// springy_mesh.rs:419-421 (a copy: the points live on the GPU).
    pub fn get_points(&mut self) -> Vec<Point> {
        self.get_points_state()
            .chunks(10)
            .map(|s| Point {
                mass: s[0],
                position: Vector3::new(s[1], s[2], s[3]),
                velocity: Vector3::new(s[4], s[5], s[6]),
                accumulated_force: Vector3::new(s[7], s[8], s[9]),
            })
            .collect()
    }

    /// Every point in the `Stateful` layout (springy_mesh.rs:242-255):
    /// [mass, position, velocity, accumulated_force], 10 f32 per point.
    pub fn get_points_state(&mut self) -> Vec<f32> {
        let n = self.counts()[0] as usize;
        let mut out = vec![0f32; 10 * n];
        check(unsafe { sys::fgb_mesh_get_points(self.0, out.as_mut_ptr()) });
        out
    }

    /// `Stateful::from_state_vector` for every point (10 f32 per point).
    pub fn set_points_state(&mut self, state: &[f32]) {
        assert_eq!(state.len(), 10 * self.counts()[0] as usize, "state vector length"); // springy_mesh.rs:205-206
        check(unsafe { sys::fgb_mesh_set_points(self.0, state.as_ptr()) });
    }

    /// springy_mesh.rs:500-513: vertex positions and the triangle index list.
    pub fn get_vertices(&mut self) -> (Vec<Vector3<f32>>, Vec<usize>) {
        let c = self.counts();
        let (n, f) = (c[0] as usize, c[2] as usize);
        let (mut pos, mut idx) = (vec![0f32; 3 * n], vec![0u32; 3 * f]);
        check(unsafe { sys::fgb_mesh_get_vertices(self.0, pos.as_mut_ptr(), idx.as_mut_ptr()) });
        (pos.chunks(3).map(|p| Vector3::new(p[0], p[1], p[2])).collect(), idx.iter().map(|&i| i as usize).collect())
    }

    /// Per-mesh wind (an extension: the reference's wind is global, config.rs:13).
    pub fn set_wind(&mut self, wind: Option<Vector3<f32>>) {
        let w = wind.map(|v| [v.x, v.y, v.z]);
        check(unsafe { sys::fgb_mesh_set_wind(self.0, w.as_ref().map_or(std::ptr::null(), |a| a.as_ptr())) });
    }

    /// The raw handle, for the extension calls of `feriphys_gb300_sys`.
    pub fn as_raw(&self) -> *mut sys::FgbMesh {
        self.0
    }
}

impl Drop for SpringyMesh {
    fn drop(&mut self) {
        unsafe {
            sys::fgb_mesh_destroy(self.0);
        }
    }
}

/// cloth.rs:9-11
pub struct Cloth {
    pub mesh: SpringyMesh,
}

impl Cloth {
    /// cloth.rs:20-113, same arguments.
    #[allow(clippy::too_many_arguments)]
    pub fn new(rows: usize, cols: usize, spacing: f32, position: Vector3<f32>, point_mass: f32,
               tensile_stiffness: f32, tensile_damping: f32, shear_stiffness: f32, shear_damping: f32,
               binding_spring_stiffness: f32, binding_spring_damping: f32, pinned_vertices: Vec<usize>) -> Self {
        let p = [position.x, position.y, position.z];
        let pins: Vec<u32> = pinned_vertices.iter().map(|&i| i as u32).collect();
        let mut m = std::ptr::null_mut();
        check(unsafe {
            sys::fgb_cloth_new(rows as u64, cols as u64, spacing, p.as_ptr(), point_mass, tensile_stiffness,
                               tensile_damping, shear_stiffness, shear_damping, binding_spring_stiffness,
                               binding_spring_damping, pins.as_ptr(), pins.len() as u64, &mut m)
        });
        Cloth { mesh: SpringyMesh(m) }
    }
}

/// collidable_mesh.rs:49-97: a static triangle soup the points collide with.
pub struct CollidableMesh {
    handle: *mut sys::FgbObstacle,
    vertex_positions: Vec<Vector3<f32>>,
    vertex_indices: Vec<usize>,
}

impl CollidableMesh {
    /// collidable_mesh.rs:57-97
    pub fn new(vertex_positions: Vec<Vector3<f32>>, vertex_indices: Vec<usize>) -> Self {
        let p: Vec<f32> = vertex_positions.iter().flat_map(|v| [v.x, v.y, v.z]).collect();
        let i: Vec<u32> = vertex_indices.iter().map(|&x| x as u32).collect();
        let mut h = std::ptr::null_mut();
        check(unsafe { sys::fgb_collidable_new(p.as_ptr(), vertex_positions.len() as u64, i.as_ptr(),
                                               i.len() as u64, &mut h) });
        CollidableMesh { handle: h, vertex_positions, vertex_indices }
    }

    /// The construction's vertices and indices (for rendering).
    pub fn get_vertices(&self) -> (&[Vector3<f32>], &[usize]) {
        (&self.vertex_positions, &self.vertex_indices)
    }
}

impl Drop for CollidableMesh {
    fn drop(&mut self) {
        unsafe {
            sys::fgb_collidable_destroy(self.handle);
        }
    }
}

/// springy/simulation.rs:10-15: the meshes, the obstacles and the config.
pub struct Simulation {
    sim: *mut sys::FgbSim,
    meshes: Vec<SpringyMesh>,
    obstacles: Vec<CollidableMesh>,
}

impl Simulation {
    /// springy/simulation.rs:17-25 (starts from `Config::default()`).
    pub fn new(meshes: Vec<SpringyMesh>, obstacles: Vec<CollidableMesh>) -> Self {
        let ms: Vec<*mut sys::FgbMesh> = meshes.iter().map(|m| m.0).collect();
        let os: Vec<*mut sys::FgbObstacle> = obstacles.iter().map(|o| o.handle).collect();
        let mut sim = std::ptr::null_mut();
        check(unsafe { sys::fgb_sim_new(ms.as_ptr(), ms.len() as u64, os.as_ptr(), os.len() as u64, &mut sim) });
        Simulation { sim, meshes, obstacles }
    }

    /// springy/simulation.rs:27-45: one step of every mesh; returns the timestep
    /// (`Duration::from_secs_f32(dt)`, line 44).
    pub fn step(&mut self) -> Duration {
        check(unsafe { sys::fgb_sim_step(self.sim, 1) });
        self.get_timestep()
    }

    /// springy/simulation.rs:47-49
    pub fn get_timestep(&self) -> Duration {
        let mut s = 0f64;
        check(unsafe { sys::fgb_sim_get_timestep(self.sim, &mut s) });
        Duration::from_secs_f64(s)
    }

    /// springy/simulation.rs:51-53 (waits for the queued steps first).
    pub fn get_meshes(&mut self) -> &mut Vec<SpringyMesh> {
        check(unsafe { sys::fgb_sim_synchronize(self.sim, std::ptr::null_mut()) });
        &mut self.meshes
    }

    /// springy/simulation.rs:55-57
    pub fn get_obstacles(&self) -> &Vec<CollidableMesh> {
        &self.obstacles
    }

    /// springy/simulation.rs:59-77: the UI's eight fields become the step's config.
    pub fn sync_sim_config_from_ui(&mut self, ui_config: &Config) {
        let c = ui_config.to_raw();
        check(unsafe { sys::fgb_sim_set_config(self.sim, &c) });
    }

    /// The configuration the next step uses.
    pub fn get_config(&self) -> Config {
        let mut c = sys::FgbConfig::default();
        check(unsafe { sys::fgb_sim_get_config(self.sim, &mut c) });
        Config::from_raw(&c)
    }

    /// The raw handle, for the extension calls of `feriphys_gb300_sys`.
    pub fn as_raw(&self) -> *mut sys::FgbSim {
        self.sim
    }
}

impl Drop for Simulation {
    fn drop(&mut self) {
        unsafe {
            sys::fgb_sim_destroy(self.sim);
        }
    }
}
