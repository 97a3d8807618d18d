/*
 * feriphys_gb300 -- GB300-native (sm_103a) spring-mass-damper cloth step.
 *
 * C ABI of the drop-in for feriphys's springy-mesh simulation path.  Every
 * entry point mirrors one item of the reference's Rust API (cited as
 * file:line relative to the reference project root); the reference has no FFI
 * of its own, so these are the calls its Rust host would bind through an
 * extern "C" block, with a build.rs that compiles this library.
 *
 * Conventions
 *  - Every function returns 0 (FGB_OK) on success or a negative fgb_status;
 *    fgb_last_error() gives a message for the calling thread.  The reference
 *    panics where these return an error.
 *  - Handles own their device memory and CUDA stream.  A handle is not
 *    thread-safe: drive it from one host thread at a time.
 *  - Host buffers are caller-owned and copied in/out; vertex indices are
 *    uint32 (the reference uses usize; meshes stay below 2^31 vertices).
 *  - Points use the reference's Stateful layout (springy_mesh.rs:242-255):
 *    10 floats per point [mass, px, py, pz, vx, vy, vz, Fx, Fy, Fz].
 *  - Arithmetic is f32 like the reference (cgmath Vector3<f32>); a mesh can
 *    be switched to f64 for the FP64 rerun used to state rounding error.
 */
#ifndef FERIPHYS_GB300_H
#define FERIPHYS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum fgb_status {
  FGB_OK = 0,
  FGB_EINVAL = -1,       /* bad argument (null pointer, bad size, bad dt)  */
  FGB_EINDEX = -2,       /* vertex index out of range                       */
  FGB_ENONMANIFOLD = -3, /* an edge has more than two faces (springy_mesh.rs:339) */
  FGB_ECUDA = -4,        /* CUDA runtime error (message has the CUDA text)  */
  FGB_ESTATE = -5,       /* call not valid in the handle's current state   */
  FGB_ENOMEM = -6,       /* host or device allocation failed               */
  FGB_ECHECK = -7        /* a device-side check failed (see message)       */
} fgb_status;

/* state.rs:4-8 */
typedef enum fgb_integration { FGB_EULER = 0, FGB_RK4 = 1 } fgb_integration;

/* springy/config.rs:9-18.  gravity is a FORCE added to every point
 * (springy_mesh.rs:194-196); drag/lift have no air density
 * (springy_mesh.rs:636-646). */
typedef struct fgb_config {
  int32_t integration; /* fgb_integration */
  float dt;            /* seconds */
  float gravity[3];
  float wind[3];
  float lift_coefficient;
  float drag_coefficient;
  float coefficient_of_restitution;
  float coefficient_of_friction;
} fgb_config;

/* StrutKey + SpringConfig (springy_mesh.rs:38-42, 96-107): per-edge override
 * of the default stiffness/damping used by SpringyMesh::new. */
typedef struct fgb_spring_override {
  uint32_t a, b;
  float stiffness, damping;
} fgb_spring_override;

typedef struct fgb_mesh fgb_mesh;
typedef struct fgb_obstacle fgb_obstacle;
typedef struct fgb_sim fgb_sim;

/* Message for the last failing call on this thread ("" if none). */
const char* fgb_last_error(void);

/* Config::default() -- springy/config.rs:20-32 (Rk4, dt = 1 ms, g = (0,-10,0),
 * Cl = Cd = 1, e = 0.95, mu = 0.3). */
int fgb_config_default(fgb_config* out);

/* ---------------------------------------------------------------- meshes -- */

/* SpringyMesh::new -- springy_mesh.rs:267-401.  positions: 3*n_vertices
 * floats; indices: triangles (3 per face, trailing remainder ignored like
 * itertools::tuples); mass: TOTAL mass (split evenly, line 277); overrides
 * may be NULL.  Struts are de-duplicated in triangle order; stiffness and
 * damping are scaled by 1/rest_length (lines 83-84).  Torsional springs are
 * not built (the reference's force for them is disabled, lines 518-519). */
int fgb_mesh_new(const float* positions, uint64_t n_vertices, const uint32_t* indices, uint64_t n_indices,
                 float mass, float default_stiffness, float default_damping,
                 const fgb_spring_override* overrides, uint64_t n_overrides, fgb_mesh** out);

/* fgb_mesh_new with the strut de-duplication, the face/strut adjacency and
 * the strut constants built on the current GPU (a radix sort of the edge
 * keys instead of springy_mesh.rs:284-345's hash map) -- for meshes of
 * millions of vertices.  Same arguments, same errors, and the same mesh bit
 * for bit (strut order, constants, rest lengths, adjacency).  Extension with
 * no reference counterpart. */
int fgb_mesh_new_device(const float* positions, uint64_t n_vertices, const uint32_t* indices, uint64_t n_indices,
                        float mass, float default_stiffness, float default_damping,
                        const fgb_spring_override* overrides, uint64_t n_overrides, fgb_mesh** out);

/* Cloth::new -- springy/cloth.rs:20-113 (rows, cols >= 2).  Builds the grid,
 * its triangles, the shear overrides, the pins and the binding struts. */
int fgb_cloth_new(uint64_t rows, uint64_t cols, float spacing, const float position[3], float point_mass,
                  float tensile_stiffness, float tensile_damping, float shear_stiffness, float shear_damping,
                  float binding_stiffness, float binding_damping, const uint32_t* pinned, uint64_t n_pinned,
                  fgb_mesh** out);

/* SpringyMesh::add_strut -- springy_mesh.rs:403-413 (vertex order kept). */
int fgb_mesh_add_strut(fgb_mesh* m, uint32_t a, uint32_t b, float stiffness, float damping);

/* SpringyMesh::add_pin -- springy_mesh.rs:415-417. */
int fgb_mesh_add_pin(fgb_mesh* m, uint32_t index);

/* add_strut / add_pin applied n times in order (one call for large meshes;
 * same result as the loop). */
int fgb_mesh_add_struts(fgb_mesh* m, const uint32_t* a, const uint32_t* b, const float* stiffness,
                        const float* damping, uint64_t n);
int fgb_mesh_add_pins(fgb_mesh* m, const uint32_t* index, uint64_t n);

/* Counts: out[0] points, out[1] struts, out[2] faces, out[3] pins. */
int fgb_mesh_counts(const fgb_mesh* m, uint64_t out[4]);

/* Per-strut stiffness/damping/rest length and vertex pair, in strut order
 * (the reference keeps these private; exposed for parity checks).  Any
 * pointer may be NULL. */
int fgb_mesh_get_struts(const fgb_mesh* m, float* kcl /*3*S*/, uint32_t* ab /*2*S*/);

/* Replace per-strut stiffness and damping (already length-scaled, strut
 * order).  Extension with no reference counterpart: lets a caller build
 * per-strut random stiffness without an override map. */
int fgb_mesh_set_strut_params(fgb_mesh* m, const float* stiffness, const float* damping);

/* SpringyMesh::get_points -- springy_mesh.rs:419-421, in the Stateful layout
 * (10 floats per point). */
int fgb_mesh_get_points(fgb_mesh* m, float* out);

/* Stateful::from_state_vector for every point -- springy_mesh.rs:204-221. */
int fgb_mesh_set_points(fgb_mesh* m, const float* in);

/* Positions only (3 floats per point), and the same in f64 for an f64 mesh. */
int fgb_mesh_get_positions(fgb_mesh* m, float* out);
int fgb_mesh_get_points_f64(fgb_mesh* m, double* out);

/* SpringyMesh::get_vertices -- springy_mesh.rs:500-513 (positions 3*N,
 * indices 3*F; either pointer may be NULL). */
int fgb_mesh_get_vertices(fgb_mesh* m, float* positions, uint32_t* indices);

/* Headless render export (replaces the per-frame host rebuild of
 * ColoredMesh::from_springy_mesh, graphics/model.rs:72-90, 142-186).
 * fgb_mesh_export_vertices writes, into the caller's DEVICE buffer of
 * 9 * N floats, each vertex as ColoredVertex {position, color, normal}
 * (model.rs:20-24) straight from the simulation's device state; the normal is
 * graphics/util.rs:178-199's: the sum in face order of (p_a - p_b) x
 * (p_a - p_c) over the vertex's faces, normalised.  color: 3 floats or NULL
 * (white).  fgb_mesh_export_indices writes the static index buffer (3 * F
 * uint32, so no 65,535-vertex cap as with the reference's u16 indices) into
 * a device buffer once.  stream: a cudaStream_t or NULL for the mesh's own;
 * the vertex export is asynchronous on it (ordered after the mesh's queued
 * steps); the index export returns when the copy is done. */
int fgb_mesh_export_vertices(fgb_mesh* m, void* device_out, const float* color, void* stream);
int fgb_mesh_export_indices(fgb_mesh* m, void* device_out, void* stream);

/* Select the step implementation: 0 = automatic (grid kernel when the mesh
 * is a Cloth::new grid, else the general gather), 1 = general gather,
 * 2 = grid kernel (fails with FGB_ESTATE if the mesh is not a grid),
 * 3 = the grid kernel's untiled form (one thread per vertex, no shared
 * memory; a cross-check of the tiled one), 4 = the general gather over its
 * plain incidence lists (a cross-check of the compact lists path 1 reads
 * when the mesh fits them).  All give identical results; fgb_mesh_get_path
 * reports 4 as 1. */
int fgb_mesh_set_path(fgb_mesh* m, int path);

/* Which path the next step uses (1 general, 2 grid); decided on the host. */
int fgb_mesh_get_path(fgb_mesh* m, int* path);

/* Arithmetic precision of the device state: 32 (default) or 64 (FP64
 * rerun of the same step on the GPU; general gather path only). */
int fgb_mesh_set_precision(fgb_mesh* m, int bits);

/* Phase hooks used by Simulation::step (springy/simulation.rs:27-45):
 * accumulate_forces (springy_mesh.rs:515-525), State::euler_step/rk4_step
 * into the mesh's staging points (state.rs:75-106), update_points with the
 * staged points (springy_mesh.rs:423-497) and clear_forces (656-660).
 * fgb_sim_step runs the fused equivalent in one launch. */
int fgb_mesh_accumulate_forces(fgb_mesh* m, const fgb_config* cfg);
int fgb_mesh_integrate(fgb_mesh* m, int32_t integration, float dt);
int fgb_mesh_update_points(fgb_mesh* m, fgb_obstacle* const* obstacles, uint64_t n_obstacles,
                           const fgb_config* cfg);
int fgb_mesh_clear_forces(fgb_mesh* m);

/* Wait for the mesh's stream. */
int fgb_mesh_synchronize(fgb_mesh* m);

int fgb_mesh_destroy(fgb_mesh* m);

/* -------------------------------------------------------------- obstacles -- */

/* CollidableMesh::new -- collidable_mesh.rs:57-97 (triangle soup; a triangle
 * that repeats a vertex is rejected like the reference's panic at 81-89). */
int fgb_collidable_new(const float* positions, uint64_t n_vertices, const uint32_t* indices, uint64_t n_indices,
                       fgb_obstacle** out);
/* Counts: out[0] vertices, out[1] edges, out[2] faces. */
int fgb_collidable_counts(const fgb_obstacle* o, uint64_t out[3]);
int fgb_collidable_destroy(fgb_obstacle* o);

/* ------------------------------------------------------------- simulation -- */

/* Simulation::new -- springy/simulation.rs:17-25 (starts from
 * Config::default()).  The simulation borrows the meshes and obstacles:
 * step it only while they live.  fgb_sim_destroy never touches them, so the
 * handles may be destroyed in any order.  Every mesh must have been created
 * with the same CUDA device current (a mesh belongs to the device current at
 * its creation); meshes of different devices give FGB_EINVAL, and so does
 * a mesh listed twice (the reference's Simulation owns each mesh once). */
int fgb_sim_new(fgb_mesh* const* meshes, uint64_t n_meshes, fgb_obstacle* const* obstacles, uint64_t n_obstacles,
                fgb_sim** out);

/* sync_sim_config_from_ui -- springy/simulation.rs:64-77 (headless form). */
int fgb_sim_set_config(fgb_sim* s, const fgb_config* cfg);
int fgb_sim_get_config(const fgb_sim* s, fgb_config* out);

/* Simulation::step repeated n_steps times -- springy/simulation.rs:27-45.
 * Asynchronous: returns once the launches are queued. */
int fgb_sim_step(fgb_sim* s, uint64_t n_steps);

/* Per-mesh wind (3 floats), or NULL to use the simulation's Config.wind.
 * Extension with no reference counterpart: the reference's wind is global
 * per Simulation (springy/config.rs:13); equivalent to one Simulation per
 * mesh. */
int fgb_mesh_set_wind(fgb_mesh* m, const float* wind);

/* Batched stepping: a simulation with two or more Cloth::new grid meshes
 * advances all of them with one kernel launch per step (largest cloths
 * first, tiles pulled from a shared work list); a call with n_steps >= 2 is
 * captured once as a CUDA graph and replayed (1 = default; 0 = plain
 * launches).  Extension with no reference counterpart (the reference steps
 * meshes one after another, springy/simulation.rs:28); results are
 * identical to stepping each mesh alone. */
int fgb_sim_set_graphs(fgb_sim* s, int enabled);

/* Launch form of the batched step: -1 (default) lets the autotuner choose,
 * 0 one CTA per tile, 1 persistent CTAs pulling tiles from a work counter. */
int fgb_sim_set_batch_mode(fgb_sim* s, int mode);

/* Tile of the batched step: 32 vertices wide and tile_rows = 4, 8 or 12
 * tall (each with its own block size and resident CTAs per SM), or 0
 * (default) to let the autotuner time all three on the batch.  Extension
 * with no reference counterpart; results are identical for every tile. */
int fgb_sim_set_batch_tile(fgb_sim* s, int tile_rows);

/* out[0] meshes in the batch, out[1] work items (tiles), out[2] launch form
 * chosen by the autotuner (0 one CTA per tile, 1 persistent; -1 not yet
 * tuned), out[3] persistent CTAs, out[4] tile rows.  The choice is cached
 * per GPU in $FGB_AUTOTUNE_CACHE (default ~/.cache/feriphys_gb300/autotune.txt). */
int fgb_sim_batch_info(const fgb_sim* s, int64_t out[5]);

/* Collision search: 1 (default) uses an exact broad phase over the obstacle
 * faces (candidates visited in face order, so the first hit is unchanged);
 * 0 tests every face for every point like collidable_mesh.rs:107-169.
 * Extension with no reference counterpart (the results are identical). */
int fgb_sim_set_collision_broadphase(fgb_sim* s, int enabled);

/* Issue the simulation's work (every mesh) on the caller's CUDA stream
 * (a cudaStream_t passed as void*); NULL returns to the meshes' own streams.
 * Extension with no reference counterpart: lets a host application order the
 * step with its own GPU work and time it with its own events. */
int fgb_sim_set_stream(fgb_sim* s, void* stream);

/* Allocation-free step (no counterpart in the reference).  For hosts that
 * cannot let a library allocate device memory once they are running -- game
 * engines and renderers that own all GPU memory through their own
 * allocators, and real-time loops that cannot afford cudaMalloc/cudaFree,
 * which may synchronise the whole device.  Advances every mesh of a
 * simulation n_steps times with the batched persistent kernel, keeping its
 * scratch (work counter, cloth table, tile list) in a fixed 4 MiB array that
 * every GPU loading this library holds until exit: it fits 80 bytes per cloth
 * plus 16 bytes per 32x8 tile (e.g. 4096 cloths of 16..128 vertices a side
 * need 2.3 MB); larger batches fail with FGB_EINVAL.  Inputs
 * and outputs are the meshes' device state, as for fgb_sim_step.  All meshes
 * must be Cloth::new grids on the f32 grid path, already prepared by one
 * fgb_sim_step(sim, 0) during set-up (else FGB_ESTATE); this call uploads
 * nothing and allocates nothing.  Its first call on a device looks up the
 * array's device address, so make that first call before any stream capture.
 * Every call reuses the same array: calls that overlap on the GPU (other
 * streams or threads) race.  stream: a cudaStream_t, or NULL for the
 * simulation's own stream; the call returns when the steps have finished.
 * The calling thread's current device is the same on return as on entry, and
 * regular fgb_sim_step calls on the same simulation may come before or after
 * it. */
int fgb_sim_step_static(fgb_sim* s, uint64_t n_steps, void* stream);

/* Simulation::get_timestep -- springy/simulation.rs:47-49, as
 * Duration::from_secs_f32(dt).as_secs_f64(). */
int fgb_sim_get_timestep(const fgb_sim* s, double* seconds);

/* Wait for every queued step; then report whether any stepped vertex went
 * non-finite since the last call (*nonfinite = 1).  May be NULL. */
int fgb_sim_synchronize(fgb_sim* s, int* nonfinite);

int fgb_sim_destroy(fgb_sim* s);


/* ---- Learned surrogate (no counterpart in the reference) -----------------
 * A per-vertex MLP 54 -> 128 -> 128 -> 3 (tanh-form GELU, bf16 weights, f32
 * accumulation on the tensor cores) that predicts, for a vertex of a
 * Cloth::new grid, its velocity change over one coarse step of `ratio` fine
 * steps of the simulation's dt, from its 8-neighbour stencil (the
 * neighbours' positions relative to the vertex, minus the same at rest, and
 * relative velocities), pin flag, relative wind and normal.  Training
 * data comes from the simulation's own fine steps on the GPU; training
 * (forward, backward, Adam) and inference are CUDA kernels of this library.
 * The fine step stays the reference: fgb_sim_step_surrogate checks each cloth's
 * energy and maximum strain after every coarse step and reverts a failing
 * cloth to `ratio` fine steps.
 *
 * Public parameter layout (f32, row-major, rows = outputs): W1[128][54],
 * b1[128], W2[128][128], b2[128], W3[3][128], b3[3] (23939 floats).
 * The network sees standardised inputs (x - in_mean) / in_std and predicts
 * standardised outputs; y * out_std + out_mean is the velocity change times
 * T / h (T the coarse step, h the cloth's rest spacing). */
typedef struct fgb_surrogate fgb_surrogate;

/* Per-cloth check after every coarse step.  E = sum m|v|^2/2 - g.p + sum over
 * struts k(|d| - L)^2/2 (g: the gravity force of a point), strain = the
 * largest |(|d| - L) / L|.  A cloth fails when
 *   E_new > E_old + energy_growth * (|E_start| + W h) + energy_abs
 * (E_start: the cloth's energy when the call began; W h: its weight times its
 * rest spacing, the energy of lifting it by one spacing -- a scale fixed for
 * the call, so the allowed growth adds up linearly, never geometrically),
 * when its strain exceeds max_strain, or when either is not finite. */
typedef struct fgb_surrogate_check {
  int32_t enabled;      /* 0: no checks, no fallback */
  float energy_growth;
  float energy_abs;     /* J */
  float max_strain;
} fgb_surrogate_check;

/* New network on the current device: Xavier-uniform weights from `seed`,
 * zero biases, identity normalisation, empty dataset. */
int fgb_surrogate_new(uint64_t seed, fgb_surrogate** out);
int fgb_surrogate_destroy(fgb_surrogate* g);
int fgb_surrogate_get_params(fgb_surrogate* g, float* out /* 23939 */);
int fgb_surrogate_set_params(fgb_surrogate* g, const float* in /* 23939 */);
/* in_mean[54], in_std[54], out_mean[3], out_std[3]; any may be NULL on get. */
int fgb_surrogate_set_normalization(fgb_surrogate* g, const float* in_mean, const float* in_std,
                                    const float* out_mean, const float* out_std);
int fgb_surrogate_get_normalization(const fgb_surrogate* g, float* in_mean, float* in_std, float* out_mean,
                                    float* out_std);
/* Raw (unstandardised) inputs of every vertex of a grid mesh for coarse step
 * `coarse_dt` and wind `wind[3]` (NULL: the mesh's wind or zero): out[n][54]. */
int fgb_surrogate_features(fgb_surrogate* g, fgb_mesh* m, float coarse_dt, const float* wind, float* out);
/* Network outputs y[n][3] for standardised inputs x[n][54] (host buffers). */
int fgb_surrogate_forward(fgb_surrogate* g, const float* x, uint64_t n, float* y);
/* Gradient of the mean squared error mean((y - t)^2) over n rows (n a
 * multiple of 128) in the public layout; *loss = that mean.  Nothing changes. */
int fgb_surrogate_gradients(fgb_surrogate* g, const float* x, const float* t, uint64_t n, float* grad, float* loss);
/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) on host rows; *loss = the
 * batch's mean squared error before the step. */
int fgb_surrogate_train_batch(fgb_surrogate* g, const float* x, const float* t, uint64_t n, float lr, float* loss);
/* Device ring of training transitions (one row per vertex and coarse step). */
int fgb_surrogate_dataset_reserve(fgb_surrogate* g, uint64_t capacity_rows);
/* Runs n_coarse x ratio fine steps of the simulation (fgb_sim_step) and
 * records, before each coarse step, every vertex's inputs and, after it, its
 * velocity change; the oldest rows are overwritten when the ring is full. */
int fgb_surrogate_collect(fgb_surrogate* g, fgb_sim* s, uint32_t ratio, uint64_t n_coarse);
/* out[0] = rows held, out[1] = capacity. */
int fgb_surrogate_dataset_info(const fgb_surrogate* g, uint64_t out[2]);
/* Copies rows [first, first + n) of the ring: feat[n][54], tgt[n][3]. */
int fgb_surrogate_dataset_get(fgb_surrogate* g, uint64_t first, uint64_t n, float* feat, float* tgt);
/* Sets the normalisation to the dataset's per-feature mean and standard
 * deviation (a standard deviation below 1e-6 becomes 1). */
int fgb_surrogate_fit_normalization(fgb_surrogate* g);
/* n_steps Adam steps on batches of `batch` rows (a multiple of 128) drawn
 * from the dataset with a seeded hash; losses[n_steps] (may be NULL). */
int fgb_surrogate_train(fgb_surrogate* g, uint64_t n_steps, uint64_t batch, float lr, uint64_t seed,
                        float* losses);

/* n_coarse coarse steps of every mesh (all Cloth::new grids on the f32 grid
 * path) with the surrogate: T = ratio * dt, v' = v + dv, p' = p + (v + v') T / 2,
 * collision response against the obstacles over T, pinned vertices
 * unchanged.  With chk->enabled, a cloth whose energy or strain check fails
 * after a coarse step is reverted and advanced by `ratio` fine steps instead;
 * *n_fallbacks (may be NULL) receives the number of such reverts.  An
 * accumulated force carried in by fgb_mesh_set_points does not enter a
 * coarse step (the network sees positions and velocities only) and is
 * cleared by it, as Simulation::step's clear_forces would. */
int fgb_sim_step_surrogate(fgb_sim* s, fgb_surrogate* g, uint32_t ratio, uint64_t n_coarse,
                           const fgb_surrogate_check* chk, uint64_t* n_fallbacks);
/* Energy and maximum strain of each mesh's current state (out[2 * n_meshes]),
 * as the checks compute them. */
int fgb_sim_energy(fgb_sim* s, float* out);

#ifdef __cplusplus
}
#endif

#endif /* FERIPHYS_GB300_H */
