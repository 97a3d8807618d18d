"""feriphys_gb300 -- GB300-native spring-mass-damper cloth step.

A Python mirror of feriphys's springy-simulation API over the C ABI in
include/feriphys_gb300.h (libferiphys_gb300.so, hand-written CUDA for
sm_103a).  Names follow the reference (file:line relative to its root):

    Cloth.new            springy/cloth.rs:20-113
    SpringyMesh.new      springy/springy_mesh.rs:267-401  (+ add_strut, add_pin,
                         get_points, get_vertices, accumulate_forces,
                         update_points, clear_forces)
    CollidableMesh.new   collidable_mesh.rs:57-97
    Simulation.new       springy/simulation.rs:17-25      (+ step, get_timestep,
                         get_meshes, get_obstacles, set_config)
    Config, Integration  springy/config.rs:9-33, state.rs:4-8

Extensions with no reference counterpart: per-mesh wind and batched
stepping controls on Simulation, Simulation.step_static (no allocation after
set-up), SpringyMesh.new(..., build_on_device=True) (strut de-dup on the GPU),
SpringyMesh.export_vertices / export_indices (render buffers written into
device memory), and the learned surrogate (Surrogate, SurrogateCheck,
Simulation.step_surrogate, Simulation.energy).

There is no CPU fallback: importing the package loads the CUDA library (it is
built first when missing or stale and nvcc is available) and raises if it
cannot.
"""
from __future__ import annotations

import ctypes as C
import enum
import os

import numpy as np

from . import build as _build

__all__ = ["Integration", "Config", "SpringyMesh", "Cloth", "CollidableMesh", "Simulation", "FgbError",
           "Surrogate", "SurrogateCheck", "library_path", "POINT_FIELDS", "N_FEATURES", "N_PARAMS"]

N_FEATURES = 54
N_PARAMS = 128 * 54 + 128 + 128 * 128 + 128 + 3 * 128 + 3

POINT_FIELDS = ("mass", "px", "py", "pz", "vx", "vy", "vz", "fx", "fy", "fz")


class FgbError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__("fgb error %d: %s" % (code, message))
        self.code = code


class Integration(enum.IntEnum):
    Euler = 0
    Rk4 = 1


class Config(C.Structure):
    """springy/config.rs Config.  gravity is a force per point (not m*g)."""

    _fields_ = [
        ("integration", C.c_int32),
        ("dt", C.c_float),
        ("gravity", C.c_float * 3),
        ("wind", C.c_float * 3),
        ("lift_coefficient", C.c_float),
        ("drag_coefficient", C.c_float),
        ("coefficient_of_restitution", C.c_float),
        ("coefficient_of_friction", C.c_float),
    ]

    @classmethod
    def default(cls) -> "Config":
        c = cls()
        _check(_lib().fgb_config_default(C.byref(c)))
        return c

    @classmethod
    def make(cls, integration=Integration.Euler, dt=1e-3, gravity=(0.0, -10.0, 0.0), wind=(0.0, 0.0, 0.0),
             lift_coefficient=1.0, drag_coefficient=1.0, coefficient_of_restitution=0.95,
             coefficient_of_friction=0.3) -> "Config":
        c = cls()
        c.integration = int(integration)
        c.dt = float(dt)
        c.gravity[:] = [float(v) for v in gravity]
        c.wind[:] = [float(v) for v in wind]
        c.lift_coefficient = float(lift_coefficient)
        c.drag_coefficient = float(drag_coefficient)
        c.coefficient_of_restitution = float(coefficient_of_restitution)
        c.coefficient_of_friction = float(coefficient_of_friction)
        return c


class SurrogateCheck(C.Structure):
    """fgb_surrogate_check: per-cloth energy and strain limits of a coarse step."""

    _fields_ = [
        ("enabled", C.c_int32),
        ("energy_growth", C.c_float),
        ("energy_abs", C.c_float),
        ("max_strain", C.c_float),
    ]

    @classmethod
    def make(cls, energy_growth=0.05, energy_abs=1e-3, max_strain=0.25, enabled=True) -> "SurrogateCheck":
        return cls(1 if enabled else 0, energy_growth, energy_abs, max_strain)


class _Override(C.Structure):
    _fields_ = [("a", C.c_uint32), ("b", C.c_uint32), ("stiffness", C.c_float), ("damping", C.c_float)]


_LIB = None


def library_path() -> str:
    return _build.LIB


def _declare(l):
    P, U64, U32, F, I = C.c_void_p, C.c_uint64, C.c_uint32, C.c_float, C.c_int
    pp = C.POINTER(C.c_void_p)
    cfg = C.POINTER(Config)
    sig = {
        "fgb_last_error": (C.c_char_p, []),
        "fgb_config_default": (I, [cfg]),
        "fgb_mesh_new": (I, [P, U64, P, U64, F, F, F, P, U64, pp]),
        "fgb_cloth_new": (I, [U64, U64, F, P, F, F, F, F, F, F, F, P, U64, pp]),
        "fgb_mesh_new_device": (I, [P, U64, P, U64, F, F, F, P, U64, pp]),
        "fgb_mesh_add_strut": (I, [P, U32, U32, F, F]),
        "fgb_mesh_add_pin": (I, [P, U32]),
        "fgb_mesh_add_struts": (I, [P, P, P, P, P, U64]),
        "fgb_mesh_add_pins": (I, [P, P, U64]),
        "fgb_mesh_counts": (I, [P, P]),
        "fgb_mesh_get_struts": (I, [P, P, P]),
        "fgb_mesh_set_strut_params": (I, [P, P, P]),
        "fgb_mesh_get_points": (I, [P, P]),
        "fgb_mesh_set_points": (I, [P, P]),
        "fgb_mesh_get_positions": (I, [P, P]),
        "fgb_mesh_get_points_f64": (I, [P, P]),
        "fgb_mesh_get_vertices": (I, [P, P, P]),
        "fgb_mesh_export_vertices": (I, [P, P, P, P]),
        "fgb_mesh_export_indices": (I, [P, P, P]),
        "fgb_mesh_set_path": (I, [P, I]),
        "fgb_mesh_get_path": (I, [P, C.POINTER(C.c_int)]),
        "fgb_mesh_set_precision": (I, [P, I]),
        "fgb_mesh_accumulate_forces": (I, [P, cfg]),
        "fgb_mesh_integrate": (I, [P, C.c_int32, F]),
        "fgb_mesh_update_points": (I, [P, P, U64, cfg]),
        "fgb_mesh_clear_forces": (I, [P]),
        "fgb_mesh_synchronize": (I, [P]),
        "fgb_mesh_destroy": (I, [P]),
        "fgb_collidable_new": (I, [P, U64, P, U64, pp]),
        "fgb_collidable_counts": (I, [P, P]),
        "fgb_collidable_destroy": (I, [P]),
        "fgb_sim_new": (I, [P, U64, P, U64, pp]),
        "fgb_sim_set_config": (I, [P, cfg]),
        "fgb_sim_get_config": (I, [P, cfg]),
        "fgb_sim_step": (I, [P, U64]),
        "fgb_sim_step_static": (I, [P, U64, P]),
        "fgb_sim_set_stream": (I, [P, P]),
        "fgb_sim_set_collision_broadphase": (I, [P, I]),
        "fgb_mesh_set_wind": (I, [P, P]),
        "fgb_sim_set_graphs": (I, [P, I]),
        "fgb_sim_set_batch_mode": (I, [P, I]),
        "fgb_sim_set_batch_tile": (I, [P, I]),
        "fgb_sim_batch_info": (I, [P, P]),
        "fgb_sim_get_timestep": (I, [P, C.POINTER(C.c_double)]),
        "fgb_sim_synchronize": (I, [P, C.POINTER(C.c_int)]),
        "fgb_sim_destroy": (I, [P]),
        "fgb_surrogate_new": (I, [U64, pp]),
        "fgb_surrogate_destroy": (I, [P]),
        "fgb_surrogate_get_params": (I, [P, P]),
        "fgb_surrogate_set_params": (I, [P, P]),
        "fgb_surrogate_set_normalization": (I, [P, P, P, P, P]),
        "fgb_surrogate_get_normalization": (I, [P, P, P, P, P]),
        "fgb_surrogate_features": (I, [P, P, F, P, P]),
        "fgb_surrogate_forward": (I, [P, P, U64, P]),
        "fgb_surrogate_gradients": (I, [P, P, P, U64, P, P]),
        "fgb_surrogate_train_batch": (I, [P, P, P, U64, F, P]),
        "fgb_surrogate_dataset_reserve": (I, [P, U64]),
        "fgb_surrogate_collect": (I, [P, P, U32, U64]),
        "fgb_surrogate_dataset_info": (I, [P, P]),
        "fgb_surrogate_dataset_get": (I, [P, U64, U64, P, P]),
        "fgb_surrogate_fit_normalization": (I, [P]),
        "fgb_surrogate_train": (I, [P, U64, U64, F, U64, P]),
        "fgb_sim_step_surrogate": (I, [P, P, U32, U64, C.POINTER(SurrogateCheck), C.POINTER(C.c_uint64)]),
        "fgb_sim_energy": (I, [P, P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(l, name)
        fn.restype = res
        fn.argtypes = args


def _lib():
    global _LIB
    if _LIB is None:
        path = _build.LIB
        try:
            path = _build.build()
        except RuntimeError as e:  # no nvcc: use a prebuilt library if there is one
            if not os.path.exists(path):
                raise ImportError("libferiphys_gb300.so is missing and cannot be built: %s" % e) from None
        l = C.CDLL(path)
        _declare(l)
        _LIB = l
    return _LIB


def _check(rc: int):
    if rc != 0:
        raise FgbError(rc, _lib().fgb_last_error().decode())


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _out_array(out, shape, dtype=np.float32):
    """A caller's output buffer as the library writes it (a pinned one by the
    GPU directly): exactly the expected dtype and size, C-contiguous and
    writeable; a fresh array when ``out`` is None."""
    size = int(np.prod(shape))
    if out is None:
        return np.empty(shape, dtype)
    if (not isinstance(out, np.ndarray) or out.dtype != dtype or out.size != size or not out.flags.c_contiguous
            or not out.flags.writeable):
        raise ValueError("out must be a writeable C-contiguous %s array of %d elements" % (np.dtype(dtype).name, size))
    return out


def _f32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1))


def _u32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint32).reshape(-1))


class SpringyMesh:
    """A GPU-backed springy mesh (springy_mesh.rs:258-661)."""

    def __init__(self, handle: int):
        self._h = C.c_void_p(handle)

    @classmethod
    def new(cls, vertex_positions, vertex_indices, mass, default_stiffness, default_damping,
            strut_overrides=None, build_on_device=False) -> "SpringyMesh":
        """SpringyMesh::new.  strut_overrides: {(a, b): (stiffness, damping)} or
        a pair of arrays (pairs[n, 2], kc[n, 2]), or None.  build_on_device:
        de-duplicate the struts on the GPU (fgb_mesh_new_device, same mesh)."""
        pos = _f32(vertex_positions)
        idx = _u32(vertex_indices)
        ov = None
        nov = 0
        if strut_overrides is not None:
            if isinstance(strut_overrides, dict):
                items = list(strut_overrides.items())
                pairs = np.array([k for k, _ in items], np.uint32).reshape(-1, 2)
                kc = np.array([v for _, v in items], np.float32).reshape(-1, 2)
            else:
                pairs = np.asarray(strut_overrides[0], np.uint32).reshape(-1, 2)
                kc = np.asarray(strut_overrides[1], np.float32).reshape(-1, 2)
            nov = len(pairs)
            ov = (_Override * max(1, nov))()
            arr = np.ctypeslib.as_array(C.cast(ov, C.POINTER(C.c_uint32)), shape=(max(1, nov) * 4,))
            rec = arr.view(np.uint32).reshape(-1, 4)[:nov]
            rec[:, 0:2] = pairs
            rec[:, 2:4] = kc.view(np.uint32)
        h = C.c_void_p()
        fn = _lib().fgb_mesh_new_device if build_on_device else _lib().fgb_mesh_new
        _check(fn(_ptr(pos), pos.size // 3, _ptr(idx), idx.size, float(mass), float(default_stiffness),
                  float(default_damping), C.cast(ov, C.c_void_p) if ov is not None else None, nov, C.byref(h)))
        return cls(h.value)

    def __del__(self):
        try:
            if self._h and _LIB is not None:
                _LIB.fgb_mesh_destroy(self._h)
                self._h = None
        except Exception:
            pass

    def add_strut(self, vertex_indices, stiffness, damping):
        a, b = vertex_indices
        _check(_lib().fgb_mesh_add_strut(self._h, int(a), int(b), float(stiffness), float(damping)))

    def add_pin(self, pin_index):
        _check(_lib().fgb_mesh_add_pin(self._h, int(pin_index)))

    def add_struts(self, pairs, stiffness, damping):
        """add_strut for each row of pairs [n, 2], in order."""
        pairs = np.asarray(pairs, np.uint32).reshape(-1, 2)
        n = len(pairs)
        a = np.ascontiguousarray(pairs[:, 0])
        b = np.ascontiguousarray(pairs[:, 1])
        k = np.ascontiguousarray(np.broadcast_to(np.asarray(stiffness, np.float32), (n,)))
        c = np.ascontiguousarray(np.broadcast_to(np.asarray(damping, np.float32), (n,)))
        _check(_lib().fgb_mesh_add_struts(self._h, _ptr(a), _ptr(b), _ptr(k), _ptr(c), n))

    def add_pins(self, pins):
        p = _u32(pins)
        _check(_lib().fgb_mesh_add_pins(self._h, _ptr(p), p.size))

    def counts(self):
        out = np.zeros(4, np.uint64)
        _check(_lib().fgb_mesh_counts(self._h, _ptr(out)))
        return tuple(int(v) for v in out)

    @property
    def n_points(self) -> int:
        return self.counts()[0]

    def get_points(self, out=None) -> np.ndarray:
        """Points as [n, 10] float32 in the Stateful::as_state layout."""
        out = _out_array(out, (self.n_points, 10))
        _check(_lib().fgb_mesh_get_points(self._h, _ptr(out)))
        return out

    def get_points_f64(self) -> np.ndarray:
        out = np.empty((self.n_points, 10), np.float64)
        _check(_lib().fgb_mesh_get_points_f64(self._h, _ptr(out)))
        return out

    def set_points(self, points):
        """Stateful::from_state_vector for every point ([n, 10] float32)."""
        pts = np.ascontiguousarray(points, dtype=np.float32)
        if pts.size != 10 * self.n_points:
            raise ValueError("expected %d floats" % (10 * self.n_points))
        _check(_lib().fgb_mesh_set_points(self._h, _ptr(pts)))

    def get_positions(self, out=None) -> np.ndarray:
        """Positions as [n, 3] float32 (a pinned ``out`` is written by the GPU directly)."""
        out = _out_array(out, (self.n_points, 3))
        _check(_lib().fgb_mesh_get_positions(self._h, _ptr(out)))
        return out

    def get_vertices(self):
        """SpringyMesh::get_vertices: (positions [n, 3], indices [3F])."""
        n, _, f, _ = self.counts()
        pos = np.empty((n, 3), np.float32)
        idx = np.empty(3 * f, np.uint32)
        _check(_lib().fgb_mesh_get_vertices(self._h, _ptr(pos), _ptr(idx)))
        return pos, idx

    def export_vertices(self, device_ptr: int, color=None, stream_handle=None):
        """Write ColoredVertex {position, color, normal} (9 f32 per vertex) into
        a device buffer (e.g. ``tensor.data_ptr()`` of a CUDA tensor)."""
        col = None if color is None else _f32(color)
        _check(_lib().fgb_mesh_export_vertices(self._h, C.c_void_p(device_ptr), _ptr(col),
                                               C.c_void_p(stream_handle) if stream_handle else None))

    def export_indices(self, device_ptr: int, stream_handle=None):
        """Write the static uint32 index buffer (3 per face) into a device buffer."""
        _check(_lib().fgb_mesh_export_indices(self._h, C.c_void_p(device_ptr),
                                              C.c_void_p(stream_handle) if stream_handle else None))

    def get_struts(self):
        """(kcl [S, 3]: stiffness, damping, rest length; ab [S, 2])."""
        s = self.counts()[1]
        kcl = np.empty((s, 3), np.float32)
        ab = np.empty((s, 2), np.uint32)
        _check(_lib().fgb_mesh_get_struts(self._h, _ptr(kcl), _ptr(ab)))
        return kcl, ab

    def set_strut_params(self, stiffness, damping):
        k = _f32(stiffness)
        c = _f32(damping)
        if k.size != self.counts()[1] or c.size != k.size:
            raise ValueError("one stiffness and damping per strut expected")
        _check(_lib().fgb_mesh_set_strut_params(self._h, _ptr(k), _ptr(c)))

    def set_path(self, path: int):
        """0 auto, 1 general gather, 2 grid (32x8 tiles), 3 grid (one thread per vertex),
        4 general gather over the plain incidence lists."""
        _check(_lib().fgb_mesh_set_path(self._h, int(path)))

    def get_path(self) -> int:
        p = C.c_int()
        _check(_lib().fgb_mesh_get_path(self._h, C.byref(p)))
        return p.value

    def set_wind(self, wind):
        """Per-mesh wind (extension); None returns to the simulation's wind."""
        if wind is None:
            _check(_lib().fgb_mesh_set_wind(self._h, None))
        else:
            w = _f32(wind)
            _check(_lib().fgb_mesh_set_wind(self._h, _ptr(w)))

    def set_precision(self, bits: int):
        _check(_lib().fgb_mesh_set_precision(self._h, int(bits)))

    # phase hooks of Simulation::step
    def accumulate_forces(self, config: Config):
        _check(_lib().fgb_mesh_accumulate_forces(self._h, C.byref(config)))

    def integrate(self, integration, dt):
        """State::euler_step / rk4_step into the mesh's staged points."""
        _check(_lib().fgb_mesh_integrate(self._h, int(integration), float(dt)))

    def update_points(self, obstacles, config: Config):
        arr = (C.c_void_p * max(1, len(obstacles)))(*[o._h for o in obstacles])
        _check(_lib().fgb_mesh_update_points(self._h, arr, len(obstacles), C.byref(config)))

    def clear_forces(self):
        _check(_lib().fgb_mesh_clear_forces(self._h))

    def synchronize(self):
        _check(_lib().fgb_mesh_synchronize(self._h))


class Cloth:
    """springy/cloth.rs Cloth: ``Cloth.new(...).mesh`` is a SpringyMesh."""

    def __init__(self, mesh: SpringyMesh):
        self.mesh = mesh

    @classmethod
    def new(cls, rows, cols, spacing, position, point_mass, tensile_stiffness, tensile_damping, shear_stiffness,
            shear_damping, binding_spring_stiffness, binding_spring_damping, pinned_vertices=()) -> "Cloth":
        p = _f32(position)
        pins = _u32(pinned_vertices)
        h = C.c_void_p()
        _check(_lib().fgb_cloth_new(int(rows), int(cols), float(spacing), _ptr(p), float(point_mass),
                                    float(tensile_stiffness), float(tensile_damping), float(shear_stiffness),
                                    float(shear_damping), float(binding_spring_stiffness),
                                    float(binding_spring_damping), _ptr(pins) if pins.size else None, pins.size,
                                    C.byref(h)))
        return cls(SpringyMesh(h.value))


class CollidableMesh:
    """collidable_mesh.rs CollidableMesh (static triangle obstacle)."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle)

    @classmethod
    def new(cls, vertex_positions, vertex_indices) -> "CollidableMesh":
        pos = _f32(vertex_positions)
        idx = _u32(vertex_indices)
        h = C.c_void_p()
        _check(_lib().fgb_collidable_new(_ptr(pos), pos.size // 3, _ptr(idx), idx.size, C.byref(h)))
        return cls(h.value)

    def counts(self):
        out = np.zeros(3, np.uint64)
        _check(_lib().fgb_collidable_counts(self._h, _ptr(out)))
        return tuple(int(v) for v in out)

    def __del__(self):
        try:
            if self._h and _LIB is not None:
                _LIB.fgb_collidable_destroy(self._h)
                self._h = None
        except Exception:
            pass


class Simulation:
    """springy/simulation.rs Simulation over GPU-backed meshes."""

    def __init__(self, handle, meshes, obstacles):
        self._h = C.c_void_p(handle)
        self._meshes = list(meshes)  # the C simulation borrows these
        self._obstacles = list(obstacles)

    @classmethod
    def new(cls, meshes, obstacles) -> "Simulation":
        meshes = list(meshes)
        obstacles = list(obstacles)
        ma = (C.c_void_p * max(1, len(meshes)))(*[m._h for m in meshes])
        oa = (C.c_void_p * max(1, len(obstacles)))(*[o._h for o in obstacles])
        h = C.c_void_p()
        _check(_lib().fgb_sim_new(ma, len(meshes), oa, len(obstacles), C.byref(h)))
        return cls(h.value, meshes, obstacles)

    def __del__(self):
        try:
            if self._h and _LIB is not None:
                _LIB.fgb_sim_destroy(self._h)
                self._h = None
        except Exception:
            pass

    def set_config(self, config: Config):
        """Headless form of sync_sim_config_from_ui (simulation.rs:64-77)."""
        _check(_lib().fgb_sim_set_config(self._h, C.byref(config)))

    def get_config(self) -> Config:
        c = Config()
        _check(_lib().fgb_sim_get_config(self._h, C.byref(c)))
        return c

    def step(self, n_steps: int = 1) -> float:
        """Simulation::step (n_steps times, queued asynchronously); returns the
        simulated seconds of one step like the reference's Duration."""
        _check(_lib().fgb_sim_step(self._h, int(n_steps)))
        return self.get_timestep()

    def set_batch_mode(self, mode: int):
        """-1 autotuned (default), 0 one CTA per tile, 1 persistent."""
        _check(_lib().fgb_sim_set_batch_mode(self._h, int(mode)))

    def set_batch_tile(self, tile_rows: int):
        """0 autotuned (default), or batch tiles 32 wide and 4, 8 or 12 rows tall."""
        _check(_lib().fgb_sim_set_batch_tile(self._h, int(tile_rows)))

    def set_graphs(self, enabled: bool):
        _check(_lib().fgb_sim_set_graphs(self._h, 1 if enabled else 0))

    def batch_info(self):
        """(meshes in the batch, work items, launch form, persistent CTAs, tile rows)."""
        out = np.zeros(5, np.int64)
        _check(_lib().fgb_sim_batch_info(self._h, _ptr(out)))
        return tuple(int(v) for v in out)

    def set_collision_broadphase(self, enabled: bool):
        """True (default): exact broad phase; False: test every obstacle face."""
        _check(_lib().fgb_sim_set_collision_broadphase(self._h, 1 if enabled else 0))

    def set_stream(self, stream_handle):
        """Issue every mesh's work on an external cudaStream_t (an integer
        handle, e.g. torch.cuda.current_stream().cuda_stream); None resets."""
        _check(_lib().fgb_sim_set_stream(self._h, C.c_void_p(stream_handle) if stream_handle else None))

    def step_static(self, n_steps: int = 1, stream_handle=None):
        """fgb_sim_step_static: the batched step with its scratch in a fixed
        array, for hosts that cannot allow device allocations after set-up
        (call ``step(0)`` once during set-up first)."""
        _check(_lib().fgb_sim_step_static(self._h, int(n_steps),
                                          C.c_void_p(stream_handle) if stream_handle else None))

    def get_timestep(self) -> float:
        s = C.c_double()
        _check(_lib().fgb_sim_get_timestep(self._h, C.byref(s)))
        return s.value

    def get_meshes(self):
        return list(self._meshes)

    def get_obstacles(self):
        return list(self._obstacles)

    def synchronize(self) -> bool:
        """Wait for queued steps; True when a vertex went non-finite since the last call."""
        bad = C.c_int()
        _check(_lib().fgb_sim_synchronize(self._h, C.byref(bad)))
        return bool(bad.value)

    def step_surrogate(self, surrogate: "Surrogate", ratio: int, n_coarse: int = 1, check=None) -> int:
        """n_coarse coarse steps of ratio fine steps each with the learned
        surrogate; with a SurrogateCheck, failing cloths fall back to the fine
        step.  Returns the number of fallbacks."""
        n = C.c_uint64()
        _check(_lib().fgb_sim_step_surrogate(self._h, surrogate._h, int(ratio), int(n_coarse),
                                             C.byref(check) if check is not None else None, C.byref(n)))
        return int(n.value)

    def energy(self) -> np.ndarray:
        """[n_meshes, 2]: energy and maximum strain of each mesh's state."""
        out = np.zeros((len(self._meshes), 2), np.float32)
        _check(_lib().fgb_sim_energy(self._h, _ptr(out)))
        return out


class Surrogate:
    """Learned per-vertex surrogate of the cloth step (no reference
    counterpart): MLP 54 -> 128 -> 128 -> 3 trained and run by CUDA kernels
    (tcgen05 tensor cores, bf16 weights, f32 accumulation)."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle)

    @classmethod
    def new(cls, seed: int = 0) -> "Surrogate":
        h = C.c_void_p()
        _check(_lib().fgb_surrogate_new(int(seed), C.byref(h)))
        return cls(h.value)

    def __del__(self):
        try:
            if self._h and _LIB is not None:
                _LIB.fgb_surrogate_destroy(self._h)
                self._h = None
        except Exception:
            pass

    def get_params(self) -> np.ndarray:
        out = np.zeros(N_PARAMS, np.float32)
        _check(_lib().fgb_surrogate_get_params(self._h, _ptr(out)))
        return out

    def set_params(self, params):
        p = _f32(params)
        if p.size != N_PARAMS:
            raise ValueError("expected %d parameters" % N_PARAMS)
        _check(_lib().fgb_surrogate_set_params(self._h, _ptr(p)))

    def set_normalization(self, in_mean, in_std, out_mean, out_std):
        a, b, c, d = _f32(in_mean), _f32(in_std), _f32(out_mean), _f32(out_std)
        _check(_lib().fgb_surrogate_set_normalization(self._h, _ptr(a), _ptr(b), _ptr(c), _ptr(d)))

    def get_normalization(self):
        a, b = np.zeros(N_FEATURES, np.float32), np.zeros(N_FEATURES, np.float32)
        c, d = np.zeros(3, np.float32), np.zeros(3, np.float32)
        _check(_lib().fgb_surrogate_get_normalization(self._h, _ptr(a), _ptr(b), _ptr(c), _ptr(d)))
        return a, b, c, d

    def features(self, mesh: SpringyMesh, coarse_dt: float, wind=None) -> np.ndarray:
        n = mesh.n_points
        out = np.zeros((n, N_FEATURES), np.float32)
        w = None if wind is None else _f32(wind)
        _check(_lib().fgb_surrogate_features(self._h, mesh._h, float(coarse_dt), _ptr(w), _ptr(out)))
        return out

    def forward(self, x) -> np.ndarray:
        x = np.ascontiguousarray(np.asarray(x, np.float32).reshape(-1, N_FEATURES))
        y = np.zeros((x.shape[0], 3), np.float32)
        _check(_lib().fgb_surrogate_forward(self._h, _ptr(x), x.shape[0], _ptr(y)))
        return y

    def gradients(self, x, t):
        x = np.ascontiguousarray(np.asarray(x, np.float32).reshape(-1, N_FEATURES))
        t = np.ascontiguousarray(np.asarray(t, np.float32).reshape(-1, 3))
        g = np.zeros(N_PARAMS, np.float32)
        loss = C.c_float()
        _check(_lib().fgb_surrogate_gradients(self._h, _ptr(x), _ptr(t), x.shape[0], _ptr(g), C.byref(loss)))
        return g, float(loss.value)

    def train_batch(self, x, t, lr: float) -> float:
        x = np.ascontiguousarray(np.asarray(x, np.float32).reshape(-1, N_FEATURES))
        t = np.ascontiguousarray(np.asarray(t, np.float32).reshape(-1, 3))
        loss = C.c_float()
        _check(_lib().fgb_surrogate_train_batch(self._h, _ptr(x), _ptr(t), x.shape[0], float(lr), C.byref(loss)))
        return float(loss.value)

    def reserve(self, capacity_rows: int):
        _check(_lib().fgb_surrogate_dataset_reserve(self._h, int(capacity_rows)))

    def collect(self, sim: Simulation, ratio: int, n_coarse: int):
        _check(_lib().fgb_surrogate_collect(self._h, sim._h, int(ratio), int(n_coarse)))

    def dataset_info(self):
        out = np.zeros(2, np.uint64)
        _check(_lib().fgb_surrogate_dataset_info(self._h, _ptr(out)))
        return int(out[0]), int(out[1])

    def dataset(self, first: int, n: int):
        f = np.zeros((n, N_FEATURES), np.float32)
        t = np.zeros((n, 3), np.float32)
        _check(_lib().fgb_surrogate_dataset_get(self._h, int(first), int(n), _ptr(f), _ptr(t)))
        return f, t

    def fit_normalization(self):
        _check(_lib().fgb_surrogate_fit_normalization(self._h))

    def train(self, n_steps: int, batch: int = 65536, lr: float = 1e-3, seed: int = 0) -> np.ndarray:
        losses = np.zeros(max(1, int(n_steps)), np.float32)
        _check(_lib().fgb_surrogate_train(self._h, int(n_steps), int(batch), float(lr), int(seed), _ptr(losses)))
        return losses[: int(n_steps)]
