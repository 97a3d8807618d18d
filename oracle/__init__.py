"""The oracle: a CPU restatement of feriphys's cloth step (test infrastructure).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this package, and only as the oracle the GPU results are compared with (or the
timed CPU baseline); the shipped
library never routes through it.  The C++ restatement lives in
``springy_oracle.cpp`` (see its header for the reference file:line map); this
module builds it with g++ and wraps it with ctypes.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "springy_oracle.cpp")
_LIB = os.path.join(_HERE, "liboracle.so")
_lock = threading.Lock()
_lib = None

# -ffp-contract=off: the reference (Rust) never fuses a*b+c; gcc on aarch64
# would otherwise contract by default.
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math"]


def build(force: bool = False) -> str:
    """Compile the restatement into oracle/liboracle.so (idempotent)."""
    with _lock:
        if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(_SRC):
            tmp = _LIB + ".tmp%d" % os.getpid()
            subprocess.check_call(["g++", *CXXFLAGS, "-o", tmp, _SRC])
            os.replace(tmp, _LIB)
    return _LIB


class Config(C.Structure):
    """Mirror of springy/config.rs:9-33 (integration 0 = Euler, 1 = Rk4)."""

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
        lib().oracle_config_default(C.byref(c))
        return c

    @classmethod
    def make(cls, integration=0, dt=1e-3, gravity=(0.0, -10.0, 0.0), wind=(0.0, 0.0, 0.0),
             lift=1.0, drag=1.0, restitution=0.95, friction=0.3) -> "Config":
        c = cls()
        c.integration = int(integration)
        c.dt = float(dt)
        c.gravity[:] = [float(v) for v in gravity]
        c.wind[:] = [float(v) for v in wind]
        c.lift_coefficient = float(lift)
        c.drag_coefficient = float(drag)
        c.coefficient_of_restitution = float(restitution)
        c.coefficient_of_friction = float(friction)
        return c


def _declare(l):
    P, U64, F, I = C.c_void_p, C.c_uint64, C.c_float, C.c_int
    pp = C.POINTER(C.c_void_p)
    sig = {
        "oracle_last_error": (C.c_char_p, []),
        "oracle_config_default": (I, [C.POINTER(Config)]),
        "oracle_duration_roundtrip": (F, [F]),
        "oracle_mesh_new": (I, [P, U64, P, U64, F, F, F, P, P, U64, pp]),
        "oracle_cloth_new": (I, [U64, U64, F, P, F, F, F, F, F, F, F, P, U64, pp]),
        "oracle_mesh_widen": (I, [P, pp]),
        "oracle_mesh_free": (I, [P]),
        "oracle_mesh_add_strut": (I, [P, U64, U64, F, F]),
        "oracle_mesh_add_pin": (I, [P, U64]),
        "oracle_mesh_add_struts": (I, [P, P, P, P, P, U64]),
        "oracle_mesh_add_pins": (I, [P, P, U64]),
        "oracle_mesh_counts": (I, [P, P]),
        "oracle_mesh_get_points_f32": (I, [P, P]),
        "oracle_mesh_get_points_f64": (I, [P, P]),
        "oracle_mesh_set_points_f32": (I, [P, P]),
        "oracle_mesh_get_struts": (I, [P, P, P, P]),
        "oracle_mesh_get_faces": (I, [P, P, P]),
        "oracle_mesh_set_strut_params": (I, [P, P, P]),
        "oracle_mesh_get_pins": (I, [P, P]),
        "oracle_mesh_face_normal": (I, [P, U64, P]),
        "oracle_mesh_face_angle": (I, [P, U64, I, P]),
        "oracle_mesh_accumulate_forces": (I, [P, C.POINTER(Config)]),
        "oracle_mesh_clear_forces": (I, [P]),
        "oracle_mesh_integrate": (I, [P, I, F, P]),
        "oracle_mesh_update_points": (I, [P, P, P, U64, C.POINTER(Config)]),
        "oracle_collidable_new": (I, [P, U64, P, U64, pp]),
        "oracle_collidable_free": (I, [P]),
        "oracle_collidable_counts": (I, [P, P]),
        "oracle_collidable_get": (I, [P, P, P]),
        "oracle_collided_faces": (I, [P, U64, P, P, U64, F, P]),
        "oracle_sim_new": (I, [P, U64, P, U64, pp]),
        "oracle_sim_free": (I, [P]),
        "oracle_sim_set_config": (I, [P, C.POINTER(Config)]),
        "oracle_sim_step": (I, [P, U64]),
        "oracle_state_test_euler": (I, [P, F, P]),
        "oracle_state_test_rk4": (I, [P, F, P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(l, name)
        fn.restype = res
        fn.argtypes = args


def lib():
    global _lib
    if _lib is None:
        l = C.CDLL(build())
        _declare(l)
        _lib = l
    return _lib


class OracleError(RuntimeError):
    pass


def _ck(rc):
    if rc != 0:
        raise OracleError(lib().oracle_last_error().decode())


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _f32(a, n=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1))
    return a


def _u32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint32).reshape(-1))


def duration_roundtrip(x: float) -> float:
    """Duration::from_secs_f32(x).as_secs_f32() as modern Rust computes it."""
    return float(lib().oracle_duration_roundtrip(float(x)))


class SpringyMesh:
    """springy_mesh.rs SpringyMesh (f32, or f64 after ``widen()``)."""

    def __init__(self, handle, prec=32):
        self._h = C.c_void_p(handle)
        self.prec = prec

    @classmethod
    def new(cls, positions, indices, mass, stiffness, damping, overrides=None):
        """SpringyMesh::new; ``overrides`` = (pairs[n,2], kc[n,2]) or None."""
        pos = _f32(positions)
        idx = _u32(indices)
        ov_ab = ov_kc = None
        nov = 0
        if overrides is not None:
            ov_ab = _u32(overrides[0])
            ov_kc = _f32(overrides[1])
            nov = ov_ab.size // 2
        h = C.c_void_p()
        _ck(lib().oracle_mesh_new(_ptr(pos), pos.size // 3, _ptr(idx), idx.size, mass, stiffness, damping,
                                  _ptr(ov_ab), _ptr(ov_kc), nov, C.byref(h)))
        return cls(h.value)

    @classmethod
    def cloth(cls, rows, cols, spacing, position, point_mass, tk, tc, sk, sc, bk, bc, pinned=()):
        """Cloth::new (cloth.rs:20-113); returns the cloth's mesh."""
        p = _f32(position)
        pins = np.ascontiguousarray(np.asarray(pinned, dtype=np.uint64).reshape(-1))
        h = C.c_void_p()
        _ck(lib().oracle_cloth_new(rows, cols, spacing, _ptr(p), point_mass, tk, tc, sk, sc, bk, bc,
                                   _ptr(pins) if pins.size else None, pins.size, C.byref(h)))
        return cls(h.value)

    def widen(self) -> "SpringyMesh":
        h = C.c_void_p()
        _ck(lib().oracle_mesh_widen(self._h, C.byref(h)))
        return SpringyMesh(h.value, 64)

    def __del__(self):
        try:
            if self._h and _lib is not None:
                _lib.oracle_mesh_free(self._h)
                self._h = None
        except Exception:
            pass

    def add_strut(self, a, b, k, c):
        _ck(lib().oracle_mesh_add_strut(self._h, a, b, k, c))

    def add_pin(self, i):
        _ck(lib().oracle_mesh_add_pin(self._h, i))

    def add_struts(self, pairs, k, c):
        pairs = np.asarray(pairs, np.uint32).reshape(-1, 2)
        n = len(pairs)
        a = np.ascontiguousarray(pairs[:, 0])
        b = np.ascontiguousarray(pairs[:, 1])
        kk = np.ascontiguousarray(np.broadcast_to(np.asarray(k, np.float32), (n,)))
        cc = np.ascontiguousarray(np.broadcast_to(np.asarray(c, np.float32), (n,)))
        _ck(lib().oracle_mesh_add_struts(self._h, _ptr(a), _ptr(b), _ptr(kk), _ptr(cc), n))

    def add_pins(self, pins):
        p = _u32(pins)
        _ck(lib().oracle_mesh_add_pins(self._h, _ptr(p), p.size))

    def counts(self):
        out = np.zeros(4, np.uint64)
        _ck(lib().oracle_mesh_counts(self._h, _ptr(out)))
        return tuple(int(v) for v in out)

    @property
    def n_points(self):
        return self.counts()[0]

    def get_points(self):
        """Points as [n, 10] in the Stateful::as_state layout [m, p, v, F]."""
        n = self.n_points
        if self.prec == 32:
            out = np.zeros((n, 10), np.float32)
            _ck(lib().oracle_mesh_get_points_f32(self._h, _ptr(out)))
        else:
            out = np.zeros((n, 10), np.float64)
            _ck(lib().oracle_mesh_get_points_f64(self._h, _ptr(out)))
        return out

    def set_points(self, pts):
        pts = np.ascontiguousarray(np.asarray(pts, np.float32).reshape(-1))
        _ck(lib().oracle_mesh_set_points_f32(self._h, _ptr(pts)))

    def get_struts(self):
        s = self.counts()[1]
        kcl = np.zeros((s, 3), np.float32)
        ab = np.zeros((s, 2), np.uint64)
        fc = np.zeros((s, 2), np.int64)
        _ck(lib().oracle_mesh_get_struts(self._h, _ptr(kcl), _ptr(ab), _ptr(fc)))
        return kcl, ab, fc

    def set_strut_params(self, k, c):
        k = _f32(k)
        c = _f32(c)
        _ck(lib().oracle_mesh_set_strut_params(self._h, _ptr(k), _ptr(c)))

    def get_faces(self):
        f = self.counts()[2]
        st = np.zeros((f, 3), np.uint64)
        vs = np.zeros((f, 3), np.uint64)
        _ck(lib().oracle_mesh_get_faces(self._h, _ptr(st), _ptr(vs)))
        return st, vs

    def get_pins(self):
        n = self.counts()[3]
        out = np.zeros(n, np.uint64)
        if n:
            _ck(lib().oracle_mesh_get_pins(self._h, _ptr(out)))
        return out

    def face_normal(self, f):
        out = np.zeros(3, np.float32)
        _ck(lib().oracle_mesh_face_normal(self._h, f, _ptr(out)))
        return out

    def face_angle(self, f, k):
        out = C.c_float()
        _ck(lib().oracle_mesh_face_angle(self._h, f, k, C.byref(out)))
        return np.float32(out.value)

    def accumulate_forces(self, cfg: Config):
        _ck(lib().oracle_mesh_accumulate_forces(self._h, C.byref(cfg)))

    def clear_forces(self):
        _ck(lib().oracle_mesh_clear_forces(self._h))

    def integrate(self, integration, dt):
        out = np.zeros((self.n_points, 10), np.float32)
        _ck(lib().oracle_mesh_integrate(self._h, integration, dt, _ptr(out)))
        return out

    def update_points(self, new_points, obstacles, cfg: Config):
        np_ = np.ascontiguousarray(np.asarray(new_points, np.float32).reshape(-1))
        arr = (C.c_void_p * max(1, len(obstacles)))(*[o._h for o in obstacles])
        _ck(lib().oracle_mesh_update_points(self._h, _ptr(np_), arr, len(obstacles), C.byref(cfg)))


class CollidableMesh:
    """collidable_mesh.rs CollidableMesh."""

    def __init__(self, positions, indices):
        pos = _f32(positions)
        idx = _u32(indices)
        h = C.c_void_p()
        _ck(lib().oracle_collidable_new(_ptr(pos), pos.size // 3, _ptr(idx), idx.size, C.byref(h)))
        self._h = h

    def __del__(self):
        try:
            if self._h and _lib is not None:
                _lib.oracle_collidable_free(self._h)
                self._h = None
        except Exception:
            pass

    def counts(self):
        out = np.zeros(3, np.uint64)
        _ck(lib().oracle_collidable_counts(self._h, _ptr(out)))
        return tuple(int(v) for v in out)

    def faces(self):
        nf = self.counts()[2]
        out = np.zeros((nf, 3, 3), np.float32)
        _ck(lib().oracle_collidable_get(self._h, _ptr(out), None))
        return out

    def edges(self):
        ne = self.counts()[1]
        out = np.zeros((ne, 2, 3), np.float32)
        _ck(lib().oracle_collidable_get(self._h, None, _ptr(out)))
        return out


def collided_faces(obstacles, old_p, new_p, dt):
    """First-hit flattened face index (or -1) per segment."""
    old_p = _f32(old_p)
    new_p = _f32(new_p)
    n = old_p.size // 3
    out = np.zeros(n, np.int64)
    arr = (C.c_void_p * max(1, len(obstacles)))(*[o._h for o in obstacles])
    _ck(lib().oracle_collided_faces(arr, len(obstacles), _ptr(old_p), _ptr(new_p), n, dt, _ptr(out)))
    return out


class Simulation:
    """springy/simulation.rs Simulation (starts from Config::default())."""

    def __init__(self, meshes, obstacles):
        self.meshes = list(meshes)
        self.obstacles = list(obstacles)
        ma = (C.c_void_p * max(1, len(self.meshes)))(*[m._h for m in self.meshes])
        oa = (C.c_void_p * max(1, len(self.obstacles)))(*[o._h for o in self.obstacles])
        h = C.c_void_p()
        _ck(lib().oracle_sim_new(ma, len(self.meshes), oa, len(self.obstacles), C.byref(h)))
        self._h = h

    def __del__(self):
        try:
            if self._h and _lib is not None:
                _lib.oracle_sim_free(self._h)
                self._h = None
        except Exception:
            pass

    def set_config(self, cfg: Config):
        _ck(lib().oracle_sim_set_config(self._h, C.byref(cfg)))

    def step(self, n=1):
        _ck(lib().oracle_sim_step(self._h, n))


def state_test_euler(pv6, h):
    a = _f32(pv6)
    out = np.zeros(6, np.float32)
    _ck(lib().oracle_state_test_euler(_ptr(a), h, _ptr(out)))
    return out


def state_test_rk4(yth, h):
    a = _f32(yth)
    out = np.zeros(3, np.float32)
    _ck(lib().oracle_state_test_rk4(_ptr(a), h, _ptr(out)))
    return out
