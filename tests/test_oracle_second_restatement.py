"""A second, independent restatement of the reference's Simulation::step in
float32 numpy (pure-Python loops: small cloths only), checked against the
oracle's C++ restatement bit for bit over whole steps -- gravity, strut
springs and dampers, drag and lift with the corner-angle split, pins,
explicit Euler and the plane collision response together.  The reference's
own tests pin these pieces one at a time; this pins their composition.

Followed line by line (paths relative to the reference project root):
  springy/simulation.rs:27-45   step: accumulate, State, euler_step, update_points, clear
  springy/springy_mesh.rs:515-551, 629-654   forces; 118-172 face normal/area/angles
  springy/springy_mesh.rs:194-196, 223-255   gravity as force, Stateful derivative/as_state
  state.rs:75-106, utils.rs:5-21              euler_step S + S' h and the frozen-force
                                              "rk4_step", element by element
  springy/springy_mesh.rs:423-497             collision response, pin restore
  collidable_mesh.rs:40-47, 107-169           face normal, plane distance, first-hit search
cgmath 0.18 (the reference's vector library): dot = (x x' + y y') + z z',
magnitude = sqrt(dot), normalize(v) = v * (1 / |v|), angle(a, b) =
atan2(|a x b|, a . b), Vector3 / s componentwise."""
import ctypes
import ctypes.util
import math
from fractions import Fraction

import numpy as np
import pytest

f = np.float32
PI = f(math.pi)

# Rust's f32::atan2 (behind cgmath's angle) is the platform libm's atan2f;
# numpy's float32 arctan2 is its own vectorised approximation and differs
# from it in the last bit on a large share of inputs.
_LIBM = ctypes.util.find_library("m")
_atan2f = None
if _LIBM:
    _atan2f = ctypes.CDLL(_LIBM).atan2f
    _atan2f.restype = ctypes.c_float
    _atan2f.argtypes = [ctypes.c_float, ctypes.c_float]


def atan2f(y, x):
    return f(_atan2f(float(y), float(x)))


def dot(a, b):
    return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]


def cross(a, b):
    return np.array([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]], f)


def magnitude(v):
    return np.sqrt(dot(v, v))


def normalize(v):
    return v * (f(1.0) / magnitude(v))


def angle(a, b):
    return atan2f(magnitude(cross(a, b)), dot(a, b))


def duration_secs(dt):
    """Duration::from_secs_f32(dt).as_secs_f32(): whole nanoseconds (nearest,
    ties to even), rebuilt as f32(nanos) / f32(1e9) below one second."""
    ns = Fraction(float(dt)) * 10 ** 9
    q, r = divmod(ns.numerator, ns.denominator)
    if 2 * r > ns.denominator or (2 * r == ns.denominator and q % 2):
        q += 1
    return f(q) / f(1e9)


class Obstacle:
    def __init__(self, v0, v1, v2):
        self.v0, self.v1, self.v2 = (np.array(v, f) for v in (v0, v1, v2))

    def normal(self):
        return normalize(cross(self.v1 - self.v0, self.v2 - self.v0))

    def distance(self, p):
        return dot(p - self.v0, self.normal())


def collided_face(faces, old, new, dtd):
    for face in faces:
        old_velocity = (new - old) / dtd
        d0, d1 = face.distance(old), face.distance(new)
        if np.signbit(d0) == np.signbit(d1):
            continue
        fr = d0 / (d0 - d1)
        cp = old + (dtd * fr) * old_velocity
        n = face.normal()
        if n[0] >= n[1] and n[0] >= n[2]:  # the eliminated coordinate becomes +0.0
            keep = np.array([False, True, True])
        elif n[1] >= n[0] and n[1] >= n[2]:
            keep = np.array([True, False, True])
        else:
            keep = np.array([True, True, False])
        a, b, c, p = (np.where(keep, v, f(0.0)).astype(f) for v in (face.v0, face.v1, face.v2, cp))
        o0 = not np.signbit(dot(cross(b - a, p - a), n))
        o1 = not np.signbit(dot(cross(c - b, p - b), n))
        o2 = not np.signbit(dot(cross(a - c, p - c), n))
        if o0 == o1 and o1 == o2:
            return face
    return None


def step(pts, struts, faces, pins, obstacles, cfg):
    """One Simulation::step of one mesh on Stateful points [n, 10] (f32);
    returns the new points and the obstacle faces hit."""
    pts = pts.copy()
    P, V, F = pts[:, 1:4], pts[:, 4:7], pts[:, 7:10]
    g, wind = np.array(cfg["gravity"], f), np.array(cfg["wind"], f)
    cd, cl, dt = f(cfg["drag"]), f(cfg["lift"]), f(cfg["dt"])
    # accumulate_forces
    for i in range(len(pts)):
        F[i] = F[i] + g
    for (a, b), (k, c, L) in struts:
        u = normalize(P[b] - P[a])
        sf = (k * (magnitude(P[b] - P[a]) - L)) * u
        F[a] = F[a] + sf
        F[b] = F[b] + f(-1.0) * sf
        df = (c * dot(V[b] - V[a], u)) * u
        F[a] = F[a] + df
        F[b] = F[b] + f(-1.0) * df
    for i0, i1, i2 in faces:
        avg = ((V[i0] + V[i1]) + V[i2]) / f(3.0)
        rv = avg - wind
        cr = cross(P[i1] - P[i0], P[i2] - P[i0])
        area = magnitude(cr) / f(2.0)
        n = normalize(cross(P[i1] - P[i0], P[i2] - P[i0]))
        eff = area * abs(dot(n, rv))
        drag = ((f(-1.0) * cd) * eff) * rv
        lift = ((f(-1.0) * cl) * eff) * (rv * magnitude(cross(n, rv)))
        w = [angle(P[i2] - P[i0], P[i1] - P[i0]), angle(P[i0] - P[i1], P[i2] - P[i1]),
             angle(P[i1] - P[i2], P[i0] - P[i2])]
        for v, wk in zip((i0, i1, i2), w):
            F[v] = F[v] + (wk / PI) * (drag + lift)
    for p in pins:
        F[p] = 0.0
    # State::euler_step (S + S' h) or rk4_step, with S' = [0, v, F / m, 0, 0, 0]
    old = pts.copy()

    def deriv(S):
        d = np.zeros_like(S)
        d[:, 1:4] = S[:, 4:7]
        d[:, 4:7] = S[:, 7:10] / S[:, 0:1]
        return d

    if cfg.get("integration", 0) == 0:
        new = pts + deriv(pts) * dt
    else:  # k1..k4 from re-built states; the force is carried, not re-evaluated
        k1 = deriv(pts)
        k2 = deriv(pts + k1 * (dt * f(0.5)))
        k3 = deriv(pts + k2 * (dt * f(0.5)))
        k4 = deriv(pts + k3 * dt)
        h6, h3 = dt / f(6.0), dt / f(3.0)
        new = pts + (((h6 * k1 + h3 * k2) + h3 * k3) + h6 * k4)
    # update_points: first obstacle face crossed, response; then pins restored
    dtd = duration_secs(dt)
    e, mu = f(cfg["restitution"]), f(cfg["friction"])
    hits = []
    for i in range(len(new)):
        op, ov, oF, om = old[i, 1:4], old[i, 4:7], old[i, 7:10], old[i, 0]
        face = collided_face(obstacles, op, new[i, 1:4], dtd)
        if face is None:
            continue
        hits.append(face)
        d0, d1 = face.distance(op), face.distance(new[i, 1:4])
        fr = d0 / (d0 - d1)
        cp = op + (dt * fr) * ov
        vc = ov + ((dt * fr) * oF) / om
        n = face.normal()
        vcn = dot(vc, n) * n
        vct = vc - vcn
        vrn = (f(-1.0) * vcn) * e
        mt = magnitude(vct)
        if np.all(vct == 0) or np.isnan(mt):
            vrt = np.zeros(3, f)
        else:
            vrt = vct - normalize(vct) * np.fmin(mu * magnitude(vcn), mt)
        new[i, 1:4] = cp + n * f(1e-4)
        new[i, 4:7] = vrn + vrt
    for p in pins:
        new[p] = old[p]
    new[:, 7:10] = 0.0  # clear_forces
    return new, hits


@pytest.mark.skipif(_atan2f is None, reason="no libm to take atan2f from")
@pytest.mark.parametrize("integration", [0, 1])
def test_second_restatement_matches_the_oracle(orc, integration):
    rows, cols, s = 6, 5, f(0.1)
    pins = [rows * cols - cols, rows * cols - 1]
    mesh = orc.SpringyMesh.cloth(rows, cols, float(s), (0.0, 0.0, 0.0), 0.01, 500.0 * s, 0.5 * s, 250.0 * s,
                                 0.5 * s, 50.0 * s, 0.5 * s, pins)
    kcl, ab, _ = mesh.get_struts()
    struts = [((int(a), int(b)), (kcl[j, 0], kcl[j, 1], kcl[j, 2])) for j, (a, b) in enumerate(ab)]
    faces = [tuple(int(v) for v in fv) for fv in mesh.get_faces()[1]]
    pin_list = [int(p) for p in mesh.get_pins()]
    y = -0.3005  # just below the bottom row (y = -rows/2 * s): it is crossed within a few steps
    plane_pos = np.array([[-3, y, 3], [3, y, 3], [3, y, -3], [-3, y, -3]], f)
    plane_idx = np.array([0, 1, 2, 0, 2, 3], np.uint32)
    obstacles = [Obstacle(plane_pos[plane_idx[3 * t]], plane_pos[plane_idx[3 * t + 1]], plane_pos[plane_idx[3 * t + 2]])
                 for t in range(2)]
    cfg = dict(gravity=(0.0, -0.0981, 0.0), wind=(2.0, 0.0, 1.0), drag=0.6, lift=0.3, dt=f(1.0 / 1200.0),
               restitution=0.3, friction=0.2, integration=integration)
    sim = orc.Simulation([mesh], [orc.CollidableMesh(plane_pos, plane_idx)])
    sim.set_config(orc.Config.make(integration, cfg["dt"], cfg["gravity"], cfg["wind"], cfg["lift"], cfg["drag"],
                                   cfg["restitution"], cfg["friction"]))
    pts = mesh.get_points()
    hits = 0
    for k in range(30):
        pts, h = step(pts, struts, faces, pin_list, obstacles, cfg)
        hits += len(h)
        sim.step(1)
        ref = mesh.get_points()
        assert pts[:, 1:7].tobytes() == ref[:, 1:7].tobytes(), "step %d: max diff %g" % (
            k, float(np.abs(pts[:, 1:7].astype(np.float64) - ref[:, 1:7]).max()))
    assert hits > 0  # the bottom row reached the plane: the collision response ran too


def _plane(axis, at):
    """Two triangles of the plane {coordinate axis = at} whose normal points
    along +axis (collidable_mesh.rs face winding)."""
    if axis == 0:
        q = [[at, -3, -3], [at, 3, -3], [at, 3, 3], [at, -3, 3]]
    elif axis == 1:
        q = [[-3, at, 3], [3, at, 3], [3, at, -3], [-3, at, -3]]
    else:
        q = [[-3, -3, at], [3, -3, at], [3, 3, at], [-3, 3, at]]
    return np.array(q, f), np.array([0, 1, 2, 0, 2, 3], np.uint32)


@pytest.mark.skipif(_atan2f is None, reason="no libm to take atan2f from")
def test_every_projection_axis_of_the_collision_search(orc):
    """A floor (+y), and walls facing +x and +z that the wind pushes the cloth
    through: the search drops x, y or z by the reference's signed normal
    comparisons, and both restatements agree bit for bit."""
    rows, cols, s = 6, 5, f(0.1)
    mesh = orc.SpringyMesh.cloth(rows, cols, float(s), (0.0, 0.0, 0.0), 0.01, 500.0 * s, 0.5 * s, 250.0 * s,
                                 0.5 * s, 50.0 * s, 0.5 * s, [rows * cols - cols])
    kcl, ab, _ = mesh.get_struts()
    struts = [((int(a), int(b)), (kcl[j, 0], kcl[j, 1], kcl[j, 2])) for j, (a, b) in enumerate(ab)]
    faces = [tuple(int(v) for v in fv) for fv in mesh.get_faces()[1]]
    pin_list = [int(p) for p in mesh.get_pins()]
    planes = [_plane(1, -0.3005), _plane(0, 0.15002), _plane(2, 0.00002)]
    obstacles = [Obstacle(pos[idx[3 * t]], pos[idx[3 * t + 1]], pos[idx[3 * t + 2]]) for pos, idx in planes
                 for t in range(2)]
    cfg = dict(gravity=(0.0, -0.0981, 0.0), wind=(3.0, 0.0, 3.0), drag=0.6, lift=0.3, dt=f(1.0 / 1200.0),
               restitution=0.3, friction=0.2)
    sim = orc.Simulation([mesh], [orc.CollidableMesh(pos, idx) for pos, idx in planes])
    sim.set_config(orc.Config.make(0, cfg["dt"], cfg["gravity"], cfg["wind"], cfg["lift"], cfg["drag"],
                                   cfg["restitution"], cfg["friction"]))
    pts = mesh.get_points()
    axes = set()
    for k in range(40):
        pts, hit = step(pts, struts, faces, pin_list, obstacles, cfg)
        for face in hit:
            axes.add(int(np.argmax(np.abs(face.normal()))))
        sim.step(1)
        ref = mesh.get_points()
        assert pts[:, 1:7].tobytes() == ref[:, 1:7].tobytes(), "step %d: max diff %g" % (
            k, float(np.abs(pts[:, 1:7].astype(np.float64) - ref[:, 1:7]).max()))
    assert axes == {0, 1, 2}, axes
