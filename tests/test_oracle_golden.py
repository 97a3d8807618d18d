"""Pins the oracle (the C++ restatement) to the reference.

Part 1 replays the assertions of the reference's own unit tests
(tests/golden/reference_unit_goldens.json, each entry citing its file:line).
Part 2 checks hand-derived known answers for the terms no reference test
pins: strut spring/damper forces, per-face drag/lift with the angle split,
gravity-as-force, pins, explicit Euler / frozen-force RK4 and the plane
collision response (springy_mesh.rs:423-551, 629-660; state.rs:75-106).
"""
import json
import math
import os

import numpy as np
import pytest

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_unit_goldens.json")))
F32 = np.float32


# ----------------------------------------------------------- reference tests ---
def test_ctor_triangle(orc):
    g = GOLD["ctor_triangle"]
    m = orc.SpringyMesh.new(g["positions"], g["indices"], g["mass"], g["stiffness"], g["damping"])
    assert m.counts()[:3] == (g["n_points"], g["n_struts"], g["n_faces"])
    st, vs = m.get_faces()
    assert st[0].tolist() == g["face0_struts"] and vs[0].tolist() == g["face0_vertices"]
    pts = m.get_points()
    assert pts[0, 0] == F32(1.0) / F32(3.0)
    assert pts[0, 1:].tolist() == [0.0] * 9
    assert pts[1, 1:4].tolist() == [2.0, 0.0, 0.0] and pts[1, 4:7].tolist() == [0.0] * 3
    kcl, _, _ = m.get_struts()
    assert kcl[0, 0] == F32(2.0) * (F32(1.0) / F32(2.0))
    assert kcl[0, 1] == F32(3.0) * (F32(1.0) / F32(2.0))
    assert kcl[0, 2] == F32(g["strut0_length"])


def test_face_angles_exact(orc):
    g = GOLD["face_angles"]
    t = GOLD["ctor_triangle"]
    m = orc.SpringyMesh.new(t["positions"], t["indices"], t["mass"], t["stiffness"], t["damping"])
    assert m.face_angle(0, 0) == F32(math.pi) / F32(2.0)
    assert m.face_angle(0, 1) == F32(g["angle1"])
    assert m.face_angle(0, 2) == F32(g["angle2"])


def test_strip_ctor(orc):
    g = GOLD["strip"]
    m = orc.SpringyMesh.new(g["positions"], g["indices"], g["mass"], g["stiffness"], g["damping"])
    assert m.counts()[:3] == (g["n_points"], g["n_struts"], g["n_faces"])
    st, vs = m.get_faces()
    assert vs.tolist() == g["face_vertices"]
    assert st.tolist() == g["face_struts"]
    _, ab, fc = m.get_struts()
    assert ab.tolist() == g["strut_vertices"]
    want = [[a, -1 if b is None else b] for a, b in g["strut_faces"]]
    assert fc.tolist() == want
    for f, n in enumerate(g["face_normals"]):
        assert m.face_normal(f).tolist() == [float(v) for v in n]


def test_get_vertices(orc):
    g = GOLD["get_vertices"]
    m = orc.SpringyMesh.new(g["positions"], g["indices"], 1.0, 2.0, 3.0)
    assert m.get_points()[:, 1:4].tolist() == [[float(v) for v in p] for p in g["positions"]]
    assert m.get_faces()[1].reshape(-1).tolist() == g["indices"]


def test_euler_step_exact(orc):
    g = GOLD["euler_step"]
    out = orc.state_test_euler(g["initial_state"], g["h"])
    assert out[:3].tolist() == g["expected_position"]
    assert out[3:].tolist() == g["expected_velocity"]


def test_rk4_step(orc):
    g = GOLD["rk4_step"]
    s = np.asarray(g["initial_state"], np.float32)
    for y, t in zip(g["expected_y"], g["expected_t"]):
        s = orc.state_test_rk4(s, g["h"])
        assert abs(float(s[0]) - y) < g["acceptable_error"]
        assert s[1] == F32(t) and s[2] == F32(g["h"])


def test_collidable_ctor(orc):
    g = GOLD["collidable_ctor"]
    o = orc.CollidableMesh(g["positions"], g["indices"])
    assert o.counts() == (g["n_vertices"], g["n_edges"], g["n_faces"])
    edges = o.edges().tolist()
    for e in g["edges_contained"]:
        assert [[float(v) for v in p] for p in e] in edges
    assert o.faces().tolist() == [[[float(v) for v in p] for p in f] for f in g["faces"]]


def test_collidable_rejects_degenerate_triangle(orc):
    # collidable_mesh.rs:81-89 indexes verts_indices[1] of a one-element edge set: panics.
    with pytest.raises(orc.OracleError):
        orc.CollidableMesh([[0, 0, 0], [1, 0, 0]], [0, 0, 1])


def test_duration_roundtrip(orc):
    # Duration::from_secs_f32 rounds to whole nanoseconds; as_secs_f32 rebuilds an f32.
    assert orc.duration_roundtrip(F32(1 / 600)) == F32(1666667) / F32(1e9)
    assert orc.duration_roundtrip(F32(0.001)) == F32(0.001)
    assert orc.duration_roundtrip(F32(0.0)) == 0.0
    assert orc.duration_roundtrip(F32(1.5)) == F32(1.5)


# --------------------------------------------------------- known answers (f64) ---
def _two_vertex(orc, k=40.0, c=0.3, mass=0.02):
    m = orc.SpringyMesh.new([[0, 0, 0], [0.5, 0, 0]], [], mass, 1.0, 1.0)
    m.add_strut(0, 1, k, c)
    return m


def test_strut_spring_damper_known_answer(orc):
    k, c, mass = 40.0, 0.3, 0.02
    m = _two_vertex(orc, k, c, mass)
    pts = m.get_points()
    pts[1, 1:4] = [0.55, 0.1, -0.05]
    pts[0, 4:7] = [0.2, -0.1, 0.3]
    pts[1, 4:7] = [-0.4, 0.25, 0.1]
    m.set_points(pts)
    g = np.array([0.0, -0.0981, 0.0])
    cfg = orc.Config.make(gravity=g, wind=(0, 0, 0), lift=0, drag=0)
    m.accumulate_forces(cfg)
    got = m.get_points().astype(np.float64)
    L = 0.5
    ke, ce = k / L, c / L
    p0, p1 = pts[0, 1:4].astype(np.float64), pts[1, 1:4].astype(np.float64)
    v0, v1 = pts[0, 4:7].astype(np.float64), pts[1, 4:7].astype(np.float64)
    d = p1 - p0
    u = d / np.linalg.norm(d)
    fs = ke * (np.linalg.norm(d) - L) * u
    fd = ce * np.dot(v1 - v0, u) * u
    np.testing.assert_allclose(got[0, 7:10], g + fs + fd, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(got[1, 7:10], g - fs - fd, rtol=1e-5, atol=1e-6)
    # Euler: p' = p + v h, v' = v + F/m h (state.rs:75-83); RK4 with frozen forces
    # is the exact constant-acceleration update p + v h + a h^2/2 (state.rs:86-106).
    h = 1e-3
    for integ in (0, 1):
        nxt = m.integrate(integ, h).astype(np.float64)
        a = got[:, 7:10] / got[:, :1]
        ph = got[:, 1:4] + got[:, 4:7] * h + (0.5 * a * h * h if integ else 0.0)
        np.testing.assert_allclose(nxt[:, 1:4], ph, rtol=1e-6, atol=1e-7)
        np.testing.assert_allclose(nxt[:, 4:7], got[:, 4:7] + a * h, rtol=1e-5, atol=1e-6)
        assert (nxt[:, 0] == got[:, 0]).all()


def test_face_aero_known_answer(orc):
    # One right-isosceles face in the xy-plane (normal +z) at rest in uniform wind.
    m = orc.SpringyMesh.new([[0, 0, 0], [1, 0, 0], [0, 1, 0]], [0, 1, 2], 0.03, 10.0, 0.5)
    w = np.array([2.0, 0.5, 1.0])
    cd, cl = 0.6, 0.3
    cfg = orc.Config.make(gravity=(0, 0, 0), wind=w, lift=cl, drag=cd)
    m.accumulate_forces(cfg)
    F = m.get_points()[:, 7:10].astype(np.float64)
    rv = -w
    n = np.array([0.0, 0.0, 1.0])
    eff = 0.5 * abs(np.dot(n, rv))
    drag = -cd * eff * rv
    lift = -cl * eff * rv * np.linalg.norm(np.cross(n, rv))
    tot = drag + lift
    for i, frac in enumerate([0.5, 0.25, 0.25]):
        np.testing.assert_allclose(F[i], frac * tot, rtol=2e-6, atol=1e-7)


def test_pins_and_gravity_force(orc):
    m = orc.SpringyMesh.new([[0, 0, 0], [1, 0, 0], [0, 1, 0]], [0, 1, 2], 0.03, 10.0, 0.5)
    m.add_pin(2)
    sim = orc.Simulation([m], [])
    cfg = orc.Config.make(integration=0, dt=0.01, gravity=(0, -0.5, 0), wind=(0, 0, 0), lift=0, drag=0)
    sim.set_config(cfg)
    before = m.get_points().copy()
    sim.step(3)
    after = m.get_points()
    assert (after[2] == before[2]).all()          # pinned: restored each step
    assert (after[:, 7:10] == 0).all()            # clear_forces
    # first step: gravity is a force, a = g/m (springy_mesh.rs:194-196)
    m2 = orc.SpringyMesh.new([[0, 0, 0], [1, 0, 0], [0, 1, 0]], [0, 1, 2], 0.03, 10.0, 0.5)
    s2 = orc.Simulation([m2], [])
    s2.set_config(cfg)
    s2.step(1)
    v = m2.get_points()[:, 4:7]
    np.testing.assert_allclose(v[:, 1], -0.5 / 0.01 * 0.01, rtol=1e-6)


def _floor(y=-1.0, half=5.0):
    pos = [[-half, y, half], [half, y, half], [half, y, -half], [-half, y, -half]]
    return pos, [0, 1, 2, 0, 2, 3]


def test_plane_collision_known_answer(orc):
    pos, idx = _floor(-1.0)
    floor = orc.CollidableMesh(pos, idx)
    assert floor.faces().shape == (2, 3, 3)
    m = orc.SpringyMesh.new([[0.1, -0.99, 0.2]], [], 0.01, 1.0, 1.0)
    pts = m.get_points()
    v = np.array([1.0, -10.0, 0.5])
    pts[0, 4:7] = v
    m.set_points(pts)
    e, mu, h = 0.3, 0.2, 0.005
    g = np.array([0.0, -0.0981, 0.0])
    cfg = orc.Config.make(integration=0, dt=h, gravity=g, wind=(0, 0, 0), lift=0, drag=0,
                          restitution=e, friction=mu)
    sim = orc.Simulation([m], [floor])
    sim.set_config(cfg)
    sim.step(1)
    got = m.get_points()[0].astype(np.float64)
    p = np.array([0.1, -0.99, 0.2])
    mass = float(F32(0.01))
    d_old = p[1] + 1.0
    d_new = (p + v * h)[1] + 1.0
    f = d_old / (d_old - d_new)
    n = np.array([0.0, 1.0, 0.0])
    cp = p + h * f * v
    vc = v + h * f * g / mass
    vn = np.dot(vc, n) * n
    vt = vc - vn
    vr = -e * vn + vt - vt / np.linalg.norm(vt) * min(mu * np.linalg.norm(vn), np.linalg.norm(vt))
    np.testing.assert_allclose(got[1:4], cp + n * 1e-4, rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(got[4:7], vr, rtol=1e-5, atol=1e-6)


def test_first_hit_order(orc):
    # Two stacked floors: a vertex that crosses both planes collides with the
    # first face in flattened obstacle order (springy_mesh.rs:429-433).
    a = orc.CollidableMesh(*_floor(-1.0))
    b = orc.CollidableMesh(*_floor(-1.5))
    old = np.array([[0.1, -0.9, 0.1]], np.float32)
    new = np.array([[0.1, -1.7, 0.1]], np.float32)
    assert orc.collided_faces([a, b], old, new, 0.01)[0] in (0, 1)
    assert orc.collided_faces([b, a], old, new, 0.01)[0] in (0, 1)
    miss = np.array([[9.0, -1.7, 9.0]], np.float32)
    assert orc.collided_faces([a, b], miss * [1, 0, 1] + [0, -0.9, 0], miss, 0.01)[0] == -1


def test_cloth_builder_counts(orc):
    # cloth.rs:63-110: 3(r-1)(c-1) + (r-1) + (c-1) triangle struts, 2(r-2)(c-2) binding.
    for r, c in [(2, 2), (3, 5), (32, 32)]:
        m = orc.SpringyMesh.cloth(r, c, 0.1, (0, 0, 0), 0.01, 500, 0.5, 250, 0.5, 50, 0.5, [])
        tri = 3 * (r - 1) * (c - 1) + (r - 1) + (c - 1)
        assert m.counts()[:3] == (r * c, tri + 2 * max(r - 2, 0) * max(c - 2, 0), 2 * (r - 1) * (c - 1))
    m = orc.SpringyMesh.cloth(32, 32, 1 / 31, (0, 0, 0), 0.01, 500, 0.5, 250, 0.5, 50, 0.5, [])
    assert m.counts()[1] == 4745  # 1,984 structural + 961 shear + 1,800 binding


def test_cloth_builder_rejects_small(orc):
    with pytest.raises(orc.OracleError):
        orc.SpringyMesh.cloth(1, 5, 0.1, (0, 0, 0), 0.01, 1, 1, 1, 1, 1, 1, [])
