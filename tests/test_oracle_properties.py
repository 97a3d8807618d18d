"""Properties of the oracle's step that hold whatever the cloth (the
reference's own tests pin components, not whole steps): internal strut forces
cancel pairwise (springy_mesh.rs:533-551 adds fs to one end and -fs to the
other), a cloth at its rest shape with nothing acting on it stays there bit
for bit, a rigid translation of a free cloth translates its step, and the
total momentum of a free cloth without external forces is conserved by the
explicit Euler step (state.rs:75-83)."""
import numpy as np

F32 = np.float32


def _cloth(orc, rows=12, cols=9, pins=()):
    s = 1.0 / (cols - 1)
    return orc.SpringyMesh.cloth(rows, cols, s, (0.0, 0.0, 0.0), 0.01, 500.0 * s, 0.5 * s, 250.0 * s, 0.5 * s,
                                 50.0 * s, 0.5 * s, list(pins))


def _free_config(orc, dt=1.0 / 6000.0):
    # no gravity, no wind, no aerodynamics: only the struts act
    return orc.Config.make(0, dt, (0.0, 0.0, 0.0), (0.0, 0.0, 0.0), 0.0, 0.0, 0.3, 0.2)


def _perturb(mesh, seed, dpos=2e-3, vel=0.05):
    rng = np.random.default_rng(seed)
    pts = mesh.get_points().copy()
    pts[:, 1:4] += rng.normal(0.0, dpos, (len(pts), 3)).astype(F32)
    pts[:, 4:7] = rng.normal(0.0, vel, (len(pts), 3)).astype(F32)
    mesh.set_points(pts)
    return pts


def test_internal_forces_cancel(orc):
    mesh = _cloth(orc)
    _perturb(mesh, 1)
    mesh.accumulate_forces(_free_config(orc))
    F = mesh.get_points()[:, 7:10].astype(np.float64)
    assert np.abs(F).sum() > 0
    net = np.abs(F.sum(0)).max()
    assert net <= 1e-5 * np.abs(F).sum(), (net, np.abs(F).sum())


def test_rest_shape_stays_at_rest_bit_for_bit(orc):
    mesh = _cloth(orc, pins=[0, 5])
    start = mesh.get_points().copy()
    plane = orc.CollidableMesh(np.array([[-3, -1.5, 3], [3, -1.5, 3], [3, -1.5, -3], [-3, -1.5, -3]], F32),
                               np.array([0, 1, 2, 0, 2, 3], np.uint32))
    sim = orc.Simulation([mesh], [plane])
    sim.set_config(orc.Config.make(0, 1.0 / 600.0, (0.0, 0.0, 0.0), (0.0, 0.0, 0.0), 0.5, 0.6, 0.3, 0.2))
    sim.step(25)
    end = mesh.get_points()
    assert end[:, 1:4].tobytes() == start[:, 1:4].tobytes()
    assert np.array_equal(end[:, 4:7], np.zeros_like(end[:, 4:7]))


def test_translation_moves_the_step_along(orc):
    shift = np.array([0.75, -0.5, 0.25], F32)
    a, b = _cloth(orc), _cloth(orc)
    pts = _perturb(a, 2)
    moved = pts.copy()
    moved[:, 1:4] += shift
    b.set_points(moved)
    cfg = _free_config(orc)
    for m in (a, b):
        sim = orc.Simulation([m], [])
        sim.set_config(cfg)
        sim.step(5)
    pa = a.get_points()[:, 1:4].astype(np.float64)
    pb = b.get_points()[:, 1:4].astype(np.float64) - shift.astype(np.float64)
    assert np.abs(pa - pb).max() <= 1e-5 * np.abs(pa).max()
    va, vb = a.get_points()[:, 4:7], b.get_points()[:, 4:7]
    assert np.abs(va - vb).max() <= 1e-3 * np.abs(va).max()


def test_momentum_of_a_free_cloth_is_conserved(orc):
    mesh = _cloth(orc)
    pts = _perturb(mesh, 3)
    m = pts[:, 0:1].astype(np.float64)
    p0 = (m * pts[:, 4:7].astype(np.float64)).sum(0)
    sim = orc.Simulation([mesh], [])
    sim.set_config(_free_config(orc))
    sim.step(20)
    end = mesh.get_points()
    p1 = (m * end[:, 4:7].astype(np.float64)).sum(0)
    scale = (m * np.abs(end[:, 4:7].astype(np.float64))).sum()
    assert np.abs(p1 - p0).max() <= 1e-5 * scale, (p0, p1, scale)
