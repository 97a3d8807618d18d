"""Parity of the CUDA step against the oracle (GPU tests).

Error measure: relative position error = max_i |p_gpu_i - p_ref_i| / max_i |p_ref_i|
(the same for velocities).  Bars: 1e-5 per step against the f32 oracle,
1e-3 after 1000 steps; bit-identical when the aerodynamic terms are off
(the f32 step leaves the reference's arithmetic only in the face terms'
corner angles); the grid-stencil and general-gather kernels must agree bit
for bit with each other.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PER_STEP_TOL = 1e-5
LONG_TOL = 1e-3


@pytest.fixture(scope="module")
def fgb():
    import feriphys_gb300

    feriphys_gb300._lib()
    return feriphys_gb300


@pytest.fixture(scope="module")
def W():
    from feriphys_gb300 import workloads

    return workloads


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def both(scene, fgb, orc, W, path=0):
    g = W.build(scene, fgb)
    g[1].set_path(path)
    o = W.build(scene, orc)
    return g, o


def compare_steps(g, o, steps, tol, reset=True):
    """Step both sides `steps` times.  With reset, the GPU state is set to the
    oracle's before every step, so each step is checked on identical input
    (the per-step bar); without it the trajectories drift freely."""
    gsim, gm, _ = g
    osim, om, _ = o
    worst = 0.0
    for s in range(steps):
        if reset:
            gm.set_points(om.get_points())
        gsim.step(1)
        osim.step(1)
        gp, op = gm.get_points(), om.get_points()
        e = max(rel(gp[:, 1:4], op[:, 1:4]), rel(gp[:, 4:7], op[:, 4:7]))
        assert np.isfinite(op).all()
        assert e <= tol, "step %d: relative error %.3g > %.3g" % (s + 1, e, tol)
        worst = max(worst, e)
    return worst


@pytest.mark.parametrize("path", [1, 2, 3])
def test_c0_per_step(fgb, orc, W, path):
    g, o = both(W.c0(), fgb, orc, W, path)
    assert g[1].get_path() == min(path, 2)
    worst = compare_steps(g, o, 120, PER_STEP_TOL)
    print("c0 path %d: worst per-step relative error %.3g" % (path, worst))


def test_c0_free_trajectory(fgb, orc, W):
    # Without resets the GPU and oracle trajectories separate only through
    # the corner angles' last bits; at the configured dt=1/600 explicit Euler
    # is unstable, which amplifies that, so the bar here is the long-horizon
    # one.
    g, o = both(W.c0(), fgb, orc, W)
    worst = compare_steps(g, o, 100, LONG_TOL, reset=False)
    print("c0 free trajectory: worst relative error over 100 steps %.3g" % worst)


@pytest.mark.parametrize("path", [1, 2, 3])
def test_c0_aero_off_bit_exact(fgb, orc, W, path):
    sc = W.c0()
    sc.config["drag_coefficient"] = 0.0
    sc.config["lift_coefficient"] = 0.0
    g, o = both(sc, fgb, orc, W, path)
    for _ in range(40):
        g[0].step(1)
        o[0].step(1)
    assert g[1].get_points().tobytes() == o[1].get_points().tobytes()


@pytest.mark.parametrize("rows,cols", [(24, 24), (2, 2), (3, 5), (37, 29), (9, 70), (70, 95), (41, 63), (5, 33)])
def test_step_forms_bit_identical(fgb, W, rows, cols):
    """General gather (1), tiled grid (2), untiled grid (3) kernels and the
    general gather over its plain incidence lists (4) agree bit for bit,
    including cloths that do not fill whole 32x8 tiles."""
    s = 1.0 / 31
    lt, ls, lb = s, s * 2 ** 0.5, 2 * s
    args = (rows, cols, s, (0.0, 0.0, 0.0), 0.01, 500 * lt, 0.5 * lt, 250 * ls, 0.5 * ls, 50 * lb, 0.5 * lb)
    pins = [rows * cols - 1]
    out = []
    for path in (1, 2, 3, 4):
        mesh = fgb.Cloth.new(*args, pins).mesh
        mesh.set_path(path)
        sim = fgb.Simulation.new([mesh], [fgb.CollidableMesh.new(*W.plane(-0.3))])
        sim.set_config(fgb.Config.make(**W.cloth_config(1.0 / 1200.0)))
        p = mesh.get_points()
        p[:, 4:7] = np.random.default_rng(rows * cols).normal(0, 0.5, (rows * cols, 3))  # exercise dampers
        mesh.set_points(p)
        sim.step(40)
        out.append(mesh.get_points().tobytes())
    assert all(o == out[0] for o in out)


def test_c0_long_horizon(fgb, orc, W):
    # dt = 1/6000 keeps explicit Euler stable over 1000 steps (at the config's
    # 1/600 the reference's own step diverges near step 135).
    g, o = both(W.c0(dt=1.0 / 6000.0), fgb, orc, W)
    g[0].step(1000)
    o[0].step(1000)
    gp, op = g[1].get_points(), o[1].get_points()
    assert np.isfinite(op).all()
    assert rel(gp[:, 1:4], op[:, 1:4]) <= LONG_TOL


@pytest.mark.parametrize("path", [1, 2])
def test_rk4(fgb, orc, W, path):
    g, o = both(W.c0(n=16, integration=1), fgb, orc, W, path)
    compare_steps(g, o, 30, PER_STEP_TOL)


def _drop_scene(W, n=20, y0=-1.2, vy=-3.0):
    """A horizontal cloth falling onto a sphere standing on the plane, so that
    many vertices collide with both obstacles."""
    sc = W.c0(n=n, dt=1.0 / 600.0)
    sc.pins = np.zeros(0, np.uint32)
    sc.obstacles = [W.plane(-1.5), W.uv_sphere((0.02, -1.35, 0.01), 0.25, 16, 8)]
    return sc, y0, vy


def _lay_flat(mesh, y0, vy):
    p = mesh.get_points()
    x, y = p[:, 1].copy(), p[:, 2].copy()
    p[:, 1], p[:, 2], p[:, 3] = x, np.float32(y0), y
    p[:, 5] = np.float32(vy)
    mesh.set_points(p)


@pytest.mark.parametrize("path", [1, 2, 3])
def test_collisions_plane_and_sphere(fgb, orc, W, path):
    sc, y0, vy = _drop_scene(W)
    g, o = both(sc, fgb, orc, W, path)
    _lay_flat(g[1], y0, vy)
    _lay_flat(o[1], y0, vy)
    moved_up = 0
    for s in range(60):
        before = o[1].get_points()
        g[0].step(1)
        o[0].step(1)
        gp, op = g[1].get_points(), o[1].get_points()
        moved_up += int((op[:, 5] > 0).sum())
        assert rel(gp[:, 1:4], op[:, 1:4]) <= PER_STEP_TOL, s
        assert rel(gp[:, 4:7], op[:, 4:7]) <= PER_STEP_TOL, s
        # continue both from the oracle state so every step is checked on identical input
        g[1].set_points(op)
    assert moved_up > 0  # collisions actually happened


def test_collision_search_bit_exact_aero_off(fgb, orc, W):
    sc, y0, vy = _drop_scene(W)
    sc.config["drag_coefficient"] = 0.0
    sc.config["lift_coefficient"] = 0.0
    g, o = both(sc, fgb, orc, W, 2)
    _lay_flat(g[1], y0, vy)
    _lay_flat(o[1], y0, vy)
    g[0].step(80)
    o[0].step(80)
    assert g[1].get_points().tobytes() == o[1].get_points().tobytes()


def _random_mesh(rng, n_side=9):
    xs, ys = np.meshgrid(np.arange(n_side), np.arange(n_side))
    pos = np.stack([xs.ravel() * 0.05, ys.ravel() * 0.05, np.zeros(n_side * n_side)], 1)
    pos += rng.normal(0, 0.004, pos.shape)
    idx = []
    for r in range(n_side - 1):
        for c in range(n_side - 1):
            i = r * n_side + c
            if rng.random() < 0.5:
                idx += [i, i + 1, i + n_side, i + 1, i + n_side + 1, i + n_side]
            else:
                idx += [i, i + 1, i + n_side + 1, i, i + n_side + 1, i + n_side]
    return pos.astype(np.float32), np.array(idx, np.uint32)


@pytest.mark.parametrize("integration", [0, 1])
def test_general_mesh(fgb, orc, W, integration):
    rng = np.random.default_rng(3)
    pos, idx = _random_mesh(rng)
    pairs = idx[:12].reshape(-1, 2)
    # nominal (k, c) overrides: effective k ~ 160-320 N/m, c ~ 0.2-0.6 N.s/m on 5 cm struts
    kc = np.stack([rng.uniform(8.0, 16.0, len(pairs)), rng.uniform(0.01, 0.03, len(pairs))], 1).astype(np.float32)
    cfg = W.cloth_config(1.0 / 1200.0, integration)
    g = fgb.SpringyMesh.new(pos, idx, 0.81, 12.0, 0.02, (pairs, kc))
    o = orc.SpringyMesh.new(pos, idx, 0.81, 12.0, 0.02, (pairs, kc))
    for m, add in ((g, lambda a, b: g.add_strut((a, b), 3.0, 0.01)), (o, lambda a, b: o.add_strut(a, b, 3.0, 0.01))):
        add(0, 20)
        add(40, 3)
        m.add_pin(80)
    assert g.get_path() == 1
    obs = [W.plane(-0.05, 1.0)]
    gs = fgb.Simulation.new([g], [fgb.CollidableMesh.new(*obs[0])])
    os_ = orc.Simulation([o], [orc.CollidableMesh(*obs[0])])
    gs.set_config(fgb.Config.make(**cfg))
    c = cfg
    os_.set_config(orc.Config.make(c["integration"], c["dt"], c["gravity"], c["wind"], c["lift_coefficient"],
                                   c["drag_coefficient"], c["coefficient_of_restitution"],
                                   c["coefficient_of_friction"]))
    compare_steps((gs, g, None), (os_, o, None), 100, PER_STEP_TOL)


@pytest.mark.parametrize("bits,spread", [(32, False), (64, False), (32, True)])
def test_general_lists_bit_identical(fgb, W, bits, spread):
    """The general gather over its compact incidence lists (path 1) and over
    the plain CSR lists (path 4) give the same bits, in f32 and f64, for the
    fused step and for accumulate_forces, on a random mesh with (k, c)
    overrides and extra struts.  spread: the mesh's vertices scattered over
    6000 ids (the rest free points without struts), so that neighbour offsets
    exceed the 16-bit strut words and the 32-bit form is read."""
    rng = np.random.default_rng(5)
    pos, idx = _random_mesh(rng)
    if spread:
        ids = rng.permutation(6000)[:len(pos)].astype(np.uint32)
        big = rng.uniform(-1.0, 1.0, (6000, 3)).astype(np.float32)
        big[ids] = pos
        pos, idx = big, ids[idx]
    pairs = idx[:12].reshape(-1, 2)
    kc = np.stack([rng.uniform(8.0, 16.0, len(pairs)), rng.uniform(0.01, 0.03, len(pairs))], 1).astype(np.float32)
    cfg = fgb.Config.make(**W.cloth_config(1.0 / 1200.0))
    out = []
    for path in (1, 4):
        m = fgb.SpringyMesh.new(pos, idx, 0.81, 12.0, 0.02, (pairs, kc))
        m.add_strut((int(idx[0]), int(idx[20])), 3.0, 0.01)
        m.add_strut((int(idx[40]), int(idx[3])), 3.0, 0.01)
        m.add_pin(int(idx[80]))
        m.set_path(path)
        m.set_precision(bits)
        sim = fgb.Simulation.new([m], [fgb.CollidableMesh.new(*W.plane(-0.05, 1.0))])
        sim.set_config(cfg)
        p = m.get_points()
        p[:, 4:7] = rng.normal(0, 0.3, (len(p), 3)) if path == 1 else out[0][2]
        m.set_points(p)
        vel = p[:, 4:7].copy()
        sim.step(50)
        got = m.get_points_f64() if bits == 64 else m.get_points()
        m.accumulate_forces(cfg)
        forces = m.get_points_f64() if bits == 64 else m.get_points()
        assert m.get_path() == 1
        out.append((got.tobytes(), forces.tobytes(), vel))
    assert out[0][0] == out[1][0]
    assert out[0][1] == out[1][1]


def test_phase_hooks_match_oracle(fgb, orc, W):
    sc, y0, vy = _drop_scene(W, n=12)
    (gsim, gm, gobs), (osim, om, oobs) = both(sc, fgb, orc, W, 1)
    _lay_flat(gm, y0, vy)
    _lay_flat(om, y0, vy)
    c = sc.config
    gcfg = fgb.Config.make(**c)
    ocfg = orc.Config.make(c["integration"], c["dt"], c["gravity"], c["wind"], c["lift_coefficient"],
                           c["drag_coefficient"], c["coefficient_of_restitution"], c["coefficient_of_friction"])
    for _ in range(20):
        gm.accumulate_forces(gcfg)
        om.accumulate_forces(ocfg)
        gp, op = gm.get_points(), om.get_points()
        assert rel(gp[:, 7:10], op[:, 7:10]) <= PER_STEP_TOL
        gm.integrate(0, c["dt"])
        staged = om.integrate(0, c["dt"])
        gm.update_points(gobs, gcfg)
        om.update_points(staged, oobs, ocfg)
        gp, op = gm.get_points(), om.get_points()
        assert rel(gp[:, 1:7], op[:, 1:7]) <= PER_STEP_TOL
        assert rel(gp[:, 7:10], op[:, 7:10]) <= PER_STEP_TOL
        gm.clear_forces()
        om.clear_forces()
        gm.set_points(om.get_points())


def test_f64_rerun(fgb, orc, W):
    sc = W.c0(n=16, dt=1.0 / 6000.0)
    g = W.build(sc, fgb)
    g[1].set_precision(64)
    o = W.build(sc, orc)
    o64m = o[1].widen()
    o64 = orc.Simulation([o64m], o[2])
    c = sc.config
    o64.set_config(orc.Config.make(c["integration"], c["dt"], c["gravity"], c["wind"], c["lift_coefficient"],
                                   c["drag_coefficient"], c["coefficient_of_restitution"],
                                   c["coefficient_of_friction"]))
    g[0].step(200)
    o64.step(200)
    assert rel(g[1].get_points_f64()[:, 1:7], o64m.get_points()[:, 1:7]) <= 1e-10
    # and the f32 step sits within the per-step bar of the f64 rerun
    f32 = W.build(sc, fgb)
    f32[0].step(1)
    g2 = W.build(sc, fgb)
    g2[1].set_precision(64)
    g2[0].step(1)
    assert rel(f32[1].get_points()[:, 1:4], g2[1].get_points_f64()[:, 1:4]) <= PER_STEP_TOL


def test_points_round_trip_device(fgb, W):
    sim, m, _ = W.build(W.c0(n=8), fgb)
    sim.step(3)
    p = m.get_points()
    p[:, 4:7] += 0.25
    m.set_points(p)
    assert m.get_points().tobytes() == p.tobytes()
    pos, idx = m.get_vertices()
    assert (pos == p[:, 1:4]).all() and idx.size == 3 * 2 * 7 * 7


@pytest.mark.parametrize("n", [8, 97])
def test_points_round_trip_pinned_host(fgb, W, n):
    """Pinned host rows are read and written by the conversion kernels across
    the host link directly; odd sizes exercise the partial last block."""
    torch = pytest.importorskip("torch")
    sim, m, _ = W.build(W.c0(n=n), fgb)
    sim.step(3)
    p = m.get_points()
    p[:, 4:7] += 0.25
    p[:, 7:10] = np.random.default_rng(0).normal(size=(len(p), 3)).astype(np.float32)
    buf = torch.empty(p.shape, dtype=torch.float32, pin_memory=True)
    host = buf.numpy()
    host[:] = p
    m.set_points(host)
    host[:] = 0
    m.get_points(out=host)
    assert host.tobytes() == p.tobytes()
    # and the next step uses the forces that came in that way, as from pageable memory
    sim2, m2, _ = W.build(W.c0(n=n), fgb)
    sim2.step(3)
    m2.set_points(p.copy())
    sim.step(1)
    sim2.step(1)
    assert m.get_points().tobytes() == m2.get_points().tobytes()


def test_nonfinite_flag(fgb, W):
    sc = W.c0(n=8)
    sim, m, _ = W.build(sc, fgb)
    assert not sim.synchronize()
    p = m.get_points()
    p[3, 1] = np.inf
    m.set_points(p)
    sim.step(2)
    assert sim.synchronize()
    assert not sim.synchronize()  # the flag resets once read


def test_c1_full_size_first_steps(fgb, orc, W):
    sc = W.c1()
    g, o = both(sc, fgb, orc, W)
    assert g[1].get_path() == 2
    compare_steps(g, o, 2, PER_STEP_TOL)


def test_c1_determinism(fgb, W):
    sc = W.c1(n=256)
    a = W.build(sc, fgb)
    b = W.build(sc, fgb)
    a[0].step(20)
    b[0].step(20)
    assert a[1].get_points().tobytes() == b[1].get_points().tobytes()
