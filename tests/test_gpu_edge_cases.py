"""Edge cases of the step against the oracle (GPU tests).

* A mesh with no points, and a simulation with no meshes, step without
  error and stay empty.
* One simulation over three meshes of different kinds -- a Cloth::new grid
  (tiled kernel), a general SpringyMesh (gather kernel) and an empty mesh --
  steps each as the reference steps them one after another
  (simulation.rs:27-45): bit-identical with drag and lift off, within the
  per-step bar with them on.
* The smallest cloth (2 x 2) with every point pinned does not move, bit for
  bit.
* A degenerate (zero-area) triangle makes the reference's face normal
  0 * (1/0) = NaN, so its three vertices go non-finite; the GPU step gives
  NaN at exactly the same points and raises its non-finite flag.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PER_STEP_TOL = 1e-5


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


def oracle_config(orc, c):
    return orc.Config.make(c["integration"], c["dt"], c["gravity"], c["wind"], c["lift_coefficient"],
                           c["drag_coefficient"], c["coefficient_of_restitution"], c["coefficient_of_friction"])


def small_mesh(rng, n_side=6):
    xs, ys = np.meshgrid(np.arange(n_side), np.arange(n_side))
    pos = np.stack([xs.ravel() * 0.05, np.zeros(n_side * n_side), ys.ravel() * 0.05], 1)
    pos += rng.normal(0, 0.003, pos.shape)
    idx = []
    for r in range(n_side - 1):
        for c in range(n_side - 1):
            i = r * n_side + c
            idx += [i, i + 1, i + n_side, i + 1, i + n_side + 1, i + n_side]
    return pos.astype(np.float32), np.array(idx, np.uint32)


def test_empty_mesh_and_empty_simulation(fgb, W):
    empty = fgb.SpringyMesh.new(np.zeros((0, 3), np.float32), np.zeros(0, np.uint32), 1.0, 10.0, 0.1)
    sim = fgb.Simulation.new([empty], [fgb.CollidableMesh.new(*W.plane(-1.0))])
    sim.set_config(fgb.Config.make(**W.cloth_config(1.0 / 600.0)))
    sim.step(5)
    assert not sim.synchronize()
    assert empty.get_points().shape == (0, 10)
    nothing = fgb.Simulation.new([], [])
    nothing.step(3)
    assert not nothing.synchronize()


@pytest.mark.parametrize("aero", [False, True])
def test_mixed_meshes_in_one_simulation(fgb, orc, W, aero):
    rng = np.random.default_rng(11)
    pos, idx = small_mesh(rng)
    cfg = W.cloth_config(1.0 / 3000.0)
    if not aero:
        cfg["drag_coefficient"] = 0.0
        cfg["lift_coefficient"] = 0.0
    s = 1.0 / 15
    cloth_args = (12, 9, s, (-0.3, 0.2, 0.0), 0.01, 500 * s, 0.5 * s, 250 * s, 0.5 * s, 50 * s, 0.5 * s)
    pins = [0, 8]
    empty_pos, empty_idx = np.zeros((0, 3), np.float32), np.zeros(0, np.uint32)
    sides = {}
    for name, api in (("gpu", fgb), ("oracle", orc)):
        if api is fgb:
            cloth = fgb.Cloth.new(*cloth_args, pins).mesh
        else:
            cloth = orc.SpringyMesh.cloth(*cloth_args, pinned=pins)
        general = api.SpringyMesh.new(pos, idx, 0.5, 12.0, 0.02)
        empty = api.SpringyMesh.new(empty_pos, empty_idx, 1.0, 10.0, 0.1)
        general.add_pin(3)
        obstacles = [W.plane(-0.25)]
        if api is fgb:
            sim = fgb.Simulation.new([cloth, empty, general], [fgb.CollidableMesh.new(*o) for o in obstacles])
            sim.set_config(fgb.Config.make(**cfg))
        else:
            sim = orc.Simulation([cloth, empty, general], [orc.CollidableMesh(*o) for o in obstacles])
            sim.set_config(oracle_config(orc, cfg))
        sides[name] = (sim, cloth, general)
    assert sides["gpu"][1].get_path() == 2 and sides["gpu"][2].get_path() == 1
    for k in range(20):
        for sim, _, _ in sides.values():
            sim.step(1)
        for j in (1, 2):
            g, o = sides["gpu"][j].get_points(), sides["oracle"][j].get_points()
            assert np.isfinite(o).all()
            if aero:
                e = max(rel(g[:, 1:4], o[:, 1:4]), rel(g[:, 4:7], o[:, 4:7]))
                assert e <= PER_STEP_TOL, (k, j, e)
                sides["gpu"][j].set_points(o)  # re-base: the per-step bar
            else:
                assert g.tobytes() == o.tobytes(), (k, j)


def test_fully_pinned_smallest_cloth_stays_put(fgb, W):
    s = 0.1
    mesh = fgb.Cloth.new(2, 2, s, (0.0, 0.0, 0.0), 0.01, 500 * s, 0.5 * s, 250 * s, 0.5 * s, 50 * s, 0.5 * s,
                         [0, 1, 2, 3]).mesh
    sim = fgb.Simulation.new([mesh], [fgb.CollidableMesh.new(*W.plane(-1.0))])
    sim.set_config(fgb.Config.make(**W.cloth_config(1.0 / 600.0)))
    before = mesh.get_points()
    sim.step(10)
    after = mesh.get_points()
    assert after[:, 1:7].tobytes() == before[:, 1:7].tobytes()


def test_degenerate_face_goes_non_finite_like_the_reference(fgb, orc, W):
    pos = np.array([[0, 0, 0], [0.1, 0, 0], [0.2, 0, 0],   # collinear: zero area
                    [0, 0.1, 0], [0.1, 0.1, 0.01], [0.2, 0.12, 0]], np.float32)
    idx = np.array([0, 1, 2, 0, 4, 3, 1, 5, 4], np.uint32)
    cfg = W.cloth_config(1.0 / 600.0)
    g = fgb.SpringyMesh.new(pos, idx, 0.3, 10.0, 0.05)
    o = orc.SpringyMesh.new(pos, idx, 0.3, 10.0, 0.05)
    gs = fgb.Simulation.new([g], [])
    gs.set_config(fgb.Config.make(**cfg))
    os_ = orc.Simulation([o], [])
    os_.set_config(oracle_config(orc, cfg))
    gs.step(1)
    os_.step(1)
    gp, op = g.get_points(), o.get_points()
    bad_ref = ~np.isfinite(op[:, 1:7]).all(1)
    assert bad_ref[[0, 1, 2]].all()  # the degenerate face's vertices
    assert np.array_equal(~np.isfinite(gp[:, 1:7]).all(1), bad_ref)
    ok = ~bad_ref
    assert rel(gp[ok][:, 1:7], op[ok][:, 1:7]) <= PER_STEP_TOL
    assert gs.synchronize()  # the non-finite flag
