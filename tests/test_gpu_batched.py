"""Batched stepping (many Cloth::new grids in one launch per step) gives
exactly the results of stepping every cloth alone: bit for bit, for both
launch forms, with and without CUDA-graph capture, with per-cloth wind, a
general (non-grid) mesh in the same simulation, and cloths too small for
interior tiles.  A few cloths are also checked against the oracle, one
reference Simulation per cloth (the reference's wind is per Simulation)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fgb():
    import feriphys_gb300

    feriphys_gb300._lib()
    return feriphys_gb300


def _batch(W, n=24, seed=1):
    b = W.c2(n_cloths=n, lo=2, hi=70, seed=seed)
    # make sure tiny and tile-edge sizes are present
    extra = W.c2(n_cloths=4, lo=2, hi=2, seed=seed + 1).cloths + W.c2(n_cloths=2, lo=36, hi=36, seed=seed + 2).cloths
    b.cloths.extend(extra)
    return b


def _alone(fgb, W, batch, steps):
    out = []
    for args, pins, wind in batch.cloths:
        m = fgb.Cloth.new(*args, pins).mesh
        sim = fgb.Simulation.new([m], [fgb.CollidableMesh.new(p, i) for p, i in batch.obstacles])
        cfg = dict(batch.config)
        cfg["wind"] = wind
        sim.set_config(fgb.Config.make(**cfg))
        sim.step(steps)
        out.append(m.get_points().tobytes())
    return out


@pytest.mark.parametrize("mode,graphs", [(0, True), (1, True), (1, False), (-1, True)])
def test_batched_equals_alone(fgb, mode, graphs):
    from feriphys_gb300 import workloads as W

    batch = _batch(W)
    sim, meshes, _ = W.build_batch(batch, fgb)
    sim.set_batch_mode(mode)
    sim.set_graphs(graphs)
    sim.step(1)
    sim.step(12)  # graph-captured when enabled
    sim.step(7)
    info = sim.batch_info()
    assert info[0] == len(meshes) and info[1] > len(meshes) and info[2] in (0, 1)
    ref = _alone(fgb, W, batch, 20)
    got = [m.get_points().tobytes() for m in meshes]
    assert got == ref


@pytest.mark.parametrize("tile_rows,mode", [(4, 1), (12, 1), (12, 0), (0, -1)])
def test_every_tile_height_equals_alone(fgb, tile_rows, mode):
    """32x4, 32x8 and 32x12 tiles (and the autotuner's pick) give every cloth
    the bits of stepping it alone."""
    from feriphys_gb300 import workloads as W

    batch = _batch(W)
    sim, meshes, _ = W.build_batch(batch, fgb)
    sim.set_batch_tile(tile_rows)
    sim.set_batch_mode(mode)
    sim.step(1)
    sim.step(12)
    sim.step(7)
    info = sim.batch_info()
    assert info[4] == tile_rows if tile_rows else info[4] in (4, 8, 12)
    ref = _alone(fgb, W, batch, 20)
    got = [m.get_points().tobytes() for m in meshes]
    assert got == ref


def test_batch_with_general_mesh_and_forces(fgb):
    from feriphys_gb300 import workloads as W

    batch = _batch(W, n=6, seed=3)
    sim, meshes, obs = W.build_batch(batch, fgb)
    # a general (non-grid) mesh joins the same simulation
    pos = np.array([[0, 0, 0], [0.1, 0, 0], [0, 0.1, 0], [0.1, 0.1, 0.02]], np.float32)
    g = fgb.SpringyMesh.new(pos, [0, 1, 2, 1, 3, 2], 0.04, 10.0, 0.1)
    sim2 = fgb.Simulation.new(meshes + [g], obs)
    sim2.set_config(fgb.Config.make(**batch.config))
    # carried accumulated force on one cloth (Stateful point with F != 0)
    p = meshes[0].get_points()
    p[:, 7:10] = 0.001
    meshes[0].set_points(p)
    sim2.step(10)
    m0 = fgb.Cloth.new(*batch.cloths[0][0], batch.cloths[0][1]).mesh
    s0 = fgb.Simulation.new([m0], [fgb.CollidableMesh.new(pp, ii) for pp, ii in batch.obstacles])
    cfg = dict(batch.config)
    cfg["wind"] = batch.cloths[0][2]
    s0.set_config(fgb.Config.make(**cfg))
    q = m0.get_points()
    q[:, 7:10] = 0.001
    m0.set_points(q)
    s0.step(10)
    assert meshes[0].get_points().tobytes() == m0.get_points().tobytes()
    assert np.isfinite(g.get_points()).all()


def test_batched_against_oracle(fgb, orc):
    from feriphys_gb300 import workloads as W

    batch = W.c2(n_cloths=5, lo=8, hi=40, seed=7)
    sim, meshes, _ = W.build_batch(batch, fgb)
    for i, (args, pins, wind) in enumerate(batch.cloths):
        om = orc.SpringyMesh.cloth(*args, pins)
        os_ = orc.Simulation([om], [orc.CollidableMesh(p, ix) for p, ix in batch.obstacles])
        c = batch.config
        os_.set_config(orc.Config.make(c["integration"], c["dt"], c["gravity"], wind, c["lift_coefficient"],
                                       c["drag_coefficient"], c["coefficient_of_restitution"],
                                       c["coefficient_of_friction"]))
        meshes[i]._oracle = (os_, om)
    for step in range(30):
        for m in meshes:
            m.set_points(m._oracle[1].get_points())
        sim.step(1)
        for m in meshes:
            m._oracle[0].step(1)
            gp, op = m.get_points().astype(np.float64), m._oracle[1].get_points().astype(np.float64)
            err = np.abs(gp[:, 1:7] - op[:, 1:7]).max() / np.abs(op[:, 1:7]).max()
            assert err <= 1e-5, (step, err)
