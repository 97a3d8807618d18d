"""Long-horizon parity on a scene shaped like the large plain configuration.

A 128 x 128 cloth with the large configuration's features -- seeded N(0, 1e-3)
position noise, per-strut stiffness within +-10%, the top row pinned, wind,
drag and lift, a plane and a 32 x 16 UV sphere (collidable_mesh.rs:107-169)
-- stepped 1000 times at dt = 1/6000 s (explicit Euler is stable there; at
the configured 1/600 the reference's own step diverges) on the GPU and in the
oracle, free-running (no re-basing).  The sphere (radius 0.3 m) stands just
in front of the hanging cloth and the cloth's free vertices start at 1 m/s
towards it, so a growing patch of the cloth runs into the sphere's faces; the
oracle counts those hits (springy_mesh.rs:423-497 through the first-hit
search) so the test knows the collision path ran.

Bars: relative position error <= 1e-3 after 1000 steps with the aerodynamic
terms on (the only differences are the face corner angles' last bits), and
bit-identical states over 200 steps with drag and lift off.  The oracle trajectories run in
worker processes (spawned, CUDA-free) while the GPU steps.
"""
import concurrent.futures as cf
import multiprocessing as mp

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LONG_TOL = 1e-3
N = 128
DT = 1.0 / 6000.0
CHECKPOINTS = (100, 250, 500, 1000)
COUNT_EVERY = 5  # the oracle counts obstacle hits on every 5th step
LAUNCH = 1.0  # m/s along +z


def _scene(aero: bool):
    """The large configuration's cloth at 128 x 128, with its sphere moved in
    front of the cloth (centre 0.32 m along +z, 0.25 m below the cloth
    centre) so that the cloth, launched towards it, runs into it."""
    from feriphys_gb300 import workloads as W

    sc = W.c1(n=N, dt=DT)
    centre = sc.positions.astype(np.float64).mean(0)
    sc.obstacles = [W.plane(-1.5), W.uv_sphere((centre[0], centre[1] - 0.25, centre[2] + 0.32), 0.3, 32, 16)]
    if not aero:
        sc.config["drag_coefficient"] = 0.0
        sc.config["lift_coefficient"] = 0.0
    return sc


def _build(sc, api):
    """The scene through an API, every free vertex launched at 1 m/s along +z."""
    from feriphys_gb300 import workloads as W

    sim, mesh, obstacles = W.build(sc, api)
    p = mesh.get_points()
    free = np.ones(len(p), bool)
    free[sc.pins] = False
    p[free, 6] = np.float32(LAUNCH)
    mesh.set_points(p)
    return sim, mesh, obstacles


def oracle_trajectory(aero: bool, steps: int, checkpoints):
    """Runs in a worker process: the oracle's points at each checkpoint and
    the number of first hits on the plane (faces 0-1) and on the sphere
    (faces 2..) over the counted steps.  A counted step is the reference's
    Simulation::step through its own phases (accumulate_forces, the State
    integration, update_points, clear_forces) with the first-hit search run on
    the same segments in between."""
    import oracle

    sc = _scene(aero)
    sim, mesh, obstacles = _build(sc, oracle)
    c = sc.config
    cfg = oracle.Config.make(c["integration"], c["dt"], c["gravity"], c["wind"], c["lift_coefficient"],
                             c["drag_coefficient"], c["coefficient_of_restitution"], c["coefficient_of_friction"])
    out, hits = {}, {"plane": 0, "sphere": 0}
    for s in range(1, steps + 1):
        if s % COUNT_EVERY == 0:
            old = mesh.get_points()
            mesh.accumulate_forces(cfg)
            new = mesh.integrate(c["integration"], c["dt"])
            f = oracle.collided_faces(obstacles, old[:, 1:4], new[:, 1:4], c["dt"])
            pinned = np.zeros(len(old), bool)
            pinned[sc.pins] = True
            f = f[~pinned]  # update_points restores pinned points whatever they hit
            hits["plane"] += int(((f >= 0) & (f < 2)).sum())
            hits["sphere"] += int((f >= 2).sum())
            mesh.update_points(new, obstacles, cfg)
            mesh.clear_forces()
        else:
            sim.step(1)
        if s in checkpoints:
            out[s] = mesh.get_points()
    return out, hits


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


@pytest.fixture(scope="module")
def fgb():
    import feriphys_gb300

    feriphys_gb300._lib()
    return feriphys_gb300


@pytest.fixture(scope="module")
def oracle_runs(orc):
    """Both oracle trajectories, started together in two spawned workers."""
    ctx = mp.get_context("spawn")
    with cf.ProcessPoolExecutor(max_workers=2, mp_context=ctx) as ex:
        aero = ex.submit(oracle_trajectory, True, CHECKPOINTS[-1], CHECKPOINTS)
        plain = ex.submit(oracle_trajectory, False, 200, (200,))
        yield {"aero": aero, "plain": plain}


def test_c1_style_1000_steps_with_sphere(fgb, oracle_runs):
    sim, mesh, _ = _build(_scene(True), fgb)
    assert mesh.get_path() == 2  # the tiled grid kernel
    gpu, done = {}, 0
    for c in CHECKPOINTS:
        sim.step(c - done)
        done = c
        gpu[c] = mesh.get_points()
    assert not sim.synchronize()
    ref, hits = oracle_runs["aero"].result()
    assert hits["sphere"] > 0, hits  # the sphere's faces were crossed
    for c in CHECKPOINTS:
        assert np.isfinite(ref[c]).all()
        e = _rel(gpu[c][:, 1:4], ref[c][:, 1:4])
        print("step %d: relative position error %.3g (obstacle hits on counted steps: %s)" % (c, e, hits))
        assert e <= LONG_TOL, (c, e)


def test_c1_style_aero_off_bit_exact_200_steps(fgb, oracle_runs):
    sim, mesh, _ = _build(_scene(False), fgb)
    sim.step(200)
    ref, hits = oracle_runs["plain"].result()
    assert hits["sphere"] > 0, hits
    assert mesh.get_points().tobytes() == ref[200].tobytes()
