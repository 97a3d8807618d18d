"""The collision broad phase reproduces the reference's full first-hit
search (collidable_mesh.rs:107-169) bit for bit.

Free points (no struts, no faces, no forces) move in a straight line during
one step, so each point is one query segment.  Segments are aimed at
obstacle vertices, edges and interiors from both sides with tiny to large
offsets, plus long segments that must take the fallback path.  Results with
the broad phase on and off must be identical, and equal to the oracle's.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fgb():
    import feriphys_gb300

    feriphys_gb300._lib()
    return feriphys_gb300


def _segments(rng, faces, n):
    """faces: [F, 3, 3].  Returns (old positions, velocities) aimed at faces."""
    F = len(faces)
    f = rng.integers(0, F, n)
    tri = faces[f].astype(np.float64)
    kind = rng.integers(0, 4, n)
    bary = rng.dirichlet([1.0, 1.0, 1.0], n)
    # vertices, edge points (one barycentric coordinate exactly 0), interiors
    v = rng.integers(0, 3, n)
    bary[kind == 0] = np.eye(3)[v[kind == 0]]
    e = kind == 1
    bary[e, v[e]] = 0.0
    bary[e] /= bary[e].sum(1, keepdims=True)
    target = np.einsum("nk,nkd->nd", bary, tri)
    nrm = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    side = rng.choice([-1.0, 1.0], n)
    off = 10.0 ** rng.uniform(-7, -2, n)
    direction = nrm * -side[:, None] + rng.normal(0, 0.3, (n, 3))
    step = 10.0 ** rng.uniform(-6, -2.5, n)
    step[kind == 3] = 10.0 ** rng.uniform(-1, 0.5, (kind == 3).sum())  # long: fallback path
    old = target + nrm * side[:, None] * off[:, None] - direction * 0.5 * step[:, None]
    new = old + direction * step[:, None]
    return old, new


def _points(old, new, dt):
    n = len(old)
    pts = np.zeros((n, 10), np.float32)
    pts[:, 0] = 0.01
    pts[:, 1:4] = old.astype(np.float32)
    pts[:, 4:7] = ((new - old) / dt).astype(np.float32)
    return pts


def _run(api, pts, obstacles, dt, broadphase=None):
    n = len(pts)
    cfg = dict(integration=0, dt=dt, gravity=(0, 0, 0), wind=(0, 0, 0), lift_coefficient=0.0,
               drag_coefficient=0.0, coefficient_of_restitution=0.3, coefficient_of_friction=0.2)
    if api.__name__ == "oracle":
        m = api.SpringyMesh.new(pts[:, 1:4], [], 0.01 * n, 1.0, 1.0)
        m.set_points(pts)
        obs = [api.CollidableMesh(p, i) for p, i in obstacles]
        sim = api.Simulation([m], obs)
        sim.set_config(api.Config.make(0, dt, (0, 0, 0), (0, 0, 0), 0.0, 0.0, 0.3, 0.2))
    else:
        m = api.SpringyMesh.new(pts[:, 1:4], [], 0.01 * n, 1.0, 1.0)
        m.set_points(pts)
        obs = [api.CollidableMesh.new(p, i) for p, i in obstacles]
        sim = api.Simulation.new([m], obs)
        sim.set_config(api.Config.make(**cfg))
        sim.set_collision_broadphase(broadphase)
    sim.step(1)
    return m.get_points()


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_broadphase_equals_full_search(fgb, orc, seed):
    from feriphys_gb300 import workloads as W

    rng = np.random.default_rng(seed)
    obstacles = [W.plane(-1.5), W.uv_sphere((0.013, -0.52, 0.007), 0.3, 32, 16),
                 W.uv_sphere((0.4, -0.9, -0.2), 0.11, 12, 6)]
    faces = np.concatenate([p[i.reshape(-1, 3)] for p, i in obstacles])
    old, new = _segments(rng, faces, 200_000)
    dt = float(np.float32(1.0 / 600.0))
    pts = _points(old, new, dt)
    a = _run(fgb, pts, obstacles, dt, broadphase=True)
    b = _run(fgb, pts, obstacles, dt, broadphase=False)
    hit = (b[:, 4:7] != pts[:, 4:7]).any(1)
    assert hit.sum() > 1000  # many collisions exercised
    assert a.tobytes() == b.tobytes()
    o = _run(orc, pts[:20000], obstacles, dt)
    assert a[:20000].tobytes() == o.tobytes()
