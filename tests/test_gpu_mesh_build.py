"""SpringyMesh::new built on the GPU (fgb_mesh_new_device) is the host build
bit for bit: strut order, ends, constants and rest lengths, the grid
detection, the errors, and the first steps of the simulation."""
import time

import numpy as np
import pytest

import feriphys_gb300 as fgb
from feriphys_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def build_pair(pos, idx, mass, k, c, ov=None):
    t0 = time.perf_counter()
    a = fgb.SpringyMesh.new(pos, idx, mass, k, c, ov)
    t1 = time.perf_counter()
    b = fgb.SpringyMesh.new(pos, idx, mass, k, c, ov, build_on_device=True)
    t2 = time.perf_counter()
    return a, b, t1 - t0, t2 - t1


def same_mesh(a, b):
    ka, aa = a.get_struts()
    kb, ab = b.get_struts()
    assert np.array_equal(aa, ab)
    assert np.array_equal(ka.view(np.uint32), kb.view(np.uint32))
    pa, ia = a.get_vertices()
    pb, ib = b.get_vertices()
    assert np.array_equal(ia, ib) and np.array_equal(pa, pb)
    assert a.counts() == b.counts()


def test_large_cloth_with_overrides():
    n = 1024
    pos = W.grid_positions(n, n, 1.0 / (n - 1)).astype(np.float64)
    pos += np.random.default_rng(0).normal(0, 1e-3, pos.shape)
    pos = pos.astype(np.float32)
    idx = W.cloth_indices(n, n)
    rng = np.random.default_rng(1)
    t = rng.integers(0, len(idx) // 3, 5000)
    pairs = np.stack([idx[3 * t], idx[3 * t + 1]], 1)
    pairs = np.concatenate([pairs, pairs[:100, ::-1], np.array([[0, 5 * n]])])  # duplicates (last wins), a non-edge
    kc = rng.uniform(1, 3, (len(pairs), 2)).astype(np.float32)
    a, b, th, td = build_pair(pos, idx, 0.01 * n * n, 1.0, 0.5, (pairs, kc))
    print("1024^2 mesh: host build %.3f s, device build %.3f s" % (th, td))
    same_mesh(a, b)
    assert a.get_path() == b.get_path()


def test_cloth_detected_as_grid_and_steps_identically():
    sc = W.c1(n=96, seed=3)
    meshes = []
    for dev in (False, True):
        m = fgb.SpringyMesh.new(sc.positions, sc.indices, sc.mass, 1.0, 1.0, build_on_device=dev)
        m.add_pins(sc.pins)
        m.add_struts(sc.extra_struts, 1.0, 1.0)
        _, ab = m.get_struts()
        k, c = sc.strut_params(ab)
        m.set_strut_params(k, c)
        meshes.append(m)
    same_mesh(*meshes)
    pts = []
    for m in meshes:
        sim = fgb.Simulation.new([m], [fgb.CollidableMesh.new(p, i) for p, i in sc.obstacles])
        sim.set_config(fgb.Config.make(**sc.config))
        sim.step(5)
        assert m.get_path() == 2
        pts.append(m.get_points())
    assert np.array_equal(pts[0], pts[1])


def test_irregular_mesh():
    rng = np.random.default_rng(4)
    rows, cols = 40, 37
    pos = rng.normal(size=(rows * cols, 3)).astype(np.float32)
    tri = []
    for r in range(rows - 1):
        for c in range(cols - 1):
            i = r * cols + c
            if rng.random() < 0.5:
                tri += [i, i + 1, i + cols, i + 1, i + cols + 1, i + cols]
            else:
                tri += [i, i + 1, i + cols + 1, i, i + cols + 1, i + cols]
    tri = np.array(tri, np.uint32).reshape(-1, 3)
    tri = tri[rng.permutation(len(tri))]
    perm = rng.permutation(rows * cols).astype(np.uint32)
    idx = perm[tri].reshape(-1)
    a, b, _, _ = build_pair(pos, np.concatenate([idx, [0, 1]]), 3.0, 2.0, 0.1)  # trailing partial triangle dropped
    same_mesh(a, b)


@pytest.mark.parametrize("case", ["nonmanifold", "index"])
def test_errors_match(case):
    pos = np.zeros((6, 3), np.float32)
    if case == "nonmanifold":
        idx = np.array([0, 1, 2, 1, 0, 3, 0, 1, 4, 2, 3, 5], np.uint32)
        code = -3
    else:
        idx = np.array([0, 1, 2, 1, 9, 3], np.uint32)
        code = -2
    msgs = []
    for dev in (False, True):
        with pytest.raises(fgb.FgbError) as e:
            fgb.SpringyMesh.new(pos, idx, 1.0, 1.0, 1.0, build_on_device=dev)
        assert e.value.code == code
        msgs.append(str(e.value))
    assert msgs[0] == msgs[1]
