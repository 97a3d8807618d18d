"""CPU-side checks of the C ABI (no GPU needed).

The shared library must load and export every function include/*.h
declares; host-side mesh construction (SpringyMesh::new de-dup order,
Strut::new scaling, Cloth::new layout, overrides, add_strut) must be
bit-identical to the oracle's; errors map to the documented status codes.
"""
import ctypes as C
import glob
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def fgb():
    import feriphys_gb300

    feriphys_gb300._lib()
    return feriphys_gb300


def _declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\*?(fgb_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(fgb):
    lib = C.CDLL(fgb.library_path())
    declared = _declared_functions()
    assert len(declared) >= 30
    missing = [n for n in declared if not hasattr(lib, n)]
    assert not missing, missing


def _rand_mesh(rng, n_side=6, jitter=0.02):
    xs, ys = np.meshgrid(np.arange(n_side), np.arange(n_side))
    pos = np.stack([xs.ravel() * 0.1, ys.ravel() * 0.1, np.zeros(n_side * n_side)], 1)
    pos += rng.normal(0, jitter, pos.shape)
    idx = []
    for r in range(n_side - 1):
        for c in range(n_side - 1):
            i = r * n_side + c
            if rng.random() < 0.5:
                idx += [i, i + 1, i + n_side, i + 1, i + n_side + 1, i + n_side]
            else:
                idx += [i, i + 1, i + n_side + 1, i, i + n_side + 1, i + n_side]
    return pos.astype(np.float32), np.array(idx, np.uint32)


def test_springy_construction_matches_oracle(fgb, orc):
    rng = np.random.default_rng(1)
    pos, idx = _rand_mesh(rng)
    pairs = np.array([[idx[0], idx[1]], [idx[4], idx[3]], [7, 13]], np.uint32)
    kc = np.array([[11.0, 0.25], [13.0, 0.5], [17.0, 0.75]], np.float32)
    g = fgb.SpringyMesh.new(pos, idx, 0.37, 500.0, 0.5, (pairs, kc))
    o = orc.SpringyMesh.new(pos, idx, 0.37, 500.0, 0.5, (pairs, kc))
    g.add_strut((0, 14), 50.0, 0.125)
    o.add_strut(0, 14, 50.0, 0.125)
    assert g.counts()[:3] == o.counts()[:3]
    gk, gab = g.get_struts()
    ok, oab, _ = o.get_struts()
    assert (gab.astype(np.uint64) == oab).all()
    assert gk.tobytes() == ok.tobytes()  # bit-identical k, c, L
    _, gidx = g.get_vertices()
    assert (gidx.astype(np.uint64) == o.get_faces()[1].reshape(-1)).all()
    assert g.get_points().tobytes() == o.get_points().tobytes()


@pytest.mark.parametrize("rows,cols", [(2, 2), (2, 5), (3, 3), (5, 4), (32, 32)])
def test_cloth_construction_matches_oracle(fgb, orc, rows, cols):
    pins = [rows * cols - cols, rows * cols - 1]
    args = (rows, cols, 1 / 31, (0.1, -0.2, 0.3), 0.01, 16.1, 0.016, 11.4, 0.023, 3.2, 0.032)
    g = fgb.Cloth.new(*args, pins).mesh
    o = orc.SpringyMesh.cloth(*args, pins)
    assert g.counts() == o.counts()
    gk, gab = g.get_struts()
    ok, oab, _ = o.get_struts()
    assert (gab.astype(np.uint64) == oab).all()
    assert gk.tobytes() == ok.tobytes()
    assert g.get_points().tobytes() == o.get_points().tobytes()
    assert g.get_path() == 2  # recognised as a Cloth::new grid


def test_grid_detection_on_plain_springy_mesh(fgb, orc):
    # The same triangles passed through SpringyMesh::new are still a grid
    # once the binding struts are added in Cloth::new's order.
    o = orc.SpringyMesh.cloth(6, 7, 0.1, (0, 0, 0), 0.01, 1, 1, 1, 1, 1, 1, [])
    pts = o.get_points()[:, 1:4]
    idx = o.get_faces()[1].reshape(-1)
    g = fgb.SpringyMesh.new(pts, idx, 0.42, 1.0, 1.0)
    assert g.get_path() == 1  # binding struts still missing
    for r in range(4):
        for c in range(5):
            i = r * 7 + c
            g.add_strut((i, i + 2), 1.0, 1.0)
            g.add_strut((i, i + 14), 1.0, 1.0)
    assert g.get_path() == 2
    g.add_strut((0, 41), 1.0, 1.0)  # an extra strut: general gather
    assert g.get_path() == 1
    with pytest.raises(fgb.FgbError):
        g.set_path(2)
        g.get_path()


def test_error_codes(fgb):
    with pytest.raises(fgb.FgbError) as e:
        fgb.SpringyMesh.new([[0, 0, 0], [1, 0, 0], [0, 1, 0]], [0, 1, 5], 1.0, 1.0, 1.0)
    assert e.value.code == -2
    # a fan of three triangles on one edge: more than two faces per strut
    pos = [[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1]]
    with pytest.raises(fgb.FgbError) as e:
        fgb.SpringyMesh.new(pos, [0, 1, 2, 0, 1, 3, 0, 1, 4], 1.0, 1.0, 1.0)
    assert e.value.code == -3
    with pytest.raises(fgb.FgbError) as e:
        fgb.Cloth.new(1, 4, 0.1, (0, 0, 0), 0.01, 1, 1, 1, 1, 1, 1)
    assert e.value.code == -1
    # more than 2^31 - 1 vertices, including a product that wraps to 0 in 64 bits
    for rows, cols in ((1 << 16, 1 << 16), (1 << 32, 1 << 32), (2, 1 << 40)):
        with pytest.raises(fgb.FgbError) as e:
            fgb.Cloth.new(rows, cols, 0.1, (0, 0, 0), 0.01, 1, 1, 1, 1, 1, 1)
        assert e.value.code == -1
    m = fgb.SpringyMesh.new([[0, 0, 0], [1, 0, 0], [0, 1, 0]], [0, 1, 2], 1.0, 1.0, 1.0)
    with pytest.raises(fgb.FgbError) as e:
        m.add_pin(3)
    assert e.value.code == -2
    with pytest.raises(fgb.FgbError) as e:
        m.add_strut((0, 9), 1.0, 1.0)
    assert e.value.code == -2
    with pytest.raises(fgb.FgbError) as e:
        fgb.CollidableMesh.new([[0, 0, 0], [1, 0, 0]], [0, 0, 1])
    assert e.value.code == -1
    with pytest.raises(fgb.FgbError) as e:  # one mesh twice in one simulation
        fgb.Simulation.new([m, m], [])
    assert e.value.code == -1
    sim = fgb.Simulation.new([m], [])
    for bad in (-1.0, float("nan"), float("inf")):
        with pytest.raises(fgb.FgbError) as e:
            sim.set_config(fgb.Config.make(dt=bad))
        assert e.value.code == -1


def test_config_default_and_timestep(fgb, orc):
    c = fgb.Config.default()
    o = orc.Config.default()
    assert bytes(c) == bytes(o)
    m = fgb.SpringyMesh.new([[0, 0, 0], [1, 0, 0], [0, 1, 0]], [0, 1, 2], 1.0, 1.0, 1.0)
    sim = fgb.Simulation.new([m], [])
    assert sim.get_timestep() == 0.001
    sim.set_config(fgb.Config.make(dt=np.float32(1 / 600)))
    assert sim.get_timestep() == 0.001666667  # whole nanoseconds, like Duration


def test_collidable_counts_match_oracle(fgb, orc):
    pos = [[0, 0, 0], [1, 0, 0], [-1, 1, 0], [0, 1, 0]]
    idx = [0, 3, 2, 0, 1, 3]
    assert fgb.CollidableMesh.new(pos, idx).counts() == orc.CollidableMesh(pos, idx).counts()


def test_output_buffers_are_checked_before_the_library_writes(fgb):
    m = fgb.SpringyMesh.new([[0, 0, 0], [1, 0, 0], [0, 1, 0]], [0, 1, 2], 1.0, 1.0, 1.0)
    wrong = (np.empty((2, 10), np.float32), np.empty((3, 10), np.float64), np.empty((10, 3), np.float32).T,
             np.empty((3, 10), np.float32)[:, ::-1], [[0.0] * 10] * 3)
    for out in wrong:
        with pytest.raises(ValueError):
            m.get_points(out=out)
    ro = np.empty((3, 10), np.float32)
    ro.flags.writeable = False
    with pytest.raises(ValueError):
        m.get_points(out=ro)
    for out in (np.empty((4, 3), np.float32), np.empty((3, 3), np.int32)):
        with pytest.raises(ValueError):
            m.get_positions(out=out)


def test_points_round_trip_host(fgb):
    m = fgb.SpringyMesh.new([[0, 0, 0], [1, 0, 0], [0, 1, 0]], [0, 1, 2], 3.0, 1.0, 1.0)
    p = m.get_points()
    assert p[:, 0].tolist() == [1.0, 1.0, 1.0]
    p[:, 4:10] = np.arange(18, dtype=np.float32).reshape(3, 6)
    m.set_points(p)
    assert (m.get_points() == p).all()


def test_extension_entry_points_reject_bad_arguments(fgb):
    """The surrogate, export and static-step entry points validate their
    arguments on the host before touching a device."""
    lib = fgb._lib()
    null = None
    f = (C.c_float * 64)()
    u = (C.c_uint64 * 2)()
    assert lib.fgb_surrogate_new(0, null) == -1
    assert lib.fgb_surrogate_get_params(null, f) == -1
    assert lib.fgb_surrogate_set_params(null, f) == -1
    assert lib.fgb_surrogate_set_normalization(null, f, f, f, f) == -1
    assert lib.fgb_surrogate_get_normalization(null, f, f, f, f) == -1
    assert lib.fgb_surrogate_forward(null, f, 1, f) == -1
    assert lib.fgb_surrogate_gradients(null, f, f, 128, f, null) == -1
    assert lib.fgb_surrogate_train_batch(null, f, f, 128, C.c_float(1e-3), null) == -1
    assert lib.fgb_surrogate_dataset_reserve(null, 10) == -1
    assert lib.fgb_surrogate_collect(null, null, 10, 1) == -1
    assert lib.fgb_surrogate_dataset_info(null, u) == -1
    assert lib.fgb_surrogate_fit_normalization(null) == -1
    assert lib.fgb_surrogate_train(null, 1, 128, C.c_float(1e-3), 0, null) == -1
    assert lib.fgb_sim_step_surrogate(null, null, 10, 1, null, null) == -1
    assert lib.fgb_sim_energy(null, f) == -1
    assert lib.fgb_mesh_export_vertices(null, f, null, null) == -1
    assert lib.fgb_mesh_export_indices(null, f, null) == -1
    assert lib.fgb_surrogate_destroy(null) == 0
    assert "null" in lib.fgb_last_error().decode()
    assert lib.fgb_sim_set_batch_tile(null, 8) == -1
    sim = fgb.Simulation.new([], [])
    for bad in (-1, 1, 5, 16):
        assert lib.fgb_sim_set_batch_tile(sim._h, bad) == -1
        assert "tile_rows" in lib.fgb_last_error().decode()
    for ok in (0, 4, 8, 12):
        assert lib.fgb_sim_set_batch_tile(sim._h, ok) == 0


def test_device_build_rejects_bad_input_before_the_gpu(fgb):
    pos = np.zeros((4, 3), np.float32)
    with pytest.raises(fgb.FgbError) as e:
        fgb.SpringyMesh.new(pos, np.array([0, 1, 7], np.uint32), 1.0, 1.0, 1.0, build_on_device=True)
    assert e.value.code == -2 and "out of range" in str(e.value)
