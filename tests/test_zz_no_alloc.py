"""The allocation-free step, fgb_sim_step_static, called through the C ABI.

It serves hosts that cannot let a library allocate device memory once they
run (engines and renderers owning all GPU memory through their own
allocators, real-time loops that cannot afford cudaMalloc/cudaFree).  Its
results must match the regular batched step, fgb_sim_step, on the same
cloths, for two calls in a row (the second call finds the fixed scratch
array holding the first call's contents).  This file is collected last so a
run stopping at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5  # the per-step bar of the parity tests


@pytest.fixture(scope="module")
def fgb():
    import feriphys_gb300

    feriphys_gb300._lib()
    return feriphys_gb300


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def test_static_step_matches_regular_step(fgb):
    from feriphys_gb300 import workloads as W

    batch = W.c2(n_cloths=12, lo=2, hi=70, seed=11)
    sim_a, meshes_a, _ = W.build_batch(batch, fgb)   # regular entry point
    sim_b, meshes_b, _ = W.build_batch(batch, fgb)   # allocation-free entry point
    sim_a.step(0)
    sim_b.step(0)  # set-up: uploads state, topology and obstacles
    lib = fgb._lib()
    for call in range(2):
        sim_a.step(3)
        rc = lib.fgb_sim_step_static(sim_b._h, C.c_uint64(3), None)
        assert rc == 0, lib.fgb_last_error().decode()
        for ma, mb in zip(meshes_a, meshes_b):
            pa, pb = ma.get_points(), mb.get_points()
            assert np.isfinite(pb).all()
            assert _rel(pb[:, 1:7], pa[:, 1:7]) <= TOL, call


def test_static_step_rejects_unprepared_and_oversized(fgb):
    from feriphys_gb300 import workloads as W

    lib = fgb._lib()
    batch = W.c2(n_cloths=2, lo=8, hi=8, seed=2)
    sim, _, _ = W.build_batch(batch, fgb)
    assert lib.fgb_sim_step_static(sim._h, C.c_uint64(1), None) == -5  # not prepared: uploads nothing
    # 50,000 tiny cloths need 50,000 x (80 + 16) bytes > the fixed 4 MiB: rejected before any device work
    args = W.c2(n_cloths=1, lo=2, hi=2, seed=3).cloths[0]
    meshes = [fgb.Cloth.new(*args[0], args[1]).mesh for _ in range(50000)]
    big = fgb.Simulation.new(meshes, [])
    rc = lib.fgb_sim_step_static(big._h, C.c_uint64(1), None)
    assert rc == -1 and b"scratch" in lib.fgb_last_error()
