"""The allocation-free step, fgb_sim_step_static, called through the C ABI.

It serves hosts that cannot let a library allocate device memory once they
run (engines and renderers owning all GPU memory through their own
allocators, real-time loops that cannot afford cudaMalloc/cudaFree).  Its
results must equal the regular batched step's, fgb_sim_step, on the same
cloths bit for bit, for two calls in a row (the second call finds the fixed
scratch array holding the first call's contents), the second call must leave
the device's free memory unchanged, and regular calls may follow it.  This file is collected last so a
run stopping at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fgb():
    import feriphys_gb300

    feriphys_gb300._lib()
    return feriphys_gb300


def _same_bits(a, b):
    """Bit-for-bit equality of two float32 point arrays (NaN-safe)."""
    return np.array_equal(np.ascontiguousarray(a, np.float32).view(np.uint32),
                          np.ascontiguousarray(b, np.float32).view(np.uint32))


def _free_device_bytes():
    import torch

    return torch.cuda.mem_get_info()[0]  # cudaMemGetInfo on the current device


def test_static_step_matches_regular_step(fgb):
    """Both entry points run the batched kernel over 32 x 8 tiles, so the
    results agree bit for bit; the second static call allocates no device
    memory (the free bytes cudaMemGetInfo reports do not change)."""
    from feriphys_gb300 import workloads as W

    batch = W.c2(n_cloths=12, lo=2, hi=70, seed=11)
    sim_a, meshes_a, _ = W.build_batch(batch, fgb)   # regular entry point
    sim_b, meshes_b, _ = W.build_batch(batch, fgb)   # allocation-free entry point
    sim_a.set_batch_tile(8)  # the allocation-free step's tile height
    sim_a.step(0)
    sim_b.step(0)  # set-up: uploads state, topology and obstacles
    lib = fgb._lib()
    _free_device_bytes()  # the first query may set up the runtime's own context state
    for call in range(2):
        sim_a.step(3)
        free_before = _free_device_bytes()
        rc = lib.fgb_sim_step_static(sim_b._h, C.c_uint64(3), None)
        free_after = _free_device_bytes()
        assert rc == 0, lib.fgb_last_error().decode()
        if call == 1:  # the first call may load the library's device code; the second allocates nothing
            assert free_after == free_before, (free_before, free_after)
        for ma, mb in zip(meshes_a, meshes_b):
            pa, pb = ma.get_points(), mb.get_points()
            assert np.isfinite(pb).all()
            assert _same_bits(pb, pa), call


def test_regular_step_after_static_step(fgb):
    """Regular and allocation-free calls mixed on one simulation (an odd number
    of static steps swaps its meshes' buffers against the regular batch's
    parity) give the same bits as a simulation stepped only regularly."""
    from feriphys_gb300 import workloads as W

    batch = W.c2(n_cloths=9, lo=3, hi=60, seed=5)
    sim_a, meshes_a, _ = W.build_batch(batch, fgb)   # regular steps only
    sim_b, meshes_b, _ = W.build_batch(batch, fgb)   # regular, static, regular
    for s in (sim_a, sim_b):
        s.set_batch_tile(8)
        s.step(0)
        s.step(2)
    lib = fgb._lib()
    sim_a.step(3)
    assert lib.fgb_sim_step_static(sim_b._h, C.c_uint64(3), None) == 0, lib.fgb_last_error().decode()
    sim_a.step(4)
    sim_b.step(4)
    sim_a.step(1)
    sim_b.step(1)
    for ma, mb in zip(meshes_a, meshes_b):
        assert _same_bits(mb.get_points(), ma.get_points())


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
