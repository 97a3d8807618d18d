"""The C++ mirror of the reference's API (include/feriphys_gb300.hpp) compiles
against the C ABI and behaves like the reference's types on the host:
tests/cpp/host_api.cpp, built with g++ and run (no GPU needed)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_mirror_builds_and_runs(tmp_path):
    import feriphys_gb300

    lib = feriphys_gb300.library_path()
    feriphys_gb300._lib()
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "host_api")
    libdir = os.path.dirname(lib)
    cmd = [gxx, "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "host_api.cpp"), "-o", exe, "-L", libdir, "-lferiphys_gb300",
           "-Wl,-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr


def test_sim_rejects_meshes_of_different_devices(tmp_path):
    """fgb_sim_new refuses meshes created on different devices (white-box:
    tests/cpp/sim_devices.cpp marks a mesh's device through the internal
    handle layout; no GPU, no launch)."""
    import feriphys_gb300

    lib = feriphys_gb300.library_path()
    feriphys_gb300._lib()
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    from feriphys_gb300 import build as fbuild

    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(fbuild._nvcc())), "include")
    exe = str(tmp_path / "sim_devices")
    libdir = os.path.dirname(lib)
    cmd = [gxx, "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(ROOT, "feriphys_gb300", "csrc"), "-I", cuda_inc,
           os.path.join(ROOT, "tests", "cpp", "sim_devices.cpp"), "-o", exe, "-L", libdir, "-lferiphys_gb300",
           "-Wl,-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr


def test_compact_incidence_lists_decode_to_the_csr(tmp_path):
    """The general gather's compact lists (mesh_build.h: CompactTopo) decode
    to the plain CSR lists on cloth grids and a random triangle soup, and a
    mesh beyond their limits is refused (tests/cpp/compact_topo.cpp calls the
    library's internal builders; no GPU)."""
    import feriphys_gb300

    lib = feriphys_gb300.library_path()
    feriphys_gb300._lib()
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "compact_topo")
    libdir = os.path.dirname(lib)
    cmd = [gxx, "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(ROOT, "feriphys_gb300", "csrc"), os.path.join(ROOT, "tests", "cpp", "compact_topo.cpp"),
           "-o", exe, "-L", libdir, "-lferiphys_gb300", "-Wl,-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr


def test_tile_lists_cover_every_tile_once(tmp_path):
    """The single-cloth kernel's blockIdx -> tile mapping and the batched
    kernel's work items list every tile of a cloth exactly once, ring tiles
    first, and run the unchecked interior form only where every neighbour
    within two vertices exists (tests/cpp/tile_cover.cpp, over every cloth
    shape up to 140 x 140 and larger ones, tile heights 4, 8 and 12; no GPU)."""
    import feriphys_gb300

    lib = feriphys_gb300.library_path()
    feriphys_gb300._lib()
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    from feriphys_gb300 import build as fbuild

    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(fbuild._nvcc())), "include")
    exe = str(tmp_path / "tile_cover")
    libdir = os.path.dirname(lib)
    cmd = [gxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(ROOT, "feriphys_gb300", "csrc"), "-I", cuda_inc,
           os.path.join(ROOT, "tests", "cpp", "tile_cover.cpp"), "-o", exe, "-L", libdir, "-lferiphys_gb300",
           "-Wl,-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
