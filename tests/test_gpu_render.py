"""Headless render export: fgb_mesh_export_vertices / _export_indices write
the reference's ColoredVertex buffer and a u32 index buffer into device
memory; checked bit for bit against oracle/render_oracle.py, including a
cloth beyond the reference's 65,535-vertex u16 index cap."""
import numpy as np
import pytest

import feriphys_gb300 as fgb
from feriphys_gb300 import workloads as W
from oracle import render_oracle as RO

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def export(mesh, color):
    n, _, f, _ = mesh.counts()
    buf = torch.zeros(n * 9, dtype=torch.float32, device="cuda")
    idx = torch.zeros(f * 3, dtype=torch.int32, device="cuda")
    mesh.export_vertices(buf.data_ptr(), color)
    mesh.export_indices(idx.data_ptr())
    torch.cuda.synchronize()
    return buf.cpu().numpy().reshape(n, 9), idx.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("rows,cols", [(40, 30), (300, 250)])
def test_export_matches_oracle(rows, cols):
    sc = W.c0(n=rows, dt=1.0 / 6000.0)
    args = (rows, cols) + sc.cloth_args[2:]
    mesh = fgb.Cloth.new(*args, np.array([rows * cols - 1], np.uint32)).mesh
    sim = fgb.Simulation.new([mesh], [])
    sim.set_config(fgb.Config.make(**sc.config))
    sim.step(25)
    color = (0.2, 0.5, 0.9)
    got, idx = export(mesh, color)
    pos, ref_idx = mesh.get_vertices()
    assert np.array_equal(idx, ref_idx.reshape(-1))
    assert idx.max() == rows * cols - 1
    ref = RO.colored_vertices(pos, ref_idx, color)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_export_general_mesh():
    rng = np.random.default_rng(1)
    sc = W.c1(n=24, seed=2)
    sim, mesh, _ = W.build(sc, fgb)
    mesh.set_path(1)
    sim.step(5)
    got, idx = export(mesh, None)
    pos, ref_idx = mesh.get_vertices()
    ref = RO.colored_vertices(pos, ref_idx, (1.0, 1.0, 1.0))
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
