"""CPU restatement of the reference's render-vertex build -- TEST
INFRASTRUCTURE ONLY (the oracle of fgb_mesh_export_vertices).

ColoredMesh::from_springy_mesh (graphics/model.rs:72-90) takes
SpringyMesh::get_vertices (springy_mesh.rs:500-513), computes per-vertex
normals with graphics/util.rs:178-199 -- every face (a, b, c) in order adds
(p_a - p_b) x (p_a - p_c) to the normals of a, b and c; each sum is then
normalised (cgmath: v * (1 / |v|)) -- and zips position, color and normal into
ColoredVertex (model.rs:20-24, 170-186): 9 f32 per vertex.
"""
from __future__ import annotations

import numpy as np


def _cross(a, b):
    return np.stack([a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1],
                     a[:, 2] * b[:, 0] - a[:, 0] * b[:, 2],
                     a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]], 1)


def normals(positions, indices):
    """get_normals in f32; every vertex's contributions are added in face order."""
    p = np.asarray(positions, np.float32).reshape(-1, 3)
    tri = np.asarray(indices, np.int64).reshape(-1, 3)
    fn = _cross(p[tri[:, 0]] - p[tri[:, 1]], p[tri[:, 0]] - p[tri[:, 2]]).astype(np.float32)
    acc = np.zeros_like(p)
    # face-major order of (vertex, contribution): np.add.at applies repeated
    # indices in array order, i.e. per vertex in ascending face order
    np.add.at(acc, tri.reshape(-1), np.repeat(fn, 3, axis=0))
    mag = np.sqrt((acc[:, 0] * acc[:, 0] + acc[:, 1] * acc[:, 1]) + acc[:, 2] * acc[:, 2])
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = np.float32(1.0) / mag
    return acc * inv[:, None]


def colored_vertices(positions, indices, color):
    """[n, 9]: position, color, normal."""
    p = np.asarray(positions, np.float32).reshape(-1, 3)
    out = np.zeros((len(p), 9), np.float32)
    out[:, 0:3] = p
    out[:, 3:6] = np.asarray(color, np.float32)
    out[:, 6:9] = normals(p, indices)
    return out
