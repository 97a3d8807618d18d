"""The render oracle's vectorised normal sum equals a literal face loop
(graphics/util.rs:178-199) bit for bit."""
import numpy as np

from oracle import render_oracle as RO


def test_vectorised_normals_equal_the_face_loop():
    rng = np.random.default_rng(0)
    rows, cols = 6, 5
    pos = rng.normal(size=(rows * cols, 3)).astype(np.float32)
    tri = []
    for r in range(rows - 1):
        for c in range(cols - 1):
            i = r * cols + c
            tri += [i + 1, i + cols, i]
    for r in range(1, rows):
        for c in range(cols - 1):
            i = r * cols + c
            tri += [i - cols + 1, i + 1, i]
    acc = np.zeros((rows * cols, 3), np.float32)
    for a, b, c in np.asarray(tri).reshape(-1, 3):
        e1 = pos[a] - pos[b]
        e2 = pos[a] - pos[c]
        fn = np.array([e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]],
                      np.float32)
        acc[a] = acc[a] + fn
        acc[b] = acc[b] + fn
        acc[c] = acc[c] + fn
    ref = np.stack([v * (np.float32(1) / np.sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2])) for v in acc])
    got = RO.normals(pos, tri)
    assert np.array_equal(got.view(np.uint32), ref.astype(np.float32).view(np.uint32))
    cv = RO.colored_vertices(pos, tri, (0.1, 0.2, 0.3))
    assert cv.shape == (rows * cols, 9) and np.array_equal(cv[:, :3], pos)
