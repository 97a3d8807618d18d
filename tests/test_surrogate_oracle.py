"""The surrogate's CPU oracle pinned on its own (no GPU): bf16 rounding
against torch's conversion, the backward pass against central finite
differences in float64, known feature values of an undeformed cloth, and the
closed form of a first Adam step."""
import numpy as np
import pytest

from oracle import surrogate_oracle as SO


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    x = np.concatenate([
        rng.standard_normal(20000).astype(np.float32) * np.float32(10.0) ** rng.integers(-8, 8, 20000).astype(np.float32),
        np.array([0.0, -0.0, 1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 65504.0, 3.4e38, -1e-40, np.inf, -np.inf],
                 np.float32),
    ])
    ref = torch.from_numpy(x).to(torch.bfloat16).float().numpy()
    got = SO.bf16(x)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    # ties go to even
    assert SO.bf16(np.float32(1.0 + 2 ** -8)) == np.float32(1.0)
    assert SO.bf16(np.float32(1.0 + 3 * 2 ** -8)) == np.float32(1.0 + 2 ** -6)


def _small_problem(seed, n=8):
    rng = np.random.default_rng(seed)
    p = rng.standard_normal(SO.N_HID * SO.N_FEAT + SO.N_HID + SO.N_HID ** 2 + SO.N_HID + 3 * SO.N_HID + 3) * 0.1
    x = rng.standard_normal((n, SO.N_FEAT))
    t = rng.standard_normal((n, 3))
    return p, x, t


def test_backward_matches_finite_differences():
    p, x, t = _small_problem(1)
    g, loss = SO.gradients(p, x, t, rounding=False, dtype=np.float64)
    y = SO.forward(p, x, rounding=False, dtype=np.float64)
    assert loss == pytest.approx(np.mean((y - t) ** 2), rel=1e-12)
    rng = np.random.default_rng(2)
    idx = np.concatenate([rng.choice(p.size, 300, replace=False), np.arange(p.size - 3, p.size)])
    eps = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        fp = np.mean((SO.forward(pp, x, rounding=False, dtype=np.float64) - t) ** 2)
        fm = np.mean((SO.forward(pm, x, rounding=False, dtype=np.float64) - t) ** 2)
        fd = (fp - fm) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_rounded_gradient_close_to_exact():
    p, x, t = _small_problem(3, n=256)
    g32, _ = SO.gradients(p.astype(np.float32), x.astype(np.float32), t.astype(np.float32))
    g64, _ = SO.gradients(p, x, t, rounding=False, dtype=np.float64)
    rel = np.linalg.norm(g32 - g64) / np.linalg.norm(g64)
    assert rel < 2e-2, rel


def test_features_of_undeformed_cloth():
    rows, cols, h, T = 4, 5, 0.1, 0.01
    pos = np.zeros((rows * cols, 4), np.float32)
    for r in range(rows):
        for c in range(cols):
            pos[r * cols + c] = (c * h, r * h, 0.0, 0.01)
    rest = pos[:, :3].copy()
    vel = np.zeros((rows * cols, 4), np.float32)
    vel[0, 3] = 1.0
    wind = (2.0, 0.0, 1.0)
    f = SO.features(pos, vel, rows, cols, h, T, wind, rest)
    interior = f[1 * cols + 2]
    assert np.all(f[:, :48] == 0)  # at rest: no deformation, no relative velocity
    s = np.float32(T) / np.float32(h)
    assert np.allclose(interior[49:52], np.array(wind, np.float32) * s)
    assert interior[52] == pytest.approx(0.5, abs=1e-6) and interior[53] == pytest.approx(0.5, abs=1e-6)
    assert f[0, 48] == 1.0 and f[0, 52] == pytest.approx(0.5, abs=1e-6)
    # stretch the right neighbour of the interior vertex by 0.02 in x
    moved = pos.copy()
    moved[1 * cols + 3, 0] += np.float32(0.02)
    g = SO.features(moved, vel, rows, cols, h, T, wind, rest)[1 * cols + 2]
    k = SO.NEIGHBOURS.index((0, 1))
    assert g[3 * k] == pytest.approx(0.2, rel=1e-5) and np.all(np.delete(g[:24], 3 * k) == 0)


def test_first_adam_step_closed_form():
    rng = np.random.default_rng(4)
    p = rng.standard_normal(100).astype(np.float32)
    g = rng.standard_normal(100).astype(np.float32)
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    p1, m1, v1 = SO.adam(p, g, m, v, 1, 1e-3)
    assert np.allclose(m1, 0.1 * g, rtol=1e-6)
    assert np.allclose(v1, 0.001 * g * g, rtol=1e-4)  # 1 - 0.999 in f32 is 0.0010000467
    assert np.allclose(p1, p - 1e-3 * np.sign(g), atol=1e-6)
