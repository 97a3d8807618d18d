"""The learned surrogate's CUDA kernels against the CPU oracle
(oracle/surrogate_oracle.py): input features, the tensor-core forward pass,
the gradient of the training loss (the gradient check), one Adam step, data
collection, the coarse step, the energy/strain checks and the fine-step
fallback; and what a trained network gains over the method without it.

Tolerances: features are the same f32 operations as the oracle (1e-6
relative; the two angles 2e-6 absolute); network outputs and gradients differ
from the oracle only by f32 summation order inside the MMAs and the hardware
tanh approximation in GELU, which can move a bf16 rounding by one unit
(outputs within 1e-2 of their scale, gradients within 3e-2 relative L2 per
parameter block with cosine similarity >= 0.999).
"""
import numpy as np
import pytest

import feriphys_gb300 as fgb
from feriphys_gb300 import workloads as W
from oracle import surrogate_oracle as SO

pytestmark = pytest.mark.gpu

BLOCKS = [("W1", 128 * 54), ("b1", 128), ("W2", 128 * 128), ("b2", 128), ("W3", 3 * 128), ("b3", 3)]


def rand_params(seed, scale=1.0):
    rng = np.random.default_rng(seed)
    parts = [rng.normal(0, scale / np.sqrt(54), 128 * 54), rng.normal(0, 0.1, 128),
             rng.normal(0, scale / np.sqrt(128), 128 * 128), rng.normal(0, 0.1, 128),
             rng.normal(0, scale / np.sqrt(128), 3 * 128), rng.normal(0, 0.1, 3)]
    return np.concatenate(parts).astype(np.float32)


def blocks(v):
    out, o = {}, 0
    for name, n in BLOCKS:
        out[name] = v[o:o + n]
        o += n
    return out


def cloth_state(mesh, pins):
    pts = mesh.get_points()
    n = len(pts)
    pos = np.zeros((n, 4), np.float32)
    vel = np.zeros((n, 4), np.float32)
    pos[:, :3], pos[:, 3] = pts[:, 1:4], pts[:, 0]
    vel[:, :3] = pts[:, 4:7]
    vel[np.asarray(pins, np.int64), 3] = 1.0
    return pos, vel


def perturbed_cloth(rows, cols, s, seed, pins):
    args = (rows, cols, s, (0.0, 0.0, 0.0), 0.01, 500.0 * s, 0.5 * s, 250.0 * s * 2 ** 0.5, 0.5 * s * 2 ** 0.5,
            50.0 * 2 * s, 0.5 * 2 * s)
    mesh = fgb.Cloth.new(*args, np.asarray(pins, np.uint32)).mesh
    rng = np.random.default_rng(seed)
    pts = mesh.get_points()
    pts[:, 1:4] += rng.normal(0, 0.2 * s, (len(pts), 3)).astype(np.float32)
    pts[:, 4:7] = rng.normal(0, 0.3, (len(pts), 3)).astype(np.float32)
    pts[np.asarray(pins, np.int64), 4:7] = 0.0
    mesh.set_points(pts)
    return args, mesh


def test_features_match_oracle():
    rows, cols, s = 20, 13, 0.05
    pins = [rows * cols - 1, rows * cols - cols]
    _, mesh = perturbed_cloth(rows, cols, s, 1, pins)
    sur = fgb.Surrogate.new(0)
    T, wind = 0.01, (1.0, -0.5, 2.0)
    got = sur.features(mesh, T, wind)
    pos, vel = cloth_state(mesh, pins)
    h = SO.spacing(W.grid_positions(rows, cols, s), rows, cols)
    ref = SO.features(pos, vel, rows, cols, h, np.float32(T), wind, W.grid_positions(rows, cols, s))
    assert np.all(np.abs(got[:, :52] - ref[:, :52]) <= 1e-6 * np.maximum(1.0, np.abs(ref[:, :52])))
    assert np.abs(got[:, 52:] - ref[:, 52:]).max() <= 2e-6
    assert np.all(got[pins, 48] == 1.0) and got[:, 48].sum() == len(pins)


def test_forward_matches_oracle():
    p = rand_params(2)
    sur = fgb.Surrogate.new(0)
    sur.set_params(p)
    assert np.array_equal(sur.get_params(), p)
    x = np.random.default_rng(3).normal(size=(300, 54)).astype(np.float32)  # not a multiple of 128
    y = sur.forward(x)
    ref = SO.forward(p, x)
    scale = np.sqrt(np.mean(ref ** 2))
    err = np.abs(y - ref).max() / scale
    assert err <= 1e-2, err


def test_gradients_match_oracle():
    p = rand_params(4)
    sur = fgb.Surrogate.new(0)
    sur.set_params(p)
    rng = np.random.default_rng(5)
    n = 128 * 200  # more tiles than SMs: some CTAs accumulate two tiles in tensor memory
    x = rng.normal(size=(n, 54)).astype(np.float32)
    t = rng.normal(size=(n, 3)).astype(np.float32)
    g, loss = sur.gradients(x, t)
    gr, loss_r = SO.gradients(p, x, t)
    assert loss == pytest.approx(loss_r, rel=1e-3)
    G, R = blocks(g), blocks(gr)
    for name, _ in BLOCKS:
        a, b = G[name].astype(np.float64), R[name].astype(np.float64)
        rel = np.linalg.norm(a - b) / np.linalg.norm(b)
        cos = a @ b / (np.linalg.norm(a) * np.linalg.norm(b))
        assert rel <= 3e-2 and cos >= 0.999, (name, rel, cos)


def test_adam_step_matches_oracle():
    p = rand_params(6)
    sur = fgb.Surrogate.new(0)
    sur.set_params(p)
    rng = np.random.default_rng(7)
    n, lr = 128 * 16, 1e-3
    x = rng.normal(size=(n, 54)).astype(np.float32)
    t = rng.normal(size=(n, 3)).astype(np.float32)
    gr, _ = SO.gradients(p, x, t)
    sur.train_batch(x, t, lr)
    p1 = sur.get_params()
    ref, _, _ = SO.adam(p, gr, np.zeros_like(p), np.zeros_like(p), 1, lr)
    off = np.abs(p1 - ref) > 0.1 * lr
    assert off.mean() <= 0.01, off.mean()
    assert np.abs(p1 - p).max() <= 1.01 * lr * 1.0001


def test_training_reduces_loss():
    rng = np.random.default_rng(8)
    n = 8192
    x = rng.normal(size=(n, 54)).astype(np.float32)
    t = np.tanh(0.8 * x[:, :3] + 0.5 * x[:, 3:6] * x[:, 6:9]).astype(np.float32)
    sur = fgb.Surrogate.new(9)
    losses = [sur.train_batch(x, t, 1e-3) for _ in range(300)]
    assert np.isfinite(losses).all()
    assert losses[-1] < 0.3 * losses[0], (losses[0], losses[-1])


def small_scene(n=16, dt=1.0 / 6000.0, obstacles=True):
    sc = W.c0(n=n, dt=dt, obstacles=obstacles)
    sim, mesh, obs = W.build(sc, fgb)
    return sc, sim, mesh, obs


def test_collect_matches_oracle_and_normalization():
    sc, sim, mesh, _ = small_scene()
    n, ratio = sc.rows * sc.cols, 5
    dt = np.float32(sc.config["dt"])
    T = np.float32(ratio) * dt
    h = SO.spacing(W.grid_positions(sc.rows, sc.cols, sc.cloth_args[2]), sc.rows, sc.cols)
    wind = sc.config["wind"]
    sur = fgb.Surrogate.new(0)
    sur.reserve(10 * n)
    for k in range(2):
        pos, vel = cloth_state(mesh, sc.pins)
        sur.collect(sim, ratio, 1)
        pos1, vel1 = cloth_state(mesh, sc.pins)
        f, t = sur.dataset(k * n, n)
        ref = SO.features(pos, vel, sc.rows, sc.cols, h, T, wind, W.grid_positions(sc.rows, sc.cols, sc.cloth_args[2]))
        assert np.all(np.abs(f[:, :52] - ref[:, :52]) <= 1e-6 * np.maximum(1.0, np.abs(ref[:, :52])))
        s = T / h
        tref = (vel1[:, :3] - vel[:, :3]) * s
        assert np.allclose(t, tref, rtol=1e-6, atol=1e-7)
    assert sur.dataset_info() == (2 * n, 10 * n)
    for first, rows in ((2 * n, 1), ((1 << 64) - 1, 2)):  # past the end; an end that wraps in 64 bits
        with pytest.raises(fgb.FgbError) as e:
            sur.dataset(first, rows)
        assert e.value.code == -2
    sur.fit_normalization()
    f, t = sur.dataset(0, 2 * n)
    m, sd, om, osd = sur.get_normalization()
    fm, fs = f.astype(np.float64).mean(0), f.astype(np.float64).std(0)
    fs = np.where(fs < 1e-6, 1.0, fs)
    assert np.allclose(m, fm, rtol=1e-4, atol=1e-6) and np.allclose(sd, fs, rtol=1e-4, atol=1e-6)
    assert np.allclose(om, t.astype(np.float64).mean(0), rtol=1e-4, atol=1e-8)


def test_coarse_step_matches_oracle():
    sc, sim, mesh, _ = small_scene(obstacles=False)
    p = rand_params(10, scale=0.5)
    sur = fgb.Surrogate.new(0)
    sur.set_params(p)
    rng = np.random.default_rng(11)
    in_mean = rng.normal(0, 0.1, 54).astype(np.float32)
    in_std = rng.uniform(0.5, 2.0, 54).astype(np.float32)
    out_mean = rng.normal(0, 0.01, 3).astype(np.float32)
    out_std = rng.uniform(0.01, 0.05, 3).astype(np.float32)
    sur.set_normalization(in_mean, in_std, out_mean, out_std)
    ratio = 10
    T = np.float32(ratio) * np.float32(sc.config["dt"])
    h = SO.spacing(W.grid_positions(sc.rows, sc.cols, sc.cloth_args[2]), sc.rows, sc.cols)
    pos, vel = cloth_state(mesh, sc.pins)
    assert sim.step_surrogate(sur, ratio, 1) == 0
    pos1, vel1 = cloth_state(mesh, sc.pins)
    rest = W.grid_positions(sc.rows, sc.cols, sc.cloth_args[2])
    rp, rv = SO.coarse_step(pos, vel, sc.rows, sc.cols, h, T, sc.config["wind"], rest, p, in_mean, in_std, out_mean,
                            out_std)
    dv = np.abs(rv[:, :3] - vel[:, :3]).max()
    assert dv > 0
    assert np.abs(vel1[:, :3] - rv[:, :3]).max() <= 1e-2 * dv + 1e-7
    assert np.abs(pos1[:, :3] - rp[:, :3]).max() <= 1e-2 * dv * T + 1e-6
    assert np.array_equal(pos1[sc.pins], pos[sc.pins]) and np.array_equal(vel1[sc.pins, :3], vel[sc.pins, :3])


def test_fallback_reverts_to_fine_steps():
    sc, sim, mesh, _ = small_scene()
    _, sim2, mesh2, _ = small_scene()
    sur = fgb.Surrogate.new(12)
    sur.set_normalization(np.zeros(54), np.ones(54), np.zeros(3), np.full(3, 100.0))  # wild outputs
    chk = fgb.SurrogateCheck.make(energy_growth=0.05, energy_abs=1e-6, max_strain=0.3)
    n_fb = sim.step_surrogate(sur, 10, 3, chk)
    assert n_fb == 3
    sim2.step(30)
    assert np.array_equal(mesh.get_points(), mesh2.get_points())


def test_batched_fallback_reverts_every_failing_cloth():
    batch = W.c2(n_cloths=5, lo=12, hi=70, seed=3, dt=1.0 / 6000.0)
    sim, meshes, _ = W.build_batch(batch, fgb)
    sim2, meshes2, _ = W.build_batch(batch, fgb)
    sur = fgb.Surrogate.new(14)
    sur.set_normalization(np.zeros(54), np.ones(54), np.zeros(3), np.full(3, 100.0))
    chk = fgb.SurrogateCheck.make(energy_growth=0.05, energy_abs=1e-6, max_strain=0.3)
    assert sim.step_surrogate(sur, 10, 2, chk) == 10
    sim2.step(20)
    for a, b in zip(meshes, meshes2):
        assert np.array_equal(a.get_points(), b.get_points())
    # odd ratio: no restoring copy, the masked steps end in the other buffer directly
    assert sim.step_surrogate(sur, 3, 1, chk) == 5
    sim2.step(3)
    for a, b in zip(meshes, meshes2):
        assert np.array_equal(a.get_points(), b.get_points())


def _rollout(build, sur, ratio, steps, chk, graphs):
    sim, meshes = build()
    sim.set_graphs(graphs)
    n = sim.step_surrogate(sur, ratio, steps, chk)
    return n, [m.get_points() for m in meshes]


@pytest.mark.parametrize("kind", ["single", "batch"])
def test_device_decisions_equal_host_decisions(kind):
    """The checked rollout decided on the device (one graph per coarse step,
    the fallback under a conditional node, no host wait between steps) gives
    the host-decided loop's verdicts: equal fallback counts and bit-identical
    states, with the network's outputs scaled from harmless to wild so that
    some steps (and, in a batch, some cloths) fall back and others do not;
    even and odd ratios (with and without the restoring copy)."""
    steps = 6
    if kind == "single":
        def build():
            _, sim, mesh, _ = small_scene()
            return sim, [mesh]
        cap = steps
    else:
        batch = W.c2(n_cloths=6, lo=12, hi=70, seed=5, dt=1.0 / 6000.0)

        def build():
            sim, meshes, _ = W.build_batch(batch, fgb)
            return sim, meshes
        cap = 6 * steps
    sur = fgb.Surrogate.new(21)
    chk = fgb.SurrogateCheck.make(energy_growth=1e-3, energy_abs=1e-7, max_strain=0.5)
    counts = []
    for scale in (1e-4, *np.geomspace(1e-2, 1e-1, 9), 100.0):
        sur.set_normalization(np.zeros(54), np.ones(54), np.zeros(3), np.full(3, scale))
        for ratio in (10, 3):
            n_dev, p_dev = _rollout(build, sur, ratio, steps, chk, True)
            n_host, p_host = _rollout(build, sur, ratio, steps, chk, False)
            assert n_dev == n_host, (scale, ratio)
            for a, b in zip(p_dev, p_host):
                assert np.array_equal(a, b), (scale, ratio)
            counts.append(n_dev)
    assert any(0 < c < cap for c in counts), counts


def test_energy_matches_numpy():
    sc, sim, mesh, _ = small_scene()
    sim.step(20)
    e = sim.energy()
    pts = mesh.get_points().astype(np.float64)
    kcl, ab = mesh.get_struts()
    g = np.asarray(sc.config["gravity"], np.float64)
    E = (0.5 * pts[:, 0] * (pts[:, 4:7] ** 2).sum(1)).sum() - (pts[:, 1:4] @ g).sum()
    d = np.linalg.norm(pts[ab[:, 1], 1:4] - pts[ab[:, 0], 1:4], axis=1)
    k, L = kcl[:, 0].astype(np.float64), kcl[:, 2].astype(np.float64)
    E += (0.5 * k * (d - L) ** 2).sum()
    strain = np.abs((d - L) / L).max()
    assert e[0, 0] == pytest.approx(E, rel=1e-4, abs=1e-7)
    assert e[0, 1] == pytest.approx(strain, rel=1e-4)


def rollout_error(p, f):
    p, f = p[:, 1:4].astype(np.float64), f[:, 1:4].astype(np.float64)
    return np.sqrt(((p - f) ** 2).sum(1).mean()) / np.sqrt(((f - f.mean(0)) ** 2).sum(1).mean())


def test_trained_surrogate_gains_over_the_method_without_it():
    """Train on the fine solver's own rollouts (dt = 1/6000 s), then roll the
    surrogate out for 50 coarse steps of 10 fine steps from the initial state
    and compare with the fine solver at equal simulated time.  The same coarse
    method without the network (its output replaced by the data's mean
    velocity change) must be at least twice as far off.  Over 200 coarse
    steps the reference's explicit Euler run at the coarse step goes
    non-finite on this cloth (step 135), while the checked surrogate stays
    finite."""
    ratio, n_coarse = 10, 50
    sc, sim, mesh, _ = small_scene(n=32)
    p0 = mesh.get_points()
    sur = fgb.Surrogate.new(13)
    sur.reserve(600 * 1024)
    sur.collect(sim, ratio, 500)
    sur.fit_normalization()
    losses = np.concatenate([sur.train(2000, 16384, 3e-3, seed=1), sur.train(1000, 16384, 1e-3, seed=2)])
    assert losses[-1] < 0.1 * losses[0]

    _, fine, fmesh, _ = small_scene(n=32)
    fine.step(ratio * n_coarse)
    ref = fmesh.get_points()

    _, s1, m1, _ = small_scene(n=32)
    s1.step_surrogate(sur, ratio, n_coarse)
    e_sur = rollout_error(m1.get_points(), ref)

    mean_only = fgb.Surrogate.new(0)
    mean_only.set_params(np.zeros(fgb.N_PARAMS, np.float32))
    mean_only.set_normalization(*sur.get_normalization())
    _, s2, m2, _ = small_scene(n=32)
    s2.step_surrogate(mean_only, ratio, n_coarse)
    e_mean = rollout_error(m2.get_points(), ref)

    _, s3, m3, _ = small_scene(n=32, dt=ratio / 6000.0)
    s3.step(n_coarse)
    p3 = m3.get_points()
    e_coarse = rollout_error(p3, ref) if np.isfinite(p3).all() else np.inf
    print("rollout error after %d coarse steps: surrogate %.3g, without the network %.3g, plain Euler at the "
          "coarse step %.3g" % (n_coarse, e_sur, e_mean, e_coarse))
    assert np.isfinite(e_sur)
    assert e_sur < 0.5 * e_mean
    assert np.array_equal(p0[sc.pins, 1:4], m1.get_points()[sc.pins, 1:4])

    _, s4, m4, _ = small_scene(n=32)
    fallbacks = s4.step_surrogate(sur, ratio, 200, fgb.SurrogateCheck.make())
    s3.step(200 - n_coarse)
    print("200 coarse steps: surrogate finite=%s (%d fallbacks), plain Euler at the coarse step finite=%s"
          % (np.isfinite(m4.get_points()).all(), fallbacks, np.isfinite(m3.get_points()).all()))
    assert np.isfinite(m4.get_points()).all()
    assert not np.isfinite(m3.get_points()).all()
