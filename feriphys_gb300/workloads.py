"""Synthetic cloth scenes with the shapes of the benchmark configurations.

A scene is a plain description (numpy arrays + numbers) that can be built
through this package's API or, in tests and the CPU baseline, through the
oracle.  The physical parameters of the configurations are mapped onto the
reference's Config/Cloth semantics here, in one place:

* gravity: the reference adds ``config.gravity`` as a FORCE to every point
  (springy_mesh.rs:194-196), so g = 9.81 m/s^2 on a 0.01 kg vertex is passed
  as the force (0, -0.0981, 0).
* air density: the reference's drag is ``-Cd * A_eff * v_rel`` with no air
  density (springy_mesh.rs:636-646); a drag coefficient Cd at density rho is
  passed as 0.5 * rho * Cd (same for lift).
* stiffness/damping: the reference scales a strut's constants by
  NOMINAL_STRUT_LENGTH / rest_length (springy_mesh.rs:83-84).  The configs
  give per-strut (effective) constants, so Cloth::new receives
  k_eff * nominal_length_of_the_class (spacing, spacing*sqrt(2), 2*spacing);
  the large cloth's per-strut random constants are set directly per strut.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

RHO_AIR = 1.2
G = 9.81


@dataclasses.dataclass
class Scene:
    name: str
    kind: str  # "cloth" (Cloth::new arguments) or "springy" (SpringyMesh::new arrays)
    config: dict
    cloth_args: tuple | None = None
    pins: np.ndarray | None = None
    positions: np.ndarray | None = None
    indices: np.ndarray | None = None
    mass: float = 1.0
    extra_struts: np.ndarray | None = None  # [k, 2] pairs added with add_strut (after construction)
    strut_params: object = None  # callable(ab[S,2]) -> (k[S], c[S]) applied with set_strut_params
    obstacles: list = dataclasses.field(default_factory=list)  # [(positions [V,3], indices [3F])]
    rows: int = 0
    cols: int = 0

    @property
    def n_vertices(self) -> int:
        return self.rows * self.cols if self.kind == "cloth" else len(self.positions)


def cloth_config(dt=1.0 / 600.0, integration=0, vertex_mass=0.01, wind=(2.0, 0.0, 1.0), cd=1.0, cl=0.5,
                 restitution=0.3, friction=0.2) -> dict:
    return dict(integration=integration, dt=float(np.float32(dt)), gravity=(0.0, -G * vertex_mass, 0.0),
                wind=tuple(wind), lift_coefficient=0.5 * RHO_AIR * cl, drag_coefficient=0.5 * RHO_AIR * cd,
                coefficient_of_restitution=restitution, coefficient_of_friction=friction)


def plane(y=-1.5, half=3.0):
    """Two triangles with normal +y (collidable_mesh.rs face winding)."""
    pos = np.array([[-half, y, half], [half, y, half], [half, y, -half], [-half, y, -half]], np.float32)
    return pos, np.array([0, 1, 2, 0, 2, 3], np.uint32)


def uv_sphere(center, radius, sectors=32, stacks=16):
    """UV sphere (polar axis z) with outward triangle winding: the standard
    sector/stack construction, stacks from the +z pole to the -z pole."""
    pos = []
    for i in range(stacks + 1):
        sa = math.pi / 2 - i * math.pi / stacks
        xy, z = radius * math.cos(sa), radius * math.sin(sa)
        for j in range(sectors + 1):
            ang = j * 2 * math.pi / sectors
            pos.append((center[0] + xy * math.cos(ang), center[1] + xy * math.sin(ang), center[2] + z))
    idx = []
    for i in range(stacks):
        k1, k2 = i * (sectors + 1), (i + 1) * (sectors + 1)
        for _ in range(sectors):
            if i != 0:
                idx += [k1, k2, k1 + 1]
            if i != stacks - 1:
                idx += [k1 + 1, k2, k2 + 1]
            k1 += 1
            k2 += 1
    return np.array(pos, np.float32), np.array(idx, np.uint32)


def cloth_indices(rows, cols):
    """The triangle list Cloth::new builds (cloth.rs:63-83)."""
    r, c = np.meshgrid(np.arange(rows - 1), np.arange(cols - 1), indexing="ij")
    i = (r * cols + c).ravel().astype(np.int64)
    a = np.stack([i + 1, i + cols, i], 1)
    r2, c2 = np.meshgrid(np.arange(1, rows), np.arange(cols - 1), indexing="ij")
    i2 = (r2 * cols + c2).ravel().astype(np.int64)
    b = np.stack([i2 - cols + 1, i2 + 1, i2], 1)
    return np.concatenate([a, b]).reshape(-1).astype(np.uint32)


def binding_pairs(rows, cols):
    """Binding struts in Cloth::new's order (cloth.rs:100-110)."""
    r, c = np.meshgrid(np.arange(max(rows - 2, 0)), np.arange(max(cols - 2, 0)), indexing="ij")
    i = (r * cols + c).ravel().astype(np.int64)
    return np.stack([np.stack([i, i + 2], 1), np.stack([i, i + 2 * cols], 1)], 1).reshape(-1, 2).astype(np.uint32)


def grid_positions(rows, cols, spacing, position=(0.0, 0.0, 0.0)):
    """Cloth::new's vertex positions (cloth.rs:34-55) in f32 arithmetic."""
    s = np.float32(spacing)
    c = np.arange(cols, dtype=np.float32) * s
    r = np.arange(rows, dtype=np.float32) * s
    cx = np.float32(cols) / np.float32(2.0) * s
    cy = np.float32(rows) / np.float32(2.0) * s
    pos = np.zeros((rows, cols, 3), np.float32)
    pos[:, :, 0] = (c[None, :] - cx) + np.float32(position[0])
    pos[:, :, 1] = (r[:, None] - cy) + np.float32(position[1])
    pos[:, :, 2] = np.float32(0.0) + np.float32(position[2])
    return pos.reshape(-1, 3)


def c0(n=32, side=1.0, dt=1.0 / 600.0, integration=0, obstacles=True) -> Scene:
    """Plain method, small: n x n cloth, 1 m side, structural k=500, shear 250,
    bending 50 N/m, damping 0.5 N.s/m, vertex mass 0.01 kg, top corners
    pinned, wind (2,0,1), Cd 1.0, Cl 0.5, rho 1.2, plane y=-1.5 (e 0.3, mu 0.2)."""
    s = side / (n - 1)
    lt, ls, lb = s, s * math.sqrt(2.0), 2.0 * s
    args = (n, n, s, (0.0, 0.0, 0.0), 0.01, 500.0 * lt, 0.5 * lt, 250.0 * ls, 0.5 * ls, 50.0 * lb, 0.5 * lb)
    pins = np.array([n * n - n, n * n - 1], np.uint32)
    obs = [plane(-1.5)] if obstacles else []
    return Scene("c0-%dx%d" % (n, n), "cloth", cloth_config(dt, integration), cloth_args=args, pins=pins,
                 obstacles=obs, rows=n, cols=n)


def class_params(ab, rows, cols, base_k=(500.0, 250.0, 50.0), base_c=0.5, jitter=0.1, seed=0):
    """Per-strut effective (k, c) for a Cloth-topology strut list: tensile /
    shear / binding by position in the list, k drawn uniform within +-jitter."""
    ab = np.asarray(ab, np.int64)
    S = len(ab)
    n_tri = 3 * (rows - 1) * (cols - 1) + (rows - 1) + (cols - 1)
    d = ab[:, 1] - ab[:, 0]
    cls = np.where(np.arange(S) >= n_tri, 2, np.where((d == cols) | ((d == 1) & (ab[:, 0] % cols != cols - 1)), 0, 1))
    rng = np.random.default_rng(seed + 7919)
    u = rng.uniform(1.0 - jitter, 1.0 + jitter, S)
    k = (np.asarray(base_k, np.float64)[cls] * u).astype(np.float32)
    c = np.full(S, base_c, np.float32)
    return k, c


def c1(n=1024, side=1.0, dt=1.0 / 600.0, seed=0, noise=1e-3, sphere=(32, 16), integration=0) -> Scene:
    """Plain method, large: n x n cloth (1,048,576 vertices at n=1024),
    per-strut stiffness within +-10% of the small config's, positions
    perturbed by N(0, noise), top row pinned, plane y=-1.5 plus a sphere
    r=0.3 m 0.5 m below the cloth centre."""
    s = side / (n - 1)
    pos = grid_positions(n, n, s).astype(np.float64)
    rng = np.random.default_rng(seed)
    pos += rng.normal(0.0, noise, pos.shape)
    pos = pos.astype(np.float32)
    centre = pos.astype(np.float64).mean(0)
    obs = [plane(-1.5), uv_sphere((centre[0], centre[1] - 0.5, centre[2]), 0.3, *sphere)]
    return Scene("c1-%dx%d" % (n, n), "springy", cloth_config(dt, integration), positions=pos,
                 indices=cloth_indices(n, n), mass=0.01 * n * n, extra_struts=binding_pairs(n, n),
                 strut_params=lambda ab: class_params(ab, n, n, seed=seed), pins=np.arange(n * (n - 1), n * n, dtype=np.uint32),
                 obstacles=obs, rows=n, cols=n)


@dataclasses.dataclass
class Batch:
    """Many independent cloths (one Simulation, per-cloth wind)."""
    name: str
    config: dict
    cloths: list  # [(cloth_args, pins, wind)]
    obstacles: list

    @property
    def n_vertices(self) -> int:
        return sum(a[0] * a[1] for a, _, _ in self.cloths)


def c2(n_cloths=4096, lo=16, hi=128, seed=0, dt=1.0 / 600.0, integration=0) -> Batch:
    """Batched plain: n_cloths cloths of side U{lo..hi} vertices (1 m side),
    the small config's strut constants scaled per cloth by U(0.5, 2), pins =
    one or two random corners or the top row, wind direction uniform on the
    sphere with speed U(0, 5) m/s, plane collider."""
    rng = np.random.default_rng(seed)
    cloths = []
    for _ in range(n_cloths):
        n = int(rng.integers(lo, hi + 1))
        s = 1.0 / (n - 1)
        lt, ls, lb = s, s * math.sqrt(2.0), 2.0 * s
        f = float(rng.uniform(0.5, 2.0))
        args = (n, n, s, (0.0, 0.0, 0.0), 0.01, f * 500.0 * lt, f * 0.5 * lt, f * 250.0 * ls, f * 0.5 * ls,
                f * 50.0 * lb, f * 0.5 * lb)
        corners = [n * n - n, n * n - 1, 0, n - 1]
        kind = int(rng.integers(0, 3))
        if kind == 0:
            pins = [corners[int(rng.integers(0, 4))]]
        elif kind == 1:
            pins = [int(x) for x in rng.choice(corners, 2, replace=False)]
        else:
            pins = list(range(n * n - n, n * n))
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        wind = tuple(float(v) for v in d * rng.uniform(0.0, 5.0))
        cloths.append((args, np.array(pins, np.uint32), wind))
    return Batch("c2-%d-cloths" % n_cloths, cloth_config(dt, integration), cloths, [plane(-1.5)])


def build_batch(batch: Batch, api):
    """One Simulation over all cloths of the batch (per-mesh wind)."""
    meshes = []
    for args, pins, wind in batch.cloths:
        m = api.Cloth.new(*args, pins).mesh
        m.set_wind(wind)
        meshes.append(m)
    obstacles = [api.CollidableMesh.new(p, i) for p, i in batch.obstacles]
    sim = api.Simulation.new(meshes, obstacles)
    sim.set_config(api.Config.make(**batch.config))
    return sim, meshes, obstacles


def build(scene: Scene, api):
    """Build the scene through a springy API (this package, or the oracle's
    mirror); returns (simulation, mesh, obstacles)."""
    if api.__name__ == "oracle":
        return _build_oracle(scene, api)
    cfg = api.Config.make(**scene.config)
    if scene.kind == "cloth":
        mesh = api.Cloth.new(*scene.cloth_args, scene.pins).mesh
    else:
        mesh = api.SpringyMesh.new(scene.positions, scene.indices, scene.mass, 1.0, 1.0)
        mesh.add_pins(scene.pins)
        if scene.extra_struts is not None:
            mesh.add_struts(scene.extra_struts, 1.0, 1.0)
        if scene.strut_params is not None:
            _, ab = mesh.get_struts()
            k, c = scene.strut_params(ab)
            mesh.set_strut_params(k, c)
    obstacles = [api.CollidableMesh.new(p, i) for p, i in scene.obstacles]
    sim = api.Simulation.new([mesh], obstacles)
    sim.set_config(cfg)
    return sim, mesh, obstacles


def _build_oracle(scene: Scene, orc):
    c = scene.config
    cfg = orc.Config.make(c["integration"], c["dt"], c["gravity"], c["wind"], c["lift_coefficient"],
                          c["drag_coefficient"], c["coefficient_of_restitution"], c["coefficient_of_friction"])
    if scene.kind == "cloth":
        mesh = orc.SpringyMesh.cloth(*scene.cloth_args, scene.pins)
    else:
        mesh = orc.SpringyMesh.new(scene.positions, scene.indices, scene.mass, 1.0, 1.0)
        mesh.add_pins(scene.pins)
        if scene.extra_struts is not None:
            mesh.add_struts(scene.extra_struts, 1.0, 1.0)
        if scene.strut_params is not None:
            _, ab, _ = mesh.get_struts()
            k, c_ = scene.strut_params(ab)
            mesh.set_strut_params(k, c_)
    obstacles = [orc.CollidableMesh(p, i) for p, i in scene.obstacles]
    sim = orc.Simulation([mesh], obstacles)
    sim.set_config(cfg)
    return sim, mesh, obstacles
