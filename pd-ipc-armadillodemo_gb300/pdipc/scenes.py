"""Seeded synthetic scenes for the PD-IPC cloth step.

The reference ships one hand-made scene (two 75x75 Blender cloths and a tet
armadillo, ``example/ClothArmadillo/config.xml``) and no benchmark inputs, so
the workloads here are generated: a square cloth on a regular grid split along
alternating diagonals, jittered from a counter-based SplitMix64 stream, falling
onto a subdivided icosahedron.  The same arrays feed the CUDA library and the
CPU oracle, so both see bit-identical inputs.

Conventions that mirror the reference scene set-up:
  * gravity acts along -y (``gravityForce = (0, g*m, 0)``,
    Simulator/PD-IPC/PdIpcSimulator.cpp:249-252);
  * cloth stiffness triple is (strain, bending, pin) as in the ``<type>`` line
    of config.xml read by PdIpcSimulator.h:478-483 / 519-521;
  * a static obstacle gets collision mass 1e4 per vertex
    (PdIpcSimulator.cpp:1494).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, counters: np.ndarray) -> np.ndarray:
    """SplitMix64 output for ``state = seed + (counter + 1) * golden``.

    Counter-based so any element can be generated independently (and the same
    stream is trivially reproduced in C or C++).
    """
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + (counters.astype(np.uint64) + np.uint64(1)) * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return z


def uniform01(seed: int, n: int, offset: int = 0) -> np.ndarray:
    """n doubles in [0, 1) with 53 random bits each."""
    z = splitmix64(seed, np.arange(offset, offset + n, dtype=np.uint64))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def grid_cloth(n: int, side: float = 1.0, height: float = 0.0,
               jitter: float = 1e-4, seed: int = 0,
               origin=(0.0, 0.0)) -> tuple[np.ndarray, np.ndarray]:
    """n x n vertex cloth in the x-z plane at y = ``height``.

    Vertex (r, c) has index r*n + c and sits at x = c*side/(n-1),
    z = r*side/(n-1).  Quad (r, c) is split along the diagonal chosen by the
    parity of r + c, so interior vertices alternate between degree 4 and 8.
    Every coordinate gets uniform jitter in [-jitter, jitter).
    Returns (X float64[n*n, 3], F int32[2*(n-1)^2, 3]).
    """
    if n < 2:
        raise ValueError("cloth needs at least 2x2 vertices")
    h = side / (n - 1)
    r, c = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    X = np.zeros((n * n, 3), dtype=np.float64)
    X[:, 0] = origin[0] + c.reshape(-1) * h
    X[:, 1] = height
    X[:, 2] = origin[1] + r.reshape(-1) * h
    if jitter > 0.0:
        u = uniform01(seed, 3 * n * n).reshape(n * n, 3)
        X += (2.0 * u - 1.0) * jitter
    rr, cc = np.meshgrid(np.arange(n - 1), np.arange(n - 1), indexing="ij")
    rr = rr.reshape(-1)
    cc = cc.reshape(-1)
    a = rr * n + cc
    b = a + 1
    d = a + n
    e = d + 1
    even = ((rr + cc) % 2) == 0
    F = np.empty((2 * (n - 1) * (n - 1), 3), dtype=np.int32)
    # even quads: diagonal a-e ; odd quads: diagonal b-d
    f0 = np.where(even[:, None], np.stack([a, d, e], 1), np.stack([a, d, b], 1))
    f1 = np.where(even[:, None], np.stack([a, e, b], 1), np.stack([b, d, e], 1))
    F[0::2] = f0
    F[1::2] = f1
    return X, F


_ICO_T = (1.0 + math.sqrt(5.0)) / 2.0
_ICO_V = [(-1, _ICO_T, 0), (1, _ICO_T, 0), (-1, -_ICO_T, 0), (1, -_ICO_T, 0),
          (0, -1, _ICO_T), (0, 1, _ICO_T), (0, -1, -_ICO_T), (0, 1, -_ICO_T),
          (_ICO_T, 0, -1), (_ICO_T, 0, 1), (-_ICO_T, 0, -1), (-_ICO_T, 0, 1)]
_ICO_F = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11),
          (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8),
          (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9),
          (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]


def icosphere(subdiv: int, radius: float = 1.0,
              centre=(0.0, 0.0, 0.0)) -> tuple[np.ndarray, np.ndarray]:
    """Subdivided icosahedron: V = 10*4^s + 2, F = 20*4^s.

    Midpoints are appended in first-use order while faces are visited in
    order; each face (a,b,c) becomes (a,ab,ca), (b,bc,ab), (c,ca,bc),
    (ab,bc,ca).
    """
    V = [np.array(v, dtype=np.float64) / np.linalg.norm(v) for v in _ICO_V]
    F = list(_ICO_F)
    for _ in range(subdiv):
        cache: dict[tuple[int, int], int] = {}

        def mid(i: int, j: int) -> int:
            key = (i, j) if i < j else (j, i)
            k = cache.get(key)
            if k is None:
                m = V[i] + V[j]
                V.append(m / np.linalg.norm(m))
                k = len(V) - 1
                cache[key] = k
            return k

        nf = []
        for a, b, c in F:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        F = nf
    X = np.asarray(V) * radius + np.asarray(centre, dtype=np.float64)
    return X, np.asarray(F, dtype=np.int32)


@dataclasses.dataclass
class ClothSpec:
    X: np.ndarray
    F: np.ndarray
    pins: np.ndarray
    density: float = 0.1
    k_stretch: float = 1e4
    k_bend: float = 1e-3
    k_pin: float = 1e6
    patch_dim: int = 10
    # optional (pdipc_add_cloth_ex): per-triangle stretch stiffness (nf values),
    # and a triangle strain limit of weight k_tri_strain (or per-triangle
    # tri_strain) times rest area
    tri_stretch: np.ndarray | None = None
    k_tri_strain: float = 0.0
    tri_strain: np.ndarray | None = None


@dataclasses.dataclass
class StaticSpec:
    X: np.ndarray
    F: np.ndarray
    patch_dim: int = 10


@dataclasses.dataclass
class SolidSpec:
    """A tetrahedral (volumetric) model: PdIpcVolumetricModel(strain, volume,
    position stiffness) with <density> and <patchDim>."""
    X: np.ndarray
    T: np.ndarray
    pins: np.ndarray
    density: float = 1000.0
    k_strain: float = 1e6
    k_volume: float = 1e3
    k_pin: float = 1e12
    patch_dim: int = 10


@dataclasses.dataclass
class Scene:
    name: str
    cloths: list
    statics: list
    dt: float = 1.0 / 240.0
    gravity: float = -9.8
    dhat: float = 1e-3
    kappa: float = 1e4
    lg_iterations: int = 10
    steps: int = 200
    solids: list = dataclasses.field(default_factory=list)  # simulated after the cloths

    @property
    def n_sim(self) -> int:
        return sum(c.X.shape[0] for c in self.cloths) + sum(v.X.shape[0] for v in self.solids)

    @property
    def n_total(self) -> int:
        return self.n_sim + sum(s.X.shape[0] for s in self.statics)

    def initial_positions(self) -> np.ndarray:
        """Every vertex in the library's order: cloths, tet models, static meshes."""
        return np.concatenate([c.X for c in self.cloths] + [v.X for v in self.solids] +
                              [s.X for s in self.statics])


def sphere_patch_dim(nfaces: int) -> int:
    """Grid resolution giving about two faces per patch cell on each cap."""
    return max(1, int(round(math.sqrt(nfaces / math.pi))))


def cloth_drop(n: int, subdiv: int, *, seed: int = 0, lg: int = 10,
               steps: int = 200, dhat: float = 1e-3, radius: float = 0.3,
               k_stretch: float = 1e4, k_bend: float = 1e-3,
               density: float = 0.1, k_pin: float = 1e6,
               height: float = 0.0, with_sphere: bool = True,
               name: str | None = None) -> Scene:
    """Square 1 m cloth, two adjacent corners pinned, above a fixed icosphere
    whose centre is 0.5 m below the cloth centre."""
    X, F = grid_cloth(n, 1.0, height, 1e-4, seed)
    pins = np.array([0, n - 1], dtype=np.int32)
    cloth = ClothSpec(X, F, pins, density, k_stretch, k_bend, k_pin, patch_dim=n)
    statics = []
    if with_sphere:
        SX, SF = icosphere(subdiv, radius, (0.5, height - 0.5, 0.5))
        statics.append(StaticSpec(SX, SF, patch_dim=sphere_patch_dim(SF.shape[0])))
    return Scene(name or f"cloth{n}_sphere{subdiv}", [cloth], statics,
                 dhat=dhat, lg_iterations=lg, steps=steps)


def config0(seed: int = 0) -> Scene:
    """64x64 cloth onto an icosphere (subdivision 4), 10 PD iterations, 200 steps."""
    return cloth_drop(64, 4, seed=seed, lg=10, steps=200, name="c0_cloth64_sphere4")


def config1(seed: int = 0) -> Scene:
    """512x512 cloth onto an icosphere (subdivision 6), 20 PD iterations, 100 steps."""
    return cloth_drop(512, 6, seed=seed, lg=20, steps=100, name="c1_cloth512_sphere6")


def stack(layers: int = 4, n: int = 256, subdiv: int = 5, gap: float = 5e-3,
          seed: int = 0, lg: int = 20, steps: int = 100,
          dhat: float = 5e-4, pinned: bool = False, drop: float = 0.2) -> Scene:
    """Layers of n x n cloth stacked ``gap`` apart (layer 0 lowest), each with
    its own jitter stream, falling onto a radius-0.3 m icosphere whose top is
    ``drop`` below the lowest layer's centre (0.2 m: centre 0.5 m below).  The
    layers collide with each other and with themselves (the patch broad phase
    pairs every two patches, of one model or two)."""
    cloths = []
    for L in range(layers):
        X, F = grid_cloth(n, 1.0, L * gap, 1e-4, seed + 7919 * L)
        pins = np.array([0, n - 1], dtype=np.int32) if pinned else np.zeros(0, np.int32)
        cloths.append(ClothSpec(X, F, pins, patch_dim=n))
    SX, SF = icosphere(subdiv, 0.3, (0.5, -0.3 - drop, 0.5))
    return Scene(f"stack{layers}x{n}_sphere{subdiv}", cloths,
                 [StaticSpec(SX, SF, patch_dim=sphere_patch_dim(SF.shape[0]))],
                 dhat=dhat, lg_iterations=lg, steps=steps)


def config4(seed: int = 0) -> Scene:
    """4 layers of 256x256 cloth 5 mm apart onto an icosphere (subdivision 5),
    dhat 5e-4 m, 20 PD iterations, 100 steps."""
    sc = stack(4, 256, 5, 5e-3, seed=seed, lg=20, steps=100, dhat=5e-4)
    sc.name = "c4_stack4x256_sphere5"
    return sc


def batched(count: int = 256, nmin: int = 16, nmax: int = 128, seed: int = 0,
            lg: int = 10, steps: int = 100, spacing: float = 2.0) -> Scene:
    """``count`` independent drops in one scene: cloth k has a side of
    U{nmin..nmax} vertices (1 m), stretch stiffness log-uniform in [1e3, 1e5]
    and two pinned corners, above its own icosphere (subdivision U{2..4},
    radius U(0.2, 0.4)) 0.5 m below its centre; drops sit on a square lattice
    ``spacing`` m apart so no two of them can touch."""
    u = uniform01(seed ^ 0x5EED, 4 * count).reshape(count, 4)
    side = int(math.ceil(math.sqrt(count)))
    cloths, statics = [], []
    for k in range(count):
        n = nmin + min(nmax - nmin, int(u[k, 0] * (nmax - nmin + 1)))
        ks = 10.0 ** (3.0 + 2.0 * u[k, 1])
        sub = 2 + min(2, int(u[k, 2] * 3))
        rad = 0.2 + 0.2 * u[k, 3]
        ox, oz = (k % side) * spacing, (k // side) * spacing
        X, F = grid_cloth(n, 1.0, 0.0, 1e-4, seed + 104729 * (k + 1), origin=(ox, oz))
        cloths.append(ClothSpec(X, F, np.array([0, n - 1], dtype=np.int32), k_stretch=ks, patch_dim=n))
        SX, SF = icosphere(sub, rad, (ox + 0.5, -0.5, oz + 0.5))
        statics.append(StaticSpec(SX, SF, patch_dim=sphere_patch_dim(SF.shape[0])))
    return Scene(f"batched{count}_{nmin}to{nmax}", cloths, statics, lg_iterations=lg, steps=steps)


def instance_slice(scene: Scene, first: int, last: int) -> Scene:
    """Instances [first, last) of a batched scene (cloth k with its obstacle k),
    as their own scene: what one rank steps when the batch is partitioned."""
    return Scene(f"{scene.name}[{first}:{last}]", scene.cloths[first:last], scene.statics[first:last],
                 dt=scene.dt, gravity=scene.gravity, dhat=scene.dhat, kappa=scene.kappa,
                 lg_iterations=scene.lg_iterations, steps=scene.steps)


def config2(seed: int = 0) -> Scene:
    """256 independent drops, cloth sides U{16..128}, in one context, 100 steps."""
    sc = batched(256, 16, 128, seed=seed, lg=10, steps=100)
    sc.name = "c2_batched256"
    return sc


def tet_block(nx: int, ny: int, nz: int, size=(0.2, 0.2, 0.2), origin=(0.0, 0.0, 0.0),
              jitter: float = 0.0, seed: int = 0) -> tuple[np.ndarray, np.ndarray]:
    """Box of nx*ny*nz cubes, each split into 6 tetrahedra around its main
    diagonal (a conforming Freudenthal split).  Returns (X float64[(nx+1)(ny+1)(nz+1), 3],
    T int32[6 nx ny nz, 4])."""
    g = np.stack(np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij"), -1)
    g = g.reshape(-1, 3).astype(np.float64)
    X = np.asarray(origin, np.float64) + g * (np.asarray(size, np.float64) / np.array([nx, ny, nz]))
    if jitter > 0.0:
        X += (2.0 * uniform01(seed, X.size).reshape(X.shape) - 1.0) * jitter

    def vid(i, j, k):
        return (i * (ny + 1) + j) * (nz + 1) + k

    paths = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    T = []
    for i in range(nx):
        for j in range(ny):
            for k in range(nz):
                for p in paths:
                    c = [i, j, k]
                    v = [vid(*c)]
                    for ax in p:
                        c[ax] += 1
                        v.append(vid(*c))
                    T.append(v)
    return X, np.asarray(T, dtype=np.int32)


def block_drop(n: int = 4, subdiv: int = 3, *, cloth_n: int = 0, lg: int = 10, steps: int = 100,
               size: float = 0.2, gap: float = 0.02, k_strain: float = 1e6, density: float = 1000.0,
               patch_dim: int = 8, seed: int = 0) -> Scene:
    """An n^3-cube tetrahedral block (size m, 6 tets per cube) falling from
    ``gap`` above a fixed icosphere (radius 0.3 m) and, with cloth_n > 0, a
    cloth_n x cloth_n cloth (1 m, two corners pinned) draped between them."""
    sph_top = -0.2
    X, T = tet_block(n, n, n, (size, size, size), (0.5 - size / 2, sph_top + gap, 0.5 - size / 2), 1e-5, seed)
    solid = SolidSpec(X, T, np.zeros(0, np.int32), density=density, k_strain=k_strain, patch_dim=patch_dim)
    cloths = []
    if cloth_n > 0:
        CX, CF = grid_cloth(cloth_n, 1.0, sph_top + gap / 2, 1e-4, seed + 1)
        cloths.append(ClothSpec(CX, CF, np.array([0, cloth_n - 1], dtype=np.int32), patch_dim=cloth_n))
    SX, SF = icosphere(subdiv, 0.3, (0.5, -0.5, 0.5))
    return Scene(f"block{n}_cloth{cloth_n}_sphere{subdiv}", cloths,
                 [StaticSpec(SX, SF, patch_dim=sphere_patch_dim(SF.shape[0]))],
                 lg_iterations=lg, steps=steps, solids=[solid])
