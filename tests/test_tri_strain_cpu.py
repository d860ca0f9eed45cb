"""Triangle strain limits and per-triangle stretch on the oracle (no GPU).

The triangle strain constraint is the reference's tet strain limit
(solveVolumetricStrainConstraintKernel, PdIpcGpuFunc.cu:439-599: SVD, singular
values clamped to [0.999, 1.001], R = U S' V^T, w R G to the vertices) applied
to a triangle's 3 x 2 deformation gradient.  The oracle forms it with a 3 x 3
SVD (the deformed unit normal as third column); here an independent numpy
restatement uses the thin SVD of the 3 x 2 F directly.  The two must agree to
round-off wherever F has full rank: the projection is a spectral function of F.
"""
import numpy as np

from oracle.oracle import FORM_JJ, Oracle, tri_project
from pdipc import scenes


def numpy_tri_project(x, idm, w):
    S = np.array([[-1.0, -1.0], [1.0, 0.0], [0.0, 1.0]])
    out = np.empty((x.shape[0], 3, 3))
    for e in range(x.shape[0]):
        Ds = np.stack([x[e, 1] - x[e, 0], x[e, 2] - x[e, 0]], axis=1)  # 3 x 2
        F = Ds @ idm[e]
        U, s, Vt = np.linalg.svd(F, full_matrices=False)
        P = U @ np.diag(np.clip(s, 0.999, 1.001)) @ Vt
        G = S @ idm[e]                                                 # 3 vertices x 2
        out[e] = w[e] * (G @ P.T)
    return out


def random_triangles(rng, n, stretch):
    x = rng.normal(size=(n, 3, 3))
    idm = np.empty((n, 2, 2))
    for e in range(n):
        a, b = x[e, 1] - x[e, 0], x[e, 2] - x[e, 0]
        e1 = a / np.linalg.norm(a)
        nrm = np.cross(a, b)
        e2 = np.cross(nrm, e1) / np.linalg.norm(nrm)
        Dm = np.array([[a @ e1, b @ e1], [a @ e2, b @ e2]])
        idm[e] = np.linalg.inv(Dm)
        # deform: a random rotation and stretch of the rest triangle
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        St = np.diag([stretch[e, 0], stretch[e, 1], 1.0])
        x[e] = x[e] @ (q @ St).T
    return x, idm


def test_triangle_projection_matches_numpy_thin_svd():
    rng = np.random.default_rng(5)
    n = 200
    stretch = rng.uniform(0.9, 1.1, (n, 2))     # most triangles outside [0.999, 1.001]: clamped
    x, idm = random_triangles(rng, n, stretch)
    w = rng.uniform(0.5, 2.0, n)
    mine = tri_project(x, idm, w)
    ref = numpy_tri_project(x, idm, w)
    scale = np.abs(ref).max()
    assert np.abs(mine - ref).max() < 1e-12 * scale
    # the contributions of a triangle sum to zero (translation invariance)
    assert np.abs(mine.sum(axis=1)).max() < 1e-12 * scale


def test_rest_triangle_projects_to_itself():
    rng = np.random.default_rng(6)
    x, idm = random_triangles(rng, 50, np.ones((50, 2)))  # rigidly moved: F is a rotation
    w = np.ones(50)
    mine = tri_project(x, idm, w)
    S = np.array([[-1.0, -1.0], [1.0, 0.0], [0.0, 1.0]])
    for e in range(50):
        F = np.stack([x[e, 1] - x[e, 0], x[e, 2] - x[e, 0]], axis=1) @ idm[e]
        np.testing.assert_allclose(mine[e], (S @ idm[e]) @ F.T, atol=1e-12)


def test_per_triangle_stretch_is_the_mean_over_a_vertex_s_triangles():
    sc = scenes.cloth_drop(8, 1, with_sphere=False)
    c = sc.cloths[0]
    kt = np.random.default_rng(1).uniform(1e3, 1e5, c.F.shape[0])
    c.tri_stretch = kt
    orc = Oracle(sc, "fp64", FORM_JJ, threads=2)
    lOff, lStrain = orc.table("lOff"), orc.table("lStrain")
    sums = np.zeros(c.X.shape[0])
    cnt = np.zeros(c.X.shape[0])
    for f, tri in enumerate(c.F):
        sums[tri] += kt[f]
        cnt[tri] += 1
    np.testing.assert_allclose(lStrain[lOff], sums / cnt, rtol=1e-15)


def test_uniform_per_triangle_stretch_equals_the_model_stiffness():
    sc = scenes.cloth_drop(10, 1, with_sphere=False)
    a = Oracle(sc, "fp64", FORM_JJ, threads=2)
    a.step(2)
    sc.cloths[0].tri_stretch = np.full(sc.cloths[0].F.shape[0], sc.cloths[0].k_stretch)
    b = Oracle(sc, "fp64", FORM_JJ, threads=2)
    b.step(2)
    assert np.array_equal(a.positions(), b.positions())


def test_strain_limit_holds_a_stretched_cloth_back():
    """A hanging cloth with a stiff strain limit stretches less than without it."""
    sc = scenes.cloth_drop(10, 1, with_sphere=False, k_stretch=1e2)
    free = Oracle(sc, "fp64", FORM_JJ, threads=2)
    free.step(20)
    sc.cloths[0].k_tri_strain = 1e4
    lim = Oracle(sc, "fp64", FORM_JJ, threads=2)
    lim.step(20)
    F = sc.cloths[0].F

    def max_edge_ratio(X):
        X0 = sc.cloths[0].X
        r = 0.0
        for a, b in ((0, 1), (1, 2), (2, 0)):
            r = max(r, float((np.linalg.norm(X[F[:, a]] - X[F[:, b]], axis=1) /
                              np.linalg.norm(X0[F[:, a]] - X0[F[:, b]], axis=1)).max()))
        return r

    n = sc.n_sim
    assert max_edge_ratio(lim.positions()[:n]) < max_edge_ratio(free.positions()[:n])
