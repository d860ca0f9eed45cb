"""Volumetric (tetrahedral) models on the CPU oracle: the 3x3 SVD and the
strain projection against numpy, the boundary surface of a tet block, and a
block drop in the oracle's two global-step forms."""
import numpy as np
import pytest

import pdipc
from oracle.oracle import FORM_JJ, FORM_R2, Oracle, svd3, tet_project
from oracle.oracle import tet_surface as oracle_tet_surface
from pdipc import scenes


def numpy_projection(F):
    """R = U clamp(S) V^T with U, V proper rotations and det F's sign on the
    smallest singular value, flipped positive, singular values clamped to
    [0.999, 1.001] (solveVolumetricStrainConstraintKernel)."""
    U, s, Vt = np.linalg.svd(F)
    if np.linalg.det(U) < 0:
        U[:, 2] *= -1
        s[2] *= -1
    if np.linalg.det(Vt) < 0:
        Vt[2] *= -1
        s[2] *= -1
    if np.prod(s) < 0:
        s[2] = -s[2]
    s = np.sort(s)[::-1]
    return U @ np.diag(np.clip(s, 0.999, 1.001)) @ Vt


def random_F(rng, kind):
    if kind == "general":
        return rng.normal(size=(3, 3))
    if kind == "near_rotation":
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        q *= np.sign(np.linalg.det(q))
        return q @ (np.eye(3) + 2e-3 * rng.normal(size=(3, 3)))
    if kind == "inverted":
        F = rng.normal(size=(3, 3))
        return F if np.linalg.det(F) < 0 else -F
    if kind == "repeated":
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        return q @ np.diag([1.2, 1.2, 0.7]) @ q.T
    raise ValueError(kind)


@pytest.mark.parametrize("kind", ["general", "near_rotation", "inverted", "repeated"])
def test_oracle_svd_convention(kind):
    rng = np.random.default_rng(hash(kind) % 2**32)
    for _ in range(300):
        F = random_F(rng, kind)
        U, s, V = svd3(F)
        assert abs(np.linalg.det(U) - 1) < 1e-10 and abs(np.linalg.det(V) - 1) < 1e-10
        np.testing.assert_allclose(U @ np.diag(s) @ V.T, F, atol=1e-12 * max(1.0, np.abs(F).max()))
        assert s[0] >= s[1] >= abs(s[2]) - 1e-14
        assert np.sign(s[2]) == np.sign(np.linalg.det(F)) or abs(np.linalg.det(F)) < 1e-14


@pytest.mark.parametrize("kind", ["general", "near_rotation", "inverted", "repeated"])
def test_oracle_tet_projection_matches_numpy(kind):
    rng = np.random.default_rng(7 + len(kind))
    n = 200
    x = np.empty((n, 4, 3))
    idm = np.empty((n, 3, 3))
    w = rng.uniform(0.5, 2.0, n)
    expect = np.empty((n, 4, 3))
    for e in range(n):
        F = random_F(rng, kind)
        Dm = np.eye(3) * 0.1 + 0.02 * rng.normal(size=(3, 3))
        idm[e] = np.linalg.inv(Dm)
        Ds = F @ Dm
        x0 = rng.normal(size=3)
        x[e] = np.stack([x0, x0 + Ds[:, 0], x0 + Ds[:, 1], x0 + Ds[:, 2]])
        G = np.concatenate([-idm[e].T.sum(1, keepdims=True), idm[e].T], 1)   # 3 x 4
        expect[e] = (w[e] * numpy_projection(F) @ G).T
    out = tet_project(x, idm, w)
    scale = np.abs(expect).max()
    np.testing.assert_allclose(out, expect, atol=1e-10 * scale)


def test_tet_block_surface_is_closed_and_outward(built_lib):
    X, T = scenes.tet_block(3, 2, 4, (0.3, 0.2, 0.4))
    assert T.shape[0] == 6 * 3 * 2 * 4
    D = X[T[:, 1:]] - X[T[:, :1]]
    assert np.all(np.abs(np.linalg.det(D)) > 1e-9)            # no degenerate tet
    F = oracle_tet_surface(X, T)
    assert F.shape[0] == 2 * 2 * (3 * 2 + 3 * 4 + 2 * 4)       # the box's quads, two triangles each
    np.testing.assert_array_equal(pdipc.tet_surface(X, T), F)  # library and oracle: same faces, same order
    edges = np.sort(np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]]), axis=1)
    _, counts = np.unique(edges, axis=0, return_counts=True)
    assert np.all(counts == 2)                                 # closed 2-manifold
    a, b, c = X[F[:, 0]], X[F[:, 1]], X[F[:, 2]]
    volume = np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6.0
    assert abs(volume - 0.3 * 0.2 * 0.4) < 1e-12              # outward: divergence theorem gives +V
    sc = scenes.Scene("block", [], [], solids=[scenes.SolidSpec(X, T, np.zeros(0, np.int32), patch_dim=4)])
    orc = Oracle(sc, "fp64", FORM_JJ, threads=2)
    assert orc.stats()["n_sim"] == X.shape[0]


def test_block_drop_oracle_forms_agree_and_block_stays_rigid():
    sc = scenes.block_drop(3, 2, steps=40)
    a = Oracle(sc, "fp64", FORM_JJ, threads=4)
    b = Oracle(sc, "fp64", FORM_R2, threads=4)
    T = sc.solids[0].T
    X0 = sc.solids[0].X
    rest = np.linalg.norm(X0[T[:, 1]] - X0[T[:, 0]], axis=1)
    for _ in range(4):
        a.step(10)
        b.step(10)
        assert np.abs(a.positions() - b.positions()).max() < 1e-9
    assert a.stats()["active_contacts"] > 0
    x = a.positions()[:sc.n_sim]
    length = np.linalg.norm(x[T[:, 1]] - x[T[:, 0]], axis=1)
    assert np.abs(length / rest - 1.0).max() < 0.1           # elastic under the impact, no collapse
    assert x[:, 1].min() > -0.21                              # resting on the sphere, not through it
