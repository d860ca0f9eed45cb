"""The reference's penalty / discrete-collision contact path on the CPU oracle
(PdIpcGpuFunc.cu:2933-3740: prediticeDCPositionKernel, computePenaltyForceKernal,
applyPenaltyForceForFloorKernal, computeDcdPenaltyForceKernal and
uniformPenaltyForceKernal).  The reference ships no tests for it and never
calls it, so the oracle is pinned here against independent numpy restatements
of the same formulas on small cases, and against force balance."""
import numpy as np

from oracle.oracle import FORM_JJ, Oracle
from pdipc import scenes


def crossing_scene(split_models):
    """A horizontal 8x8 grid (y = 0) crossed by a vertical one (x = 0.5); both
    one model (self pairs) or two models."""
    HX, HF = scenes.grid_cloth(8, 1.0, 0.0, 0.0, 0)
    VX, VF = scenes.grid_cloth(8, 1.0, 0.0, 0.0, 1)
    VX = np.stack([np.full(VX.shape[0], 0.5) + 1e-3 * VX[:, 1], VX[:, 0] - 0.5 + 0.03, VX[:, 2]], 1)
    none = np.zeros(0, np.int32)
    if split_models:
        cloths = [scenes.ClothSpec(HX, HF, none, patch_dim=4), scenes.ClothSpec(VX, VF, none, patch_dim=4)]
    else:
        cloths = [scenes.ClothSpec(np.concatenate([HX, VX]), np.concatenate([HF, VF + HX.shape[0]]), none,
                                   patch_dim=4)]
    return scenes.Scene("crossing", cloths, []), HF.shape[0], VF.shape[0]


def face_pairs_with_overlapping_boxes(X, F, na, nb):
    A = X[F[:na]]
    B = X[F[na:na + nb]]
    amin, amax = A.min(1), A.max(1)
    bmin, bmax = B.min(1), B.max(1)
    ov = np.all((amin[:, None, :] <= bmax[None, :, :]) & (bmin[None, :, :] <= amax[:, None, :]), axis=2)
    ia, ib = np.nonzero(ov)
    return np.stack([ia, ib + na], 1).astype(np.int32)


def numpy_tri_contact(A, B):
    p = A - A[0]
    q = B - A[0]
    e = np.array([p[1] - p[0], p[2] - p[1], p[0] - p[2]])
    f = np.array([q[1] - q[0], q[2] - q[1], q[0] - q[2]])
    n1 = np.cross(e[0], e[1])
    m1 = np.cross(f[0], f[1])
    axes = [n1, m1] + [np.cross(e[a], f[b]) for a in range(3) for b in range(3)]
    axes += [np.cross(e[a], n1) for a in range(3)] + [np.cross(f[b], m1) for b in range(3)]
    for ax in axes:
        P, Q = p @ ax, q @ ax
        if P.min() > Q.max() or Q.min() > P.max():
            return False
    return True


def numpy_dcd(X, F, pairs, model, nsim, k, kself):
    """Raw forces and hits of computeDcdPenaltyForceKernal (before averaging)."""
    force = np.zeros_like(X)
    hits = np.zeros(X.shape[0], np.int64)
    for fa, fb in pairs:
        av, bv = F[fa], F[fb]
        if np.intersect1d(av, bv).size:
            continue
        A, B = X[av], X[bv]
        if not numpy_tri_contact(A, B):
            continue
        stiff = kself if model[av[0]] == model[bv[0]] else k
        na = np.cross(A[1] - A[0], A[2] - A[0])
        na /= np.linalg.norm(na)
        nb = np.cross(B[1] - B[0], B[2] - B[0])
        nb /= np.linalg.norm(nb)
        for pv, P, qv, Q, nq in ((av, A, bv, B, nb), (bv, B, av, A, na)):
            if pv[0] >= nsim:
                continue
            for j in range(3):
                c = (P[j] - Q[1]) @ nq
                if c < 0:  # behind the plane through Q's second vertex
                    f = nq * abs(c) * stiff
                    force[pv[j]] += f
                    force[qv] -= f / 3
                    hits[pv[j]] += 1
                    hits[qv] += 1
    return force, hits


def test_floor_and_velocity_response_match_the_formula():
    sc = scenes.cloth_drop(12, 2, with_sphere=False)
    orc = Oracle(sc, "fp64", FORM_JJ, threads=2)
    rng = np.random.default_rng(4)
    x = sc.initial_positions().copy()
    x[:, 1] = rng.uniform(-0.01, 0.01, x.shape[0])
    V = rng.uniform(-1, 1, (sc.n_sim, 3))
    k, damp = 1e4, 0.3
    F, t, V2 = orc.penalty_floor(x, k, damp, V)
    below = x[:, 1] < 0
    np.testing.assert_array_equal(t, below.astype(np.int32))
    expect_F = np.zeros_like(x)
    expect_F[below, 1] = -x[below, 1] * k
    expect_F[below] -= damp * V[below]
    np.testing.assert_allclose(F, expect_F, rtol=1e-14, atol=1e-14)
    expect_V = V.copy()
    expect_V[below] = V[below] * np.array([0.9, -0.4, 0.9])  # force along +y
    np.testing.assert_allclose(V2, expect_V, rtol=1e-14, atol=1e-15)


def test_dc_prediction_matches_the_formula():
    sc = scenes.cloth_drop(12, 2)
    orc = Oracle(sc, "fp64", FORM_JJ, threads=2)
    rng = np.random.default_rng(5)
    X = sc.initial_positions()[:sc.n_sim]
    V = rng.uniform(-0.5, 0.5, (sc.n_sim, 3))
    sn, V2 = orc.penalty_predict(X, V)
    dt, g = sc.dt, sc.gravity
    expect = X + dt * (V + dt * np.array([0.0, g, 0.0]))
    pins = sc.cloths[0].pins
    expect[pins] = X[pins]
    np.testing.assert_allclose(sn, expect, rtol=0, atol=1e-14)
    free = np.setdiff1d(np.arange(sc.n_sim), pins)
    np.testing.assert_array_equal(V2[free], V[free])
    assert np.all(V2[pins] == 0)


def test_dcd_matches_numpy_for_self_and_cross_model_pairs():
    for split in (False, True):
        sc, na, nb = crossing_scene(split)
        orc = Oracle(sc, "fp64", FORM_JJ, threads=2)
        X = sc.initial_positions()
        F = np.concatenate([c.F + off for c, off in zip(sc.cloths, np.cumsum([0] + [c.X.shape[0] for c in sc.cloths])[:-1])])
        pairs = face_pairs_with_overlapping_boxes(X, F, na, nb)
        assert pairs.shape[0] > 20
        model = np.concatenate([np.full(c.X.shape[0], m) for m, c in enumerate(sc.cloths)])
        k, kself = 1e3, 2.5e3
        V0 = np.zeros((sc.n_sim, 3))
        Fo, t, _ = orc.penalty_dcd(X, pairs, k, kself, 0.0, V0)
        fn, hn = numpy_dcd(X, F, pairs, model, sc.n_sim, k, kself)
        np.testing.assert_array_equal(t, hn)
        assert t.sum() > 0
        raw = Fo * np.maximum(t, 1)[:, None]  # undo the averaging (no damping, v = 0)
        np.testing.assert_allclose(raw, fn, rtol=1e-12, atol=1e-12 * np.abs(fn).max())
        assert np.abs(raw.sum(0)).max() < 1e-9 * np.abs(raw).max()  # pushes are balanced


def test_ccd_penalty_forces_balance():
    sc = scenes.cloth_drop(16, 2)
    orc = Oracle(sc, "fp64", FORM_JJ, threads=2)
    X = sc.initial_positions().copy()
    top = X[sc.n_sim:, 1].max()
    X[:sc.n_sim, 1] += (top + 1e-3) - X[:sc.n_sim, 1].min()
    d = np.zeros_like(X)
    d[:sc.n_sim, 1] = -5e-3
    orc.broadphase(X, d)
    V0 = np.zeros((sc.n_sim, 3))
    Fo, t, V2 = orc.penalty_ccd(X, d, 1e4, 0.0, V0)
    assert t[:sc.n_sim].sum() > 0 and t[sc.n_sim:].sum() > 0      # cloth points hit sphere faces
    raw = Fo.copy()
    raw[:sc.n_sim] *= np.maximum(t[:sc.n_sim], 1)[:, None]
    assert np.abs(raw.sum(0)).max() < 1e-9 * np.abs(raw).max()
    hit = t[:sc.n_sim] > 0
    assert np.all(np.isfinite(Fo[:sc.n_sim][hit]))
