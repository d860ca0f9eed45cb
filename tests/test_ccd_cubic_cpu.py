"""The FP64 coplanarity-cubic CCD on the oracle (pdipc_params.ccd_mode).

ccd_mode 2 gives every candidate's exact first-contact time in FP64: the
roots in [0, 1] of the cubic "the four points are coplanar", the first at
which the primitives touch.  It is the FP64 CCD oracle the reference's
additive CCD (PdIpcGpuFunc.cu:2460-2607, ccd_mode 0) is held to: no contact it
finds may be missed, and the additive CCD, which stops short by its gap, may
only be earlier.  ccd_mode 1 lets the cubic lower the additive CCD's result,
which on these inputs changes nothing.  At each cubic contact time the point
lies in the triangle's plane and inside it.
"""
import numpy as np

from oracle.oracle import FORM_JJ, Oracle
from pdipc import scenes


def near_contact_state(scene, gap):
    X = scene.initial_positions()
    ns = scene.n_sim
    top = X[ns:, 1].max()
    X[:ns, 1] += (top + gap) - X[:ns, 1].min()
    return X


def setup():
    sc = scenes.cloth_drop(16, 2)
    X = near_contact_state(sc, 1.5e-3)
    dx = np.zeros_like(X)
    dx[:sc.n_sim, 1] = -8e-3
    dx[:sc.n_sim] += np.random.default_rng(3).uniform(-5e-4, 5e-4, (sc.n_sim, 3))
    return sc, X, dx


def tois(sc, X, dx, **kw):
    orc = Oracle(sc, "fp64", FORM_JJ, threads=2, **kw)
    _, pt, ee = orc.broadphase(X, dx)
    tp, te, g = orc.toi(X, X + dx, len(pt), len(ee))
    return pt, ee, tp, te, g


def test_additive_ccd_misses_no_contact_the_fp64_cubic_finds():
    sc, X, dx = setup()
    pt, ee, tp0, te0, g0 = tois(sc, X, dx)                 # the reference's additive CCD
    _, _, tpc, tec, gc = tois(sc, X, dx, ccd_mode=2)       # exact FP64 first contacts
    hit = np.concatenate([tpc, tec]) < 1.0
    accd = np.concatenate([tp0, te0])
    cubic = np.concatenate([tpc, tec])
    assert hit.sum() > 0
    assert np.all(accd[hit] < 1.0)                         # none missed
    assert np.all(accd[hit] <= cubic[hit])                 # and never past the contact
    assert g0 <= gc
    # every point-triangle contact time: in the plane and inside the triangle
    for i in np.nonzero(tpc < 1.0)[0]:
        p, a, b, c = (X[v] + tpc[i] * dx[v] for v in pt[i])
        n = np.cross(b - a, c - a)
        scale = np.linalg.norm(n) * max(np.linalg.norm(b - a), np.linalg.norm(c - a))
        assert abs(np.dot(p - a, n)) <= 1e-9 * scale
        bary = [np.dot(np.cross(b - p, c - p), n), np.dot(np.cross(c - p, a - p), n), np.dot(np.cross(a - p, b - p), n)]
        assert min(bary) >= -1e-5 * np.dot(n, n)


def test_cubic_can_only_lower_the_additive_result():
    sc, X, dx = setup()
    _, _, tp0, te0, g0 = tois(sc, X, dx)
    _, _, tp1, te1, g1 = tois(sc, X, dx, ccd_mode=1)
    assert np.all(tp1 <= tp0) and np.all(te1 <= te0)
    assert np.array_equal(tp1, tp0) and np.array_equal(te1, te0) and g1 == g0
