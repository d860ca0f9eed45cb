"""The CPU oracle on its own: internal consistency checks that need no GPU."""
import itertools

import numpy as np
import pytest

from oracle.oracle import FORM_JJ, FORM_R2, Oracle, mesh_topology
from pdipc import scenes


@pytest.fixture(scope="module")
def small():
    return scenes.cloth_drop(12, 2, steps=10)


def test_r2_form_equals_two_sweep_form_in_fp64(small):
    """The reference's materialised R2 operator (path tables) and the library's
    two weighted-Jacobi sweeps are the same linear map: FP64 trajectories agree
    to rounding."""
    a = Oracle(small, "fp64", FORM_R2, threads=2)
    b = Oracle(small, "fp64", FORM_JJ, threads=2)
    a.step(25)
    b.step(25)
    assert np.abs(a.positions() - b.positions()).max() < 1e-10


def test_thread_count_does_not_change_results(small):
    a = Oracle(small, "fp32", FORM_JJ, threads=1)
    b = Oracle(small, "fp32", FORM_JJ, threads=4)
    a.step(10)
    b.step(10)
    assert np.array_equal(a.positions(), b.positions())


def _patch_lists(scene):
    """Global patch face/point/edge lists rebuilt from per-mesh topology."""
    faces, edges, pf, pp, pe, st = [], [], [], [], [], []
    vo = fo = eo = 0
    for models, is_static in ((scene.cloths, False), (scene.statics, True)):
        for m in models:
            e, patches, owned_pts, owned_edges = mesh_topology(m.X, m.F, m.patch_dim)
            faces.append(m.F + vo)
            edges.append(e + vo)
            for p in patches:
                pf.append(p + fo)
                pp.append(np.unique(np.concatenate([owned_pts[f] for f in p]).astype(np.int64)) + vo)
                pe.append(np.unique(np.concatenate([owned_edges[f] for f in p]).astype(np.int64)) + eo)
                st.append(is_static)
            vo += m.X.shape[0]
            fo += m.F.shape[0]
            eo += e.shape[0]
    return np.concatenate(faces), np.concatenate(edges), pf, pp, pe, st


def test_broadphase_equals_brute_force(small):
    """Tree traversal + expansion == all overlapping patch pairs by brute force."""
    o = Oracle(small, "fp64", FORM_JJ, threads=2, inflation_radius=5e-3)
    X = np.concatenate([c.X for c in small.cloths] + [s.X for s in small.statics])
    rng = np.random.default_rng(1)
    dx = np.zeros_like(X)
    dx[:small.n_sim] = rng.uniform(-0.02, 0.02, (small.n_sim, 3))
    X[:small.n_sim, 1] -= 0.18  # bring the cloth near the sphere top
    pairs, pt, ee = o.broadphase(X, dx)
    faces, edges, pf, pp, pe, st = _patch_lists(small)
    infl = 5e-3
    lo, hi = [], []
    for p in pf:
        v = faces[p].reshape(-1)
        a, b = X[v], X[v] + dx[v]
        lo.append(np.minimum(a, b).min(0) - infl)
        hi.append(np.maximum(a, b).max(0) + infl)
    lo, hi = np.array(lo), np.array(hi)
    exp = []
    for a, b in itertools.combinations(range(len(pf)), 2):
        if st[a] and st[b]:
            continue
        if np.all(hi[a] >= lo[b]) and np.all(hi[b] >= lo[a]):
            exp.append((a, b))
    got = sorted(map(tuple, pairs.tolist()))
    assert got == exp
    exp_pt, exp_ee = [], []
    for a, b in exp:
        exp_pt += [(v, *faces[f]) for v in pp[a] for f in pf[b]]
        exp_pt += [(v, *faces[f]) for v in pp[b] for f in pf[a]]
        exp_ee += [(*edges[x], *edges[y]) for x in pe[a] for y in pe[b]]
    assert sorted(map(tuple, pt.tolist())) == sorted(exp_pt)
    assert sorted(map(tuple, ee.tolist())) == sorted(exp_ee)
    assert len(exp_pt) > 0 and len(exp_ee) > 0


def test_ccd_stops_a_point_before_a_triangle():
    """A vertex driven through a static triangle is stopped short of it; a
    vertex moving away gets the full step."""
    X, F = scenes.grid_cloth(2, side=0.1, jitter=0.0)       # 4 verts, 2 faces, at y=0
    tri_X = np.array([[0.0, -0.01, 0.0], [0.1, -0.01, 0.0], [0.0, -0.01, 0.1]])
    tri_F = np.array([[0, 1, 2]], np.int32)
    sc = scenes.Scene("ccd", [scenes.ClothSpec(X, F, np.array([], np.int32), patch_dim=1)],
                      [scenes.StaticSpec(tri_X, tri_F, patch_dim=1)])
    o = Oracle(sc, "fp64", FORM_JJ, threads=1)
    x0 = np.concatenate([X, tri_X])
    x1 = x0.copy()
    x1[0] = [0.02, -0.03, 0.02]   # vertex 0 crosses the plane y = -0.01
    pairs, pt, ee = o.broadphase(x0, x1 - x0)
    tp, te, g = o.toi(x0, x1, pt.shape[0], ee.shape[0])
    assert 0.0 < g < 0.98 * 0.5 + 1e-12          # plane crossed at 1/3 of the motion, times 0.98
    xc = x0 + g * (x1 - x0)
    assert xc[0, 1] > -0.01
    x1[0] = [0.02, 0.05, 0.02]
    _, _, g2 = o.toi(x0, x1, pt.shape[0], ee.shape[0])
    assert g2 == 1.0


def test_contact_pushes_apart_with_barrier_weight():
    X, F = scenes.grid_cloth(2, side=0.1, jitter=0.0)
    tri_X = np.array([[-0.05, -0.0005, -0.05], [0.2, -0.0005, -0.05], [-0.05, -0.0005, 0.2]])
    tri_F = np.array([[0, 1, 2]], np.int32)
    sc = scenes.Scene("contact", [scenes.ClothSpec(X, F, np.array([], np.int32), patch_dim=1)],
                      [scenes.StaticSpec(tri_X, tri_F, patch_dim=1)], dhat=1e-3)
    o = Oracle(sc, "fp64", FORM_JJ, threads=1)
    x = np.concatenate([X, tri_X])
    o.broadphase(x, np.zeros_like(x))
    diag, rhs, na = o.contact(x)
    assert na >= 4                                   # each cloth vertex is 5e-4 above the static triangle
    d2, dh2 = 0.0005 ** 2, 1e-6
    bar = -1e4 * (d2 - dh2) ** 2 * np.log(d2 / dh2) / dh2 ** 2
    w = diag[0]
    assert w > bar
    target = rhs[0] / w
    assert target[1] > x[0, 1] - 1e-12               # pushed up (away from the triangle)
