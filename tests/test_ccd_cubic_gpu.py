"""The FP64 coplanarity-cubic CCD on the GPU (pdipc_params.ccd_mode), through
the C ABI, against the oracle.

  * ccd_mode 2 (the cubic alone, in FP64 on the GPU in every precision mode):
    per-candidate first-contact times within 1e-9 relative of the oracle's,
    the same set of candidates in contact;
  * ccd_mode 0 (the reference's additive CCD) misses no contact the FP64 cubic
    finds, and is never later than it;
  * ccd_mode 1 (the cubic may lower the additive result) equals mode 0 here.
"""
import numpy as np
import pytest

import pdipc
from oracle.oracle import FORM_JJ, Oracle
from pdipc import scenes

pytestmark = pytest.mark.gpu


def setup():
    sc = scenes.cloth_drop(16, 2)
    X = sc.initial_positions()
    ns = sc.n_sim
    X[:ns, 1] += (X[ns:, 1].max() + 1.5e-3) - X[:ns, 1].min()
    dx = np.zeros_like(X)
    dx[:ns, 1] = -8e-3
    dx[:ns] += np.random.default_rng(3).uniform(-5e-4, 5e-4, (ns, 3))
    return sc, X, dx


def by_tuple(rows, vals):
    o = np.lexsort(np.asarray(rows).T[::-1])
    return np.asarray(rows)[o], np.asarray(vals)[o]


@pytest.mark.parametrize("prec", ["fp64", "mixed", "fp32"])
def test_cubic_times_of_impact_match_the_oracle(prec, built_lib):
    sc, X, dx = setup()
    sim = pdipc.Simulator(sc, prec, ccd_mode=2)
    _, pt, ee = sim.stage_broadphase(X, dx)
    tp, te, g = sim.stage_toi(X, X + dx, len(pt), len(ee))
    orc = Oracle(sc, "fp32" if prec == "fp32" else "fp64", FORM_JJ, threads=4, ccd_mode=2)
    _, opt, oee = orc.broadphase(X, dx)
    otp, ote, og = orc.toi(X, X + dx, len(opt), len(oee))
    for rows, mine, orows, ref in ((pt, tp, opt, otp), (ee, te, oee, ote)):
        r1, v1 = by_tuple(rows, mine)
        r2, v2 = by_tuple(orows, ref)
        assert np.array_equal(r1, r2)
        assert np.array_equal(v1 < 1.0, v2 < 1.0)
        np.testing.assert_allclose(v1, v2, rtol=1e-9, atol=0)
    assert (otp < 1).sum() + (ote < 1).sum() > 0
    assert abs(g - og) <= 1e-9 * og


def test_additive_ccd_misses_no_cubic_contact_on_the_gpu(built_lib):
    sc, X, dx = setup()
    acc = pdipc.Simulator(sc, "mixed")
    _, pt, ee = acc.stage_broadphase(X, dx)
    tp0, te0, g0 = acc.stage_toi(X, X + dx, len(pt), len(ee))
    cub = pdipc.Simulator(sc, "fp64", ccd_mode=2)
    _, cpt, cee = cub.stage_broadphase(X, dx)
    tpc, tec, gc = cub.stage_toi(X, X + dx, len(cpt), len(cee))
    r0, a0 = by_tuple(pt, tp0)
    rc, c0 = by_tuple(cpt, tpc)
    assert np.array_equal(r0, rc)
    hit = c0 < 1.0
    assert hit.sum() > 0 and np.all(a0[hit] < 1.0) and np.all(a0[hit] <= c0[hit])
    r1, a1 = by_tuple(ee, te0)
    rc1, c1 = by_tuple(cee, tec)
    assert np.array_equal(r1, rc1)
    hit = c1 < 1.0
    assert np.all(a1[hit] < 1.0) and np.all(a1[hit] <= c1[hit])
    # candidates come out of the broad phase in an order that may change from
    # run to run (atomic compaction): compare them by their vertex tuples
    one = pdipc.Simulator(sc, "mixed", ccd_mode=1)
    _, pt1, ee1 = one.stage_broadphase(X, dx)
    tp1, te1, g1 = one.stage_toi(X, X + dx, len(pt1), len(ee1))
    for rows, vals, rows1, vals1 in ((pt, tp0, pt1, tp1), (ee, te0, ee1, te1)):
        ra, va = by_tuple(rows, vals)
        rb, vb = by_tuple(rows1, vals1)
        assert np.array_equal(ra, rb) and np.array_equal(va, vb)
    assert g1 == g0
