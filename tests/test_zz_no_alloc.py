"""The no-allocation time-of-impact entry point (pdipc_stage_toi_noalloc)
against the allocating one (pdipc_stage_toi) on the same context.

Collected last (file name) so it also runs after every other GPU test has used
the device; it passes on its own as well.
"""
import numpy as np
import pytest

import pdipc
from pdipc import scenes
from pdipc.abi import PDIPC_ERR_ARG, PDIPC_ERR_OVERFLOW

pytestmark = pytest.mark.gpu


def near_contact_state(scene, gap):
    X = np.concatenate([c.X for c in scene.cloths] + [st.X for st in scene.statics])
    ns = scene.n_sim
    top = X[ns:, 1].max()
    X[:ns, 1] += (top + gap) - X[:ns, 1].min()
    return X


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_noalloc_toi_matches_stage_toi_twice(prec, built_lib):
    sc = scenes.cloth_drop(24, 3)
    sim = pdipc.Simulator(sc, prec)
    X = near_contact_state(sc, 1.5e-3)
    dx = np.zeros_like(X)
    dx[:sc.n_sim, 1] = -4e-3
    dx[:sc.n_sim] += np.random.default_rng(3).uniform(-5e-4, 5e-4, (sc.n_sim, 3))
    _, pt, ee = sim.stage_broadphase(X, dx)
    assert pt.shape[0] > 0 and ee.shape[0] > 0
    X1 = X + dx
    tp, te, tg = sim.stage_toi(X, X1, pt.shape[0], ee.shape[0])
    assert tg < 1.0
    for _ in range(2):  # two calls in a row through the same scratch
        tp2, te2, tg2 = sim.stage_toi_noalloc(X, X1, pt.shape[0], ee.shape[0])
        np.testing.assert_allclose(tp2, tp, rtol=1e-12, atol=0)
        np.testing.assert_allclose(te2, te, rtol=1e-12, atol=0)
        assert abs(tg2 - tg) <= 1e-12 * tg


def test_noalloc_toi_rejects_fp32_mode(built_lib):
    sc = scenes.cloth_drop(16, 2)
    sim = pdipc.Simulator(sc, "fp32")
    X = np.concatenate([c.X for c in sc.cloths] + [st.X for st in sc.statics])
    sim.stage_broadphase(X, np.zeros_like(X))
    with pytest.raises(pdipc.PdipcError) as e:
        sim.stage_toi_noalloc(X, X, 0, 0, per_candidate=False)
    assert e.value.status == PDIPC_ERR_ARG


def test_noalloc_toi_rejects_candidate_sets_beyond_its_scratch(built_lib):
    sc = scenes.config1()                      # 512x512 cloth: ~2e7 candidates at rest
    sim = pdipc.Simulator(sc, "mixed")
    sim.step(1)
    st = sim.stats()
    assert st["pt_candidates"] + st["ee_candidates"] > (1 << 20)
    x = sim.positions()
    with pytest.raises(pdipc.PdipcError) as e:
        sim.stage_toi_noalloc(x, x, 0, 0, per_candidate=False)
    assert e.value.status == PDIPC_ERR_OVERFLOW
    assert "exceed" in pdipc.load_library().pdipc_last_error(sim.h).decode()
