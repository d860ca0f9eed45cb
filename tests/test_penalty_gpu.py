"""The penalty / discrete-collision stages (PdIpcGpuFunc.cu:2933-3740) through
the C-ABI against the oracle: DC prediction, CCD penalty over the broad phase's
candidates, floor penalty and triangle-pair DCD penalty, each followed by the
averaging and velocity response.  Forces accumulate with atomics on the GPU
(any order) and in candidate order in the oracle: hit counts must be equal,
forces and velocities within 1e-9 relative."""
import numpy as np
import pytest

import pdipc
from oracle.oracle import FORM_JJ, Oracle
from pdipc import scenes
from pdipc.abi import PDIPC_ERR_ARG

from test_penalty_cpu import crossing_scene, face_pairs_with_overlapping_boxes

pytestmark = pytest.mark.gpu


def close(a, b, rel=1e-9):
    scale = max(1e-30, float(np.nanmax(np.abs(b))) if np.isfinite(b).any() else 1.0)
    np.testing.assert_allclose(a, b, rtol=rel, atol=rel * scale, equal_nan=True)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_prediction_and_floor(prec, built_lib):
    sc = scenes.cloth_drop(20, 2)
    sim = pdipc.Simulator(sc, prec)
    orc = Oracle(sc, prec, FORM_JJ, threads=4)
    rng = np.random.default_rng(11)
    X = sc.initial_positions()
    V = rng.uniform(-0.5, 0.5, (sc.n_sim, 3))
    s_g, v_g = sim.penalty_predict(X[:sc.n_sim], V)
    s_o, v_o = orc.penalty_predict(X[:sc.n_sim], V)
    close(s_g, s_o, 1e-12)
    close(v_g, v_o, 0)
    x = X.copy()
    x[:sc.n_sim, 1] = rng.uniform(-0.02, 0.01, sc.n_sim)
    for damping in (0.0, 0.5):
        F_g, t_g, V_g = sim.penalty_floor(x, 3e4, damping, V)
        F_o, t_o, V_o = orc.penalty_floor(x, 3e4, damping, V)
        np.testing.assert_array_equal(t_g, t_o)
        assert t_g.sum() > 0
        close(F_g, F_o)
        close(V_g, V_o)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_ccd_penalty_over_broad_phase_candidates(prec, built_lib):
    sc = scenes.cloth_drop(24, 3)
    sim = pdipc.Simulator(sc, prec)
    orc = Oracle(sc, prec, FORM_JJ, threads=4)
    X = sc.initial_positions().copy()
    top = X[sc.n_sim:, 1].max()
    X[:sc.n_sim, 1] += (top + 1.5e-3) - X[:sc.n_sim, 1].min()
    d = np.zeros_like(X)
    d[:sc.n_sim, 1] = -4e-3
    d[:sc.n_sim] += np.random.default_rng(3).uniform(-5e-4, 5e-4, (sc.n_sim, 3))
    _, pt, ee = sim.stage_broadphase(X, d)
    orc.broadphase(X, d)
    assert pt.shape[0] > 0 and ee.shape[0] > 0
    V = np.random.default_rng(8).uniform(-0.2, 0.2, (sc.n_sim, 3))
    for damping in (0.0, 0.2):
        F_g, t_g, V_g = sim.penalty_ccd(X, d, 1e4, damping, V)
        F_o, t_o, V_o = orc.penalty_ccd(X, d, 1e4, damping, V)
        np.testing.assert_array_equal(t_g, t_o)
        assert t_g[:sc.n_sim].sum() > 0
        close(F_g, F_o)
        close(V_g, V_o)


@pytest.mark.parametrize("split", [False, True])
def test_dcd_penalty_over_face_pairs(split, built_lib):
    sc, na, nb = crossing_scene(split)
    X = sc.initial_positions()
    F = np.concatenate([c.F + off for c, off in
                        zip(sc.cloths, np.cumsum([0] + [c.X.shape[0] for c in sc.cloths])[:-1])])
    pairs = face_pairs_with_overlapping_boxes(X, F, na, nb)
    V = np.random.default_rng(9).uniform(-0.1, 0.1, (sc.n_sim, 3))
    for prec in ("fp64", "mixed"):
        sim = pdipc.Simulator(sc, prec)
        orc = Oracle(sc, prec, FORM_JJ, threads=4)
        F_g, t_g, V_g = sim.penalty_dcd(X, pairs, 1e3, 2.5e3, 0.1, V)
        F_o, t_o, V_o = orc.penalty_dcd(X, pairs, 1e3, 2.5e3, 0.1, V)
        np.testing.assert_array_equal(t_g, t_o)
        assert t_g.sum() > 0
        close(F_g, F_o)
        close(V_g, V_o)


def test_dcd_rejects_face_indices_out_of_range(built_lib):
    sc, na, nb = crossing_scene(True)
    sim = pdipc.Simulator(sc, "fp64")
    with pytest.raises(pdipc.PdipcError) as e:
        sim.penalty_dcd(sc.initial_positions(), [[0, na + nb]], 1e3, 1e3, 0.0, np.zeros((sc.n_sim, 3)))
    assert e.value.status == PDIPC_ERR_ARG
