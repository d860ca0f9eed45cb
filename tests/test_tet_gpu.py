"""Volumetric (tetrahedral) models on the GPU against the CPU oracle: the
strain projection (the library's Jacobi/Givens SVD vs the oracle's one-sided
Jacobi SVD) inside whole steps, alone and with a cloth, in every precision
mode."""
import numpy as np
import pytest

import pdipc
from oracle.oracle import FORM_JJ, Oracle
from pdipc import scenes

pytestmark = pytest.mark.gpu


def run_against(scene, prec, oracle_prec, steps, every, threads=8, check_outer=True):
    sim = pdipc.Simulator(scene, prec)
    orc = Oracle(scene, oracle_prec, FORM_JJ, threads=threads)
    # FP64 solves launch per sweep; FP32 and mixed ones run the persistent kernel,
    # which projects the tets in its curvature phase
    assert (sim.stats()["pd_path"] == 0) == (prec == "fp64")
    worst, contacts = 0.0, 0
    for _ in range(steps // every):
        sim.step(every)
        orc.step(every)
        if check_outer:
            assert sim.stats()["last_outer_iters"] == orc.stats()["last_outer_iters"]
        contacts = max(contacts, orc.stats()["active_contacts"])
        worst = max(worst, float(np.abs(sim.positions() - orc.positions()).max()))
    return worst, contacts


def test_block_drop_fp64_matches_oracle(built_lib):
    worst, contacts = run_against(scenes.block_drop(3, 2), "fp64", "fp64", 40, 10)
    assert contacts > 0
    assert worst < 1e-9, worst


def test_block_drop_mixed_within_1e4_of_fp64_oracle(built_lib):
    worst, contacts = run_against(scenes.block_drop(3, 2), "mixed", "fp64", 40, 10)
    assert contacts > 0
    assert worst < 1e-4, worst


def test_block_drop_fp32_short_horizon(built_lib):
    worst, _ = run_against(scenes.block_drop(3, 2), "fp32", "fp32", 3, 1, check_outer=False)
    assert worst < 1e-4, worst


def test_block_on_cloth_fp64_matches_oracle(built_lib):
    """A tet block falling onto a pinned cloth draped above the sphere: tets,
    cloth and static mesh in one context, contact between all three.  The
    block pressing the cloth onto the sphere amplifies rounding fast (the
    contact sums are float atomics, so two GPU runs differ at 1e-16 and part by
    1e-6 to 3e-5 m within 30 steps), so each step is checked from the oracle's
    own state, and the free run against the mixed-mode bar."""
    sc = scenes.block_drop(3, 2, cloth_n=16)
    sim = pdipc.Simulator(sc, "fp64")
    orc = Oracle(sc, "fp64", FORM_JJ, threads=8)
    one_step, contacts = 0.0, 0
    for k in range(30):
        sim.set_state(orc.positions(), orc.velocities())
        sim.step(1)
        orc.step(1)
        assert sim.stats()["last_outer_iters"] == orc.stats()["last_outer_iters"], k
        contacts = max(contacts, orc.stats()["active_contacts"])
        one_step = max(one_step, float(np.abs(sim.positions() - orc.positions()).max()))
    assert contacts > 0
    assert one_step < 1e-9, one_step
    worst, _ = run_against(sc, "fp64", "fp64", 30, 10, check_outer=False)
    assert worst < 1e-4, worst


def test_block_pd_solve_matches_oracle(built_lib):
    sc = scenes.block_drop(4, 2)
    X = np.concatenate([c.X for c in sc.cloths] + [v.X for v in sc.solids] + [s.X for s in sc.statics])
    V = np.random.default_rng(2).uniform(-0.5, 0.5, (sc.n_sim, 3))
    for prec, atol in (("fp64", 1e-10), ("mixed", 1e-6)):
        xg = pdipc.Simulator(sc, prec).stage_pd(X, V)
        xo = Oracle(sc, "fp64", FORM_JJ, threads=8).stage_pd(X, V)
        assert np.abs(xg - xo).max() < atol, (prec, np.abs(xg - xo).max())


@pytest.mark.parametrize("prec,atol", [("fp32", 2e-5), ("mixed", 1e-6)])
@pytest.mark.parametrize("with_cloth", [False, True])
def test_persistent_solve_with_tets_matches_per_sweep_launches(prec, atol, with_cloth, built_lib):
    """The persistent kernel's tet projections (curvature phase, one CTA per
    tet) and their gathers give the per-sweep path's PD solve, alone and with a
    cloth in the same context."""
    sc = scenes.block_drop(3, 2, cloth_n=16) if with_cloth else scenes.block_drop(4, 2)
    a = pdipc.Simulator(sc, prec)
    b = pdipc.Simulator(sc, prec, persistent=0)
    assert a.stats()["pd_path"] in (1, 2, 3) and b.stats()["pd_path"] == 0
    X = sc.initial_positions()
    V = np.random.default_rng(12).uniform(-0.2, 0.2, (sc.n_sim, 3))
    assert np.abs(a.stage_pd(X, V) - b.stage_pd(X, V)).max() < atol
    a.step(3)
    b.step(3)
    assert np.abs(a.positions() - b.positions()).max() < 10 * atol
