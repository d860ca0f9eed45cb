"""Triangle strain limits and per-triangle stretch stiffness on the GPU,
through the C ABI (pdipc_add_cloth_ex), against the oracle.

  * the triangle strain limit (the reference's tet strain projection on a
    triangle's 3 x 2 deformation gradient, 3 x 3 SVD with the deformed normal
    appended): one outer iteration's solve from a stretched state within 1e-9 m
    (FP64), 1e-6 m (mixed, against the FP64 oracle) and 3e-5 m (FP32) of the
    oracle; 20 whole FP64 steps within 1e-6 m;
  * per-triangle stretch stiffness (a vertex's spring weight is the mean over
    its triangles): 10 whole FP64 steps within 1e-9 m of the oracle; its
    gradient (the adjoint's per-vertex stiffness gradient mapped through
    pdipc_stretch_gradient_per_triangle) against central differences of the
    per-triangle stiffnesses, 1e-4 relative.
"""
import numpy as np
import pytest

import pdipc
from oracle.oracle import FORM_JJ, Oracle
from pdipc import scenes

pytestmark = pytest.mark.gpu

ORACLE_PREC = {"fp32": "fp32", "fp64": "fp64", "mixed": "fp64"}


def strained_scene(n=24, k=2e3):
    sc = scenes.cloth_drop(n, 2, lg=10)
    sc.cloths[0].k_tri_strain = k
    return sc


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-9), ("mixed", 1e-6), ("fp32", 3e-5)])
def test_strain_limit_solve_matches_oracle(prec, tol, built_lib):
    sc = strained_scene()
    rng = np.random.default_rng(4)
    X = sc.initial_positions()
    n = sc.n_sim
    X[:n] *= np.array([1.004, 1.0, 0.997])          # stretch x, squeeze z: outside the [0.999, 1.001] band
    X[:n] += rng.uniform(-2e-4, 2e-4, (n, 3))
    V = rng.uniform(-0.05, 0.05, (n, 3))
    sim = pdipc.Simulator(sc, prec)
    xg = sim.stage_pd(X, V)[:n]
    xo = Oracle(sc, ORACLE_PREC[prec], FORM_JJ, threads=4).stage_pd(X, V)[:n]
    base = pdipc.Simulator(scenes.cloth_drop(24, 2, lg=10), prec).stage_pd(X, V)[:n]
    assert np.abs(xg - base).max() > 1e-5           # the constraint acts
    assert np.abs(xg - xo).max() < tol, np.abs(xg - xo).max()


def test_strain_limit_whole_steps_fp64(built_lib):
    sc = strained_scene(16)
    sim = pdipc.Simulator(sc, "fp64")
    orc = Oracle(sc, "fp64", FORM_JJ, threads=4)
    for _ in range(4):
        sim.step(5)
        orc.step(5)
        assert sim.stats()["last_outer_iters"] == orc.stats()["last_outer_iters"]
    assert np.abs(sim.positions() - orc.positions()).max() < 1e-6


def test_per_triangle_stretch_steps_fp64(built_lib):
    sc = scenes.cloth_drop(16, 2, lg=10)
    c = sc.cloths[0]
    c.tri_stretch = 10.0 ** (3.0 + 2.0 * np.random.default_rng(7).uniform(size=c.F.shape[0]))
    sim = pdipc.Simulator(sc, "fp64")
    orc = Oracle(sc, "fp64", FORM_JJ, threads=4)
    sim.step(10)
    orc.step(10)
    assert np.abs(sim.positions() - orc.positions()).max() < 1e-9


def test_per_triangle_stretch_gradient_matches_central_differences(built_lib):
    n_side, T = 10, 3
    rng = np.random.default_rng(21)
    base = scenes.cloth_drop(n_side, 1, with_sphere=False)
    nf = base.cloths[0].F.shape[0]
    kt = 10.0 ** (3.0 + 2.0 * rng.uniform(size=nf))

    def scene(k):
        sc = scenes.cloth_drop(n_side, 1, with_sphere=False)
        sc.cloths[0].tri_stretch = k
        return sc

    x0 = base.initial_positions()
    n = base.n_sim
    v0 = rng.uniform(-0.1, 0.1, (n, 3))
    target = x0 + rng.uniform(-0.05, 0.05, x0.shape)

    def loss_of(k):
        sim = pdipc.Simulator(scene(k), "fp64", fixed_outer=1)
        sim.set_state(x0, v0)
        sim.step(T)
        return float(0.5 * np.sum((sim.positions()[:n] - target[:n]) ** 2))

    sim = pdipc.Simulator(scene(kt), "fp64", fixed_outer=1)
    sim.set_state(x0, v0)
    sim.adjoint_record(1)
    sim.step(T)
    _, _, gk = sim.adjoint_backward(sim.positions()[:n] - target[:n])
    gtri = sim.stretch_gradient_per_triangle(gk)
    assert gtri.shape == (nf,) and np.all(np.isfinite(gtri))
    for trial in range(2):
        d = rng.normal(size=nf) * kt          # relative directions
        h = 1e-4

        def cd(s):
            return (loss_of(kt + s * d) - loss_of(kt - s * d)) / (2 * s)

        fd = (4.0 * cd(h / 2) - cd(h)) / 3.0
        ad = float(np.sum(gtri * d))
        assert abs(fd - ad) <= 1e-4 * max(abs(fd), abs(ad)), (trial, fd, ad)
