"""Discrete adjoint of recorded contact-free rollouts (plain FP64 form) through
the C-ABI, against central finite differences of the same forward.

The adjoint is the exact derivative of the executed iteration (every
local-global iteration, sweep and Chebyshev step), so with the outer-iteration
count fixed, central differences converge to it quadratically in their step:
1e-4 relative is the bar.  The forward is strongly curved (the local step
normalises spring and curvature vectors, and a short curvature vector turns
fast), so the steps are taken where the differences have converged: measured
on a GB300, one step of the 128x128 cloth, positions: relative difference
2e-2 at 1e-5, 3.4e-3 at 1e-6, 3.4e-5 at 1e-7; velocities 6e-4 at 1e-4, 6e-6 at
1e-5.  Over five steps of that cloth the differences still move by 2.6e-2
between 1e-7 and 1e-6, and over 50 they do not settle above FP64 round-off,
so the 50-step differentiable-rollout workload (128x128 cloth with the 64x64
drop's material, checkpoints every 10 steps, loss = squared distance of the
final positions to seeded targets, wrapped in a torch.autograd.Function here
only) is checked for the checkpointed replay reproducing the every-step
gradient exactly, and its one-step gradient against differences.  A ladder
of solver settings (local-global iterations x Chebyshev steps x outer
iterations) isolates the recurrences on a 10x10 cloth."""
import numpy as np
import pytest

import pdipc
from pdipc import scenes
from pdipc.abi import PDIPC_ERR_STATE

pytestmark = pytest.mark.gpu


def free_cloth(n, k_stretch=1e4, lg=10):
    """A cloth with two corners pinned and no obstacle (no contact)."""
    return scenes.cloth_drop(n, 1, with_sphere=False, k_stretch=k_stretch, lg=lg)


def make(sc, **kw):
    return pdipc.Simulator(sc, "fp64", **kw)


def rollout(sim, x0, v0, T, every=0):
    sim.set_state(x0, v0)
    if every:
        sim.adjoint_record(every)
    sim.step(T)
    return sim.positions()[:sim.n_sim].copy(), sim.velocities().copy()


def rel(a, b):
    return abs(a - b) / max(abs(a), abs(b), 1e-300)


@pytest.mark.parametrize("lg,cheby,outer", [(1, 1, 1), (1, 3, 1), (2, 4, 1), (10, 15, 2)])
def test_adjoint_matches_central_differences(lg, cheby, outer, built_lib):
    sc = free_cloth(10, lg=lg)
    kw = dict(cheby_iterations=cheby, fixed_outer=outer)
    sim = make(sc, **kw)
    rng = np.random.default_rng(lg * 100 + cheby)
    n, T = sc.n_sim, 3
    x0 = sc.initial_positions()
    v0 = rng.uniform(-0.1, 0.1, (n, 3))
    cx, cv = rng.normal(size=(n, 3)), rng.normal(size=(n, 3))
    target = x0 + rng.uniform(-0.05, 0.05, x0.shape)

    def loss(x, v):
        return float(np.sum(cx * x) + np.sum(cv * v) + 0.5 * np.sum((x - target) ** 2))

    x, v = rollout(sim, x0, v0, T, every=2)
    gx0, gv0, gk = sim.adjoint_backward(cx + (x - target), cv)
    assert np.all(np.isfinite(gx0)) and np.all(np.isfinite(gv0)) and np.all(np.isfinite(gk))
    # the backward pass leaves the state where the rollout ended
    np.testing.assert_array_equal(sim.positions()[:n], x)
    for trial in range(3):
        d = rng.normal(size=(n, 3))
        ev = 1e-5
        fd = (loss(*rollout(sim, x0, v0 + ev * d, T)) - loss(*rollout(sim, x0, v0 - ev * d, T))) / (2 * ev)
        assert rel(fd, np.sum(gv0 * d)) < 1e-4, ("v", trial, fd, np.sum(gv0 * d))
        ex = 1e-7
        fd = (loss(*rollout(sim, x0 + ex * d, v0, T)) - loss(*rollout(sim, x0 - ex * d, v0, T))) / (2 * ex)
        assert rel(fd, np.sum(gx0 * d)) < 1e-4, ("x", trial, fd, np.sum(gx0 * d))
    # the model's stretch stiffness sets every vertex's strain weight.  dL/dk is
    # small at k = 1e4 (about 6e-8 here), so the step stays at 1e-4 k, where
    # the rebuilt contexts' round-off is negligible, and Richardson
    # extrapolation of two central differences removes their h^2 error
    k = sc.cloths[0].k_stretch

    def cd(h):
        lp = loss(*rollout(make(free_cloth(10, k + h, lg), **kw), x0, v0, T))
        lm = loss(*rollout(make(free_cloth(10, k - h, lg), **kw), x0, v0, T))
        return (lp - lm) / (2 * h)

    h = 2e-4 * k
    fd = (4.0 * cd(h / 2) - cd(h)) / 3.0
    assert rel(fd, float(gk.sum())) < 1e-4, ("k", fd, float(gk.sum()))


def test_adjoint_entry_points_refuse_what_they_do_not_cover(built_lib):
    sc = free_cloth(8)
    mixed = pdipc.Simulator(sc, "mixed")
    with pytest.raises(pdipc.PdipcError) as e:
        mixed.adjoint_record(1)
    assert e.value.status == PDIPC_ERR_STATE
    sim = make(sc, fixed_outer=1)
    g = np.zeros((sc.n_sim, 3))
    with pytest.raises(pdipc.PdipcError) as e:
        sim.adjoint_backward(g)  # nothing recorded
    assert e.value.status == PDIPC_ERR_STATE
    sim.adjoint_record(1)
    sim.step(1)
    sim.set_state(sc.initial_positions())  # ends the recording
    with pytest.raises(pdipc.PdipcError) as e:
        sim.adjoint_backward(g)
    assert e.value.status == PDIPC_ERR_STATE
    # a step with contact: a cloth resting on the sphere
    drop = scenes.cloth_drop(12, 1)
    X = drop.initial_positions().copy()
    top = X[drop.n_sim:, 1].max()
    X[:drop.n_sim, 1] += top + 5e-4 - X[:drop.n_sim, 1].min()
    c = make(drop, fixed_outer=1)
    c.set_state(X, np.zeros((drop.n_sim, 3)))
    c.adjoint_record(1)
    c.step(2)
    with pytest.raises(pdipc.PdipcError) as e:
        c.adjoint_backward(np.ones((drop.n_sim, 3)))
    assert e.value.status == PDIPC_ERR_STATE


def test_differentiable_rollout_128_cloth_50_steps(built_lib):
    torch = pytest.importorskip("torch")
    sc = free_cloth(128)
    sim = make(sc, fixed_outer=3)
    n = sc.n_sim
    rng = np.random.default_rng(3)
    x0 = sc.initial_positions()
    target = torch.from_numpy(x0 + rng.uniform(-0.05, 0.05, x0.shape))
    v0 = rng.uniform(-0.1, 0.1, (n, 3))

    class Rollout(torch.autograd.Function):
        """The rollout as a differentiable function of the initial velocity."""

        @staticmethod
        def forward(ctx, v, steps, every):
            x, _ = rollout(sim, x0, v.detach().numpy(), steps, every=every)
            return torch.from_numpy(x)

        @staticmethod
        def backward(ctx, gx):
            gx0, gv0, gk = sim.adjoint_backward(gx.detach().numpy())
            Rollout.grads = (gx0, gv0, gk)
            return torch.from_numpy(gv0), None, None

    def grad_v(steps, every):
        v = torch.tensor(v0, requires_grad=True)
        loss = ((Rollout.apply(v, steps, every) - target) ** 2).sum()
        loss.backward()
        return v.grad.numpy().copy(), Rollout.grads

    # 50 steps, checkpoints every 10: the replayed segments give the gradient
    # of the every-step recording bit for bit
    g10, (gx10, _, gk10) = grad_v(50, 10)
    g1, (gx1, _, gk1) = grad_v(50, 1)
    assert np.all(np.isfinite(g10)) and np.abs(g10).max() > 0
    np.testing.assert_array_equal(g10, g1)
    np.testing.assert_array_equal(gx10, gx1)
    np.testing.assert_array_equal(gk10, gk1)
    # one step: against central differences where they have converged
    gv, (gx, _, _) = grad_v(1, 1)

    def L(xx, vv):
        x, _ = rollout(sim, xx, vv, 1)
        return float(np.sum((x - target.numpy()) ** 2))

    for trial in range(4):
        d = rng.uniform(-1.0, 1.0, (n, 3))
        ev = 1e-6
        fd = (L(x0, v0 + ev * d) - L(x0, v0 - ev * d)) / (2 * ev)
        assert rel(fd, float(np.sum(gv * d))) < 1e-4, ("v", trial, fd, float(np.sum(gv * d)))
        ex = 1e-8
        fd = (L(x0 + ex * d, v0) - L(x0 - ex * d, v0)) / (2 * ex)
        assert rel(fd, float(np.sum(gx * d))) < 1e-4, ("x", trial, fd, float(np.sum(gx * d)))


def test_adjoint_matches_the_oracle_restatement(built_lib):
    """The GPU adjoint against the oracle's sequential restatement of the same
    reverse pass on the same rollout (10x10 cloth, 10 local-global iterations x
    15 Chebyshev steps x 2 outer iterations, 3 steps): every gradient within
    1e-5 of the oracle's, norm-relative (both agree with central differences
    to about 1e-7)."""
    from oracle.oracle import FORM_JJ, Oracle

    sc = free_cloth(10)
    kw = dict(cheby_iterations=15, fixed_outer=2)
    sim = make(sc, **kw)
    orc = Oracle(sc, "fp64", FORM_JJ, threads=4, **kw)
    rng = np.random.default_rng(21)
    n, T = sc.n_sim, 3
    x0 = sc.initial_positions()
    v0 = rng.uniform(-0.1, 0.1, (n, 3))
    gx, gv = rng.normal(size=(n, 3)), rng.normal(size=(n, 3))
    rollout(sim, x0, v0, T, every=2)
    ours = sim.adjoint_backward(gx, gv)
    ref = orc.adjoint_rollout(T, x0, v0, gx, gv)
    for name, a, b in zip(("x0", "v0", "k"), ours, ref):
        assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(b), (name, np.linalg.norm(a - b), np.linalg.norm(b))


def test_adjoint_matches_the_oracle_on_the_128_cloth_50_steps(built_lib):
    """Config 3's rollout shape (128x128 cloth, 50 steps, checkpoints every 10,
    10 local-global iterations x 15 Chebyshev steps x 3 outer iterations): the
    GPU adjoint against the oracle's sequential restatement of the same reverse
    pass, every gradient within 1e-5 of the oracle's, norm-relative.  The
    oracle's adjoint is itself tied to its forward-mode tangent (the transpose
    identity to round-off, tests/test_adjoint_cpu.py), which is the check that
    holds at this length where central differences of the forward do not."""
    import os

    from oracle.oracle import FORM_JJ, Oracle

    sc = free_cloth(128)
    kw = dict(fixed_outer=3)
    sim = make(sc, **kw)
    orc = Oracle(sc, "fp64", FORM_JJ, threads=os.cpu_count() or 8, **kw)
    rng = np.random.default_rng(8)
    n, T = sc.n_sim, 50
    x0 = sc.initial_positions()
    v0 = rng.uniform(-0.1, 0.1, (n, 3))
    gx, gv = rng.normal(size=(n, 3)), rng.normal(size=(n, 3))
    rollout(sim, x0, v0, T, every=10)
    ours = sim.adjoint_backward(gx, gv)
    ref = orc.adjoint_rollout(T, x0, v0, gx, gv)
    for name, a, b in zip(("x0", "v0", "k"), ours, ref):
        assert np.all(np.isfinite(a)) and np.linalg.norm(b) > 0
        assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(b), (name, np.linalg.norm(a - b), np.linalg.norm(b))


def strained_cloth(n=10):
    """free_cloth with the triangle strain limit on every triangle."""
    sc = free_cloth(n)
    sc.cloths[0].k_tri_strain = 2e3
    return sc


def tet_scene():
    """A 2x2x2 tet block, one corner vertex pinned, no obstacle."""
    X, T = scenes.tet_block(2, 2, 2, size=(0.1, 0.1, 0.1))
    solid = scenes.SolidSpec(X, T, np.array([0], np.int32), density=500.0, k_strain=2e3, patch_dim=2)
    return scenes.Scene("tet_adjoint", [], [], solids=[solid], lg_iterations=4, steps=10)


@pytest.mark.parametrize("which", ["triangle", "tet"])
def test_adjoint_through_strain_limits_matches_central_differences(which, built_lib):
    """The strain-limit projections (the clamped 3x3 SVD of every triangle's
    or tet's deformation gradient) in the reverse pass: gradients with respect
    to initial positions and velocities against central differences of the GPU
    forward, with initial velocities large enough that most elements' singular
    values leave [0.999, 1.001] and are clamped."""
    sc = strained_cloth() if which == "triangle" else tet_scene()
    kw = dict(cheby_iterations=5, fixed_outer=2)
    sim = make(sc, **kw)
    rng = np.random.default_rng(31 if which == "triangle" else 37)
    n, T = sc.n_sim, 3
    x0 = sc.initial_positions()
    v0 = rng.uniform(-0.3, 0.3, (n, 3))
    cx, cv = rng.normal(size=(n, 3)), rng.normal(size=(n, 3))

    def loss(x, v):
        return float(np.sum(cx * x) + np.sum(cv * v))

    x, v = rollout(sim, x0, v0, T, every=2)
    gx0, gv0, _ = sim.adjoint_backward(cx, cv)
    assert np.all(np.isfinite(gx0)) and np.all(np.isfinite(gv0))
    for trial in range(3):
        d = rng.normal(size=(n, 3))
        ev = 1e-6
        fd = (loss(*rollout(sim, x0, v0 + ev * d, T)) - loss(*rollout(sim, x0, v0 - ev * d, T))) / (2 * ev)
        assert rel(fd, np.sum(gv0 * d)) < 1e-4, ("v", trial, fd, np.sum(gv0 * d))
        ex = 1e-8
        fd = (loss(*rollout(sim, x0 + ex * d, v0, T)) - loss(*rollout(sim, x0 - ex * d, v0, T))) / (2 * ex)
        assert rel(fd, np.sum(gx0 * d)) < 1e-4, ("x", trial, fd, np.sum(gx0 * d))


@pytest.mark.parametrize("which", ["triangle", "tet"])
def test_adjoint_through_strain_limits_matches_the_oracle(which, built_lib):
    """The GPU's element adjoint (k_adj_elem: its own SVD, svd3.cuh) against the
    oracle's restatement (one-sided Jacobi SVD; the clamped projection is a
    spectral function of F, so both give the same derivative to round-off),
    norm-relative within 1e-6."""
    from oracle.oracle import FORM_JJ, Oracle

    sc = strained_cloth() if which == "triangle" else tet_scene()
    kw = dict(cheby_iterations=5, fixed_outer=2)
    sim = make(sc, **kw)
    orc = Oracle(sc, "fp64", FORM_JJ, threads=4, **kw)
    rng = np.random.default_rng(41)
    n, T = sc.n_sim, 3
    x0 = sc.initial_positions()
    v0 = rng.uniform(-0.3, 0.3, (n, 3))
    gx, gv = rng.normal(size=(n, 3)), rng.normal(size=(n, 3))
    rollout(sim, x0, v0, T, every=1)
    ours = sim.adjoint_backward(gx, gv)
    ref = orc.adjoint_rollout(T, x0, v0, gx, gv)
    for name, a, b in zip(("x0", "v0"), ours[:2], ref[:2]):
        assert np.linalg.norm(a - b) <= 1e-6 * np.linalg.norm(b), (name, np.linalg.norm(a - b), np.linalg.norm(b))


def test_config3_central_differences_converge_to_the_adjoint(built_lib):
    """Config 3 as specified (128x128 cloth, 50 steps, checkpoints every 10,
    per-triangle stretch stiffness log-uniform in [1e3, 1e5], initial velocity
    uniform +/-0.1 m/s, loss = squared distance of the final positions to the
    initial grid displaced by +/-0.05 m), with three outer iterations per step
    so that the rollout is smooth.  Central differences along seeded
    directions do not converge at the specified step of 1e-4 (measured on a
    GB300: median relative difference 0.75 for velocity directions, 0.10 for
    relative stiffness directions): the rollout is strongly curved.  They
    approach the adjoint as the step shrinks (velocity 0.42 at 1e-5, 0.015 at
    1e-6; stiffness 0.005 at 1e-5), which is what is checked here."""
    rng = np.random.default_rng(2024)

    def scene(kt):
        sc = free_cloth(128)
        sc.cloths[0].tri_stretch = kt.copy()
        return sc

    nf = free_cloth(128).cloths[0].F.shape[0]
    kt = 10.0 ** (3.0 + 2.0 * rng.uniform(size=nf))
    sc = scene(kt)
    n, T = sc.n_sim, 50
    x0 = sc.initial_positions()
    v0 = rng.uniform(-0.1, 0.1, (n, 3))
    target = x0 + rng.uniform(-0.05, 0.05, x0.shape)
    sim = make(sc, fixed_outer=3)

    def L(s, vv):
        x, _ = rollout(s, x0, vv, T)
        return float(np.sum((x - target) ** 2))

    x, _ = rollout(sim, x0, v0, T, every=10)
    _, gv0, gk = sim.adjoint_backward(2.0 * (x - target))
    gkt = sim.stretch_gradient_per_triangle(gk)

    def v_err(eps, t):
        d = np.random.default_rng(100 + t).uniform(-1, 1, (n, 3))
        fd = (L(sim, v0 + eps * d) - L(sim, v0 - eps * d)) / (2 * eps)
        return rel(fd, float(np.sum(gv0 * d)))

    def k_err(eps, t):
        d = np.random.default_rng(200 + t).uniform(-1, 1, nf)
        lp = L(make(scene(kt * (1 + eps * d)), fixed_outer=3, autotune=0), v0)
        lm = L(make(scene(kt * (1 - eps * d)), fixed_outer=3, autotune=0), v0)
        return rel((lp - lm) / (2 * eps), float(np.sum(gkt * kt * d)))

    v_coarse = np.median([v_err(1e-4, t) for t in range(4)])
    v_fine = np.median([v_err(1e-6, t) for t in range(4)])
    assert v_fine < v_coarse and v_fine < 0.05, (v_coarse, v_fine)
    k_fine = [k_err(1e-5, t) for t in range(4)]
    assert np.median(k_fine) < 1e-2 and max(k_fine) < 3e-2, k_fine
