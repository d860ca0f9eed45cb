"""Parity of the CUDA library (through the C ABI) against the CPU oracle.

Tolerances:
  * integer outputs (Morton codes, sort order, patch pairs, point-triangle and
    edge-edge candidate sets) must be bit-exact;
  * FP64 mode: positions within 1e-9 m of the FP64 oracle per stage and within
    1e-5 m after whole runs with contact;
  * FP32 mode: one PD solve within 2e-5 m of the FP32 oracle (the reference's
    own float Jacobi drifts ~1e-5 m per step from FP64, so FP32 runs are compared
    over a few steps only); time of impact within 1e-5 relative;
  * mixed mode (FP64 state, FP32 local step and sweeps on the correction,
    FP64 CCD refinement and contact) is checked against the FP64 oracle: time
    of impact within 1e-6 relative, positions within 1e-4 m after whole runs.
"""
import numpy as np
import pytest

import pdipc
from oracle.oracle import FORM_JJ, FORM_R2, Oracle
from pdipc import scenes

pytestmark = pytest.mark.gpu


def small_scene(n=24, s=3, **kw):
    return scenes.cloth_drop(n, s, **kw)


# the oracle run each library mode is held to
ORACLE_PREC = {"fp32": "fp32", "fp64": "fp64", "mixed": "fp64"}


def near_contact_state(scene, gap):
    """Rest positions with the cloth lowered so its lowest point sits `gap`
    above the sphere's top vertex."""
    X = np.concatenate([c.X for c in scene.cloths] + [st.X for st in scene.statics])
    ns = scene.n_sim
    top = X[ns:, 1].max()
    X[:ns, 1] += (top + gap) - X[:ns, 1].min()
    return X


def sort_rows(a):
    return a[np.lexsort(a.T[::-1])] if a.size else a


@pytest.mark.parametrize("config", ["c1", "c2"])
def test_patch_order_is_a_stable_sort_at_full_size(config, built_lib):
    """The onesweep radix sort over many partitions (c1: about 303 k patches, c2:
    several hundred thousand over 512 meshes): the patch order equals a stable
    sort of the Morton codes, ties in patch order."""
    sc = scenes.config1() if config == "c1" else scenes.config2()
    sim = pdipc.Simulator(sc, "mixed")
    npatch = sim.stats()["n_patches"]
    assert npatch > 100000
    codes, order = sim.stage_morton(npatch)
    assert np.array_equal(order, np.argsort(codes, kind="stable"))


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_morton_codes_and_order_bitexact(prec, built_lib):
    sc = small_scene()
    sim = pdipc.Simulator(sc, prec)
    orc = Oracle(sc, prec, FORM_JJ, threads=4)
    npatch = sim.stats()["n_patches"]
    c_gpu, o_gpu = sim.stage_morton(npatch)
    c_orc, o_orc = orc.morton(npatch)
    assert np.array_equal(c_gpu, c_orc)
    assert np.array_equal(o_gpu, o_orc)


@pytest.mark.parametrize("prec", ["fp32", "fp64", "mixed"])
def test_broadphase_candidate_sets_bitexact(prec, built_lib):
    sc = small_scene()
    sim = pdipc.Simulator(sc, prec)
    orc = Oracle(sc, prec, FORM_JJ, threads=4)
    X = near_contact_state(sc, 2e-3)
    rng = np.random.default_rng(7)
    dx = np.zeros_like(X)
    dx[:sc.n_sim] = rng.uniform(-3e-3, 3e-3, (sc.n_sim, 3))
    pg, tg, eg = sim.stage_broadphase(X, dx)
    po, to, eo = orc.broadphase(X, dx)
    assert pg.shape == po.shape and tg.shape == to.shape and eg.shape == eo.shape
    assert np.array_equal(sort_rows(pg), sort_rows(po))
    assert np.array_equal(sort_rows(tg), sort_rows(to))
    assert np.array_equal(sort_rows(eg), sort_rows(eo))
    assert tg.shape[0] > 1000 and eg.shape[0] > 1000


@pytest.mark.parametrize("prec,rtol", [("fp32", 1e-5), ("fp64", 1e-12), ("mixed", 1e-6)])
def test_time_of_impact_matches(prec, rtol, built_lib):
    sc = small_scene()
    sim = pdipc.Simulator(sc, prec)
    orc = Oracle(sc, ORACLE_PREC[prec], FORM_JJ, threads=4)
    X = near_contact_state(sc, 1.5e-3)
    dx = np.zeros_like(X)
    dx[:sc.n_sim, 1] = -4e-3           # drive the cloth into the sphere
    rng = np.random.default_rng(3)
    dx[:sc.n_sim] += rng.uniform(-5e-4, 5e-4, (sc.n_sim, 3))
    pg, tg, eg = sim.stage_broadphase(X, dx)
    po, to, eo = orc.broadphase(X, dx)
    X1 = X + dx
    tpg, teg, gg = sim.stage_toi(X, X1, tg.shape[0], eg.shape[0])
    tpo, teo, go = orc.toi(X, X1, to.shape[0], eo.shape[0])
    # match candidates by their vertex tuples
    ig, io = np.lexsort(tg.T[::-1]), np.lexsort(to.T[::-1])
    jg, jo = np.lexsort(eg.T[::-1]), np.lexsort(eo.T[::-1])
    if prec == "mixed":   # only candidates that clamp are evaluated in FP64; compare those
        m = tpo[io] < 1.0
        np.testing.assert_allclose(tpg[ig][m], tpo[io][m], rtol=rtol, atol=0)
        m = teo[jo] < 1.0
        np.testing.assert_allclose(teg[jg][m], teo[jo][m], rtol=rtol, atol=0)
    else:
        np.testing.assert_allclose(tpg[ig], tpo[io], rtol=rtol, atol=0)
        np.testing.assert_allclose(teg[jg], teo[jo], rtol=rtol, atol=0)
    assert go < 1.0
    assert abs(gg - go) <= rtol * go
    # no impact the oracle finds is missed: every candidate it clamps is clamped here
    assert np.all(tpg[ig][tpo[io] < 1.0] < 1.0)
    assert np.all(teg[jg][teo[jo] < 1.0] < 1.0)


@pytest.mark.parametrize("prec,tol", [("fp32", 2e-6), ("fp64", 1e-12), ("mixed", 1e-6)])
def test_contact_projection_matches(prec, tol, built_lib):
    sc = small_scene()
    sim = pdipc.Simulator(sc, prec)
    orc = Oracle(sc, ORACLE_PREC[prec], FORM_JJ, threads=4)
    X = near_contact_state(sc, 4e-4)
    sim.stage_broadphase(X, np.zeros_like(X))
    orc.broadphase(X, np.zeros_like(X))
    dg, rg, ng = sim.stage_contact(X)
    do, ro, no = orc.contact(X)
    assert ng == no and no > 0
    scale = np.abs(do).max()
    np.testing.assert_allclose(dg, do, rtol=tol, atol=tol * scale)
    np.testing.assert_allclose(rg, ro, rtol=tol, atol=tol * np.abs(ro).max())


@pytest.mark.parametrize("prec,atol", [("fp32", 2e-5), ("fp64", 1e-10), ("mixed", 1e-6)])
def test_pd_solve_matches(prec, atol, built_lib):
    sc = small_scene(32, 2)
    sim = pdipc.Simulator(sc, prec)
    orc = Oracle(sc, ORACLE_PREC[prec], FORM_JJ, threads=4)
    X = np.concatenate([c.X for c in sc.cloths] + [s.X for s in sc.statics])
    rng = np.random.default_rng(11)
    V = rng.uniform(-0.1, 0.1, (sc.n_sim, 3))
    xg = sim.stage_pd(X, V)
    xo = orc.stage_pd(X, V)
    assert np.abs(xg - xo).max() < atol
    if prec == "fp64":   # the reference's own R2-operator form gives the same solve
        xr = Oracle(sc, "fp64", FORM_R2, threads=4).stage_pd(X, V)
        assert np.abs(xg - xr).max() < 1e-9
    # the state is untouched by the stage call
    assert np.array_equal(sim.positions(), X.astype(np.float32).astype(np.float64) if prec == "fp32" else X)


def test_fp64_run_with_contact_matches_oracle(built_lib):
    """Whole steps in FP64 (the plain FP64 GPU form) through contact: within 1e-5 m."""
    sc = scenes.cloth_drop(24, 3, height=-0.185, lg=10)  # starts 15 mm above the sphere
    sim = pdipc.Simulator(sc, "fp64")
    orc = Oracle(sc, "fp64", FORM_JJ, threads=8)
    worst = 0.0
    contacts = 0
    for k in range(6):
        sim.step(10)
        orc.step(10)
        worst = max(worst, np.abs(sim.positions() - orc.positions()).max())
        contacts = max(contacts, orc.stats()["active_contacts"])
        assert sim.stats()["last_outer_iters"] == orc.stats()["last_outer_iters"]
    assert contacts > 0
    assert worst < 1e-5, worst


def test_mixed_run_with_contact_within_1e4_of_fp64(built_lib):
    """The correction (mixed-precision) form stays within 1e-4 m of the FP64 oracle
    through contact, and converges in as few outer iterations."""
    sc = scenes.cloth_drop(24, 3, height=-0.185, lg=10)
    sim = pdipc.Simulator(sc, "mixed")
    orc = Oracle(sc, "fp64", FORM_JJ, threads=8)
    worst = 0.0
    for k in range(6):
        sim.step(10)
        orc.step(10)
        worst = max(worst, np.abs(sim.positions() - orc.positions()).max())
    assert orc.stats()["active_contacts"] > 0
    assert worst < 1e-4, worst


def test_broadphase_full_size_bitexact(built_lib):
    """512x512 cloth + subdivision-6 sphere at rest: the candidate sets of the
    library's LBVH and the oracle's heap tree are identical."""
    sc = scenes.config1()
    sim = pdipc.Simulator(sc, "fp32")
    orc = Oracle(sc, "fp32", FORM_JJ, threads=16)
    X = np.concatenate([c.X for c in sc.cloths] + [s.X for s in sc.statics])
    rng = np.random.default_rng(0)
    dx = np.zeros_like(X)
    dx[:sc.n_sim] = rng.uniform(-2e-4, 2e-4, (sc.n_sim, 3))
    pg, tg, eg = sim.stage_broadphase(X, dx)
    po, to, eo = orc.broadphase(X, dx)
    assert sim.stats()["n_patches"] == orc.stats()["n_patches"]
    assert np.array_equal(sort_rows(pg), sort_rows(po))
    assert np.array_equal(sort_rows(tg), sort_rows(to))
    assert np.array_equal(sort_rows(eg), sort_rows(eo))


def test_fp32_steps_match_oracle_short_horizon(built_lib):
    sc = small_scene(32, 3)
    sim = pdipc.Simulator(sc, "fp32")
    orc = Oracle(sc, "fp32", FORM_JJ, threads=8)
    sim.step(3)
    orc.step(3)
    assert np.abs(sim.positions() - orc.positions()).max() < 1e-4


@pytest.mark.parametrize("prec,atol", [("fp32", 2e-5), ("mixed", 1e-6)])
@pytest.mark.parametrize("n", [16, 37, 48, 160])
@pytest.mark.parametrize("variant", [1, 2, 3, 4])
def test_persistent_solve_matches_per_sweep_launches(prec, atol, n, variant, built_lib):
    """One cooperative launch per outer iteration (neighbour synchronisation or
    grid barriers; sweeps gathering from the shared-memory band, through L1 or
    L2 only) gives the same PD solve as one launch per sweep.  At 48 and 160 a
    CTA's rows reach several CTAs on each side; 37 x 37 = 1369 rows end in a
    partial 64-row window of the solve's slot order."""
    sc = small_scene(n, 2)
    a = pdipc.Simulator(sc, prec, persistent=variant)
    b = pdipc.Simulator(sc, prec, persistent=0)
    assert a.stats()["pd_path"] in (1, 2, 3) and b.stats()["pd_path"] == 0
    # the band (path 3) is the default persistent path of the mixed mode only
    assert (a.stats()["pd_path"] == 3) == (variant == 1 and prec == "mixed")
    X = np.concatenate([c.X for c in sc.cloths] + [s.X for s in sc.statics])
    V = np.random.default_rng(5).uniform(-0.1, 0.1, (sc.n_sim, 3))
    assert np.abs(a.stage_pd(X, V) - b.stage_pd(X, V)).max() < atol
    a.step(4)
    b.step(4)
    assert np.abs(a.positions() - b.positions()).max() < 10 * atol


@pytest.mark.parametrize("which", ["stack", "batched"])
def test_mixed_persistent_solve_on_multi_cloth_scenes(which, built_lib):
    """Several cloths in one context: three equal layers (the band path: CTA
    blocks and halos cross cloth boundaries) and uneven batched instances
    (whichever persistent path their offset patterns allow) give the same
    mixed-precision PD solve and steps as one launch per sweep."""
    if which == "stack":
        sc = scenes.stack(3, 24, 3, gap=2e-3, lg=10, steps=30, dhat=5e-4, drop=3e-3)
    else:
        sc = scenes.batched(6, 8, 20, seed=3, steps=60)
    a = pdipc.Simulator(sc, "mixed")
    b = pdipc.Simulator(sc, "mixed", persistent=0)
    assert a.stats()["pd_path"] in (1, 2, 3) and b.stats()["pd_path"] == 0
    if which == "stack":
        assert a.stats()["pd_path"] == 3
    X = sc.initial_positions()
    V = np.random.default_rng(6).uniform(-0.1, 0.1, (sc.n_sim, 3))
    assert np.abs(a.stage_pd(X, V) - b.stage_pd(X, V)).max() < 1e-6
    a.step(5)
    b.step(5)
    assert np.abs(a.positions() - b.positions()).max() < 1e-5


def test_graph_and_plain_launches_agree(built_lib):
    sc = small_scene(16, 2)
    a = pdipc.Simulator(sc, "fp64", use_graphs=1)
    b = pdipc.Simulator(sc, "fp64", use_graphs=0)
    a.step(5)
    b.step(5)
    assert np.array_equal(a.positions(), b.positions())


def test_checkpoint_roundtrip_and_reset(tmp_path, built_lib):
    sc = small_scene(16, 2)
    sim = pdipc.Simulator(sc, "fp32")
    sim.step(4)
    path = str(tmp_path / "frame_0004.dat")
    sim.save(path)
    x4, v4 = sim.positions(), sim.velocities()
    sim.step(3)
    sim.load(path)
    assert np.array_equal(sim.positions(), x4)
    assert np.array_equal(sim.velocities(), v4)
    raw = np.fromfile(path, dtype=np.int64, count=2)
    assert raw.tolist() == [3, sc.n_total]       # EigenMatrixIO header: rows, cols
    sim.reset()
    X = np.concatenate([c.X for c in sc.cloths] + [s.X for s in sc.statics])
    assert np.abs(sim.positions() - X).max() < 1e-6
    assert np.all(sim.velocities() == 0)


def test_nonfinite_state_is_reported(built_lib):
    sc = small_scene(8, 1)
    sim = pdipc.Simulator(sc, "fp32")
    X = sim.positions()
    X[3, 1] = np.nan
    sim.set_state(X)
    with pytest.raises(pdipc.PdipcError) as ei:
        sim.step(1)
    assert ei.value.status == pdipc.abi.PDIPC_ERR_NONFINITE


def test_animate_returns_positions_and_counts_launches(built_lib):
    sc = small_scene(16, 2)
    sim = pdipc.Simulator(sc, "fp32")
    out = sim.animate()
    assert out.shape == (sc.n_total, 3) and np.isfinite(out).all()
    st = sim.stats()
    assert st["kernel_launches"] > 10 and st["steps_done"] == 1
