"""The CUDA library (through the C ABI) against the reference's own kernels.

tests/golden/ref_kernels.npz holds outputs of the reference's PD-IPC kernels
run on the host from their sources (tests/golden/make_ref_fixtures.py).  The
library's stages must reproduce them:
  * FP64 mode vs the reference built with qeal = double: one outer
    iteration's solve within 1e-9 m (the library applies R2 as two Jacobi
    sweeps; the same linear map), times of impact within 1e-12 relative with
    the same clamping candidates, contact terms within 1e-12 relative;
  * FP32 mode vs the reference's float build: the solve within 3e-5 m
    (summation order moves one float solve ~1e-5 m), times of impact within
    1e-5 relative, contact terms within 2e-6;
  * mixed mode vs the double build: the solve within 1e-6 m; times of
    impact of the clamping candidates within 1e-6 relative.
"""
import os

import numpy as np
import pytest

import pdipc
from pdipc import scenes

pytestmark = pytest.mark.gpu

FIX = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_kernels.npz")
REF_OF = {"fp32": "fp32", "fp64": "fp64", "mixed": "fp64"}


@pytest.fixture(scope="module")
def fx():
    return dict(np.load(FIX))


def order(rows):
    return np.lexsort(np.asarray(rows).T[::-1])


@pytest.mark.parametrize("case", ["pd16", "pd20"])
@pytest.mark.parametrize("prec,tol", [("fp32", 3e-5), ("fp64", 1e-9), ("mixed", 1e-6)])
def test_pd_solve_matches_reference_kernels(fx, case, prec, tol, built_lib):
    n, s = int(fx[f"{case}_args"][0]), int(fx[f"{case}_args"][1])
    sc = scenes.cloth_drop(n, s, lg=10)
    sim = pdipc.Simulator(sc, prec)
    x = sim.stage_pd(fx[f"{case}_X"], fx[f"{case}_V"])[:sc.n_sim]
    ref = fx[f"{case}_x_{REF_OF[prec]}"]
    assert np.abs(x - ref).max() < tol, np.abs(x - ref).max()


@pytest.mark.parametrize("prec,rtol", [("fp32", 1e-5), ("fp64", 1e-12), ("mixed", 1e-6)])
def test_time_of_impact_matches_reference_kernels(fx, prec, rtol, built_lib):
    n, s = (int(v) for v in fx["coll_args"])
    sc = scenes.cloth_drop(n, s)
    sim = pdipc.Simulator(sc, prec)
    X, dx = fx["toi_X"], fx["toi_dx"]
    _, pt, ee = sim.stage_broadphase(X, dx)
    rpt, ree = fx["toi_pt"], fx["toi_ee"]
    ig, ir = order(pt), order(rpt)
    jg, jr = order(ee), order(ree)
    assert np.array_equal(pt[ig], rpt[ir]) and np.array_equal(ee[jg], ree[jr])
    tp, te, g = sim.stage_toi(X, X + dx, len(pt), len(ee))
    ref = fx[f"toi_per_{REF_OF[prec]}"]
    rp, re_ = ref[:len(rpt)][ir], ref[len(rpt):][jr]
    mp, me = tp[ig], te[jg]
    # no impact the reference finds is missed
    assert np.all(mp[rp < 1] < 1) and np.all(me[re_ < 1] < 1)
    if prec == "mixed":   # the mixed mode evaluates in FP64 only the candidates that clamp
        np.testing.assert_allclose(mp[rp < 1], rp[rp < 1], rtol=rtol, atol=0)
        np.testing.assert_allclose(me[re_ < 1], re_[re_ < 1], rtol=rtol, atol=0)
    else:
        np.testing.assert_allclose(mp, rp, rtol=rtol, atol=0)
        np.testing.assert_allclose(me, re_, rtol=rtol, atol=0)
    rg = float(fx[f"toi_global_{REF_OF[prec]}"])
    assert abs(g - rg) <= rtol * rg


@pytest.mark.parametrize("prec,tol", [("fp32", 2e-6), ("fp64", 1e-12), ("mixed", 1e-6)])
def test_contact_terms_match_reference_kernels(fx, prec, tol, built_lib):
    n, s = (int(v) for v in fx["coll_args"])
    sc = scenes.cloth_drop(n, s)
    sim = pdipc.Simulator(sc, prec)
    Xc = fx["contact_X"]
    sim.stage_broadphase(Xc, np.zeros_like(Xc))
    diag, rhs, active = sim.stage_contact(Xc)
    rd, rr = fx[f"contact_diag_{REF_OF[prec]}"], fx[f"contact_rhs_{REF_OF[prec]}"]
    assert active > 0
    np.testing.assert_allclose(diag, rd, rtol=tol, atol=tol * np.abs(rd).max())
    np.testing.assert_allclose(rhs, rr, rtol=tol, atol=tol * np.abs(rr).max())
