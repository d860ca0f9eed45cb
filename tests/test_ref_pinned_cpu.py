"""The oracle against the reference's own kernels (no GPU needed).

tests/golden/ref_kernels.npz holds outputs of the reference's PD-IPC kernels
(Simulator/PD-IPC/PdIpcGpuFunc.cu, compiled for the host by
oracle/build_ref.py, run by tests/golden/make_ref_fixtures.py) in the
reference's float configuration and its double one, on small seeded inputs:
one outer iteration's projective-dynamics solve, per-candidate and global
times of impact, and the contact diagonal and right-hand side.  The oracle
restates those kernels; here it reproduces them:
  * double: the same arithmetic in another summation order (the reference
    adds the bending terms and contact terms with atomics, the oracle in
    ascending source order) -> positions within 1e-12 m, times of impact and
    contact terms within 1e-12 relative, the same set of clamping candidates;
  * float: the reference's own configuration -> positions within 2e-5 m (one
    solve of 150 float Jacobi sweeps; summation order alone moves it ~1e-5 m),
    times of impact within 1e-5 relative, contact terms within 1e-6.
When the reference tree is present (PDIPC_REFERENCE_DIR), the last test also
rebuilds the reference kernels and checks the fixture is what they give now.
"""
import os

import numpy as np
import pytest

from oracle.oracle import FORM_JJ, FORM_R2, Oracle
from pdipc import scenes

FIX = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_kernels.npz")
PD_TOL = {"fp32": 2e-5, "fp64": 1e-12}
TOI_RTOL = {"fp32": 1e-5, "fp64": 1e-12}
CONTACT_RTOL = {"fp32": 1e-6, "fp64": 1e-12}


@pytest.fixture(scope="module")
def fx():
    return dict(np.load(FIX))


def coll_scene(fx):
    n, s = (int(v) for v in fx["coll_args"])
    return scenes.cloth_drop(n, s)


@pytest.mark.parametrize("case", ["pd16", "pd20"])
@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("form", [FORM_R2, FORM_JJ])
def test_pd_solve_matches_reference_kernels(fx, case, prec, form):
    n, s = int(fx[f"{case}_args"][0]), int(fx[f"{case}_args"][1])
    sc = scenes.cloth_drop(n, s, lg=10)
    x = Oracle(sc, prec, form, threads=4).stage_pd(fx[f"{case}_X"], fx[f"{case}_V"])[:sc.n_sim]
    ref = fx[f"{case}_x_{prec}"]
    moved = np.abs(ref - fx[f"{case}_X"][:sc.n_sim]).max()
    assert moved > 1e-4                       # the solve does move the cloth
    tol = PD_TOL[prec] * (2 if form == FORM_JJ and prec == "fp32" else 1)
    assert np.abs(x - ref).max() < tol, np.abs(x - ref).max()


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_time_of_impact_matches_reference_kernels(fx, prec):
    sc = coll_scene(fx)
    orc = Oracle(sc, prec, FORM_JJ, threads=4)
    X, dx = fx["toi_X"], fx["toi_dx"]
    _, pt, ee = orc.broadphase(X, dx)
    assert np.array_equal(pt, fx["toi_pt"]) and np.array_equal(ee, fx["toi_ee"])
    tp, te, g = orc.toi(X, X + dx, len(pt), len(ee))
    mine = np.concatenate([tp, te])
    ref = fx[f"toi_per_{prec}"]
    assert (ref < 1).sum() > 10
    assert np.array_equal(mine < 1, ref < 1)      # no impact missed, none invented
    np.testing.assert_allclose(mine, ref, rtol=TOI_RTOL[prec], atol=0)
    assert abs(g - float(fx[f"toi_global_{prec}"])) <= TOI_RTOL[prec] * g


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_contact_terms_match_reference_kernels(fx, prec):
    sc = coll_scene(fx)
    orc = Oracle(sc, prec, FORM_JJ, threads=4)
    Xc = fx["contact_X"]
    _, pt, ee = orc.broadphase(Xc, np.zeros_like(Xc))
    assert np.array_equal(pt, fx["contact_pt"]) and np.array_equal(ee, fx["contact_ee"])
    diag, rhs, active = orc.contact(Xc)
    rd, rr = fx[f"contact_diag_{prec}"], fx[f"contact_rhs_{prec}"]
    assert active > 0 and np.count_nonzero(rd) > 0
    tol = CONTACT_RTOL[prec]
    np.testing.assert_allclose(diag, rd, rtol=tol, atol=tol * np.abs(rd).max())
    np.testing.assert_allclose(rhs, rr, rtol=tol, atol=tol * np.abs(rr).max())


def test_fixture_is_what_the_reference_kernels_give(fx, tmp_path):
    """Regenerates the fixture from the reference sources (skipped where the
    reference tree is absent) and compares it with the committed one."""
    from oracle import refkern
    if not refkern.available():
        pytest.skip("reference tree not present (PDIPC_REFERENCE_DIR)")
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    script = os.path.join(root, "tests", "golden", "make_ref_fixtures.py")
    env = dict(os.environ)
    out = tmp_path / "ref_kernels.npz"
    code = ("import runpy, sys; sys.argv=['x']; m = runpy.run_path(%r, run_name='fx'); m['OUT'] = %r; "
            "import types; g = m['main'].__globals__; g['OUT'] = %r; m['main']()" % (script, str(out), str(out)))
    r = subprocess.run([sys.executable, "-c", code], cwd=root, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    new = dict(np.load(out))
    assert sorted(new) == sorted(fx)
    for k in fx:
        assert np.array_equal(new[k], fx[k]), k
