"""The autotuner (pdipc_params.autotune): the launch configuration it picks by
timing candidates at initialize computes the same steps as the default one.

Every candidate runs the same iteration.  In the FP32 form (one accumulator per
row, in column order, in every persistent configuration and in the per-sweep
kernels) positions agree to float rounding of the last solve; in the mixed
form the band path splits a row's sum between own and halo entries where the
CTA boundaries fall, which the correction form absorbs (the defect it
iterates on is small), so positions agree to 1e-8 m.  A second context of the
same shape takes the cached choice without timing.
"""
import numpy as np
import pytest

import pdipc
from pdipc import scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,tol", [("fp32", 2e-6), ("mixed", 1e-8)])
def test_tuned_and_default_plans_give_the_same_steps(prec, tol, built_lib):
    sc = scenes.cloth_drop(96, 3, lg=10)
    ref = pdipc.Simulator(sc, prec)
    tuned = pdipc.Simulator(sc, prec, autotune=1)
    t = tuned.tuning()
    d = ref.tuning()
    assert d["autotuned"] == 0 and t["autotuned"] == 1 and t["from_cache"] == 0
    assert t["candidates_timed"] >= 2
    assert 0 < t["pd_solve_ms"] <= t["pd_default_ms"]
    assert 0 < t["collision_ms"] <= t["collision_default_ms"]
    # the tuning leaves the state where it was
    assert np.array_equal(tuned.positions(), ref.positions())
    ref.step(3)
    tuned.step(3)
    err = float(np.abs(tuned.positions() - ref.positions()).max())
    assert err < tol, (err, t)
    again = pdipc.Simulator(sc, prec, autotune=1)
    a = again.tuning()
    assert a["from_cache"] == 1
    for k in ("pd_rows_per_thread", "pd_ctas", "pd_band", "pd_l1_gather", "pd_local_sync", "cand_grid",
              "traverse_block", "expand_block"):
        assert a[k] == t[k], k
