"""Persistent PD solve in launch groups, with per-instance stopping inside it.

A plan with more CTAs than the device holds at once (config 2: 256 drops,
1.6 M rows) runs as one cooperative launch per group of whole instances;
models share no matrix entry or stencil, so a group never waits for a CTA
outside it.  A CTA whose rows span two groups runs in both launches, each
time for its own rows.  Every row is still summed by the same CTA in the
same order, so splitting a small batch into small groups
(params.pd_group_ctas) must give the same bits as one launch.  Per-instance
stopping (params.instance_stop) takes stopped instances' rows out of the
persistent solve; against the per-sweep solve under the same rule the
positions agree to the FP32 sums' round-off.
"""
import numpy as np
import pytest

import pdipc
from pdipc import scenes

pytestmark = pytest.mark.gpu


def _batch(steps=40):
    return scenes.batched(12, 20, 48, seed=7, steps=steps)


@pytest.mark.parametrize("stop", [0, 1])
def test_groups_give_the_bits_of_one_launch(stop, built_lib):
    sc = _batch()
    one = pdipc.Simulator(sc, "mixed", autotune=0, instance_stop=stop)
    grp = pdipc.Simulator(sc, "mixed", autotune=0, instance_stop=stop, pd_group_ctas=32)
    t1, tg = one.tuning(), grp.tuning()
    assert t1["pd_rows_per_thread"] > 0 and t1["pd_launches"] == 1
    assert tg["pd_launches"] > 2, tg
    assert (tg["pd_rows_per_thread"], tg["pd_ctas"], tg["pd_band"]) == (t1["pd_rows_per_thread"], t1["pd_ctas"],
                                                                         t1["pd_band"])
    # before first contact the step is free of float atomics: equal bits
    for k in range(10):
        one.step(1)
        grp.step(1)
        assert one.stats()["active_contacts"] == 0
        assert one.stats()["last_outer_iters"] == grp.stats()["last_outer_iters"], k
        assert one.stats()["instance_outer_iters"] == grp.stats()["instance_outer_iters"], k
        assert np.array_equal(one.positions(), grp.positions()), k
    # through contact the contact pass sums in float atomics, whose order varies
    # from run to run and compounds over the steps: the mixed form's 1e-4 m bar
    worst = 0.0
    for _ in range(30):
        one.step(1)
        grp.step(1)
        worst = max(worst, float(np.abs(one.positions() - grp.positions()).max()))
    assert worst < 1e-4, worst
    assert grp.stats()["pd_solves"] > 0


def test_instance_stop_persistent_against_per_sweep(built_lib):
    sc = _batch()
    per = pdipc.Simulator(sc, "mixed", autotune=0, instance_stop=1, persistent=0)
    grp = pdipc.Simulator(sc, "mixed", autotune=0, instance_stop=1, pd_group_ctas=32)
    assert per.stats()["pd_path"] == 0 and grp.stats()["pd_path"] > 0
    worst = 0.0
    for k in range(20):
        per.step(1)
        grp.step(1)
        assert per.stats()["instance_outer_iters"] == grp.stats()["instance_outer_iters"], k
        worst = max(worst, float(np.abs(per.positions() - grp.positions()).max()))
    assert worst < 1e-4, worst


def test_config2_all_256_instances_in_launch_groups(built_lib):
    sc = scenes.config2()
    grp = pdipc.Simulator(sc, "mixed", autotune=0, instance_stop=1)
    per = pdipc.Simulator(sc, "mixed", autotune=0, instance_stop=1, persistent=0)
    t = grp.tuning()
    # more offset patterns than parameter space holds: each CTA's own table in shared memory
    assert t["pd_rows_per_thread"] > 0 and t["pd_launches"] > 1 and t["pd_band"] == 1, t
    worst = 0.0
    for k in range(3):
        grp.step(1)
        per.step(1)
        assert grp.stats()["instance_outer_iters"] == per.stats()["instance_outer_iters"], k
        worst = max(worst, float(np.abs(grp.positions() - per.positions()).max()))
    assert worst < 1e-5, worst
