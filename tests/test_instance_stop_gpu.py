"""Per-instance stopping (pdipc_params.instance_stop) on a batch of
independent drops.

The reference stops the outer loop of a step on one test over every vertex
of the scene (PdIpcSimulator.cpp:1776): in a batch, the instances' residuals
add up, so the batch runs more outer iterations than any instance would on
its own.  With instance_stop each simulated model takes the same test on its
own vertices, clamps its step by its own time of impact, and skips its sweeps
once it has stopped.  A batch stepped that way must equal each instance
stepped alone as its own scene (the same kernels: one launch per sweep on
both sides), position for position, with the same outer-iteration counts.
"""
import numpy as np
import pytest

import pdipc
from pdipc import scenes
from pdipc.abi import PDIPC_ERR_STATE

pytestmark = pytest.mark.gpu

# mixed: FP32 sums and float atomics of the contact pass in another order (the
# batch's candidates interleave the instances'), compounding over the steps
# after first contact (2.5e-5 m seen after 60 steps, with equal outer counts
# every step); the accuracy bar of the mixed form is 1e-4 m.  The FP64 form
# pins the logic to round-off.
TOL = {"fp64": 1e-10, "mixed": 1e-4}


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_batch_with_instance_stop_equals_each_instance_alone(prec, built_lib):
    sc = scenes.batched(6, 8, 20, seed=3, steps=60)
    steps = 60  # through first contact with the spheres
    batch = pdipc.Simulator(sc, prec, instance_stop=1, persistent=0)
    assert batch.stats()["pd_path"] == 0 and batch.stats()["instances"] == 6
    alone = [pdipc.Simulator(scenes.instance_slice(sc, k, k + 1), prec, persistent=0) for k in range(6)]
    contact = False
    for s in range(steps):
        batch.step(1)
        work = 0
        for one in alone:
            one.step(1)
            work += one.stats()["last_outer_iters"]
            contact = contact or one.stats()["active_contacts"] > 0 or one.stats()["last_toi"] < 1.0
        st = batch.stats()
        assert st["instance_outer_iters"] == work, (s, st["instance_outer_iters"], work)
        assert st["last_outer_iters"] == max(one.stats()["last_outer_iters"] for one in alone)
    xb = batch.positions()
    ns = [c.X.shape[0] for c in sc.cloths]
    off = 0
    for k, one in enumerate(alone):
        xa = one.positions()[:ns[k]]
        assert np.abs(xb[off:off + ns[k]] - xa).max() <= TOL[prec], (k, np.abs(xb[off:off + ns[k]] - xa).max())
        off += ns[k]
    assert contact


def test_instance_stop_saves_work_against_the_global_rule(built_lib):
    """The reference's rule over the whole batch (its residuals summed) runs
    at least as many outer iterations per instance as each instance's own
    rule, and more once the sum crosses the threshold the parts do not."""
    sc = scenes.batched(16, 16, 32, seed=5, steps=40)
    glob = pdipc.Simulator(sc, "mixed", persistent=0)
    inst = pdipc.Simulator(sc, "mixed", instance_stop=1)
    wg = wi = 0
    for _ in range(20):
        glob.step(1)
        inst.step(1)
        wg += glob.stats()["instance_outer_iters"]
        wi += inst.stats()["instance_outer_iters"]
    assert wi <= wg
    assert wi < wg


def test_adjoint_refuses_instance_stop(built_lib):
    sim = pdipc.Simulator(scenes.batched(2, 8, 10, seed=1), "fp64", instance_stop=1)
    with pytest.raises(pdipc.PdipcError) as e:
        sim.adjoint_record(1)
    assert e.value.status == PDIPC_ERR_STATE
