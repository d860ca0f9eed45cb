"""Device-side wait limits of the persistent solve, made to run out on purpose.

The persistent solve runs an outer iteration's whole projective-dynamics solve
in one cooperative launch whose CTAs wait on one another (neighbour flags, a
grid barrier, bulk halo copies on an mbarrier).  Every such wait is bounded by
pdipc_params.wait_limit_us.  Here the limit is set to 1 us, far below a phase,
so some wait gives up: the step must return PDIPC_ERR_CUDA (no fault, no hang),
and once the limit is back at its default the same context must step again and
match an untouched context bit for bit.  The failure is made by the limit
alone: nothing faults, traps or spins without bound.
"""
import numpy as np
import pytest

import pdipc
from pdipc import scenes
from pdipc.abi import PDIPC_ERR_CUDA

pytestmark = pytest.mark.gpu


# (precision, persistent mode, the PD path the context must take)
CASES = [
    ("fp32", 3, 1),   # grid barriers, L1 gathers, matrix from shared memory or L2
    ("fp32", 4, 1),   # neighbour waits, L1 gathers
    ("mixed", 1, 3),  # neighbour waits plus the band's bulk halo copies (sync warp)
]


@pytest.mark.parametrize("prec,mode,path", CASES)
def test_short_wait_limit_fails_cleanly_and_context_recovers(prec, mode, path, built_lib):
    sc = scenes.cloth_drop(96, 3, lg=10)
    X0 = sc.initial_positions()
    ref = pdipc.Simulator(sc, prec, persistent=mode)
    sim = pdipc.Simulator(sc, prec, persistent=mode)
    st = sim.stats()
    assert st["pd_path"] >= 1 and st["pd_ctas"] > 1, st
    if path == 3:
        assert st["pd_path"] == 3, st
    ref.step(2)

    sim.set_wait_limit(1)
    with pytest.raises(pdipc.PdipcError) as e:
        sim.step(1)
    assert e.value.status == PDIPC_ERR_CUDA
    assert "timed out" in str(e.value)

    # the context (and the CUDA context under it) stays usable
    sim.set_wait_limit(0)
    sim.set_state(X0, np.zeros((sim.n_sim, 3)))
    sim.step(2)
    assert np.array_equal(sim.positions(), ref.positions())
