"""The benchmark configurations at their stated sizes, on the GPU, against the
CPU oracle (the reference's algorithm restated in C++, run on every host core).

  * config 1 (512x512 cloth onto a subdivision-6 icosphere, 20 local-global
    iterations): the FP64 mode runs 5 whole steps free and stays within 1e-5 m
    of the FP64 oracle with the same outer-iteration count every step; the first
    step also matches the oracle's R2-operator form (the reference's own
    operator tables) within 1e-5 m; the mixed mode started from the oracle's
    state lands within 1e-4 m of the oracle's next state;
  * config 4 (4 layers of 256x256 cloth 5 mm apart onto a subdivision-5
    icosphere, dhat 5e-4 m, self-collision): the GPU runs the free fall up to
    two steps before the first step with a contact constraint or a clamped
    step, the oracle takes over that state, and each of the next 5 steps (the
    lowest layer reaching the sphere) is run by both from the oracle's state
    and held to 1e-5 m with equal outer-iteration counts;
  * config 2 (256 independent drops, sides U{16..128}, 1.6 M vertices in one
    context): FP64 for 3 whole steps against the oracle, within 1e-5 m, with
    equal outer-iteration counts, compared over every instance.
Through contact two FP64 implementations that round differently part after
tens of steps (the stopping rule is absolute and rarely fires once contact
starts), which is why the contact steps restart from the oracle's state.
"""
import os

import numpy as np
import pytest

import pdipc
from oracle.oracle import FORM_JJ, FORM_R2, Oracle
from pdipc import scenes

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 8


def test_config1_full_size_fp64_steps_and_mixed_from_oracle_state(built_lib):
    sc = scenes.config1()
    gpu = pdipc.Simulator(sc, "fp64")
    orc = Oracle(sc, "fp64", FORM_JJ, threads=THREADS)
    states = []
    worst = 0.0
    for k in range(5):
        states.append((orc.positions(), orc.velocities()))
        gpu.step(1)
        orc.step(1)
        assert gpu.stats()["last_outer_iters"] == orc.stats()["last_outer_iters"], k
        worst = max(worst, float(np.abs(gpu.positions() - orc.positions()).max()))
    assert worst < 1e-5, worst
    nexts = states[1:] + [(orc.positions(), orc.velocities())]
    orc.close()

    # the reference's own R2-operator form for the first step
    r2 = Oracle(sc, "fp64", FORM_R2, threads=THREADS)
    r2.step(1)
    err_r2 = float(np.abs(r2.positions() - nexts[0][0]).max())
    r2.close()
    assert err_r2 < 1e-5, err_r2

    # mixed precision: one step from the oracle's state, against the oracle's next state
    mixed = pdipc.Simulator(sc, "mixed")
    worst_mixed = 0.0
    for (x, v), (x1, _) in zip(states[::2], nexts[::2]):
        mixed.set_state(x, v)
        mixed.step(1)
        assert mixed.stats()["pd_path"] == 3
        worst_mixed = max(worst_mixed, float(np.abs(mixed.positions() - x1).max()))
    assert worst_mixed < 1e-4, worst_mixed


def test_config4_full_size_fp64_through_first_contact(built_lib):
    sc = scenes.config4()
    gpu = pdipc.Simulator(sc, "fp64")
    history = []
    for k in range(80):
        history.append((gpu.positions(), gpu.velocities()))
        gpu.step(1)
        if gpu.stats()["last_toi"] < 1.0 or gpu.stats()["active_contacts"] > 0:
            break
    else:
        pytest.fail("no contact within 80 steps")
    start = max(0, len(history) - 3)
    x, v = history[start]
    orc = Oracle(sc, "fp64", FORM_JJ, threads=THREADS)
    orc.set_state(x, v)
    worst, contacts = 0.0, 0
    for k in range(5):
        gpu.set_state(orc.positions(), orc.velocities())
        gpu.step(1)
        orc.step(1)
        so, sg = orc.stats(), gpu.stats()
        assert sg["last_outer_iters"] == so["last_outer_iters"], (start + k, sg["last_outer_iters"],
                                                                  so["last_outer_iters"])
        contacts = max(contacts, so["active_contacts"])
        worst = max(worst, float(np.abs(gpu.positions() - orc.positions()).max()))
    orc.close()
    assert contacts > 0
    assert worst < 1e-5, worst


def test_config2_all_256_instances_fp64_steps(built_lib):
    sc = scenes.config2()
    assert len(sc.cloths) == 256
    gpu = pdipc.Simulator(sc, "fp64")
    orc = Oracle(sc, "fp64", FORM_JJ, threads=THREADS)
    worst = 0.0
    for k in range(3):
        gpu.step(1)
        orc.step(1)
        assert gpu.stats()["last_outer_iters"] == orc.stats()["last_outer_iters"], k
        worst = max(worst, float(np.abs(gpu.positions() - orc.positions()).max()))
    orc.close()
    assert worst < 1e-5, worst
