"""Writes tests/golden/ref_kernels.npz: outputs of the reference's own PD-IPC
kernels (Simulator/PD-IPC/PdIpcGpuFunc.cu, built for the host by
oracle/build_ref.py and run through oracle/refkern.py) on small seeded inputs,
in the reference's float configuration and its USE_DOUBLE_PRECISION one.

The kernels get the oracle's initialised tables (mesh precompute, system
matrix, R1/R2 operator tables) converted to the reference's layouts, and:
  * pd_*: predictiveKernel then one outer iteration's 10 local-global
    iterations (doLocalProjection + chebyshevJacobiR2SolverHost, 15 steps)
    with no contact (PdIpcSimulator.cpp:1683-1711, 1554-1681);
  * toi_*: the per-candidate decision of getImpactOfTimeKernel and the
    clamped global time of impact (PdIpcGpuFunc.cu:2610-2742) over the
    candidates of the patch broad phase;
  * contact_*: setCollisionConstraintsKernel's collision diagonal and
    right-hand side (PdIpcGpuFunc.cu:2756-2930).
The inputs (positions, velocities, displacements) are stored beside the
outputs; the scenes are rebuilt from pdipc.scenes with the stored arguments.

Run from the repository root where the reference tree is available:
    PDIPC_REFERENCE_DIR=<reference checkout> python tests/golden/make_ref_fixtures.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "pd-ipc-armadillodemo_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

from oracle.oracle import FORM_JJ, FORM_R2, Oracle  # noqa: E402
from oracle.refkern import RefKernels, available  # noqa: E402
from pdipc import scenes  # noqa: E402

OUT = os.path.join(HERE, "ref_kernels.npz")

# (name, cloth side, sphere subdivision, jitter of the cloth's start, velocity range)
PD_CASES = [("pd16", 16, 2, 0.0, 0.1), ("pd20", 20, 2, 2e-3, 0.3)]
COLL_SCENE = (24, 3)


def near_contact_state(scene, gap):
    """Rest positions with the cloth lowered so its lowest point sits `gap`
    above the sphere's top vertex."""
    X = scene.initial_positions()
    ns = scene.n_sim
    top = X[ns:, 1].max()
    X[:ns, 1] += (top + gap) - X[:ns, 1].min()
    return X


def pd_inputs(n, s, jitter, vmax, seed):
    sc = scenes.cloth_drop(n, s, lg=10)
    rng = np.random.default_rng(seed)
    X = sc.initial_positions()
    X[:sc.n_sim] += rng.uniform(-jitter, jitter, (sc.n_sim, 3)) if jitter else 0.0
    V = rng.uniform(-vmax, vmax, (sc.n_sim, 3))
    return sc, X, V


def coll_inputs():
    sc = scenes.cloth_drop(*COLL_SCENE)
    X = near_contact_state(sc, 1.5e-3)
    dx = np.zeros_like(X)
    dx[:sc.n_sim, 1] = -4e-3
    dx[:sc.n_sim] += np.random.default_rng(3).uniform(-5e-4, 5e-4, (sc.n_sim, 3))
    Xc = near_contact_state(sc, 4e-4)
    return sc, X, dx, Xc


def main():
    if not available():
        raise SystemExit("the reference tree is not here: set PDIPC_REFERENCE_DIR")
    out = {}
    for k, (name, n, s, jit, vmax) in enumerate(PD_CASES):
        sc, X, V = pd_inputs(n, s, jit, vmax, 11 + k)
        out[f"{name}_args"] = np.array([n, s, jit, vmax])
        out[f"{name}_X"], out[f"{name}_V"] = X, V
        for var in ("fp32", "fp64"):
            rk = RefKernels(var)
            T = rk.tables(Oracle(sc, var, FORM_R2, threads=4))
            out[f"{name}_x_{var}"] = rk.pd_stage(T, X, V, sc.dt)[:sc.n_sim]
    sc, X, dx, Xc = coll_inputs()
    out["coll_args"] = np.array(COLL_SCENE)
    out["toi_X"], out["toi_dx"], out["contact_X"] = X, dx, Xc
    orc = Oracle(sc, "fp64", FORM_JJ, threads=4)
    _, pt, ee = orc.broadphase(X, dx)
    _, cpt, cee = orc.broadphase(Xc, np.zeros_like(Xc))
    out["toi_pt"], out["toi_ee"] = pt, ee
    out["contact_pt"], out["contact_ee"] = cpt, cee
    mass = orc.table("collMass")
    for var in ("fp32", "fp64"):
        rk = RefKernels(var)
        per, g = rk.toi(rk.candidate_list(pt, ee), X, X + dx)
        out[f"toi_per_{var}"], out[f"toi_global_{var}"] = per, np.array(g)
        d, r = rk.contact(rk.candidate_list(cpt, cee), Xc, mass, sc.dhat, sc.kappa, sc.dt)
        out[f"contact_diag_{var}"], out[f"contact_rhs_{var}"] = d, r
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT}: {os.path.getsize(OUT)} bytes")


if __name__ == "__main__":
    main()
