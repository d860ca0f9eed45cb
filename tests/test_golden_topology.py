"""Known-answer tests: the reference example scene's cached topology.

example/ClothArmadillo/cloth{1,2} ship boundary.dat (the sorted unique edge
list) and patchInfo.dat (the grid collision-patch partition, patchDim 50),
written by the reference's own precompute (PdIpcModel.h:219-318).  The fixture
was extracted by tests/golden/make_example_fixtures.py.  Both the CPU oracle
and the library's host precompute must reproduce them exactly.
"""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "example_cloth_topology.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def _expected(g, name):
    off, pf = g[f"{name}_patch_off"], g[f"{name}_patch_faces"]
    return g[f"{name}_edges"], [pf[off[i]:off[i + 1]] for i in range(len(off) - 1)]


@pytest.mark.parametrize("name", ["cloth1", "cloth2"])
def test_oracle_topology_matches_reference_cache(gold, name):
    from oracle.oracle import mesh_topology
    X, F = gold[f"{name}_X"], gold[f"{name}_F"]
    exp_e, exp_p = _expected(gold, name)
    edges, patches, owned_pts, owned_edges = mesh_topology(X, F, int(gold["patch_dim"]))
    assert np.array_equal(edges, exp_e)
    assert len(patches) == len(exp_p) == 2500
    for a, b in zip(patches, exp_p):
        assert np.array_equal(a, b)
    # every point and every edge is owned by exactly one face
    assert np.array_equal(np.sort(np.concatenate(owned_pts)), np.arange(X.shape[0]))
    assert np.array_equal(np.sort(np.concatenate(owned_edges)), np.arange(edges.shape[0]))


@pytest.mark.parametrize("name", ["cloth1", "cloth2"])
def test_library_topology_matches_reference_cache(gold, name, built_lib):
    import pdipc
    X, F = gold[f"{name}_X"], gold[f"{name}_F"]
    exp_e, exp_p = _expected(gold, name)
    edges, patches, owner_pt, owner_e = pdipc.mesh_topology(X, F, int(gold["patch_dim"]))
    assert np.array_equal(edges, exp_e)
    assert len(patches) == len(exp_p)
    for a, b in zip(patches, exp_p):
        assert np.array_equal(a, b)
    assert (owner_pt >= 0).all() and (owner_e >= 0).all()


def test_library_and_oracle_ownership_agree(gold, built_lib):
    import pdipc
    from oracle.oracle import mesh_topology
    X, F = gold["cloth1_X"], gold["cloth1_F"]
    _, _, owned_pts, owned_edges = mesh_topology(X, F, 50)
    _, _, owner_pt, owner_e = pdipc.mesh_topology(X, F, 50)
    ref_pt = np.empty(X.shape[0], np.int32)
    for f, lst in enumerate(owned_pts):
        ref_pt[lst] = f
    ref_e = np.empty(owner_e.shape[0], np.int32)
    for f, lst in enumerate(owned_edges):
        ref_e[lst] = f
    assert np.array_equal(ref_pt, owner_pt)
    assert np.array_equal(ref_e, owner_e)


def test_synthetic_grid_counts():
    """Grid generator sizes quoted for the workloads (V, F, E)."""
    from oracle.oracle import mesh_topology
    from pdipc import scenes
    X, F = scenes.grid_cloth(64, jitter=1e-4, seed=0)
    edges, patches, _, _ = mesh_topology(X, F, 64)
    assert (X.shape[0], F.shape[0], edges.shape[0]) == (4096, 7938, 12033)
    SX, SF = scenes.icosphere(4, 0.3)
    assert (SX.shape[0], SF.shape[0]) == (2562, 5120)
    e2, _, _, _ = mesh_topology(SX, SF, 10)
    assert e2.shape[0] == 7680
