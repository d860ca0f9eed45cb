"""The scene reader (pdipc_scene_load): a reference-format config.xml with its
OBJ, tetgen and fixed_points.txt files, written here from the seeded
generators; placement (origin, uniform, scale, translation) checked against
the same transforms in numpy; and, when the reference tree is given
($PDIPC_REFERENCE_DIR), its ClothArmadillo example scene."""
import os

import numpy as np
import pytest

import pdipc
from oracle import build_ref
from oracle.oracle import FORM_JJ, Oracle
from pdipc import scenes

_REF = build_ref.reference_dir()
EXAMPLE = os.path.join(_REF, "example", "ClothArmadillo", "config.xml") if _REF else ""


def write_obj(path, X, F):
    with open(path, "w") as f:
        for x in X:
            f.write("v %r %r %r\n" % (float(x[0]), float(x[1]), float(x[2])))
        for t in F:
            f.write(f"f {t[0] + 1}//1 {t[1] + 1}//1 {t[2] + 1}//1\n")


def write_tet(base, X, T):
    with open(base + ".node", "w") as f:
        f.write(f"{X.shape[0]}  3  0  0\n")
        for i, x in enumerate(X):
            f.write("   %d    %r  %r  %r\n" % (i + 1, float(x[0]), float(x[1]), float(x[2])))
    with open(base + ".ele", "w") as f:
        f.write(f"{T.shape[0]}  4  0\n")
        for i, t in enumerate(T):
            f.write(f"    {i + 1}    {t[0] + 1}  {t[1] + 1}  {t[2] + 1}  {t[3] + 1}\n")


def make_scene_dir(root):
    """A cloth (placed as is) above a tet block given in other units (placed by
    origin + uniform + scale + translation), with pins for both."""
    CX, CF = scenes.grid_cloth(12, 1.0, 0.0, 1e-4, 5)
    os.makedirs(os.path.join(root, "sheet"))
    write_obj(os.path.join(root, "sheet", "sheet.obj"), CX, CF)
    with open(os.path.join(root, "sheet", "fixed_points.txt"), "w") as f:
        f.write("c 2\n0\n11\n")
    BX, BT = scenes.tet_block(2, 2, 2, (30.0, 30.0, 30.0), (100.0, -7.0, 3.0))
    surf = pdipc.tet_surface(BX, BT)
    os.makedirs(os.path.join(root, "block"))
    write_obj(os.path.join(root, "block", "block.obj"), BX, surf)
    write_tet(os.path.join(root, "block", "block"), BX, BT)
    with open(os.path.join(root, "block", "fixed_points.txt"), "w") as f:
        f.write("c 1\n0\n")
    cfg = """<?xml version="1.0" ?>
<SimFramework name = "pd_ipc_simulator" run = "CUDA">
<simulator>
<!-- seeded test scene -->
<timeStep> 0.005 </timeStep>
<gravity> -9.8 </gravity>
<dhat>2e-3</dhat>
<kappa>1e5</kappa>
<object name = "sheet" nick_name = "sheet" uniform = "false" origin = "false">
<type> 0 5e3 1e-3 1e6 </type>
<patchDim> 12 </patchDim>
<scale> 1 1 1 </scale>
<translation> 0 0 0 </translation>
<rotation> 0 0 0 0</rotation>
<density> 0.1 </density>
</object>
<object name = "block" nick_name = "block" volumetric_mesh = "tet" uniform = "true" origin = "true">
<type> 1 1e5 1e3 1e8 </type>
<patchDim> 4 </patchDim>
<scale> 0.2 0.2 0.2 </scale>
<translation> 0.5 -0.2 0.5 </translation>
<rotation> 0 0 0 0</rotation>
<density> 500 </density>
</object>
</simulator>
</SimFramework>
"""
    path = os.path.join(root, "config.xml")
    with open(path, "w") as f:
        f.write(cfg)
    return path, (CX, CF), (BX, BT)


def test_reader_places_models_like_the_reference(tmp_path, built_lib):
    path, (CX, CF), (BX, BT) = make_scene_dir(str(tmp_path))
    sc = pdipc.read_scene(path)
    assert (sc.dt, sc.gravity, sc.dhat, sc.kappa) == (0.005, -9.8, 2e-3, 1e5)
    assert len(sc.cloths) == 1 and len(sc.solids) == 1 and not sc.statics
    c, v = sc.cloths[0], sc.solids[0]
    # uniform/origin off: as in the file (up to the scale-by-1 about the box centre the reference applies)
    np.testing.assert_allclose(c.X, CX, rtol=0, atol=1e-15)
    np.testing.assert_array_equal(c.F, CF)
    np.testing.assert_array_equal(c.pins, [0, 11])
    assert (c.density, c.k_stretch, c.k_bend, c.k_pin, c.patch_dim) == (0.1, 5e3, 1e-3, 1e6, 12)
    np.testing.assert_array_equal(v.T, BT)
    np.testing.assert_array_equal(v.pins, [0])
    assert (v.density, v.k_strain, v.k_volume, v.k_pin, v.patch_dim) == (500.0, 1e5, 1e3, 1e8, 4)
    # origin: box centre to 0; uniform: / largest extent; scale 0.2 about the centre; translate
    lo, hi = BX.min(0), BX.max(0)
    expect = (BX - (lo + hi) / 2) / (hi - lo).max() * 0.2 + np.array([0.5, -0.2, 0.5])
    np.testing.assert_allclose(v.X, expect, rtol=0, atol=1e-12)


def test_reader_reports_missing_files(tmp_path, built_lib):
    path = os.path.join(str(tmp_path), "config.xml")
    with open(path, "w") as f:
        f.write('<SimFramework><simulator><object name="nothing"><type> 0 1 1 1 </type></object>'
                '</simulator></SimFramework>')
    with pytest.raises(pdipc.PdipcError) as e:
        pdipc.read_scene(path)
    assert "nothing.obj" in str(e.value)


@pytest.mark.skipif(not EXAMPLE or not os.path.exists(EXAMPLE), reason="reference tree not given")
def test_reads_the_reference_cloth_armadillo_example(built_lib):
    sc = pdipc.read_scene(EXAMPLE)
    assert (sc.dt, sc.gravity, sc.dhat, sc.kappa) == (0.01, -9.8, 5e-3, 5e7)
    assert [c.X.shape[0] for c in sc.cloths] == [5625, 5625]
    assert [c.F.shape[0] for c in sc.cloths] == [10952, 10952]
    assert all(len(c.pins) == 16 and c.k_stretch == 1e6 and c.k_bend == 25 and c.density == 2500
               for c in sc.cloths)
    (arm,) = sc.solids
    assert arm.X.shape == (14779, 3) and arm.T.shape == (54855, 4)
    assert (arm.k_strain, arm.k_volume, arm.k_pin, arm.density, arm.patch_dim) == (2e6, 1e3, 1e12, 1000.0, 50)
    # uniform + origin put the surface in a unit box, scaled by 3.5 and moved by (1.5, 2.3, 1)
    ext = arm.X.max(0) - arm.X.min(0)
    assert 3.4 < ext.max() < 3.6
    orc = Oracle(sc, "fp64", FORM_JJ, threads=8)
    assert orc.stats()["n_sim"] == 5625 * 2 + 14779
    orc.step(1)
    assert orc.stats()["last_outer_iters"] >= 2


@pytest.mark.gpu
def test_scene_from_files_steps_like_the_oracle(tmp_path, built_lib):
    """The written scene through the library (FP64) and the oracle: the same
    models, and every step from the oracle's state within 1e-9 m."""
    path, _, _ = make_scene_dir(str(tmp_path))
    sc = pdipc.read_scene(path)
    sim = pdipc.Simulator(sc, "fp64")
    orc = Oracle(sc, "fp64", FORM_JJ, threads=8)
    assert sim.n_sim == orc.n_sim and sim.stats()["n_patches"] == orc.stats()["n_patches"]
    worst = 0.0
    for _ in range(40):
        sim.set_state(orc.positions(), orc.velocities())
        sim.step(1)
        orc.step(1)
        assert sim.stats()["last_outer_iters"] == orc.stats()["last_outer_iters"]
        worst = max(worst, float(np.abs(sim.positions() - orc.positions()).max()))
    assert worst < 1e-9, worst
