"""The C-ABI library loads on a host without a GPU, exports every entry point
declared in include/pdipc.h, and fails cleanly (no fallback) without a GB300."""
import ctypes as C
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "pdipc.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pdipc_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_binding_list():
    import pdipc
    assert sorted(pdipc.EXPORTS) == declared_symbols()


def test_library_exports_every_declared_symbol(built_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", built_lib], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\sT\s(pdipc_\w+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    L = C.CDLL(built_lib)
    for s in declared_symbols():
        assert hasattr(L, s)


def test_default_params_match_reference_constants(built_lib):
    import pdipc
    from pdipc.abi import Params, default_params
    L = pdipc.load_library()
    p = Params()
    L.pdipc_default_params(C.byref(p))
    q = default_params()
    for name, _ in Params._fields_:
        if name == "reserved":
            continue
        assert getattr(p, name) == getattr(q, name), name
    assert L.pdipc_abi_version() == pdipc.ABI_VERSION == 9
    assert L.pdipc_status_string(3) == b"PDIPC_ERR_OVERFLOW"


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device path")
def test_create_without_gpu_fails_loudly(built_lib):
    import pdipc
    from pdipc import scenes
    with pytest.raises(pdipc.PdipcError) as ei:
        pdipc.Simulator(scenes.cloth_drop(8, 1))
    assert ei.value.status == pdipc.PDIPC_ERR_CUDA


def test_argument_errors_are_reported(built_lib):
    import pdipc
    import numpy as np
    L = pdipc.load_library()
    assert L.pdipc_create(None, None) == 1
    assert L.pdipc_step(None, 1) == 1
    assert L.pdipc_adjoint_record(None, 1) == 1
    assert L.pdipc_adjoint_backward(None, None, None, None, None, None) == 1
    X = np.zeros((3, 3))
    F = np.array([[0, 1, 5]], np.int32)
    with pytest.raises(pdipc.PdipcError):
        pdipc.mesh_topology(X, F, 4)  # face index out of range


def test_cxx_shim_compiles_links_and_reports(built_lib, tmp_path):
    """The reference-style C++ class builds against include/ and libpdipc.so; on a
    host without a GB300 initialization() reports PDIPC_ERR_CUDA instead of aborting."""
    exe = tmp_path / "shim"
    lib_dir = os.path.dirname(built_lib)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cxx", "shim_main.cpp"), "-L" + lib_dir, "-lpdipc",
                    "-Wl,-rpath," + lib_dir, "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    if _has_gpu():
        assert "animate PDIPC_OK" in out.stdout
    else:
        assert "init PDIPC_ERR_CUDA" in out.stdout


@pytest.mark.gpu
def test_cxx_shim_animates_on_the_device(built_lib, tmp_path):
    """The reference-style C++ class (createSimulator, addClothModel,
    initialization, animate) steps a cloth on the GB300 through the C ABI: five
    animate() calls succeed and the free corner falls under gravity."""
    exe = tmp_path / "shim"
    lib_dir = os.path.dirname(built_lib)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cxx", "shim_main.cpp"), "-L" + lib_dir, "-lpdipc",
                    "-Wl,-rpath," + lib_dir, "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "init PDIPC_OK" in out.stdout and "animate PDIPC_OK" in out.stdout
    y4 = float(out.stdout.split("y4=")[1].split()[0])
    assert -0.01 < y4 < 0.0     # vertex 4 (the cloth's centre) fell, about g (5/240 s)^2 / 2
