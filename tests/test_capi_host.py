"""The C ABI library builds for sm_103a, loads, exports every entry point declared in
include/clbm_gb300.h, and fails loudly (no CPU fallback) when no GPU is present."""

import ctypes
import os
import re

import pytest
import torch

from conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "clbm_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(\w+)\s*\(", src, flags=re.M)))


def test_header_declares_the_binding_surface(pkg):
    declared = _declared()
    assert len(declared) >= 20
    assert sorted(pkg.EXPORTED) == declared


def test_library_exports_every_declared_symbol(built_pkg):
    L = ctypes.CDLL(built_pkg.lib_path())
    missing = [name for name in _declared() if not hasattr(L, name)]
    assert not missing


def test_library_is_built_for_sm103a(built_pkg):
    """Every nvcc command that produced the library (recorded by the build) targets
    sm_103a and nothing else."""
    import json
    from importlib import import_module
    b = import_module(built_pkg.__name__ + ".build")
    assert b.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    info = json.load(open(b.INFO))
    assert info["arch"] == b.ARCH
    assert len(info["commands"]) == len(b.SOURCES) + 1
    for cmd in info["commands"]:
        gencodes = [cmd[i + 1] for i, a in enumerate(cmd) if a == "-gencode"]
        assert gencodes == ["arch=compute_103a,code=sm_103a"], cmd
        assert not any(a.startswith(("-arch", "--gpu-architecture", "-code")) for a in cmd), cmd


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the no-GPU error path")
def test_no_gpu_is_an_error_not_a_fallback(built_pkg):
    with pytest.raises(built_pkg.CLBMError) as ei:
        built_pkg.Solver(16, 8, 4, 1.5)
    assert ei.value.code == 1


def test_invalid_configuration_is_rejected(built_pkg):
    with pytest.raises(built_pkg.CLBMError) as ei:
        built_pkg.Solver(2, 8, 4, 1.5)
    assert ei.value.code == 2
    with pytest.raises(built_pkg.CLBMError) as ei:
        built_pkg.Solver(16, 8, 4, 2.5)
    assert ei.value.code == 2
    with pytest.raises(ValueError):
        built_pkg.Solver(16, 8, 4, 1.5, storage="fp8")


def test_normal_build_is_not_the_bounds_checked_one(built_pkg, monkeypatch):
    """The library the package loads by default has no index tests on its hot paths (they
    are in the separate -DCLBM_CHECK library, selected by CLBM_CHECK_BUILD=1)."""
    monkeypatch.delenv("CLBM_CHECK_BUILD", raising=False)
    import importlib
    b = importlib.import_module(built_pkg.__name__ + ".build")
    assert built_pkg.lib_path() == b.LIB
    v = ctypes.c_int32(-1)
    assert built_pkg.lib().clbm_bounds_checked(ctypes.byref(v)) == 0
    assert v.value == 0
    monkeypatch.setenv("CLBM_CHECK_BUILD", "1")
    assert built_pkg.lib_path().endswith(os.path.join("_build_check", "libclbm_gb300.so"))
