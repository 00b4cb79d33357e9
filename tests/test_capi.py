"""The C ABI library loads and exports every declared entry point (no GPU)."""

import ctypes
import os
import re

import pytest

from conftest import REPO

import celeritas_gb300 as gb

HEADER = os.path.join(REPO, "include", "celeritas_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gbx_[a-z_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "gbx_stepper_step" in names
    assert "gbx_stepper_launch_action" in names
    assert len(names) >= 15


def test_library_exports_all_declared_symbols(built_lib):
    lib = ctypes.CDLL(built_lib)
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_python_bindings_cover_header():
    assert sorted(gb.EXPORTED_SYMBOLS) == declared_functions()


def test_integration_guide_maps_every_entry_point():
    """The integration guide names, for every declared entry point, the
    reference call it replaces."""
    guide = open(os.path.join(REPO, "INTEGRATION.md")).read()
    missing = [n for n in declared_functions() if n not in guide]
    assert not missing, missing


def test_errors_are_reported_without_gpu(built_lib):
    """Without a device, creation fails loudly with a message (no CPU fallback)."""
    gb.load_library(built_lib)
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:  # pragma: no cover
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(gb.GbxError):
        gb.Params(gb.physics_file("calo"), "calo")


def test_missing_physics_file_error(built_lib):
    gb.load_library(built_lib)
    with pytest.raises(gb.GbxError, match="cannot open physics file"):
        gb.Params("/nonexistent/physics.txt", "calo")


def test_unknown_geometry_error(built_lib):
    gb.load_library(built_lib)
    with pytest.raises(gb.GbxError, match="unknown geometry"):
        gb.Params(gb.physics_file("calo"), "no-such-geometry")
