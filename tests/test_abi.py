"""The C-ABI library: it builds for sm_103a, loads, exports every entry point that
include/bora_flip.h declares, and its host-only calls behave (no GPU needed)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "bora_flip.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(bora_\w+)\s*\(", text, re.M)))


def test_header_declarations_are_bound(flip_lib):
    names = declared_functions()
    assert names, "no declarations parsed"
    assert set(names) == set(flip_lib.exported_symbols()), set(names) ^ set(flip_lib.exported_symbols())


def test_library_exports_every_declared_symbol(flip_lib):
    path = flip_lib.library_path()
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (bora_\w+)", out))
    missing = set(declared_functions()) - exported
    assert not missing, missing
    lib = flip_lib.load()
    for name in declared_functions():
        assert hasattr(lib, name)


def test_default_params_mirror_flipmethod(flip_lib):
    p = flip_lib.default_params()
    # FLIPMethod::Params defaults (base/header/FLIPMethod.h:51-67)
    assert tuple(p.ext_force) == pytest.approx((0.0, -9.80665, 0.0))
    assert p.max_substeps == 1
    assert p.dt == pytest.approx(1.0 / 24.0)
    assert p.wall_level == pytest.approx(-1e30)
    assert p.enable_water_tank == 0 and p.enable_curl == 0
    assert p.voxel_size == pytest.approx(0.1)
    assert p.col_vel_scale == 1.0 and p.pts_per_cell == 8
    assert p.proj_iteration == 200 and p.redist_iteration == 80
    assert p.tolerance == pytest.approx(1e-6) and p.div_tolerance == pytest.approx(1e-5)


def test_status_strings(flip_lib):
    lib = flip_lib.load()
    for code in (0, -1, -2, -3, -4, -5, -6, 1):
        assert lib.bora_flip_status_string(code)
    assert flip_lib.status_string(-2) == "out of device memory"


def test_invalid_arguments_are_rejected(flip_lib):
    lib = flip_lib.load()
    g = flip_lib.GridDesc()
    g.nx, g.ny, g.nz = 0, 8, 8
    h = ctypes.c_void_p()
    assert lib.bora_flip_create(ctypes.byref(g), None, ctypes.byref(h)) == -1
    assert lib.bora_flip_create(None, None, ctypes.byref(h)) == -1
    assert lib.bora_flip_step(None, ctypes.c_float(0.1)) == -1
    assert lib.bora_flip_destroy(None) == -1
    p = flip_lib.default_params(enable_curl=1)
    g.nx = 8
    g.max = (ctypes.c_float * 3)(1, 1, 1)
    assert lib.bora_flip_create(ctypes.byref(g), ctypes.byref(p), ctypes.byref(h)) == -1


def test_create_without_device_reports_no_device(flip_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    g = flip_lib.GridDesc()
    g.nx = g.ny = g.nz = 16
    g.max = (ctypes.c_float * 3)(1, 1, 1)
    h = ctypes.c_void_p()
    assert flip_lib.load().bora_flip_create(ctypes.byref(g), None, ctypes.byref(h)) == -4


def test_cpp_wrapper_compiles():
    """include/BoraFLIPMethod.hpp (the FLIPMethod-shaped C++ wrapper) compiles against the
    C ABI with a plain C++ compiler."""
    src = os.path.join(ROOT, "tests", "cpp", "flipmethod_harness.cpp")
    out = os.path.join(ROOT, "tests", "cpp", "_build", "harness.o")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), "-c", src,
                        "-o", out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_scene_counts():
    from vare_gb300 import scenes
    assert scenes.config0().num_particles == 505856
    a = scenes.small(16, seed=3)
    b = scenes.small(16, seed=3)
    np.testing.assert_array_equal(a.pos, b.pos)
    assert a.pos.min() >= 0 and a.pos.max() < 16
