"""Serving layer, host side: the library exports every entry point of
include/bora_serve.h, the admission estimate behaves, a server cannot start without a
device, and the request stream has the stated distribution."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT
from vare_gb300 import flip, scenes, serve

HEADER = os.path.join(ROOT, "include", "bora_serve.h")


def declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|uint64_t)\s+(bora_serve_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def lib(flip_lib):
    return serve.load()


def test_serve_declarations_are_bound_and_exported(lib):
    names = declared()
    assert names and set(names) == set(serve.exported_symbols())
    for n in names:
        assert hasattr(lib, n)


def test_estimate_grows_with_particles_and_solver(lib):
    g = flip.GridDesc()
    g.nx = g.ny = g.nz = 64
    g.max = (ctypes.c_float * 3)(1, 1, 1)
    a = lib.bora_serve_estimate_bytes(ctypes.byref(g), 100_000, flip.SOLVER_PLAIN)
    b = lib.bora_serve_estimate_bytes(ctypes.byref(g), 200_000, flip.SOLVER_PLAIN)
    c = lib.bora_serve_estimate_bytes(ctypes.byref(g), 200_000, flip.SOLVER_MIXED)
    assert 0 < a < b < c
    # at least the two particle buffers (7 arrays of 4 bytes each)
    assert b >= 200_000 * 56
    assert lib.bora_serve_estimate_bytes(None, 10, 0) == 0


def test_default_config_and_invalid_arguments(lib):
    c = serve.ServeConfig()
    assert lib.bora_serve_default_config(ctypes.byref(c)) == 0
    assert c.hbm_budget_bytes == 120 * 10**9 and c.max_running == 64
    h = ctypes.c_void_p()
    assert lib.bora_serve_create(None, ctypes.byref(h)) == -1
    c.max_running = 0
    assert lib.bora_serve_create(ctypes.byref(c), ctypes.byref(h)) == -1
    assert lib.bora_serve_destroy(None) == -1
    assert lib.bora_serve_drain(None) == -1


def test_create_without_device_reports_no_device(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    c = serve.ServeConfig()
    lib.bora_serve_default_config(ctypes.byref(c))
    h = ctypes.c_void_p()
    assert lib.bora_serve_create(ctypes.byref(c), ctypes.byref(h)) == -4


def test_stream_distribution():
    plan = scenes.serving_plan(64)
    edges = np.array([e for e, _, _ in plan])
    steps = np.array([s for _, s, _ in plan])
    fills = np.array([f for _, _, f in plan])
    assert edges.min() >= 32 and edges.max() <= 192 and len(set(edges)) > 20
    assert steps.min() >= 50 and steps.max() <= 400
    assert fills.min() >= 0.2 and fills.max() <= 0.5
    t = scenes.serving_arrivals(64, 20.0)
    assert np.all(np.diff(t) > 0)
    assert 1.5 < t[-1] < 6.0  # 64 arrivals at 20/s
    # the generator's first request matches the plan
    sc, st = scenes.serving_request(0)
    assert sc.res[0] == plan[0][0] and st == plan[0][1]
