"""The C-ABI library without a GPU: it loads, exports every entry point that
include/gbr.h and include/gbr_replay.h declare, and its host-only functions and argument checks
behave (no kernel runs here)."""
import ctypes
import os
import re

import numpy as np
import pytest

import __graft_entry__ as graft

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def pkg():
    return graft.load_package()


@pytest.fixture(scope="module")
def lib(pkg):
    from habitat_sim_gb300 import _lib
    return _lib.load()


def declared_functions():
    names = set()
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if h.endswith(".h"):
            text = open(os.path.join(ROOT, "include", h)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(gbr_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "gbr_create" in names and "gbr_draw" in names and "gbr_add_file" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_prototypes_cover_the_header(pkg):
    from habitat_sim_gb300 import _lib
    assert sorted(_lib.PROTOTYPES) == declared_functions()


def test_config_defaults(lib, pkg):
    from habitat_sim_gb300 import _lib
    c = _lib.Config()
    lib.gbr_config_init(ctypes.byref(c))
    assert list(c.tile_size) == [128, 128] and list(c.tile_count) == [1, 1]
    assert c.max_light_count == 0 and abs(c.ambient_factor - 0.1) < 1e-7
    assert c.planes == 15 and c.draw_mode == 0 and c.scene_count == 0


def test_null_arguments_are_rejected(lib, pkg):
    from habitat_sim_gb300 import _lib
    out = ctypes.c_void_p()
    assert lib.gbr_create(None, ctypes.byref(out)) == 1
    assert b"null argument" in lib.gbr_last_error()
    assert lib.gbr_draw(None, None) == 1
    assert b"null renderer" in lib.gbr_last_error()
    c = _lib.Config()
    lib.gbr_config_init(ctypes.byref(c))
    c.max_light_count = 65
    assert lib.gbr_create(ctypes.byref(c), ctypes.byref(out)) == 1
    assert b"max_light_count" in lib.gbr_last_error()
    c.max_light_count = 0
    c.tile_size[0] = 0
    assert lib.gbr_create(ctypes.byref(c), ctypes.byref(out)) == 1


def test_create_without_gpu_fails_cleanly(lib, pkg):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from habitat_sim_gb300 import _lib
    c = _lib.Config()
    lib.gbr_config_init(ctypes.byref(c))
    out = ctypes.c_void_p()
    st = lib.gbr_create(ctypes.byref(c), ctypes.byref(out))
    assert st != 0 and not out.value
    assert lib.gbr_last_error()


@pytest.mark.parametrize("near,far", [(0.01, 10.0), (0.001, 10.0), (0.1, 100.0)])
def test_unproject_depth_matches_oracle(pkg, near, far, oracle_lib):
    """gbr_unproject_depth (host) against the oracle's restatement of
    DepthUnprojection.cpp:107-129, bit for bit, strided rows included."""
    from oracle.model import unproject_depth
    from scenarios import perspective
    p = perspective(60.0, 1.0, near, far)
    u = pkg.calculateDepthUnprojection(p)
    rng = np.random.default_rng(3)
    d = rng.uniform(0, 1, (37, 41)).astype(np.float32)
    d[::5, ::3] = 1.0
    ref = unproject_depth(u, d.copy())
    big = np.zeros((37, 64), np.float32)
    big[:, :41] = d
    got = pkg.unprojectDepth(u, big[:, :41])
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    assert (got[::5, ::3] == 0.0).all()
