"""Depth-noise model without a GPU: the Philox generator against the
Random123 known-answer vectors, the normal quantile table (the library's
host function against scipy), the float32 kernel restatement against the
reference's CPU algorithm at the reference test's tolerances
(tests/test_noise_models.py:24-51 in habitat-sim), and the C ABI checks."""
import ctypes
import hashlib
import os

import numpy as np
import pytest

import __graft_entry__ as graft
from oracle import noise as N


@pytest.fixture(scope="module")
def pkg():
    return graft.load_package()


@pytest.fixture(scope="module")
def lib(pkg):
    from habitat_sim_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="module")
def model(pkg):
    from habitat_sim_gb300 import noise
    return noise.load_model()


def test_philox_known_answers():
    """Random123's kat_vectors for philox4x32_10."""
    cases = [((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
             ((0xffffffff,) * 4, (0xffffffff,) * 2, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
             ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
              (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1))]
    for ctr, key, want in cases:
        got = N.philox4x32_10(*[np.uint32(c) for c in ctr], *key)
        assert tuple(int(g) for g in got) == want


def test_model_file(model):
    from habitat_sim_gb300 import noise
    assert model.shape == (80, 400) and model.dtype == np.float32
    digest = open(noise.MODEL_PATH + ".sha256").read().split()[0]
    assert hashlib.sha256(open(noise.MODEL_PATH, "rb").read()).hexdigest() == digest


def test_normal_table_matches_scipy(pkg, lib):
    from habitat_sim_gb300 import noise
    t = noise.normal_quantile_table()
    ref = N.normal_table()
    assert np.array_equal(t, ref)
    assert np.array_equal(t, -t[::-1]) and (np.diff(t) > 0).all()
    z = N.normals(N.philox4x32_10(np.arange(1 << 20, dtype=np.uint32), 0, 0, 0, 5, 6)[0], t)
    assert abs(z.mean()) < 3e-3 and 0.99 < z.var() < 1.0
    out = np.zeros(10, np.float32)
    assert lib.gbr_normal_quantile_table(out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), 10) == 1


@pytest.mark.parametrize("mult,tolerance", [(0.0, 1e-5), (1.0, 1e-2)])
def test_kernel_restatement_matches_reference_cpu(model, mult, tolerance):
    """The reference's own GPU-vs-CPU check: mean over 100 simulations of a
    0-20 m ramp, mean absolute difference within the tolerance."""
    depth = np.linspace(0, 20, num=256 * 256, dtype=np.float32).reshape(256, 256)
    rng = np.random.default_rng(1)
    table = N.normal_table()
    ours = np.mean([N.redwood_f32(depth, model, mult, 11, c, table=table) for c in range(100)], 0)
    ref = np.mean([N.redwood_reference_cpu(depth, model, mult, rng) for _ in range(100)], 0)
    assert np.abs(ours - ref).mean() <= tolerance
    one = N.redwood_f32(depth, model, mult, 11, 0, table=table)
    assert (one[depth >= 10.5] == 0).all() and one[0, 0] == 0     # beyond 10 m, and 0 m
    assert (one[(depth > 0.5) & (depth < 9.0)] > 0).mean() > 0.9   # the table has empty cells


def test_noise_c_abi_checks(lib, model):
    from habitat_sim_gb300 import _lib
    out = ctypes.c_void_p()
    fp = model.ctypes.data_as(_lib.c_float_p)
    assert lib.gbr_redwood_noise_create(None, 80, 400, 0, 1.0, 0, ctypes.byref(out)) == 1
    assert lib.gbr_redwood_noise_create(fp, 80, 399, 0, 1.0, 0, ctypes.byref(out)) == 1
    assert b"80 x 80 x 5" in lib.gbr_last_error()
    assert lib.gbr_redwood_noise_create(fp, 80, 400, 0, -1.0, 0, ctypes.byref(out)) == 1
    assert lib.gbr_redwood_noise_simulate_host(None, None, 1, 1, None) == 1
    assert lib.gbr_redwood_noise_set_state(None, 0, 0) == 1


def test_noise_without_gpu_fails_cleanly(pkg, model):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from habitat_sim_gb300 import noise
    with pytest.raises(pkg.GbrError):
        noise.RedwoodDepthNoiseModel(noise_multiplier=1.0)


def _reference_means():
    """Means of habitat-sim's own _simulate (run from its source by
    tests/golden/make_redwood_means.py) over the reference test's ramp."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "redwood",
                        "reference_means.npz")
    return np.load(path)


@pytest.mark.parametrize("mult,tolerance", [(0.0, 1e-5), (1.0, 1e-2)])
def test_restatements_match_reference_code(model, mult, tolerance):
    """Both restatements against the reference's own CPU code: the means of
    100 simulations of the 0-20 m ramp within the tolerances of the
    reference's GPU-versus-CPU test (tests/test_noise_models.py:24-51)."""
    ref = _reference_means()
    want = ref["mult0"] if mult == 0.0 else ref["mult1"]
    depth = np.linspace(0, 20, num=256 * 256, dtype=np.float32).reshape(256, 256)
    rng = np.random.default_rng(7)
    cpu = np.mean([N.redwood_reference_cpu(depth, model, mult, rng) for _ in range(100)], 0)
    assert np.abs(cpu - want).mean() <= tolerance
    table = N.normal_table()
    ker = np.mean([N.redwood_f32(depth, model, mult, 5, c, table=table) for c in range(100)], 0)
    assert np.abs(ker - want).mean() <= tolerance
