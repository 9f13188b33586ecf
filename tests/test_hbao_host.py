"""Ambient occlusion without a GPU: the jitter table (the library's host
function against the oracle's Mersenne-twister rebuild), the polynomial
exp2/log2 the effect is defined with, the oracle's behaviour on scenes with
known answers (an open plane is not occluded, a corner is) for the classic
and cache-aware algorithms with either blur, and the C ABI's argument checks
(include/gbr_hbao.h)."""
import ctypes

import numpy as np
import pytest

import __graft_entry__ as graft
import scenarios as S
from oracle import hbao as H


@pytest.fixture(scope="module")
def pkg():
    return graft.load_package()


@pytest.fixture(scope="module")
def lib(pkg):
    from habitat_sim_gb300 import _lib
    return _lib.load()


def test_jitter_table(lib):
    out = np.zeros(64, np.float32)
    assert lib.gbr_hbao_jitter_table(out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))) == 0
    ref = H.jitter_table()
    assert np.array_equal(out.reshape(16, 4), ref)
    ang = np.arctan2(ref[:, 1], ref[:, 0])
    assert (ang >= -1e-4).all() and (ang <= 2 * np.pi / 8 + 1e-4).all()   # [0, 2pi/8)
    assert ((ref[:, 2] >= 0) & (ref[:, 2] < 1)).all() and (ref[:, 3] == 0).all()
    assert np.allclose(np.hypot(ref[:, 0], ref[:, 1]), 1, atol=1e-4)


def test_polynomials():
    x = np.linspace(-30, 0, 20001).astype(np.float32)
    assert np.allclose(H.poly_exp2(x), np.exp2(x.astype(np.float64)), rtol=3e-7, atol=0)
    assert H.poly_exp2(np.float32(0)) == 1 and H.poly_exp2(np.float32(-200)) == 0
    a = np.linspace(1e-6, 1, 20001).astype(np.float32)
    ref = np.log2(a.astype(np.float64))
    assert (np.abs(H.poly_log2(a) - ref) <= 1e-7 + 3e-7 * np.abs(ref)).all()
    assert H.poly_log2(np.float32(1)) == 0
    assert np.allclose(H.poly_pow(a, 0.732), a.astype(np.float64) ** 0.732, rtol=2e-6)
    assert H.poly_pow(np.float32(0), 0.732) == 0 and H.poly_pow(np.float32(0.3), 0.0) == 1


def plane_depth(h, w, proj, dist, tilt=0.0):
    """Linear depth of a plane at `dist` (tilted about x) seen by `proj`."""
    y, x = np.mgrid[0:h, 0:w]
    ndc_y = (y + 0.5) / h * 2 - 1
    ty = ndc_y / proj[1, 1]
    z = dist / (1.0 + np.tan(tilt) * ty)
    return np.where(z > 0, z, 0).astype(np.float32)


def test_open_plane_not_occluded_corner_is():
    proj = S.perspective(90.0, 1.0, 0.01, 10.0)
    h = w = 48
    color = np.full((h, w, 4), 200, np.uint8)
    flat = H.hbao(color, np.full((h, w), 3.0, np.float32), proj, H.config())
    assert (flat[..., :3] >= 198).all() and (flat[..., 3] == 200).all()
    # A corner: a wall at x > 0 turning towards the camera.
    depth = np.full((h, w), 3.0, np.float32)
    xs = np.arange(w)
    depth[:, xs >= w // 2] = (3.0 - 0.12 * (xs[xs >= w // 2] - w // 2)).astype(np.float32)
    out = H.hbao(color, depth, proj, H.config())
    assert out[:, w // 2 - 2:w // 2 + 2, 0].mean() < flat[:, w // 2, 0].mean() - 5
    raw = H.hbao(color, depth, proj, H.config(no_blur=True))
    assert not np.array_equal(raw, out)
    # Orthographic projections are accepted too.
    ortho = np.eye(4, dtype=np.float32)
    ortho[2, 2], ortho[3, 2] = -2 / 9.99, -(10.01) / 9.99
    o = H.hbao(color, np.full((h, w), 3.0, np.float32), ortho, H.config())
    assert o.shape == color.shape


def test_hbao_c_abi_checks(lib, pkg):
    from habitat_sim_gb300 import _lib
    c = _lib.HbaoConfig()
    lib.gbr_hbao_config_init(ctypes.byref(c))
    assert abs(c.intensity - 0.732) < 1e-7 and abs(c.bias - 0.05) < 1e-7
    assert abs(c.radius - 1.84) < 1e-6 and c.blur_sharpness == 10.0 and c.no_blur == 0
    p = np.eye(4, dtype=np.float32)
    fp = p.ctypes.data_as(_lib.c_float_p)
    assert lib.gbr_hbao_apply(None, fp, 1, 1, 8, 8, 8, None) == 1
    assert lib.gbr_hbao_apply(ctypes.byref(c), fp, 1, 1, 8, 8, 4, None) == 1      # pitch < width
    c.special_blur = c.no_blur = 1              # the two flags exclude each other
    assert lib.gbr_hbao_apply(ctypes.byref(c), fp, 1, 1, 8, 8, 8, None) == 1
    assert b"exclude each other" in lib.gbr_last_error()
    c.special_blur = c.no_blur = 0
    c.algorithm = 7
    assert lib.gbr_hbao_apply(ctypes.byref(c), fp, 1, 1, 8, 8, 8, None) == 1
    assert b"algorithm" in lib.gbr_last_error()
    c.algorithm = 0
    c.radius = -1.0
    assert lib.gbr_hbao_apply(ctypes.byref(c), fp, 1, 1, 8, 8, 8, None) == 1
    assert lib.gbr_hbao_draw(None, ctypes.byref(c), None) == 1


def test_unquantized_jitter_rounds_to_the_table():
    f = H.jitter_table(quantized=False)
    q = H.jitter_table()
    assert np.abs(f[:, :3] - q[:, :3]).max() <= 0.5 / 32767 + 1e-7
    assert not np.array_equal(f, q)


@pytest.mark.parametrize("cache_aware", [False, True], ids=["classic", "cache_aware"])
@pytest.mark.parametrize("blur", ["bilateral", "special", "none"])
def test_variants_on_known_scenes(cache_aware, blur):
    """Every algorithm and blur: an open plane stays lit, a corner darkens."""
    proj = S.perspective(90.0, 1.0, 0.01, 10.0)
    h, w = 48, 52     # a width that is not a multiple of 4 (quarter-resolution edge)
    cfg = H.config(no_blur=blur == "none", special_blur=blur == "special", cache_aware=cache_aware)
    color = np.full((h, w, 4), 200, np.uint8)
    flat = H.hbao(color, np.full((h, w), 3.0, np.float32), proj, cfg)
    assert (flat[..., :3] >= 196).all() and (flat[..., 3] == 200).all()
    depth = np.full((h, w), 3.0, np.float32)
    xs = np.arange(w)
    depth[:, xs >= w // 2] = (3.0 - 0.12 * (xs[xs >= w // 2] - w // 2)).astype(np.float32)
    out = H.hbao(color, depth, proj, cfg)
    assert out[:, w // 2 - 2:w // 2 + 2, 0].mean() < flat[:, w // 2, 0].mean() - 5
    classic = H.hbao(color, depth, proj, H.config(no_blur=blur == "none"))
    if cache_aware or blur == "special":
        assert not np.array_equal(out, classic)
        assert np.abs(out.astype(int) - classic.astype(int)).mean() < 8   # the same effect
