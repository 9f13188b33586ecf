"""Mip levels without a GPU: the generated chain's level count
(Renderer.cpp:445-450) and 2x2 box filter, and the oracle's level-of-detail
selection on a floor receding to the horizon (minified texels average out
with mipmaps, alias without)."""
import numpy as np
import pytest

import scenarios as S
from oracle.model import OracleRenderer, generate_mips, mip_chain_levels


def test_chain_levels_and_box_filter():
    assert [mip_chain_levels(w, h) for (w, h) in [(1, 1), (2, 2), (512, 512), (64, 16), (3, 5)]] == \
        [1, 2, 10, 5, 2]
    rng = np.random.default_rng(0)
    base = rng.integers(0, 256, (2, 8, 4, 4), dtype=np.uint8)        # 2 layers, 8 x 4 (h x w)
    chain = generate_mips(base, 3)
    assert [c.shape for c in chain] == [(2, 8, 4, 4), (2, 4, 2, 4), (2, 2, 1, 4)]
    b = base.astype(np.uint32)
    want1 = (b[:, 0::2, 0::2] + b[:, 0::2, 1::2] + b[:, 1::2, 0::2] + b[:, 1::2, 1::2] + 2) >> 2
    assert np.array_equal(chain[1], want1)
    # Width 1 at level 2: the column index is clamped to the finer level.
    c1 = chain[1].astype(np.uint32)
    want2 = (c1[:, 0::2, 0:1] + c1[:, 0::2, 1:2] + c1[:, 1::2, 0:1] + c1[:, 1::2, 1:2] + 2) >> 2
    assert np.array_equal(chain[2], want2)


def floor_scene(r, tex_kwargs, size=64, pixels=None):
    """A 20 x 60 m floor with a repeating black/white checker texture (or
    the given texture levels), seen from 1 m above, looking down the corridor."""
    if pixels is None:
        y, x = np.mgrid[0:size, 0:size]
        checker = (((x // 4) + (y // 4)) % 2 * 255).astype(np.uint8)
        pixels = np.stack([checker, checker, 255 - checker // 2, np.full_like(checker, 255)], -1)
    t = r.addTexture(pixels, **tex_kwargs)
    m = r.addMaterial((1, 1, 1, 1), t)
    pos = np.array([[-10, 0, -0.5], [10, 0, -0.5], [10, 0, -60], [-10, 0, -60]], np.float32)
    uv = np.array([[0, 0], [10, 0], [10, 30], [0, 30]], np.float32)
    mesh = r.addMesh(pos, None, uv, None, np.array([0, 1, 2, 0, 2, 3], np.uint32))
    r.addNodeHierarchyTemplate("floor", [(mesh, 0, 6, m, None)])
    r.addNodeHierarchy(0, "floor")
    view = S.translation(0.0, -1.0, 0.0)
    r.updateCamera(0, S.perspective(70.0, 1.0, 0.05, 100.0), view)
    return r


def test_oracle_minification_averages_with_mipmaps():
    def render(**kw):
        r = floor_scene(OracleRenderer((96, 96), (1, 1)), kw)
        r.draw()
        return r.colorImage()[..., 0].astype(np.float64)
    plain = render(filter=1)
    mipped = render(filter=1, minFilter=2, mipFilter=2, generateMipmap=True)
    far = (slice(36, 45), slice(36, 60))    # below the horizon: heavily minified floor
    assert abs(mipped[far].mean() - 127.5) < 3
    assert mipped[far].std() < plain[far].std() / 10
    nearest = render(filter=1, minFilter=1, mipFilter=1, generateMipmap=True)
    assert not np.array_equal(nearest, mipped)
    assert abs(nearest[far].mean() - 127.5) < 12
