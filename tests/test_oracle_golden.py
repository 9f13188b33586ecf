"""Pin the CPU oracle against habitat-sim's own batch-renderer goldens.

Every scenario of ``src/tests/GfxBatchRendererTest.cpp`` is replayed on the
oracle and compared with the reference's golden screenshot using the
reference's thresholds (0/0 for uncompressed textures, 1.5/0.5 for BC1,
0.75/0.005 for the lit scenes and 95/0.07 after their rotation), plus the
known-answer pixels, depths, node ids, light ids and scene stats the
reference test asserts."""
import numpy as np
import pytest

import scenarios as S
from oracle.model import OracleRenderer, unproject_depth


def make(tile_size, tile_count, flags):
    return OracleRenderer(tile_size, tile_count, flags)


@pytest.mark.parametrize("case", range(len(S.ALL)), ids=S.ids())
def test_golden(case, oracle_lib):
    _, fn, data = S.ALL[case]
    fails = S.evaluate(fn(make, data))
    assert not fails, fails


def make_lit(tile_size, tile_count, flags, max_lights):
    return OracleRenderer(tile_size, tile_count, flags, max_light_count=max_lights)


@pytest.mark.parametrize("case", range(len(S.LIT)), ids=S.lit_ids())
def test_golden_lights(case, oracle_lib):
    _, fn, data = S.LIT[case]
    fails = S.evaluate(fn(make_lit, data))
    assert not fails, fails


def test_depth_unprojection_scene(oracle_lib):
    fails = S.evaluate(S.depth_unprojection(make, unproject_depth))
    assert not fails, fails


@pytest.mark.parametrize("row", S.UNPROJECT_DATA, ids=[r[0] for r in S.UNPROJECT_DATA])
def test_unproject_known_answers(row, oracle_lib):
    """DepthUnprojectionTest::testCpu (DepthUnprojectionTest.cpp:166-182)."""
    name, z, expected, near, far = row
    p = S.perspective(60.0, 1.0, near, far)
    # project (0.95, -0.34, -z) and map NDC z to [0, 1]
    v = np.array([0.95, -0.34, -z, 1.0], np.float64)
    clip = p.astype(np.float64).T @ v
    ndc_z = clip[2] / clip[3]
    d = np.array([[np.float32((ndc_z + 1.0) * 0.5)]], np.float32)
    unprojection = np.array([np.float32(p[2, 2] - np.float32(1)) * np.float32(0.5),
                             p[3, 2] * np.float32(0.5)], np.float32)
    unproject_depth(unprojection, d)
    assert abs(float(d[0, 0]) - expected) <= z * 0.0002


def test_linear_depth_matches_distance(oracle_lib):
    """Linear depth is -z_eye interpolated: a camera-facing square at 2.5 m reads 2.5."""
    r = make((64, 64), (1, 1), 0)
    S.add_files(r, [("batch.gltf", 0, None)])
    r.updateCamera(0, S.perspective(60.0, 1.0, 0.01, 10.0), S.camera_at_z(2.5))
    r.addNodeHierarchy(0, "square")
    r.draw()
    lin = r.linear_depth.reshape(64, 64)
    assert abs(lin[32, 32] - 2.5) < 1e-5
    assert lin[0, 0] == 0.0
