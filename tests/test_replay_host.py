"""Replay driver without a GPU: the oracle's restatement of habitat-sim's
replay Player / BatchPlayerImplementation against the reference's own
expectations (BatchReplayRendererTest.cpp:400-487), its small linear
algebra, keyframe JSON round trips, and the C ABI's host-only entry points
and argument checks (include/gbr_replay.h)."""
import ctypes
import json
import math
import os

import numpy as np
import pytest

import __graft_entry__ as graft
import scenarios as S
from oracle import replay as OR
from oracle.model import OracleRenderer

HERE = os.path.dirname(os.path.abspath(__file__))
SPHERE = os.path.join(HERE, "golden", "objects", "sphere.glb")


@pytest.fixture(scope="module")
def pkg():
    return graft.load_package()


@pytest.fixture(scope="module")
def lib(pkg):
    from habitat_sim_gb300 import _lib
    return _lib.load()


def translation(x, y, z):
    return S.translation(x, y, z)


def deletion_keyframes(pkg):
    """The three keyframes habitat-sim's Recorder writes for
    testBatchPlayerDeletion (BatchReplayRendererTest.cpp:404-449): two
    spheres; then sphere 0 deleted (sphere 2 created and deleted in the same
    frame cancels out, Recorder.cpp:166-179); then sphere 1 deleted."""
    K = pkg.Keyframe
    k0 = (K().load(SPHERE).create(0, SPHERE).create(1, SPHERE)
          .update(0, (1, 0, 0)).update(1, (0, 1, 0)))
    k1 = K().delete(0)
    k2 = K().delete(1)
    return [k0, k1, k2]


def test_batch_player_deletion_oracle(pkg):
    """BatchReplayRendererTest::testBatchPlayerDeletion on the oracle."""
    rr = OR.OracleReplayRenderer(1, resolution=(16, 16))
    rr.set_environment_keyframes(0, pkg.keyframes_to_string(deletion_keyframes(pkg)))
    t = rr.r.transformations(0)
    rr.set_environment_keyframe_index(0, 0)
    assert len(t) == 4  # two instances x (root + one mesh view)
    assert np.array_equal(t[0], translation(1, 0, 0))
    assert np.array_equal(t[2], translation(0, 1, 0))
    rr.set_environment_keyframe_index(0, 1)
    t = rr.r.transformations(0)
    assert len(t) == 2 and np.array_equal(t[0], translation(0, 1, 0))
    rr.set_environment_keyframe_index(0, 2)
    assert len(rr.r.transformations(0)) == 0
    # Going back clears and replays from the first keyframe.
    rr.set_environment_keyframe_index(0, 0)
    assert len(rr.r.transformations(0)) == 4


def test_missing_asset_info_and_unsupported_assets(pkg):
    K = pkg.Keyframe
    rr = OR.OracleReplayRenderer(1, resolution=(16, 16))
    k = (K().load("cubeSolid").create(0, "cubeSolid").create(1, SPHERE)   # no load for SPHERE
         .create(2, "cubeSolid"))
    rr.set_environment_keyframe(0, k.to_string())
    assert len(rr.r.transformations(0)) == 0
    p = rr.players[0]
    assert p.failed == {"cubeSolid", SPHERE} and not p.created
    # A material override after '?' is stripped.
    k = K().load(SPHERE).create(5, SPHERE + "?{material}").update(5, (0, 0, -2))
    rr2 = OR.OracleReplayRenderer(1, resolution=(16, 16))
    rr2.set_environment_keyframe(0, k.to_string())
    assert list(rr2.players[0].created) == [5]
    assert np.array_equal(rr2.r.transformations(0)[0], translation(0, 0, -2))


def test_quaternion_matrix_and_frames():
    rng = np.random.default_rng(5)
    for _ in range(20):
        axis = rng.normal(size=3)
        ang = rng.uniform(-180, 180)
        from habitat_sim_gb300.replay import quaternion_axis_angle
        q = tuple(np.float32(v) for v in quaternion_axis_angle(axis, ang))
        m = np.array(OR.quat_to_matrix(q), np.float64).reshape(3, 3).T   # row-major
        a = axis / np.linalg.norm(axis)
        k = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
        t = math.radians(ang)
        ref = np.eye(3) + math.sin(t) * k + (1 - math.cos(t)) * k @ k   # Rodrigues
        assert np.allclose(m, ref, atol=2e-6)
    f32 = np.float32
    assert OR.frame_to_world([f32(0), f32(1), f32(0)], [f32(0), f32(0), f32(-1)]) == (0, 0, 0, 1)
    for up, front in [((0, 0, 1), (0, -1, 0)), ((1, 0, 0), (0, 0, -1)), ((0, -1, 0), (0, 0, 1))]:
        up32 = [f32(v) for v in up]
        fr32 = [f32(v) for v in front]
        q = OR.frame_to_world(up32, fr32)
        assert np.allclose(OR.quat_rotate(q, up32), [0, 1, 0], atol=1e-6)
        assert np.allclose(OR.quat_rotate(q, fr32), [0, 0, -1], atol=1e-6)


def test_invert4_and_projection():
    rng = np.random.default_rng(7)
    for _ in range(10):
        m = np.eye(4, dtype=np.float32)
        m[:3, :3] = rng.normal(size=(3, 3)).astype(np.float32)
        m[3, :3] = rng.normal(size=3).astype(np.float32)
        inv = OR.invert4(m)
        assert np.allclose(inv.T @ m.T, np.eye(4), atol=1e-4)
    with pytest.raises(ValueError):
        OR.invert4(np.zeros((4, 4), np.float32))
    # Square sensor: the Magnum perspective of the reference's goldens.
    p = OR.sensor_projection((128, 128), 90.0, 0.01, 10.0)
    ref = S.perspective(90.0, 1.0, 0.01, 10.0)
    assert np.allclose(p, ref, rtol=1e-6, atol=0)
    # Non-square: near-plane height = width * h / w (CameraSensor.cpp:46-56).
    p = OR.sensor_projection((384, 512), 60.0, 0.1, 100.0)
    assert math.isclose(p[1, 1] / p[0, 0], 512 / 384, rel_tol=1e-6)
    o = OR.sensor_projection((64, 64), orthographic=True, near=0.01, far=10.0, ortho_scale=0.5)
    assert math.isclose(o[0, 0], 1.0) and o[2, 3] == 0 and o[3, 3] == 1


def test_environment_grid_size(lib, pkg):
    for n, want in [(1, (1, 1)), (2, (2, 1)), (4, (2, 2)), (5, (3, 2)), (10, (4, 3)),
                    (1024, (32, 32)), (1000, (32, 32))]:
        assert OR.environment_grid_size(n) == want
        assert pkg.ReplayRenderer.environment_grid_size(n) == want
    out = (ctypes.c_int32 * 2)()
    assert lib.gbr_replay_environment_grid_size(0, out) == 1


def test_keyframe_json_round_trip(pkg):
    from habitat_sim_gb300.replay import quaternion_axis_angle
    q = quaternion_axis_angle((0, 1, 0), 80.0)
    k = (pkg.Keyframe().load("a.glb", up=(0, 0, 1), front=(0, -1, 0))
         .create(3, "a.glb", scale=(2, 2, 2)).update(3, (1, 2, 3), q)
         .set_metadata(3, 7, 9).user_transform("sensor_rgb", (3.3, 1.3, 0), q)
         .set_lights([((1, 2, 3, 0), (1, 1, 1)), ((0, 1, 0, 1), (0.5, 0.5, 0.5))]))
    d = json.loads(k.to_string())["keyframe"]
    assert d["stateUpdates"][0]["state"]["absTransform"]["rotation"][0] == pytest.approx(q[3])
    parsed = OR.parse_keyframe(d)
    assert parsed["creations"][0][1]["scale"] == [2, 2, 2]
    assert parsed["metadata"] == [(3, {"object_id": 7, "semantic_id": 9})]
    t, r = parsed["user_transforms"]["sensor_rgb"]
    assert np.allclose(r, q, atol=1e-7) and np.allclose(t, (3.3, 1.3, 0))
    assert parsed["lights_changed"] and len(parsed["lights"]) == 2
    doc = json.loads(pkg.keyframes_to_string([k, pkg.Keyframe().delete(3)]))
    assert len(doc["keyframes"]) == 2 and doc["keyframes"][1]["deletions"] == [3]


def test_oracle_replay_renders_instances(pkg):
    """Two environments, each a sphere in front of a camera placed from the
    keyframe's user transform: something is drawn at the centre, with the
    sphere's base colour, and depth ~ distance minus radius."""
    K = pkg.Keyframe
    rr = OR.OracleReplayRenderer(2, resolution=(32, 48), sensor_uuid="rgb")
    for e in range(2):
        k = (K().load(SPHERE).create(0, SPHERE).update(0, (0, 0, -3.0 - e))
             .user_transform("sensor_rgb", (0, 0, 0)))
        rr.set_environment_keyframe(e, k.to_string())
        rr.set_sensor_transforms_from_keyframe(e, "sensor_")
    out = rr.render()
    for e, (c, d) in enumerate(out):
        assert c.shape == (32, 48, 4) and d.shape == (32, 48)
        assert d[16, 24] > 0 and (d == 0).any()
        assert tuple(c[16, 24, :3]) == (204, 1, 1)   # baseColorFactor (0.8, 0.0056, 0.0056)
        assert abs(d[16, 24] - (3.0 + e - 0.25)) < 0.04   # radius 0.25 m, faceted


def test_replay_config_defaults_and_errors(lib, pkg):
    from habitat_sim_gb300 import _lib
    c = _lib.ReplayConfig()
    lib.gbr_replay_config_init(ctypes.byref(c))
    assert c.num_environments == 1 and c.standalone == 1 and c.enable_hbao == 0
    assert list(c.resolution) == [128, 128] and c.hfov_degrees == 90.0
    assert abs(c.near_plane - 0.01) < 1e-9 and c.far_plane == 1000.0
    assert c.draw_mode == 1 and c.max_light_count == 0
    out = ctypes.c_void_p()
    assert lib.gbr_replay_create(None, ctypes.byref(out)) == 1
    c.standalone = 0
    assert lib.gbr_replay_create(ctypes.byref(c), ctypes.byref(out)) == 7
    c.standalone = 1
    c.num_environments = 0
    assert lib.gbr_replay_create(ctypes.byref(c), ctypes.byref(out)) == 1
    c.num_environments = 1
    c.hfov_degrees = 180.0
    assert lib.gbr_replay_create(ctypes.byref(c), ctypes.byref(out)) == 1
    assert lib.gbr_replay_render(None, None, 0, None, 0, 0, None, 0) == 1
    assert b"null replay" in lib.gbr_last_error()
    with pytest.raises(ValueError):
        pkg.ReplayRenderer(pkg.ReplayRendererConfiguration())   # no sensor


def test_replay_create_without_gpu_fails_cleanly(lib, pkg):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    cfg = pkg.ReplayRendererConfiguration()
    cfg.sensor_specifications = [pkg.CameraSensorSpec()]
    with pytest.raises(pkg.GbrError):
        pkg.ReplayRenderer.create_batch_replay_renderer(cfg)
    with pytest.raises(NotImplementedError):
        pkg.ReplayRenderer.create_classic_replay_renderer(cfg)
