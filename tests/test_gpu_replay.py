"""Batch replay renderer on the GPU (include/gbr_replay.h through
habitat_sim_gb300.ReplayRenderer) against the oracle's replay restatement:

* BatchReplayRendererTest::testBatchPlayerDeletion (node transforms after
  each keyframe);
* keyframes that load whole .glb files and composite hierarchies, with
  scales, coordinate frames, rotations, metadata, material overrides,
  unsupported primitives, incremental keyframes with deletions, cameras from
  user transforms and explicit matrices, in both draw modes: pixels
  bit-exact against the oracle;
* lights from keyframe light setups; CUDA tensor destinations; RGB
  destinations; unprojection against the classic renderer's known rays
  (BatchReplayRendererTest.cpp:210-255); error reporting and close().
"""
import math
import os

import numpy as np
import pytest

import __graft_entry__ as graft
import scenarios as S
from parity import assert_parity, compare_scene

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
OBJ = os.path.join(HERE, "golden", "objects")
SPHERE = os.path.join(OBJ, "sphere.glb")
TBOX = os.path.join(OBJ, "transform_box.glb")
NBOX = os.path.join(OBJ, "nested_box.glb")
BOXES = os.path.join(OBJ, "5boxes.glb")
COMPOSITE = os.path.join(HERE, "golden", "scenes", "batch-square-circle-triangle.gltf")


@pytest.fixture(scope="module")
def pkg():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return graft.load_package()


def make_pair(pkg, n, resolution, uuid="rgb", hfov=90.0, near=0.01, far=1000.0, lights=0,
              draw_mode=None):
    from oracle import replay as OR
    cfg = pkg.ReplayRendererConfiguration()
    cfg.num_environments = n
    cfg.sensor_specifications = [pkg.CameraSensorSpec(uuid=uuid, resolution=resolution, hfov=hfov,
                                                      near=near, far=far)]
    cfg.quiet = True
    cfg.max_light_count = lights
    if draw_mode is not None:
        cfg.draw_mode = draw_mode
    gpu = pkg.ReplayRenderer.create_batch_replay_renderer(cfg)
    cpu = OR.OracleReplayRenderer(n, resolution=resolution, sensor_uuid=uuid, hfov=hfov,
                                  near=near, far=far, max_light_count=lights)
    for r in (gpu, cpu):
        r.preload_file(COMPOSITE)    # the hierarchies "square", "circle", "triangle"
    return gpu, cpu


def test_batch_player_deletion(pkg):
    """BatchReplayRendererTest::testBatchPlayerDeletion (:400-487)."""
    from test_replay_host import deletion_keyframes
    gpu, _ = make_pair(pkg, 1, (16, 16))
    gpu.set_environment_keyframes(0, pkg.keyframes_to_string(deletion_keyframes(pkg)))
    assert gpu.environment_keyframe_count(0) == (3, -1)
    gpu.set_environment_keyframe_index(0, 0)
    t = gpu.renderer.transformations(0)
    assert t.shape == (4, 4, 4)
    assert np.array_equal(t[0], S.translation(1, 0, 0))
    assert np.array_equal(t[2], S.translation(0, 1, 0))
    gpu.set_environment_keyframe_index(0, 1)
    t = gpu.renderer.transformations(0)
    assert t.shape == (2, 4, 4) and np.array_equal(t[0], S.translation(0, 1, 0))
    gpu.set_environment_keyframe_index(0, 2)
    assert gpu.renderer.transformations(0).shape[0] == 0
    assert gpu.environment_keyframe_count(0) == (3, 2)
    gpu.set_environment_keyframe_index(0, 0)          # back: clear and replay
    assert gpu.renderer.transformations(0).shape[0] == 4
    gpu.close()


def scene_keyframes(pkg, e):
    from habitat_sim_gb300.replay import quaternion_axis_angle as qa
    rng = np.random.default_rng(100 + e)
    K = pkg.Keyframe
    k = (K().load(SPHERE).load(TBOX, up=(0, 0, 1), front=(0, -1, 0)).load(NBOX).load(BOXES)
         .load("square").load("circle").load("cubeSolid"))
    k.create(0, SPHERE, scale=(1.5, 1.5, 1.5)).create(1, TBOX).create(2, NBOX, scale=(0.4, 0.4, 0.4))
    k.create(3, BOXES).create(4, "square").create(5, "circle?{\"override\": 1}").create(6, "cubeSolid")
    for key in range(6):
        pos = (rng.uniform(-1.2, 1.2), rng.uniform(-0.8, 0.8), -rng.uniform(2.5, 5.0))
        k.update(key, pos, qa(rng.normal(size=3), rng.uniform(-180, 180)))
    k.set_metadata(1, 3, 11).set_metadata(3, 4, 22)
    k.user_transform("sensor_rgb", (0.1 * e, 0.05 * e, 0.5), qa((0, 1, 0), 4.0 * e))
    k2 = K().delete(2).create(7, SPHERE).update(7, (0.3, -0.2, -2.0)).update(0, (-0.4, 0.3, -3.0))
    k2.user_transform("sensor_rgb", (0.1 * e, 0.05 * e, 0.4), qa((1, 0, 0), -3.0))
    return k, k2


@pytest.mark.parametrize("mode", [0, 1], ids=["per_scene", "batched"])
def test_replay_matches_oracle(pkg, mode):
    n, res = 5, (48, 64)
    gpu, cpu = make_pair(pkg, n, res, hfov=75.0, near=0.05, far=50.0, draw_mode=mode)
    for e in range(n):
        k, k2 = scene_keyframes(pkg, e)
        for r in (gpu, cpu):
            r.set_environment_keyframe(e, k.to_string())
            if e < 3:                       # incremental keyframe: deletion + new instance
                r.set_environment_keyframe(e, k2.to_string())
            if e == 4:
                m = S.translation(0.2, -0.1, 0.3)
                c, s = math.cos(0.2), math.sin(0.2)
                m[0, 0], m[0, 2], m[2, 0], m[2, 2] = c, -s, s, c
                r.set_sensor_transform(e, "rgb", m)
            else:
                r.set_sensor_transforms_from_keyframe(e, "sensor_")
    colors = [np.zeros(res + (4,), np.uint8) for _ in range(n)]
    depths = [np.zeros(res, np.float32) for _ in range(n)]
    gpu.render(colors, depths)
    ref = cpu.render()
    assert_parity([compare_scene(gpu.renderer, cpu.r, pkg, e) for e in range(n)])
    for e in range(n):
        assert np.array_equal(colors[e], ref[e][0])
        assert np.array_equal(depths[e].view(np.uint32), ref[e][1].view(np.uint32))
        assert (depths[e] > 0).mean() > 0.05
    sem = np.concatenate([gpu.renderer.sceneImage(pkg.Plane.Semantic, e).ravel() for e in range(n)])
    assert {11, 22} <= set(np.unique(sem).tolist())
    # RGB destinations get the first three channels.
    rgb = [np.zeros(res + (3,), np.uint8) for _ in range(n)]
    gpu.render(rgb)
    for e in range(n):
        assert np.array_equal(rgb[e], colors[e][..., :3])
    gpu.close()


def test_replay_lights_match_oracle(pkg):
    gpu, cpu = make_pair(pkg, 2, (32, 32), lights=4)
    for e in range(2):
        k, _ = scene_keyframes(pkg, e)
        k.set_lights([((0.3, -1.0, -0.5, 0.0), (0.8, 0.7, 0.6)),
                      ((0.5, 0.5, -2.0 - e, 1.0), (2.0, 2.0, 2.0))])
        for r in (gpu, cpu):
            r.set_environment_keyframe(e, k.to_string())
            r.set_sensor_transforms_from_keyframe(e, "sensor_")
    gpu.render()
    cpu.render()
    assert_parity([compare_scene(gpu.renderer, cpu.r, pkg, e) for e in range(2)])
    assert gpu.renderer.lightColors(0).shape == (2, 3)
    gpu.close()


def test_replay_tensor_destinations(pkg):
    import torch
    n, res = 3, (32, 40)
    gpu, _ = make_pair(pkg, n, res)
    for e in range(n):
        k, _ = scene_keyframes(pkg, e)
        gpu.set_environment_keyframe(e, k.to_string())
        gpu.set_sensor_transforms_from_keyframe(e, "sensor_")
    host_c = [np.zeros(res + (4,), np.uint8) for _ in range(n)]
    host_d = [np.zeros(res, np.float32) for _ in range(n)]
    gpu.render(host_c, host_d)
    dev_c = [torch.zeros(res + (4,), dtype=torch.uint8, device="cuda") for _ in range(n)]
    dev_d = [torch.zeros(res, dtype=torch.float32, device="cuda") for _ in range(n)]
    gpu.render(dev_c, dev_d, stream=torch.cuda.current_stream())
    ct, dt = gpu.color_tensor(), gpu.depth_tensor()
    for e in range(n):
        assert np.array_equal(dev_c[e].cpu().numpy(), host_c[e])
        assert np.array_equal(dev_d[e].cpu().numpy(), host_d[e])
        assert np.array_equal(gpu.environment_view(ct, e).cpu().numpy(), host_c[e])
        assert np.array_equal(gpu.environment_view(dt, e).cpu().numpy(), host_d[e])
    assert gpu.cuda_color_buffer_device_pointer() == ct.data_ptr()
    assert gpu.cuda_depth_buffer_device_pointer() != gpu.cuda_color_buffer_device_pointer()
    del ct, dt
    gpu.close()


def test_replay_packed_destinations(pkg):
    """Views of one packed array (host or device) take the gather path and
    give the same images as separate destinations."""
    import torch
    n, res = 5, (24, 40)
    gpu, _ = make_pair(pkg, n, res)
    for e in range(n):
        k, _ = scene_keyframes(pkg, e)
        gpu.set_environment_keyframe(e, k.to_string())
        gpu.set_sensor_transforms_from_keyframe(e, "sensor_")
    sep_c = [np.zeros(res + (4,), np.uint8) for _ in range(n)]
    sep_d = [np.zeros(res, np.float32) for _ in range(n)]
    gpu.render(sep_c, sep_d)
    big_c = np.zeros((n,) + res + (4,), np.uint8)
    big_d = np.zeros((n,) + res, np.float32)
    gpu.render(list(big_c), list(big_d))
    dev_c = torch.zeros((n,) + res + (4,), dtype=torch.uint8, device="cuda")
    dev_d = torch.zeros((n,) + res, dtype=torch.float32, device="cuda")
    gpu.render(list(dev_c), list(dev_d))
    for e in range(n):
        assert np.array_equal(big_c[e], sep_c[e]) and np.array_equal(big_d[e], sep_d[e])
        assert np.array_equal(dev_c[e].cpu().numpy(), sep_c[e])
        assert np.array_equal(dev_d[e].cpu().numpy(), sep_d[e])
    # The packed arrays themselves (validated once, one gather per plane).
    big_c[...] = 0
    dev_d.zero_()
    gpu.render(big_c, dev_d)
    for e in range(n):
        assert np.array_equal(big_c[e], sep_c[e])
        assert np.array_equal(dev_d[e].cpu().numpy(), sep_d[e])
    with pytest.raises(ValueError):
        gpu.render(np.zeros((n - 1,) + res + (4,), np.uint8))
    gpu.close()


def test_replay_keyframe_batch(pkg):
    """One set_environment_keyframes_batch call equals the per-environment
    setEnvironmentKeyframe + setSensorTransformsFromKeyframe calls; a
    malformed keyframe anywhere in the batch changes no environment."""
    n, res = 5, (24, 32)
    one, _ = make_pair(pkg, n, res)
    bat, _ = make_pair(pkg, n, res)
    ks = [scene_keyframes(pkg, e) for e in range(n)]
    for e in range(n):
        one.set_environment_keyframe(e, ks[e][0].to_string())
        one.set_environment_keyframe(e, ks[e][1].to_string())
        one.set_sensor_transforms_from_keyframe(e, "sensor_")
    bat.set_environment_keyframes_batch([k.to_string() for k, _ in ks])
    bat.set_environment_keyframes_batch([k2.to_string() for _, k2 in ks], sensor_prefix="sensor_")
    a = [np.zeros(res + (4,), np.uint8) for _ in range(n)]
    b = [np.zeros(res + (4,), np.uint8) for _ in range(n)]
    one.render(a)
    bat.render(b)
    for e in range(n):
        assert np.array_equal(a[e], b[e])
        assert np.array_equal(one.renderer.transformations(e), bat.renderer.transformations(e))
    before = [bat.renderer.transformations(e).copy() for e in range(n)]
    moved = [pkg.Keyframe().update(0, (0.0, 0.0, -9.0)).to_string() for _ in range(3)]
    with pytest.raises(pkg.GbrError, match="environment 4: bad JSON"):
        bat.set_environment_keyframes_batch(moved + ["{\"keyframe\": ["], first_env=1)
    for e in range(n):
        assert np.array_equal(bat.renderer.transformations(e), before[e])
    with pytest.raises(pkg.GbrError, match="exceed the environment count"):
        bat.set_environment_keyframes_batch(moved, first_env=3)
    bat.set_environment_keyframes_batch([])
    one.close()
    bat.close()


def test_replay_keyframe_batch_threads(pkg):
    """A batch large enough to be parsed on several host threads (padded
    documents) applies the same keyframes as the per-environment calls."""
    n, res = 96, (8, 8)
    one, _ = make_pair(pkg, n, res)
    bat, _ = make_pair(pkg, n, res)
    docs = []
    for e in range(n):
        k, _ = scene_keyframes(pkg, e % 7)
        docs.append(k.to_string() + " " * 4096)
    for e in range(n):
        one.set_environment_keyframe(e, docs[e])
        one.set_sensor_transforms_from_keyframe(e, "sensor_")
    bat.set_environment_keyframes_batch(docs, sensor_prefix="sensor_")
    a = np.zeros((n,) + res + (4,), np.uint8)
    b = np.zeros((n,) + res + (4,), np.uint8)
    one.render(a)
    bat.render(b)
    assert np.array_equal(a, b)
    for e in range(n):
        assert np.array_equal(one.renderer.transformations(e), bat.renderer.transformations(e))
    one.close()
    bat.close()


def test_unproject_matches_classic_rays(pkg):
    """testUnproject's rays (BatchReplayRendererTest.cpp:210-255): sensor at
    (1, 2, 3), 512 x 384 (height x width), hfov 90."""
    cfg = pkg.ReplayRendererConfiguration()
    cfg.sensor_specifications = [pkg.CameraSensorSpec(uuid="my_rgb", resolution=(512, 384))]
    cfg.quiet = True
    r = pkg.ReplayRenderer.create_batch_replay_renderer(cfg)
    r.set_sensor_transform(0, "my_rgb", S.translation(1.0, 2.0, 3.0))
    h, w = 512, 384
    cases = [((0, 0), (-0.51544, 0.68457, -0.51544)), ((w, 0), (0.51544, 0.68457, -0.51544)),
             ((w - 1, 0), (0.513467, 0.68551, -0.51615)), ((0, h), (-0.51355, -0.68740, -0.51355)),
             ((0, h - 1), (-0.51449, -0.68599, -0.51450))]
    for pos, want in cases:
        ray = r.unproject(0, pos)
        assert np.allclose(ray.origin, (1, 2, 3))
        assert np.allclose(ray.direction, want, atol=2e-5), (pos, ray.direction)
    r.close()


def test_replay_errors_and_close(pkg):
    gpu, _ = make_pair(pkg, 2, (16, 16))
    with pytest.raises(pkg.GbrError, match="not yet called setEnvironmentKeyframe"):
        gpu.set_sensor_transforms_from_keyframe(0, "sensor_")
    k, _ = scene_keyframes(pkg, 0)
    gpu.set_environment_keyframe(0, k.to_string())
    with pytest.raises(pkg.GbrError, match="couldn't find user transform"):
        gpu.set_sensor_transforms_from_keyframe(0, "other_")
    with pytest.raises(pkg.GbrError, match="out of range"):
        gpu.set_environment_keyframe(5, k.to_string())
    with pytest.raises(pkg.GbrError, match="bad JSON"):
        gpu.set_environment_keyframe(1, "{\"keyframe\": [")
    with pytest.raises(pkg.GbrError, match="no \"keyframe\""):
        gpu.set_environment_keyframe(1, "{}")
    with pytest.raises(pkg.GbrError, match="expected 2 color"):
        gpu.render([np.zeros((16, 16, 4), np.uint8)])
    with pytest.raises(ValueError):
        gpu.render([np.zeros((8, 16, 4), np.uint8)] * 2)
    bad = pkg.Keyframe().load("missing.glb").create(0, "missing.glb")
    with pytest.raises(pkg.GbrError, match="addFile failed"):
        gpu.set_environment_keyframe(1, bad.to_string())
    assert gpu.user_transform(0, "sensor_rgb") is not None
    assert gpu.user_transform(0, "nope") is None
    gpu.clear_environment(0)
    assert gpu.renderer.transformations(0).shape[0] == 0
    assert gpu.environment_count == 2 and gpu.sensor_size(1) == (16, 16)
    gpu.close()
    gpu.close()                                     # closing twice is safe
    with pytest.raises(pkg.GbrError, match="closed"):
        gpu.set_environment_keyframe(0, k.to_string())
