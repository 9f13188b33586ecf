"""Ambient occlusion on the GPU (include/gbr_hbao.h) bit-exact against the
oracle's restatement: every scene of a batch renderer after a draw (with and
without the blur, per-scene projections), the cache-aware algorithm and the
special blur (on the tile grid, on a ragged framebuffer and on one caller
image whose width is not a multiple of 4), one caller image through
hbaoApply, and the replay renderer with enable_hbao."""
import numpy as np
import pytest

import __graft_entry__ as graft
from oracle import hbao as H

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pkg():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return graft.load_package()


@pytest.mark.parametrize("no_blur", [False, True], ids=["blur", "no_blur"])
def test_renderer_scenes_match_oracle(pkg, no_blur):
    from habitat_sim_gb300 import procedural
    wl = procedural.config0(seed=5, envs=6, resolution=48, room_subdiv=4, boxes=6)
    r = procedural.build_renderer(pkg, wl)
    projs, views = procedural.camera_poses(wl, 1)
    r.updateCameras(projs, views)
    r.draw()
    before = [r.sceneImage(pkg.Plane.Color, s) for s in range(len(projs))]
    depth = [r.sceneImage(pkg.Plane.LinearDepth, s) for s in range(len(projs))]
    cfg = pkg.HbaoConfiguration().setNoBlur(no_blur)
    r.drawHbao(cfg)
    changed = 0
    for s in range(len(projs)):
        got = r.sceneImage(pkg.Plane.Color, s)
        want = H.hbao(before[s], depth[s], projs[s], H.config(no_blur=no_blur))
        assert np.array_equal(got, want), (s, int((got != want).any(-1).sum()))
        changed += int((got != before[s]).any(-1).sum())
    assert changed > 0
    # Depth planes are untouched.
    for s in range(len(projs)):
        assert np.array_equal(r.sceneImage(pkg.Plane.LinearDepth, s), depth[s])


def test_ragged_scenes_match_oracle(pkg):
    """A ragged framebuffer (64/128/256 px scenes, per-scene field of view):
    every scene darkened in the same launches equals the oracle on it."""
    from habitat_sim_gb300 import procedural
    wl = procedural.config2(envs=5, scenes=2, tri_range=(2e4, 3e4), texture_size=64)
    r = procedural.build_renderer(pkg, wl)
    projs, views = procedural.camera_poses(wl, 2)
    r.updateCameras(projs, views)
    r.draw()
    n = len(projs)
    before = [r.sceneImage(pkg.Plane.Color, s) for s in range(n)]
    depth = [r.sceneImage(pkg.Plane.LinearDepth, s) for s in range(n)]
    assert len({b.shape for b in before}) > 1          # mixed resolutions
    r.drawHbao(pkg.HbaoConfiguration())
    for s in range(n):
        got = r.sceneImage(pkg.Plane.Color, s)
        want = H.hbao(before[s], depth[s], projs[s], H.config())
        assert np.array_equal(got, want), (s, int((got != want).any(-1).sum()))


@pytest.mark.parametrize("algorithm,blur", [("cache_aware", "bilateral"), ("cache_aware", "none"),
                                            ("cache_aware", "special"), ("classic", "special")])
def test_variants_match_oracle(pkg, algorithm, blur):
    """HbaoType::CacheAware and HbaoFlag::UseAoSpecialBlur on every scene of
    a tile grid and of a ragged framebuffer."""
    from habitat_sim_gb300 import procedural
    ca = algorithm == "cache_aware"
    cfg = pkg.HbaoConfiguration().setAlgorithm(pkg.HbaoType.CacheAware if ca else pkg.HbaoType.Classic)
    cfg.setNoBlur(blur == "none").setUseSpecialBlur(blur == "special")
    want_cfg = H.config(no_blur=blur == "none", special_blur=blur == "special", cache_aware=ca)
    for wl in (procedural.config0(seed=6, envs=4, resolution=48, room_subdiv=4, boxes=6),
               procedural.config2(envs=5, scenes=2, tri_range=(2e4, 3e4), texture_size=64)):
        r = procedural.build_renderer(pkg, wl)
        projs, views = procedural.camera_poses(wl, 3)
        r.updateCameras(projs, views)
        r.draw()
        n = len(projs)
        before = [r.sceneImage(pkg.Plane.Color, s) for s in range(n)]
        depth = [r.sceneImage(pkg.Plane.LinearDepth, s) for s in range(n)]
        r.drawHbao(cfg)
        for s in range(n):
            got = r.sceneImage(pkg.Plane.Color, s)
            want = H.hbao(before[s], depth[s], projs[s], want_cfg)
            assert np.array_equal(got, want), (algorithm, blur, s, int((got != want).any(-1).sum()))
        r.close()


@pytest.mark.parametrize("special", [False, True], ids=["bilateral", "special"])
def test_cache_aware_apply_ragged_edge(pkg, special):
    """One caller image 50 x 37: the quarter-resolution layers overhang the
    image, and their texels beyond it read as the far plane."""
    import torch
    import scenarios as S
    rng = np.random.default_rng(8)
    h, w = 37, 50
    proj = S.perspective(80.0, w / h, 0.05, 20.0)
    y, x = np.mgrid[0:h, 0:w]
    depth = (1.5 + 0.04 * x + 0.4 * np.cos(y / 4.0)).astype(np.float32)
    depth[rng.uniform(size=depth.shape) < 0.05] = 0.0
    color = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    cfg = pkg.HbaoConfiguration().setAlgorithm(pkg.HbaoType.CacheAware).setUseSpecialBlur(special)
    dt = torch.from_numpy(depth).cuda()
    ct = torch.from_numpy(color).cuda()
    pkg.hbaoApply(cfg, proj, dt, ct)
    want = H.hbao(color, depth, proj, H.config(special_blur=special, cache_aware=True))
    assert np.array_equal(ct.cpu().numpy(), want)


def test_hbao_apply_one_image(pkg):
    import torch
    import scenarios as S
    rng = np.random.default_rng(4)
    h, w = 40, 56
    proj = S.perspective(70.0, w / h, 0.05, 20.0)
    y, x = np.mgrid[0:h, 0:w]
    depth = (2.0 + 0.03 * x + 0.5 * np.sin(y / 5.0)).astype(np.float32)
    depth[rng.uniform(size=depth.shape) < 0.05] = 0.0          # background holes
    color = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    cfg = pkg.HbaoConfiguration().setRadius(0.7).setIntensity(1.5)
    dt = torch.from_numpy(depth).cuda()
    ct = torch.from_numpy(color).cuda()
    pkg.hbaoApply(cfg, proj, dt, ct)
    want = H.hbao(color, depth, proj, H.config(radius=0.7, intensity=1.5))
    assert np.array_equal(ct.cpu().numpy(), want)


def test_replay_enable_hbao(pkg):
    from oracle import replay as OR
    from test_gpu_replay import COMPOSITE, scene_keyframes
    n, res = 3, (32, 48)
    cfg = pkg.ReplayRendererConfiguration()
    cfg.num_environments = n
    cfg.sensor_specifications = [pkg.CameraSensorSpec(uuid="rgb", resolution=res, far=50.0)]
    cfg.quiet = True
    cfg.enable_hbao = True
    gpu = pkg.ReplayRenderer.create_batch_replay_renderer(cfg)
    cpu = OR.OracleReplayRenderer(n, resolution=res, sensor_uuid="rgb", far=50.0)
    for r in (gpu, cpu):
        r.preload_file(COMPOSITE)
    for e in range(n):
        k, _ = scene_keyframes(pkg, e)
        for r in (gpu, cpu):
            r.set_environment_keyframe(e, k.to_string())
            r.set_sensor_transforms_from_keyframe(e, "sensor_")
    colors = [np.zeros(res + (4,), np.uint8) for _ in range(n)]
    gpu.render(colors)
    ref = cpu.render()
    for e in range(n):
        want = H.hbao(ref[e][0], ref[e][1], cpu.projection, H.config())
        assert np.array_equal(colors[e], want)
    gpu.close()
