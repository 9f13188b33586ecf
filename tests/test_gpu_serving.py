"""Serving extensions of the C ABI and the serving loop (GPU tests).

* scene sources: a scene bound to another scene's content renders exactly
  what that scene renders with the same camera, in both draw modes;
* disabled scenes: not drawn, their framebuffer rectangle keeps its pixels;
* resource removal: device ranges go back to the free lists and are reused,
  draws and hierarchy adds that still need a removed resource fail with
  GBR_ERROR_STATE, and the pixels of content loaded into reused ranges are
  exact;
* the serving loop: every request served in a mixed batch is bit-identical
  to the same request rendered alone and to the oracle, with and without
  eviction under a small device budget, and after the launch shape is tuned.
"""
import numpy as np
import pytest

import __graft_entry__ as graft

pytestmark = pytest.mark.gpu

STATE = 7
INVALID = 1


@pytest.fixture(scope="module")
def pkg():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return graft.load_package()


@pytest.fixture(scope="module")
def mods(pkg):
    from habitat_sim_gb300 import procedural, server
    return procedural, server


def _renderer(pkg, tile, count, mode=1):
    cfg = pkg.RendererConfiguration().setTileSizeCount(tile, count).setDrawMode(mode)
    return pkg.RendererStandalone(cfg, pkg.RendererStandaloneConfiguration().setFlags(
        pkg.RendererStandaloneFlags.QuietLog))


def _planes(pkg, r, s):
    return [r.sceneImage(p, s).copy() for p in (pkg.Plane.Color, pkg.Plane.Depth,
                                                pkg.Plane.LinearDepth, pkg.Plane.Semantic)]


def _same(a, b):
    return all(np.array_equal(x.view(np.uint8), y.view(np.uint8)) for x, y in zip(a, b))


def _add_asset(r, asset, name, scene):
    """The server's loading of a catalog scene (texture array, mesh, one
    material per layer, one mesh view per object), then an instance in `scene`."""
    from habitat_sim_gb300 import server
    mesh, tex = server.add_asset(r, asset, name)
    if scene is not None:
        r.addNodeHierarchy(scene, name)
    return mesh, tex


@pytest.mark.parametrize("mode,graph", [(0, False), (1, False), (1, True)],
                         ids=["per_scene", "batched", "graph"])
def test_scene_sources(pkg, mods, mode, graph):
    procedural, server = mods
    cat = server.SceneCatalog(2, seed=11, tri_range=(4e3, 2e4))
    r = _renderer(pkg, (96, 80), (2, 2), mode)
    for s in range(2):
        _add_asset(r, cat.asset(s), f"a{s}", s)
    proj = procedural.projection(90.0, 96, 80)
    views = [server.pose_view(0.5, 1.2, 0.3, 0.4 + s, -0.1, 0.05) for s in range(2)]
    r.updateCameras([proj] * 4, views + views)
    r.setSceneSources([0, 1], first=2)
    r.draw(graph=graph)
    for s in range(2):
        assert _same(_planes(pkg, r, s), _planes(pkg, r, s + 2))
        assert (r.sceneImage(pkg.Plane.Semantic, s + 2) > 0).any()
    # Re-binding takes effect at the next draw, without any other change.
    r.setSceneSources([1, 0], first=2)
    r.updateCameras([proj] * 2, views[::-1], first=2)
    r.draw(graph=graph)
    for s in range(2):
        assert _same(_planes(pkg, r, s), _planes(pkg, r, 3 - s))
    with pytest.raises(pkg.GbrError):
        r.setSceneSources([4], first=0)
    with pytest.raises(pkg.GbrError):
        r.setSceneSources([0, 0], first=3)
    r.close()


@pytest.mark.parametrize("graph", [False, True], ids=["plain", "graph"])
def test_disabled_scene_keeps_pixels(pkg, mods, graph):
    procedural, server = mods
    cat = server.SceneCatalog(1, seed=12, tri_range=(4e3, 1e4))
    r = _renderer(pkg, (64, 64), (2, 1))
    _add_asset(r, cat.asset(0), "a", 0)
    r.setSceneSources([0], first=1)
    proj = procedural.projection(90.0, 64, 64)
    v0 = server.pose_view(0.0, 1.2, 0.0, 0.0, 0.0, 0.0)
    v1 = server.pose_view(0.0, 1.2, 0.0, 2.0, 0.0, 0.0)
    r.updateCameras([proj, proj], [v0, v0])
    r.draw(graph=graph)
    before = _planes(pkg, r, 1)
    r.setSceneEnabled(1, False)
    r.updateCameras([proj, proj], [v1, v1])
    r.draw(graph=graph)
    assert _same(before, _planes(pkg, r, 1))          # untouched
    assert not _same(before, _planes(pkg, r, 0))      # scene 0 moved on
    alone = r.lastDrawStats()["visible_draws"]
    assert alone >= 1
    r.setSceneEnabled(1, True)
    r.draw(graph=graph)
    assert _same(_planes(pkg, r, 0), _planes(pkg, r, 1))
    assert r.lastDrawStats()["visible_draws"] == 2 * alone   # same source and camera
    r.close()


def test_remove_and_reuse_ranges(pkg, mods):
    procedural, server = mods
    cat = server.SceneCatalog(3, seed=13, tri_range=(5e3, 2e4))
    a, b = cat.asset(0), cat.asset(1)
    r = _renderer(pkg, (80, 80), (2, 1))
    assert r.memoryUsage() == (4, 4)                   # the reserved white texel
    m0, t0 = _add_asset(r, a, "a", 0)
    live_a = r.memoryUsage()[0] - 4
    assert live_a == a.device_bytes()
    _add_asset(r, b, "b", 1)
    live_ab, reserved_ab = r.memoryUsage()
    proj = procedural.projection(90.0, 80, 80)
    view = server.pose_view(-1.0, 1.5, 1.0, 0.7, -0.2, 0.0)
    r.updateCameras([proj, proj], [view, view])
    r.draw()

    # Removing what scene 0 still draws: the next draw fails, and so does
    # adding a hierarchy whose mesh is gone.
    r.removeMesh(m0)
    with pytest.raises(pkg.GbrError) as e:
        r.draw()
    assert e.value.status == STATE
    with pytest.raises(pkg.GbrError) as e:
        r.addNodeHierarchy(1, "a")
    assert e.value.status == STATE
    r.removeTexture(t0)
    r.removeNodeHierarchyTemplate("a")
    assert not r.hasNodeHierarchy("a")
    r.clear(0)
    assert r.memoryUsage()[0] == live_ab - live_a
    for bad in (lambda: r.removeMesh(m0), lambda: r.removeTexture(t0), lambda: r.removeTexture(0)):
        with pytest.raises(pkg.GbrError) as e:
            bad()
        assert e.value.status == INVALID
    with pytest.raises(pkg.GbrError):
        r.removeNodeHierarchyTemplate("a")

    # The same content again lands in the released ranges: nothing grows.
    _add_asset(r, a, "a2", 0)
    assert r.memoryUsage() == (live_ab, reserved_ab)
    r.draw()
    got = _planes(pkg, r, 0)
    fresh = _renderer(pkg, (80, 80), (1, 1))
    _add_asset(fresh, a, "a", 0)
    fresh.updateCamera(0, proj, view)
    fresh.draw()
    assert _same(got, _planes(pkg, fresh, 0))
    fresh.close()
    r.close()


def _alone(pkg, procedural, asset, req):
    c = req.resolution
    r = _renderer(pkg, (c, c), (1, 1))
    _add_asset(r, asset, "s", 0)
    r.updateCamera(0, procedural.projection(req.hfov, c, c), req.view)
    r.draw()
    out = (r.sceneImage(pkg.Plane.Color, 0), r.sceneImage(pkg.Plane.LinearDepth, 0),
           r.sceneImage(pkg.Plane.Semantic, 0))
    r.close()
    return out


def _oracle(procedural, asset, req):
    from oracle.model import OracleRenderer
    c = req.resolution
    o = OracleRenderer((c, c), (1, 1))
    _add_asset(o, asset, "s", 0)
    o.updateCamera(0, procedural.projection(req.hfov, c, c), req.view)
    o.draw()
    return (o.scene_image(o.color, 0).view(np.uint8).reshape(c, c, 4),
            o.scene_image(o.linear_depth, 0), o.scene_image(o.semantic, 0))


def _check(req, ref):
    color, lin, sem = ref
    assert np.array_equal(req.color, color)
    assert np.array_equal(req.depth.view(np.uint32), lin.view(np.uint32))
    assert np.array_equal(req.semantic, sem.view(np.uint32))


def test_serving_mix_matches_alone_and_oracle(pkg, mods):
    """Textured scenes (1-5 layers of bilinear noise, one material per layer,
    one mesh view per object), as the serving benchmark's catalog has them."""
    procedural, server = mods
    cat = server.SceneCatalog(6, seed=14, tri_range=(2e3, 2e4), texture_side=64, tris_per_layer=4000,
                              pool_bytes=1 << 22)
    assert max(cat.asset(s).texture.shape[0] for s in range(6)) > 1
    reqs = server.random_requests(cat, 48, rate=0, seed=3)
    srv = server.RenderServer(pkg, cat, slots={64: 8, 128: 6, 256: 2}, max_resident=8)
    stats = srv.serve(reqs, realtime=False)
    assert stats["requests"] == 48 and stats["steps"] >= 48 // 16
    assert stats["evictions"] == 0 and stats["loads"] == len({q.scene for q in reqs})
    assert stats["p99_ms"] >= stats["p50_ms"] > 0
    for q in reqs:
        assert q.color.shape == (q.resolution, q.resolution, 4)
        assert (q.semantic > 0).any()
    for q in reqs[::4]:
        _check(q, _alone(pkg, procedural, cat.asset(q.scene), q))
    for q in reqs[:3]:
        _check(q, _oracle(procedural, cat.asset(q.scene), q))
    srv.close()


def test_serving_tune_then_mix_matches_alone(pkg, mods):
    """The launch shape chosen by closed-loop throughput is one of the
    autotuner's candidates, and requests served with it (plane sets
    alternating, copy-back on the second stream) are bit-identical to the
    same requests rendered alone."""
    procedural, server = mods
    from habitat_sim_gb300 import autotune
    cat = server.SceneCatalog(4, seed=17, tri_range=(2e3, 1e4), texture_side=32, tris_per_layer=4000,
                              pool_bytes=1 << 20)
    srv = server.RenderServer(pkg, cat, slots={64: 4, 128: 4, 256: 2}, max_resident=4)
    warm = server.random_requests(cat, 4, rate=0, seed=6)
    for s, q in enumerate(warm):
        q.scene = s
    srv.serve(warm, realtime=False, keep_images=False)
    tuning, trials = srv.tune(lambda: server.random_requests(cat, 30, rate=0, seed=7), reps=1)
    timed = [t for t in trials if "requests_per_s" in t]
    assert len(timed) >= len(autotune.BATCHED_SPACE) and all(t["requests_per_s"] > 0 for t in timed)
    shape = {k: tuning[k] for k in ("threads", "region_width", "region_height", "small_area", "ctas_per_sm")}
    assert shape in [{k: c[k] for k in shape} for c in autotune.BATCHED_SPACE]
    reqs = server.random_requests(cat, 40, rate=0, seed=8)
    stats = srv.serve(reqs, realtime=False)
    assert stats["requests"] == 40 and stats["loads"] == 0
    for q in reqs[::3]:
        _check(q, _alone(pkg, procedural, cat.asset(q.scene), q))
    srv.close()


def test_serving_eviction_under_small_budget(pkg, mods):
    procedural, server = mods
    cat = server.SceneCatalog(8, seed=15, tri_range=(3e3, 3e4), texture_side=32, tris_per_layer=6000,
                              pool_bytes=1 << 20)
    sizes = [cat.asset(s).device_bytes() for s in range(8)]
    budget = int(2.2 * max(sizes))
    reqs = server.random_requests(cat, 40, rate=0, seed=4, zipf=0.8)
    srv = server.RenderServer(pkg, cat, slots={64: 2, 128: 2, 256: 1}, max_resident=3,
                              budget_bytes=budget)
    stats = srv.serve(reqs, realtime=False)
    assert stats["evictions"] > 0 and stats["loads"] > len({q.scene for q in reqs})
    assert srv.residency.bytes <= budget
    assert srv.r.memoryUsage()[0] == 4 + srv.residency.bytes
    for q in reqs[::3]:
        _check(q, _alone(pkg, procedural, cat.asset(q.scene), q))
    srv.close()


def test_serving_realtime_poisson(pkg, mods):
    procedural, server = mods
    cat = server.SceneCatalog(4, seed=16, tri_range=(2e3, 1e4))
    reqs = server.random_requests(cat, 60, rate=300.0, seed=5)
    srv = server.RenderServer(pkg, cat, slots={64: 4, 128: 4, 256: 2}, max_resident=4)
    stats = srv.serve(reqs, realtime=True)
    assert stats["requests"] == 60
    assert all(q.done >= q.arrival for q in reqs)
    assert stats["elapsed_s"] >= reqs[-1].arrival
    srv.close()
