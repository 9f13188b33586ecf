"""CUDA renderer vs the CPU oracle, through the C ABI (GPU tests).

* every golden scenario of habitat-sim's GfxBatchRendererTest, in the
  per-scene and the batched draw modes, against the reference screenshots
  and bit for bit against the oracle;
* seeded procedural workloads (the benchmark configurations at test sizes,
  and the full 1024-env configuration through size-independent properties);
* clipping edge cases, empty and cleared scenes, determinism, DLPack views,
  readback rectangles, device depth unprojection, error reporting.
"""
import math

import numpy as np
import pytest

import __graft_entry__ as graft
import scenarios as S
from parity import assert_parity, compare_scene

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pkg():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return graft.load_package()


@pytest.fixture(scope="module")
def procedural(pkg):
    from habitat_sim_gb300 import procedural
    return procedural


def gpu_factory(pkg, mode):
    def make(tile_size, tile_count, flags):
        cfg = (pkg.RendererConfiguration().setTileSizeCount(tile_size, tile_count)
               .setFlags(flags).setDrawMode(mode))
        return pkg.RendererStandalone(cfg, pkg.RendererStandaloneConfiguration().setFlags(
            pkg.RendererStandaloneFlags.QuietLog))
    return make


@pytest.mark.parametrize("mode", [0, 1], ids=["per_scene", "batched"])
@pytest.mark.parametrize("case", range(len(S.ALL)), ids=S.ids())
def test_golden(pkg, case, mode):
    from oracle.model import OracleRenderer
    _, fn, data = S.ALL[case]
    made = []

    def make(tile_size, tile_count, flags):
        r = gpu_factory(pkg, mode)(tile_size, tile_count, flags)
        made.append(r)
        return r
    fails = S.evaluate(fn(make, data))
    assert not fails, fails
    # Bit-exact against the oracle running the same scenario.
    oracle_checks = fn(lambda ts, tc, fl: OracleRenderer(ts, tc, fl), data)
    gpu_checks = fn(gpu_factory(pkg, mode), data)
    for g, c in zip(gpu_checks, oracle_checks):
        if g.kind == "image":
            assert np.array_equal(g.image, c.image), g.golden


def lit_factory(pkg, mode):
    def make(tile_size, tile_count, flags, max_lights):
        cfg = (pkg.RendererConfiguration().setTileSizeCount(tile_size, tile_count)
               .setFlags(flags).setDrawMode(mode).setMaxLightCount(max_lights))
        return pkg.RendererStandalone(cfg, pkg.RendererStandaloneConfiguration().setFlags(
            pkg.RendererStandaloneFlags.QuietLog))
    return make


@pytest.mark.parametrize("mode", [0, 1], ids=["per_scene", "batched"])
@pytest.mark.parametrize("case", range(len(S.LIT)), ids=S.lit_ids())
def test_golden_lights(pkg, case, mode):
    """GfxBatchRendererTest::lights / clearLights against the reference's
    golden images at its thresholds, and bit for bit against the oracle."""
    from oracle.model import OracleRenderer
    _, fn, data = S.LIT[case]
    gpu_checks = fn(lit_factory(pkg, mode), data)
    fails = S.evaluate(gpu_checks)
    assert not fails, fails
    oracle_checks = fn(lambda ts, tc, fl, ml: OracleRenderer(ts, tc, fl, max_light_count=ml), data)
    for g, c in zip(gpu_checks, oracle_checks):
        if g.kind == "image":
            assert np.array_equal(g.image, c.image), g.golden


def test_lights_errors(pkg):
    r = lit_factory(pkg, 1)((32, 32), (1, 1), 0, 0)
    r.addEmptyNode(0)
    with pytest.raises(pkg.GbrError) as e:
        r.addLight(0, 0, pkg.RendererLightType.Point)
    assert e.value.status == 7
    r = lit_factory(pkg, 1)((32, 32), (1, 1), 0, 2)
    with pytest.raises(pkg.GbrError) as e:
        r.addLight(0, 0, pkg.RendererLightType.Point)   # no node 0 yet
    assert e.value.status == 1
    r.addEmptyNode(0)
    assert r.addLight(0, 0, pkg.RendererLightType.Directional) == 0
    assert r.lightColors(0).shape == (1, 3) and (r.lightColors(0) == 1).all()
    assert np.isinf(r.lightRanges(0)).all()


def test_depth_unprojection_scene(pkg):
    fails = S.evaluate(S.depth_unprojection(gpu_factory(pkg, 1), pkg.unprojectDepth))
    assert not fails, fails


def _parity(pkg, procedural, wl, envs=None, modes=(0, 1), graph=False, steps=(0,),
            require_exact=True):
    from oracle.model import OracleRenderer
    gpu = procedural.build_renderer(pkg, wl, envs=envs)
    cpu = procedural.build_oracle(OracleRenderer, wl, envs=envs)
    n = gpu.sceneCount()
    results = []
    for step in steps:
        poses = procedural.camera_poses(wl, step)
        procedural.set_cameras(gpu, wl, poses, envs)
        procedural.set_cameras(cpu, wl, poses, envs)
        cpu.draw(threads=8)
        for mode in modes:
            gpu.draw(mode=mode, graph=graph and mode == 1)
            results += [compare_scene(gpu, cpu, pkg, s) for s in range(n)]
    assert_parity(results, require_exact)
    return gpu, cpu


def test_config0_full(pkg, procedural):
    """16 envs, 128^2, the 49k-triangle room + 20 boxes, two pose sets."""
    wl = procedural.config0()
    _parity(pkg, procedural, wl, steps=(0, 1))


def test_config0_graph(pkg, procedural):
    wl = procedural.config0(envs=8)
    _parity(pkg, procedural, wl, modes=(1,), graph=True, steps=(0, 1, 2))


def test_config1_subset(pkg, procedural):
    """Textured instancing: 8 of the 1024 envs (two per scene) at full detail."""
    wl = procedural.config1(envs=1024)
    _parity(pkg, procedural, wl, envs=[0, 1, 2, 3, 512, 513, 1022, 1023])


def test_ragged_mixed_resolution(pkg, procedural):
    """Per-env resolution from {64,128,256}^2 and hfov U(60,110) in one batch."""
    wl = procedural.config2(envs=24, scenes=3, tri_range=(2e4, 1.5e5))
    _parity(pkg, procedural, wl)


def test_config3_scan_subset(pkg, procedural):
    """Scan-like rooms (noisy tessellated shell, value-noise colours,
    Voronoi ids per vertex) at 5 cm edges, 256^2, three steps of the random
    walk, both draw modes."""
    wl = procedural.config3(envs=6, scenes=2, edge=0.05)
    _parity(pkg, procedural, wl, steps=(0, 1, 7))


def test_split_work_items_match_per_scene_and_oracle(pkg, procedural):
    """A 150k-triangle scene in a 64 x 64 viewport beside 100 scenes of 2k
    triangles at 128 x 128: the batched form cuts a viewport into smaller
    regions when a region would outweigh half a CTA's share of the step (the
    heavy scene's into 32 x 32 regions).  Every scene of the batched draw
    (graph) equals the per-scene draw, and the heavy scene and a few light
    ones equal the oracle."""
    from habitat_sim_gb300 import server
    from oracle.model import OracleRenderer
    heavy, light = server.serving_scene(99, 150000), server.serving_scene(7, 2000)
    viewports = [(64, 64)] + [(128, 128)] * 100
    cfg = pkg.RendererConfiguration().setViewports(viewports)
    gpu = pkg.RendererStandalone(cfg, pkg.RendererStandaloneConfiguration().setFlags(
        pkg.RendererStandaloneFlags.QuietLog))
    cpu_scenes = [0, 1, 50, 100]
    cpu = OracleRenderer(viewports=[viewports[s] for s in cpu_scenes])
    for r in (gpu, cpu):
        server.add_asset(r, heavy, "heavy")
        server.add_asset(r, light, "light")
    gpu.addNodeHierarchy(0, "heavy")
    for s in range(1, len(viewports)):
        gpu.addNodeHierarchy(s, "light")
    cpu.addNodeHierarchy(0, "heavy")
    for k in range(1, len(cpu_scenes)):
        cpu.addNodeHierarchy(k, "light")
    rng = np.random.default_rng(12)
    n = len(viewports)
    views = server.pose_views(rng.uniform(-5, 5, n), rng.uniform(0.5, 2.5, n), rng.uniform(-5, 5, n),
                              rng.uniform(0, 2 * math.pi, n), np.radians(rng.uniform(-30, 30, n)),
                              np.zeros(n))
    projs = np.stack([procedural.projection(90.0, w, h) for (w, h) in viewports])
    gpu.updateCameras(projs, views)
    cpu.updateCameras(projs[cpu_scenes], views[cpu_scenes])
    cpu.draw(threads=4)
    planes = (pkg.Plane.Color, pkg.Plane.Depth, pkg.Plane.LinearDepth, pkg.Plane.Semantic)
    gpu.draw(mode=1, graph=True)
    batched = [[gpu.sceneImage(p, s).copy() for p in planes] for s in range(n)]
    assert_parity([compare_scene(_Subset(gpu, cpu_scenes), cpu, pkg, k) for k in range(len(cpu_scenes))])
    gpu.draw(mode=0)
    for s in range(n):
        for p, a in zip(planes, batched[s]):
            assert np.array_equal(a.view(np.uint8), gpu.sceneImage(p, s).view(np.uint8)), (s, p)
    assert (batched[0][3] > 0).any()


def test_config2_full_scale_sample(pkg, procedural):
    """The full uneven-batching workload (4096 envs, 64 scenes of 20k-2M
    triangles, mixed 64/128/256 px, hfov U(60, 110)): 16 envs spanning the
    three resolution classes -- the envs of the largest scenes first -- equal
    the oracle, rendered in one batched step with the other envs of their
    ragged framebuffer."""
    from oracle.model import OracleRenderer
    wl = procedural.config2()
    tri = wl.triangles_per_env()
    sample = []
    for c, k in ((64, 5), (128, 6), (256, 5)):
        envs = sorted((e for e in range(wl.envs) if wl.viewports[e][0] == c), key=lambda e: -int(tri[e]))
        sample += envs[:k - 2] + envs[-2:]
    sample = sorted(sample)
    assert max(int(tri[e]) for e in sample) == int(tri.max()) > 1e6   # the largest scene is in
    gpu = procedural.build_renderer(pkg, wl, mode=1, envs=sample)
    cpu = procedural.build_oracle(OracleRenderer, wl, envs=sample)
    poses = procedural.camera_poses(wl, 5)
    procedural.set_cameras(gpu, wl, poses, sample)
    procedural.set_cameras(cpu, wl, poses, sample)
    cpu.draw(threads=8)
    gpu.draw(mode=1, graph=True)
    assert_parity([compare_scene(gpu, cpu, pkg, k) for k in range(len(sample))])


def test_config3_full_density_scene(pkg, procedural):
    """Two 5M-triangle scan rooms at full density: 16 walking envs in one
    batched step equal the per-scene path and the same step with occlusion
    culling off; eight envs (four per room) equal the oracle."""
    from oracle.model import OracleRenderer
    wl = procedural.config3(envs=16, scenes=2)
    gpu = procedural.build_renderer(pkg, wl, mode=1)
    poses = procedural.camera_poses(wl, 3)
    procedural.set_cameras(gpu, wl, poses)
    gpu.draw(mode=1, graph=True)
    planes = (pkg.Plane.Color, pkg.Plane.Depth, pkg.Plane.LinearDepth, pkg.Plane.Semantic)
    ref = [gpu.sceneImage(p, s).copy() for s in range(16) for p in planes]
    gpu.draw(mode=0)
    assert all(np.array_equal(a.view(np.uint8), gpu.sceneImage(p, s).view(np.uint8))
               for a, (s, p) in zip(ref, [(s, p) for s in range(16) for p in planes]))
    gpu.setTuning(occlusion_culling=0)
    gpu.draw(mode=1)
    assert all(np.array_equal(a.view(np.uint8), gpu.sceneImage(p, s).view(np.uint8))
               for a, (s, p) in zip(ref, [(s, p) for s in range(16) for p in planes]))
    sample = [0, 1, 4, 7, 9, 10, 13, 14]
    cpu = procedural.build_oracle(OracleRenderer, wl, envs=sample)
    procedural.set_cameras(cpu, wl, poses, sample)
    cpu.draw(threads=8)
    assert_parity([compare_scene(_Subset(gpu, sample), cpu, pkg, k) for k in range(len(sample))])


class _Subset:
    """The GPU renderer seen through a list of its scenes (for compare_scene)."""

    def __init__(self, r, scenes):
        self.r, self.scenes = r, scenes

    def sceneImage(self, plane, k):
        return self.r.sceneImage(plane, self.scenes[k])


def look_view(x, y, z, yaw, pitch):
    """View matrix ([col][row] float32) of a camera at (x, y, z) turned by yaw
    about +y, then pitch about its x axis."""
    cy, sy, cp, sp = math.cos(yaw), math.sin(yaw), math.cos(pitch), math.sin(pitch)
    ry = np.array([[cy, 0, sy, 0], [0, 1, 0, 0], [-sy, 0, cy, 0], [0, 0, 0, 1]])
    rx = np.array([[1, 0, 0, 0], [0, cp, -sp, 0], [0, sp, cp, 0], [0, 0, 0, 1]])
    t = np.eye(4)
    t[:3, 3] = [x, y, z]
    cam_to_world = t @ ry @ rx
    return np.linalg.inv(cam_to_world).T.astype(np.float32)


def _wall_hugging_workload(procedural):
    wl = procedural.config0(seed=11, envs=6, resolution=96, room_subdiv=8, boxes=4)
    return wl


def test_near_plane_and_guard_band(pkg, procedural):
    """Cameras 1-5 mm from walls and inside boxes: triangles cross the near
    plane and project far outside the viewport (clipping paths)."""
    from oracle.model import OracleRenderer
    wl = _wall_hugging_workload(procedural)
    gpu = procedural.build_renderer(pkg, wl)
    cpu = procedural.build_oracle(OracleRenderer, wl)
    projs, views = procedural.camera_poses(wl, 0)
    spots = [(-3.999, 1.0, 0.0, 0.3), (3.995, 2.999, 3.9, 2.0), (0.0, 0.005, 0.0, 1.0),
             (0.0, 1.25, -3.998, math.pi), (2.0, 1.0, 3.999, 0.01), (-3.99, 0.002, -3.99, 0.8)]
    for e, (x, y, z, yaw) in enumerate(spots):
        views[e] = look_view(x, y, z, yaw, -1.0 if e % 2 else 0.0)
    gpu.updateCameras(projs, views)
    cpu.updateCameras(projs, views)
    cpu.draw()
    results = []
    for mode in (0, 1):
        gpu.draw(mode=mode)
        results += [compare_scene(gpu, cpu, pkg, s) for s in range(wl.envs)]
    assert_parity(results)


def test_huge_triangle_guard_band(pkg):
    """A 2-triangle quad 1e5 m wide crossing the near plane and the guard band."""
    from oracle.model import OracleRenderer
    pos = np.array([[-1e5, -1, -1e5], [1e5, -1, -1e5], [1e5, -1, 1e5], [-1e5, -1, 1e5]],
                   np.float32)
    col = np.array([[1, 0, 0, 1], [0, 1, 0, 1], [0, 0, 1, 1], [1, 1, 1, 1]], np.float32)
    idx = np.array([0, 3, 2, 0, 2, 1], np.uint32)  # faces +y
    proj = S.perspective(90.0, 1.0, 0.01, 10.0)
    outs = []
    for r in (gpu_factory(pkg, 1)((64, 64), (2, 1), 0), OracleRenderer((64, 64), (2, 1), 0)):
        m = r.addMesh(pos, col, None, None, idx)
        r.addNodeHierarchyTemplate("floor", [(m, 0, 6, 0, None)])
        for s in range(2):
            r.addNodeHierarchy(s, "floor")
        r.updateCamera(0, proj, S.translation(0.0, 0.0, 0.0))
        tilt = np.eye(4, dtype=np.float32)
        c, s_ = np.float32(math.cos(0.7)), np.float32(math.sin(0.7))
        tilt[1, 1], tilt[1, 2], tilt[2, 1], tilt[2, 2] = c, s_, -s_, c
        r.updateCamera(1, proj, tilt)
        r.draw()
        outs.append(r)
    gpu, cpu = outs
    res = [compare_scene(gpu, cpu, pkg, s) for s in range(2)]
    assert_parity(res)
    assert (gpu.colorImage()[..., 3] == 255).all()


@pytest.mark.parametrize("mode", [0, 1], ids=["per_scene", "batched"])
def test_queue_overflow_many_big_triangles(pkg, mode):
    """3072 viewport-sized triangles at random (and some equal) depths: one
    round of 256 threads queues more large triangles than the shared queue
    holds, so the rest go through the spill area; bit-exact against the
    oracle, depth ties resolved by draw order."""
    from oracle.model import OracleRenderer
    rng = np.random.default_rng(11)
    n = 3072
    z = rng.uniform(-3.0, -1.0, n).astype(np.float32)
    z[::7] = np.float32(-2.0)                          # coplanar groups: ties
    cx, cy = rng.uniform(-0.5, 0.5, (2, n)).astype(np.float32)
    pos = np.zeros((3 * n, 3), np.float32)
    for k, (dx, dy) in enumerate([(-3.0, -3.0), (3.0, -3.0), (0.0, 3.0)]):
        pos[k::3, 0] = (cx + dx) * -z
        pos[k::3, 1] = (cy + dy) * -z
        pos[k::3, 2] = z
    col = rng.uniform(0, 1, (3 * n, 4)).astype(np.float32)
    col[:, 3] = 1.0
    idx = np.arange(3 * n, dtype=np.uint32)
    proj = S.perspective(60.0, 1.0, 0.1, 10.0)
    outs = []
    for r in (gpu_factory(pkg, mode)((64, 64), (2, 1), 0), OracleRenderer((64, 64), (2, 1), 0)):
        if hasattr(r, "setTuning"):
            r.setTuning(threads=256, region_width=64, region_height=64)
        m = r.addMesh(pos, col, None, None, idx)
        r.addNodeHierarchyTemplate("stack", [(m, 0, 3 * n, 0, None)])
        for s in range(2):
            r.addNodeHierarchy(s, "stack")
        r.updateCamera(0, proj, S.translation(0.0, 0.0, 0.0))
        r.updateCamera(1, proj, S.translation(0.3, -0.2, 0.5))
        r.draw()
        outs.append(r)
    gpu, cpu = outs
    assert_parity([compare_scene(gpu, cpu, pkg, s) for s in range(2)])
    assert (gpu.colorImage()[..., 3] == 255).all()


def test_empty_and_cleared_scenes(pkg, procedural):
    wl = procedural.config0(seed=3, envs=4, resolution=32, room_subdiv=4, boxes=2)
    gpu = procedural.build_renderer(pkg, wl)
    procedural.set_cameras(gpu, wl, procedural.camera_poses(wl, 0))
    gpu.clear(1)
    gpu.clear(3)
    gpu.draw()
    for s in (1, 3):
        assert (gpu.sceneImage(pkg.Plane.Color, s).view(np.uint32) == 0xFF1F1F1F).all()
        assert (gpu.sceneImage(pkg.Plane.Depth, s) == 1.0).all()
        assert (gpu.sceneImage(pkg.Plane.LinearDepth, s) == 0.0).all()
        assert (gpu.sceneImage(pkg.Plane.Semantic, s) == 0).all()
    assert (gpu.sceneImage(pkg.Plane.Semantic, 0) > 0).any()


def test_no_file_added(pkg):
    """renderNoFileAdded (GfxBatchRendererTest.cpp:1724-1735)."""
    r = gpu_factory(pkg, 0)((64, 48), (2, 2), 0)
    r.draw()
    assert (r.colorImage().reshape(-1, 4) == [31, 31, 31, 255]).all()


def test_deterministic_and_modes_agree(pkg, procedural):
    wl = procedural.config1(envs=16, instances=60)
    gpu = procedural.build_renderer(pkg, wl)
    procedural.set_cameras(gpu, wl, procedural.camera_poses(wl, 5))
    imgs = []
    for mode, graph in ((0, False), (1, False), (1, True), (1, True)):
        gpu.draw(mode=mode, graph=graph)
        imgs.append((gpu.colorImage(), gpu.linearDepthImage(), gpu.semanticImage()))
    for other in imgs[1:]:
        for a, b in zip(imgs[0], other):
            assert np.array_equal(a, b)


def test_dlpack_and_device_pointers(pkg, procedural):
    import torch
    wl = procedural.config0(seed=5, envs=4, resolution=64, room_subdiv=8, boxes=3)
    gpu = procedural.build_renderer(pkg, wl)
    procedural.set_cameras(gpu, wl, procedural.camera_poses(wl, 0))
    gpu.draw(stream=torch.cuda.current_stream())
    col = gpu.colorTensor()
    assert col.is_cuda and col.dtype == torch.uint8 and tuple(col.shape) == (128, 128, 4)
    assert np.array_equal(col.cpu().numpy(), gpu.colorImage())
    assert np.array_equal(gpu.linearDepthTensor().cpu().numpy(), gpu.linearDepthImage())
    assert np.array_equal(gpu.semanticTensor().cpu().numpy().astype(np.uint32),
                          gpu.semanticImage())
    ptr = gpu.colorCudaBufferDevicePointer()
    assert ptr == col.data_ptr()
    dep = gpu.depthTensor()
    assert gpu.depthCudaBufferDevicePointer() == dep.data_ptr()
    expected = gpu.colorImage().copy()
    gpu.close()  # the tensor keeps the renderer's memory alive
    assert np.array_equal(col.cpu().numpy(), expected)


def test_image_into_rectangles(pkg, procedural):
    wl = procedural.config0(seed=6, envs=4, resolution=48, room_subdiv=8, boxes=3)
    gpu = procedural.build_renderer(pkg, wl)
    procedural.set_cameras(gpu, wl, procedural.camera_poses(wl, 0))
    gpu.draw()
    full = gpu.colorImage()
    part = np.empty((20, 30, 4), np.uint8)
    gpu.colorImageInto(((10, 5), (40, 25)), part)
    assert np.array_equal(part, full[5:25, 10:40])
    dpart = np.empty((48, 48), np.float32)
    gpu.depthImageInto(((48, 48), (96, 96)), dpart)
    assert np.array_equal(dpart, gpu.depthImage()[48:96, 48:96])
    with pytest.raises(pkg.GbrError):
        gpu.colorImageInto(((0, 0), (97, 10)), np.empty((10, 97, 4), np.uint8))


@pytest.mark.parametrize("graph", [False, True], ids=["plain", "graph"])
def test_double_buffer_async_readback(pkg, procedural, graph):
    """Double-buffered planes with asynchronous readback: each step's images
    (read while the next step draws) equal a single-buffered renderer's
    synchronous images of the same poses; a ragged layout reads one row."""
    import torch
    wl = procedural.config0(seed=8, envs=6, resolution=64, room_subdiv=16, boxes=6)
    ref = procedural.build_renderer(pkg, wl, mode=1)
    dbl = procedural.build_renderer(pkg, wl, mode=1, double_buffer=True)
    fbw, fbh = dbl.framebufferSize()
    rect = ((0, 0), (fbw, fbh))
    bufs = [(torch.empty((fbh, fbw, 4), dtype=torch.uint8, pin_memory=True).numpy(),
             torch.empty((fbh, fbw), dtype=torch.float32, pin_memory=True).numpy(),
             torch.empty((fbh, fbw), dtype=torch.int32, pin_memory=True).numpy())
            for _ in range(4)]
    planes = (pkg.Plane.Color, pkg.Plane.LinearDepth, pkg.Plane.Semantic)
    for k in range(4):
        procedural.set_cameras(dbl, wl, procedural.camera_poses(wl, k))
        dbl.draw(graph=graph)
        for p, b in zip(planes, bufs[k]):
            dbl.imageIntoAsync(p, rect, b)
    dbl.readbackWait()
    for k in range(4):
        procedural.set_cameras(ref, wl, procedural.camera_poses(wl, k))
        ref.draw(graph=graph)
        assert np.array_equal(bufs[k][0], ref.colorImage())
        assert np.array_equal(bufs[k][1].view(np.uint32), ref.linearDepthImage().view(np.uint32))
        assert np.array_equal(bufs[k][2].view(np.uint32), ref.semanticImage())
    # the synchronous calls read the last draw's set
    assert np.array_equal(dbl.colorImage(), ref.colorImage())
    wl2 = procedural.config2(envs=5, scenes=2, tri_range=(2e4, 4e4))
    rag = procedural.build_renderer(pkg, wl2, mode=1, double_buffer=True)
    procedural.set_cameras(rag, wl2, procedural.camera_poses(wl2, 0))
    rag.draw(graph=graph)
    n = rag.framebufferSize()[0]
    row = np.empty((1, n, 4), np.uint8)
    rag.imageIntoAsync(pkg.Plane.Color, ((0, 0), (n, 1)), row)
    rag.readbackWait()
    off, _, w, h = rag.sceneViewport(3)
    assert np.array_equal(row[0, off:off + w * h].reshape(h, w, 4),
                          rag.sceneImage(pkg.Plane.Color, 3))


@pytest.mark.parametrize("ragged", [False, True], ids=["tiles", "ragged"])
def test_scenes_into_async(pkg, procedural, ragged):
    """Packed batched readback into host arrays and device tensors equals
    the per-scene readback, for a sub-range of scenes."""
    import torch
    wl = procedural.config0(seed=7, envs=7, resolution=40, room_subdiv=4, boxes=3)
    if ragged:
        wl.viewports = [(40, 40)] * wl.envs
        wl.uniform = False
    r = procedural.build_renderer(pkg, wl)
    procedural.set_cameras(r, wl, procedural.camera_poses(wl, 2))
    r.draw()
    first, count = 2, 5
    for plane, dt, shape in ((pkg.Plane.Color, np.uint8, (40, 40, 4)),
                             (pkg.Plane.LinearDepth, np.float32, (40, 40)),
                             (pkg.Plane.Semantic, np.uint32, (40, 40))):
        host = np.zeros((count,) + shape, dt)
        r.scenesIntoAsync(plane, first, count, host)
        tdt = {np.uint8: torch.uint8, np.float32: torch.float32, np.uint32: torch.int32}[dt]
        dev = torch.zeros((count,) + shape, dtype=tdt, device="cuda")
        r.scenesIntoAsync(plane, first, count, dev)
        r.readbackWait()
        for i in range(count):
            want = r.sceneImage(plane, first + i)
            assert np.array_equal(host[i], want)
            assert np.array_equal(dev[i].cpu().numpy().view(dt), want)
    with pytest.raises(pkg.GbrError):
        r.scenesIntoAsync(pkg.Plane.Color, 5, 5, np.zeros((5, 40, 40, 4), np.uint8))


@pytest.mark.parametrize("kw", [
    dict(filter=1, minFilter=1, mipFilter=1, generateMipmap=True),
    dict(filter=1, minFilter=2, mipFilter=1, generateMipmap=True),
    dict(filter=0, minFilter=1, mipFilter=2, generateMipmap=True),
    dict(filter=1, minFilter=2, mipFilter=2, generateMipmap=True),
    dict(filter=1, minFilter=1, mipFilter=0),
    dict(filter=0, minFilter=2, mipFilter=2, levels=True),
], ids=["nn", "ln", "nl", "ll", "min_nearest_no_mips", "given_levels"])
def test_mipmapped_floor_matches_oracle(pkg, kw):
    """A checkered floor receding to the horizon (minified far away): level
    of detail, level selection and filtering bit-exact against the oracle."""
    from oracle.model import OracleRenderer, generate_mips
    from test_mipmaps_host import floor_scene
    kw = dict(kw)
    if kw.pop("levels", False):
        y, x = np.mgrid[0:64, 0:64]
        rng = np.random.default_rng(3)
        base = rng.integers(0, 256, (1, 64, 64, 4), dtype=np.uint8)
        chain = [c[0] for c in generate_mips(base, 5)]   # 5 of the 7 possible levels
        kw.update(levels=True)
    outs = []
    for r in (gpu_factory(pkg, 1)((96, 96), (1, 1), 0), OracleRenderer((96, 96), (1, 1), 0)):
        if kw.get("levels"):
            k2 = dict(kw)
            k2["levels"] = len(chain)
            floor_scene(r, k2, pixels=chain)
        else:
            floor_scene(r, kw)
        r.draw()
        outs.append(r)
    gpu, cpu = outs
    assert_parity([compare_scene(gpu, cpu, pkg, 0)])


def test_unproject_device_matches_host(pkg):
    import torch
    p = S.perspective(60.0, 1.0, 0.01, 10.0)
    u = pkg.calculateDepthUnprojection(p)
    d = torch.rand(64, 80, device="cuda")
    d[::7, ::5] = 1.0
    host = d.cpu().numpy().copy()
    pkg.unprojectDepthDevice(u, d)
    torch.cuda.synchronize()
    pkg.unprojectDepth(u, host)
    assert np.array_equal(d.cpu().numpy().view(np.uint32), host.view(np.uint32))


def test_errors(pkg, procedural):
    r = gpu_factory(pkg, 0)((32, 32), (1, 1), 0)
    assert r.addFile("/nonexistent/file.gltf") is False
    with pytest.raises(pkg.GbrError) as e:
        r.addNodeHierarchy(0, "nothing")
    assert e.value.status == 2
    with pytest.raises(pkg.GbrError) as e:
        r.addNodeHierarchy(5, "nothing")
    assert e.value.status == 1
    with pytest.raises(pkg.GbrError):
        r.addMesh(np.zeros((3, 3)), indices=np.array([0, 1, 3]))
    # A large index array is checked on the host's worker pool: the first bad
    # index is reported, and nothing is added.
    idx = np.tile(np.array([0, 1, 2], np.uint32), 200000)
    idx[456791] = 3
    idx[500000] = 7
    live = r.memoryUsage()[0]
    with pytest.raises(pkg.GbrError) as e:
        r.addMesh(np.zeros((3, 3), np.float32), indices=idx)
    assert e.value.status == 1 and "index 456791 out of range for 3 vertices" in str(e.value)
    assert r.memoryUsage()[0] == live
    idx[456791] = idx[500000] = 2
    assert r.addMesh(np.zeros((3, 3), np.float32), indices=idx) >= 0
    with pytest.raises(pkg.GbrError):
        r.setTuning(threads=100)


def test_config1_full_size_properties(pkg, procedural):
    """All 1024 envs of the textured-instancing workload in one batched
    step: every pixel written, ids and depths in range, the batched output
    equals the per-scene output, and sampled envs equal the oracle."""
    from oracle.model import OracleRenderer
    wl = procedural.config1()
    gpu = procedural.build_renderer(pkg, wl, mode=1)
    poses = procedural.camera_poses(wl, 3)
    procedural.set_cameras(gpu, wl, poses)
    gpu.draw(mode=1, graph=True)
    col, lin, sem = gpu.colorImage(), gpu.linearDepthImage(), gpu.semanticImage()
    valid_ids = (sem == 0) | (sem == 1) | ((sem >= 1000) & (sem < 1200))
    assert valid_ids.all()
    assert ((lin == 0) | ((lin >= 0.0099) & (lin <= 10.0))).all()
    assert ((sem == 0) == (lin == 0)).all()
    gpu.draw(mode=0)
    assert np.array_equal(col, gpu.colorImage())
    assert np.array_equal(sem, gpu.semanticImage())
    # Occlusion culling of chunks is exact: switching it off changes no pixel.
    dep = gpu.depthImage()
    gpu.setTuning(occlusion_culling=0)
    gpu.draw(mode=1, graph=True)
    assert np.array_equal(col, gpu.colorImage())
    assert np.array_equal(dep.view(np.uint32), gpu.depthImage().view(np.uint32))
    assert np.array_equal(lin.view(np.uint32), gpu.linearDepthImage().view(np.uint32))
    assert np.array_equal(sem, gpu.semanticImage())
    gpu.setTuning(occlusion_culling=1)
    sample = [0, 137, 500, 1023]
    cpu = procedural.build_oracle(OracleRenderer, wl, envs=sample)
    procedural.set_cameras(cpu, wl, poses, sample)
    cpu.draw(threads=8)
    res = []
    for slot, e in enumerate(sample):
        _, _, w, h = gpu.sceneViewport(e)
        for plane, arr in ((pkg.Plane.Color, cpu.color), (pkg.Plane.LinearDepth, cpu.linear_depth),
                           (pkg.Plane.Semantic, cpu.semantic)):
            g = gpu.sceneImage(plane, e)
            c = cpu.scene_image(arr, slot)
            if plane == pkg.Plane.Color:
                c = c.view(np.uint8).reshape(g.shape)
            res.append(np.array_equal(g, c))
    assert all(res), res
