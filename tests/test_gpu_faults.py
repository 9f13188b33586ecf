"""Host-side fault injection (GPU tests that fault, trap or hang nothing).

* Device allocations made to fail: a renderer with a device-memory limit
  refuses an addMesh, an addTexture and a first draw with
  GBR_ERROR_OUT_OF_MEMORY, stays usable, and once the limit is lifted the
  same renderer draws output bit-identical to a renderer that never failed.
* Scene records damaged on the device after the host validated them (a
  parent index out of range, a parent cycle): the prepare kernel sets the
  device status word instead of reading out of bounds, the next readback
  returns GBR_ERROR_DEVICE, and the following draw, from the host's records
  uploaded again, is bit-identical to the undamaged one.
"""
import numpy as np
import pytest

import __graft_entry__ as graft

pytestmark = pytest.mark.gpu

OOM, DEVICE = 5, 6


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


def _planes(pkg, r, n):
    return [r.sceneImage(p, s).copy() for s in range(n)
            for p in (pkg.Plane.Color, pkg.Plane.Depth, pkg.Plane.LinearDepth, pkg.Plane.Semantic)]


def _same(a, b):
    return len(a) == len(b) and all(np.array_equal(x.view(np.uint8), y.view(np.uint8)) for x, y in zip(a, b))


def test_allocation_failures_leave_the_renderer_usable(pkg, procedural):
    wl = procedural.config0(seed=3, envs=4, resolution=64, room_subdiv=16, boxes=6)
    poses = procedural.camera_poses(wl, 0)
    good = procedural.build_renderer(pkg, wl, mode=pkg.DrawMode.Batched)
    procedural.set_cameras(good, wl, poses)
    good.draw(mode=pkg.DrawMode.Batched)
    want = _planes(pkg, good, wl.envs)
    good.close()

    cfg = pkg.RendererConfiguration().setTileSizeCount(wl.viewports[0], procedural.grid_for(wl.envs))
    r = pkg.RendererStandalone(cfg, pkg.RendererStandaloneConfiguration().setFlags(
        pkg.RendererStandaloneFlags.QuietLog))
    held, limit = r.deviceMemory()
    assert held > 0 and limit == 0
    r.setDeviceMemoryLimit(held + 4096)
    # A mesh and a texture larger than the headroom are refused.
    n = 100_000
    pos = np.random.default_rng(0).uniform(-1, 1, (n, 3)).astype(np.float32)
    idx = np.arange(3 * (n // 3), dtype=np.uint32)
    with pytest.raises(pkg.GbrError) as e:
        r.addMesh(pos, None, None, None, idx)
    assert e.value.status == OOM
    with pytest.raises(pkg.GbrError) as e:
        r.addTexture(np.zeros((256, 256, 4), np.uint8), 1, 0, 0)
    assert e.value.status == OOM
    assert r.deviceMemory()[0] <= held + 4096
    # Lifted: the workload's resources and scenes go in, then the first draw
    # (which allocates the scene records) is refused under a new limit.
    r.setDeviceMemoryLimit(0)
    procedural.populate(r, wl)
    procedural.set_cameras(r, wl, poses)
    r.setDeviceMemoryLimit(r.deviceMemory()[0])
    with pytest.raises(pkg.GbrError) as e:
        r.draw(mode=pkg.DrawMode.Batched)
    assert e.value.status == OOM
    r.setDeviceMemoryLimit(0)
    r.draw(mode=pkg.DrawMode.Batched)
    assert _same(_planes(pkg, r, wl.envs), want)
    r.close()


@pytest.mark.parametrize("parent,bit", [(10_000, "out of range"), ("self", "deeper than 64")])
def test_device_reports_damaged_scene_records(pkg, procedural, parent, bit):
    wl = procedural.config0(seed=4, envs=4, resolution=64, room_subdiv=16, boxes=6)
    poses = procedural.camera_poses(wl, 1)
    r = procedural.build_renderer(pkg, wl, mode=pkg.DrawMode.Batched)
    procedural.set_cameras(r, wl, poses)
    r.draw(mode=pkg.DrawMode.Batched)
    want = _planes(pkg, r, wl.envs)
    node = len(r.transformations(2)) - 1
    r.debugCorruptParent(2, node, node if parent == "self" else parent)
    r.draw(mode=pkg.DrawMode.Batched)
    with pytest.raises(pkg.GbrError) as e:
        r.sceneImage(pkg.Plane.Color, 0)
    assert e.value.status == DEVICE
    assert bit in str(e.value)
    # The host's records are uploaded again: the next draw is the undamaged one.
    r.draw(mode=pkg.DrawMode.Batched)
    assert _same(_planes(pkg, r, wl.envs), want)
    r.close()
