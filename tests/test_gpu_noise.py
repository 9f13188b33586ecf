"""Redwood depth noise on the GPU (include/gbr_noise.h): bit-exact against
the oracle's float32 restatement for the same seed and call counter, the
reference's own statistical GPU-vs-CPU test (tests/test_noise_models.py in
habitat-sim), device and host entry points agreeing, and the batched form
over a renderer's linear-depth plane."""
import numpy as np
import pytest

import __graft_entry__ as graft
from oracle import noise as N

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pkg():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return graft.load_package()


@pytest.fixture(scope="module")
def noise(pkg):
    from habitat_sim_gb300 import noise
    return noise


def depth_cases():
    rng = np.random.default_rng(3)
    ramp = np.linspace(0, 20, num=256 * 256, dtype=np.float32).reshape(256, 256)
    odd = rng.uniform(0.0, 12.0, (97, 131)).astype(np.float32)
    odd[rng.uniform(size=odd.shape) < 0.1] = 0.0
    tall = rng.uniform(0.2, 9.0, (300, 2)).astype(np.float32)
    return [ramp, odd, tall]


@pytest.mark.parametrize("mult", [0.0, 1.0, 2.5])
def test_bit_exact_against_oracle(noise, mult):
    table = N.normal_table()
    model = noise.load_model()
    impl = noise.RedwoodNoiseModelGPUImpl(model, 0, mult, seed=0x1234_5678_9abc)
    for depth in depth_cases():
        for _ in range(2):
            seed, call = impl.get_state()
            got = impl.simulate_from_cpu(depth)
            want = N.redwood_f32(depth, model, mult, seed, call, table=table)
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), \
                (depth.shape, call, int((got != want).sum()))
            assert impl.get_state() == (seed, call + 1)
    impl.close()


def test_reference_gpu_cpu_comparison(noise):
    """habitat-sim's test_compare_gpu_cpu_redwood_depth: 100 simulations of
    a 0-20 m ramp, mean absolute difference of the means."""
    depth = np.linspace(0, 20, num=256 * 256, dtype=np.float32).reshape(256, 256)
    model = noise.load_model()
    rng = np.random.default_rng(2)
    for mult, tol in [(0.0, 1e-5), (1.0, 1e-2)]:
        gpu = noise.RedwoodDepthNoiseModel(noise_multiplier=mult, gpu_device_id=0)
        g = np.mean(np.stack([gpu(depth) for _ in range(100)]), 0)
        c = np.mean(np.stack([N.redwood_reference_cpu(depth, model, mult, rng) for _ in range(100)]), 0)
        assert np.abs(g - c).mean() <= tol


def test_reference_code_comparison(noise):
    """The same statistical test against habitat-sim's own CPU code: the
    means of 100 GPU simulations of the ramp against the means of its
    _simulate, run from the reference's source when the fixture was made
    (tests/golden/make_redwood_means.py)."""
    import os
    ref = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "redwood",
                               "reference_means.npz"))
    depth = np.linspace(0, 20, num=256 * 256, dtype=np.float32).reshape(256, 256)
    for mult, tol, want in [(0.0, 1e-5, ref["mult0"]), (1.0, 1e-2, ref["mult1"])]:
        gpu = noise.RedwoodDepthNoiseModel(noise_multiplier=mult, gpu_device_id=0, seed=31)
        g = np.mean(np.stack([gpu(depth) for _ in range(100)]), 0)
        assert np.abs(g - want).mean() <= tol


def test_device_and_host_paths_agree(noise):
    import torch
    depth = depth_cases()[1]
    m = noise.RedwoodDepthNoiseModel(noise_multiplier=1.0, seed=9)
    m._impl.set_state(9, 40)
    host = m(depth)
    m._impl.set_state(9, 40)
    dev = m(torch.from_numpy(depth).cuda())
    torch.cuda.synchronize()
    assert np.array_equal(dev.cpu().numpy(), host)
    a, b = m(depth), m(depth)
    assert not np.array_equal(a, b)          # the call counter advances


def test_renderer_plane_tiles(pkg, noise):
    """Every environment of a tile-grid renderer noised in one launch equals
    the oracle on that environment's linear depth, image index = scene."""
    import torch
    from habitat_sim_gb300 import procedural
    wl = procedural.config0(seed=3, envs=6, resolution=48, room_subdiv=4, boxes=4)
    r = procedural.build_renderer(pkg, wl)
    procedural.set_cameras(r, wl, procedural.camera_poses(wl, 0))
    r.draw()
    m = noise.RedwoodNoiseModelGPUImpl(noise.load_model(), 0, 1.0, seed=77)
    out = m.apply_to_renderer(r)
    torch.cuda.synchronize()
    plane = r.linearDepthTensor().cpu().numpy()
    got = out.cpu().numpy()
    (tw, th), (tx, _) = r.tileSize(), r.tileCount()
    table = N.normal_table()
    for s in range(r.sceneCount()):
        x0, y0 = (s % tx) * tw, (s // tx) * th
        want = N.redwood_f32(plane[y0:y0 + th, x0:x0 + tw], m._model, 1.0, 77, 0, image=s, table=table)
        assert np.array_equal(got[y0:y0 + th, x0:x0 + tw], want)
    assert m.get_state() == (77, 1)


def test_renderer_plane_ragged(pkg, noise):
    """A ragged (mixed-resolution) framebuffer: every scene noised in one
    launch from the per-scene layout equals the oracle on that scene, image
    index = scene, and equals the tile form's noise of the same image."""
    import torch
    from habitat_sim_gb300 import procedural
    wl = procedural.config2(envs=7, scenes=2, tri_range=(2e4, 3e4), texture_size=64)
    r = procedural.build_renderer(pkg, wl)
    procedural.set_cameras(r, wl, procedural.camera_poses(wl, 0))
    r.draw()
    m = noise.RedwoodNoiseModelGPUImpl(noise.load_model(), 0, 1.0, seed=5)
    out = m.apply_to_renderer(r)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    table = N.normal_table()
    for s in range(r.sceneCount()):
        off, pitch, w, h = r.sceneViewport(s)
        depth = r.sceneImage(pkg.Plane.LinearDepth, s)
        want = N.redwood_f32(depth, m._model, 1.0, 5, 0, image=s, table=table)
        img = np.lib.stride_tricks.as_strided(got.reshape(-1)[off:], shape=(h, w), strides=(4 * pitch, 4))
        assert np.array_equal(img, want), s
    assert m.get_state() == (5, 1)
    # Bad layouts are rejected before any launch.
    src = r.linearDepthTensor()
    with pytest.raises(pkg.GbrError, match="bad layout of image 1"):
        m.simulate_images(src.data_ptr(), out.data_ptr(), [(0, 8, 8, 8), (0, 4, 8, 8)])
    m.close()

