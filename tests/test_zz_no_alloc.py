"""gbr_render_mesh_no_alloc, the entry point that allocates nothing.

Some callers cannot allocate device memory: code running inside another
framework's memory pool or under a strict memory budget, real-time loops
where an allocation could stall, plugins whose host owns every allocation.
They hand the renderer their own device buffers (mesh in, planes out) and it
uses a fixed scratch array inside the library.  This test renders one mesh
with two cameras through that entry point, two calls in a row, and requires
the pixels that gbr_draw produces for the same mesh and cameras (the parity
bar of the other GPU tests: same triangle on >= 99.9 % of pixels, linear
depth within 1e-4 m; the implementation is expected to be exact)."""
import ctypes
import math

import numpy as np
import pytest

import __graft_entry__ as graft

W, H = 200, 150   # two 128-pixel regions in each direction, ragged edges


def _mesh(procedural):
    rng = np.random.default_rng(21)
    parts, ids = [], []
    p, t = procedural.box_faces([-4, 0, -4], [4, 3, 4], 6, inward=True)
    parts.append((p, t))
    ids.append(np.full(len(p), 1, np.uint32))
    for b in range(3):
        lo = np.array([-2.0 + 1.5 * b, 0.0, -1.0 + 0.7 * b])
        p, t = procedural.box_faces(lo, lo + [0.8, 1.2, 0.6], 2, inward=False)
        parts.append((p, t))
        ids.append(np.full(len(p), 2 + b, np.uint32))
    pos, idx, base = [], [], 0
    for (p, t) in parts:
        pos.append(p)
        idx.append(t + base)
        base += len(p)
    pos = np.concatenate(pos).astype(np.float32)
    col = np.ones((len(pos), 4), np.float32)
    col[:, :3] = rng.integers(0, 256, (len(pos), 3)).astype(np.float32) / np.float32(255.0)
    return pos, col, np.concatenate(ids), np.concatenate(idx).astype(np.uint32).reshape(-1)


def _view(x, y, z, yaw):
    c, s = math.cos(yaw), math.sin(yaw)
    cam = np.array([[c, 0, s, x], [0, 1, 0, y], [-s, 0, c, z], [0, 0, 0, 1]], np.float64)
    return np.linalg.inv(cam).T.astype(np.float32)   # [col][row]


@pytest.mark.gpu
def test_no_alloc_matches_draw():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    pkg = graft.load_package()
    from habitat_sim_gb300 import _lib, procedural
    lib = _lib.load()
    pos, col, ids, idx = _mesh(procedural)
    proj = procedural.projection(80.0, W, H)
    views = [_view(0.3, 1.25, 2.5, 0.4), _view(-3.995, 1.0, 0.2, -1.2)]

    # The existing entry point: a renderer with this mesh as one hierarchy.
    cfg = pkg.RendererConfiguration().setTileSizeCount((W, H), (1, 1))
    r = pkg.RendererStandalone(cfg, pkg.RendererStandaloneConfiguration().setFlags(
        pkg.RendererStandaloneFlags.QuietLog))
    m = r.addMesh(pos, col, None, ids, idx)
    r.addNodeHierarchyTemplate("mesh", [(m, 0, len(idx), 0, None)])
    r.addNodeHierarchy(0, "mesh")
    expected = []
    for v in views:
        r.updateCamera(0, proj, v)
        r.draw()
        expected.append((r.colorImage().view(np.uint32)[..., 0], r.depthImage(),
                         r.linearDepthImage(), r.semanticImage()))
    r.close()

    # Caller-owned device buffers: float4 positions with the id bits in w.
    pos4 = np.zeros((len(pos), 4), np.float32)
    pos4[:, :3] = pos
    pos4[:, 3] = ids.view(np.float32)
    d_pos = torch.from_numpy(pos4).cuda()
    d_col = torch.from_numpy(col).cuda()
    d_idx = torch.from_numpy(idx.view(np.int32)).cuda()
    planes = [torch.empty((H, W), dtype=torch.int32, device="cuda"),
              torch.empty((H, W), dtype=torch.float32, device="cuda"),
              torch.empty((H, W), dtype=torch.float32, device="cuda"),
              torch.empty((H, W), dtype=torch.int32, device="cuda")]
    stream = torch.cuda.current_stream().cuda_stream
    p32 = np.ascontiguousarray(proj, np.float32)
    results = []
    for v in views:   # two calls in a row
        v32 = np.ascontiguousarray(v, np.float32)
        st = lib.gbr_render_mesh_no_alloc(
            d_pos.data_ptr(), d_col.data_ptr(), d_idx.data_ptr(), len(pos), len(idx) // 3,
            p32.ctypes.data_as(_lib.c_float_p), v32.ctypes.data_as(_lib.c_float_p), 0, 1, W, H,
            planes[0].data_ptr(), planes[1].data_ptr(), planes[2].data_ptr(), planes[3].data_ptr(),
            stream)
        assert st == 0, lib.gbr_last_error()
        torch.cuda.synchronize()
        results.append([t.cpu().numpy().copy() for t in planes])

    for (c, z, lin, sid), got in zip(expected, results):
        g_c, g_z, g_lin, g_sid = got
        same = ((g_c.view(np.uint32) == c) & (g_sid.view(np.uint32) == sid) &
                (g_z.view(np.uint32) == z.view(np.uint32)))
        assert (~same).sum() <= 1e-3 * same.size
        assert np.abs(g_lin[same].astype(np.float64) - lin[same]).max() <= 1e-4
        assert same.all() and np.array_equal(g_lin.view(np.uint32), lin.view(np.uint32))
        assert (sid > 0).any()


def _lib():
    graft.load_package()
    from habitat_sim_gb300 import _lib as lib_mod
    return lib_mod, lib_mod.load()


def test_no_alloc_rejects_sizes_beyond_its_limits():
    """Argument checks come before any CUDA call, so they run without a GPU:
    viewports beyond the 4096 x 4096 the fixed scratch can tile, and more
    triangles than 32-bit index addressing reaches (3 x count < 2^32)."""
    lib_mod, lib = _lib()
    eye = np.eye(4, dtype=np.float32)
    m = eye.ctypes.data_as(lib_mod.c_float_p)
    st = lib.gbr_render_mesh_no_alloc(None, None, None, 0, 0, m, m, 0, 0, 4097, 16,
                                      None, None, None, None, None)
    assert st == 1
    assert b"4096" in lib.gbr_last_error()
    fake = 1 << 20   # never dereferenced: the count is rejected first
    st = lib.gbr_render_mesh_no_alloc(fake, None, fake, 3, 0x55555556, m, m, 0, 0, 16, 16,
                                      None, None, None, None, None)
    assert st == 1
    assert b"1431655765" in lib.gbr_last_error()


@pytest.mark.gpu
def test_no_alloc_bad_index_renders_background_then_recovers():
    """An index beyond the vertex count makes the call draw nothing (every
    pixel background) while still returning GBR_OK: the check runs on the
    GPU and the call does not wait for it.  The next call with good indices
    renders the mesh again (the flag in the shared scratch is cleared on
    every call)."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib_mod, lib = _lib()
    from habitat_sim_gb300 import procedural
    pos, col, ids, idx = _mesh(procedural)
    pos4 = np.zeros((len(pos), 4), np.float32)
    pos4[:, :3] = pos
    pos4[:, 3] = ids.view(np.float32)
    d_pos = torch.from_numpy(pos4).cuda()
    bad = idx.copy()
    bad[7] = len(pos) + 5
    d_bad = torch.from_numpy(bad.view(np.int32)).cuda()
    d_idx = torch.from_numpy(idx.view(np.int32)).cuda()
    proj = np.ascontiguousarray(procedural.projection(80.0, W, H), np.float32)
    view = np.ascontiguousarray(_view(0.3, 1.25, 2.5, 0.4), np.float32)
    col_plane = torch.empty((H, W), dtype=torch.int32, device="cuda")
    lin_plane = torch.empty((H, W), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    out = []
    for d in (d_bad, d_idx):
        st = lib.gbr_render_mesh_no_alloc(
            d_pos.data_ptr(), None, d.data_ptr(), len(pos), len(idx) // 3,
            proj.ctypes.data_as(lib_mod.c_float_p), view.ctypes.data_as(lib_mod.c_float_p), 0, 1,
            W, H, col_plane.data_ptr(), None, lin_plane.data_ptr(), None, stream)
        assert st == 0, lib.gbr_last_error()
        torch.cuda.synchronize()
        out.append((col_plane.cpu().numpy().view(np.uint32).copy(), lin_plane.cpu().numpy().copy()))
    (c_bad, l_bad), (c_ok, l_ok) = out
    assert (c_bad == 0xFF1F1F1F).all() and (l_bad == 0).all()
    assert (c_ok != 0xFF1F1F1F).all() and (l_ok > 0).all()   # the camera is inside the room
