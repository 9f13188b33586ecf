"""Parity metric between the CUDA renderer and the oracle.

A pixel *matches* when colour, semantic id and window depth are bit-equal
(the same triangle won it in both); for matched pixels linear depth must
agree within 1e-4 m.  At most 0.1 % of pixels may mismatch (edge ties).
The implementation targets exact equality, which the tests also report."""
import numpy as np

DEPTH_TOL_M = 1e-4
MISMATCH_FRAC = 1e-3


def compare_scene(gpu, cpu, pkg, scene):
    c_g = gpu.sceneImage(pkg.Plane.Color, scene)
    c_c = cpu.scene_image(cpu.color, scene).view(np.uint8).reshape(c_g.shape)
    s_g = gpu.sceneImage(pkg.Plane.Semantic, scene)
    s_c = cpu.scene_image(cpu.semantic, scene)
    z_g = gpu.sceneImage(pkg.Plane.Depth, scene)
    z_c = cpu.scene_image(cpu.depth, scene)
    l_g = gpu.sceneImage(pkg.Plane.LinearDepth, scene)
    l_c = cpu.scene_image(cpu.linear_depth, scene)
    same = ((c_g == c_c).all(-1) & (s_g == s_c) &
            (z_g.view(np.uint32) == z_c.view(np.uint32)))
    mismatch = int((~same).sum())
    dl = np.abs(l_g.astype(np.float64) - l_c.astype(np.float64))
    max_dl = float(dl[same].max()) if same.any() else 0.0
    exact = (mismatch == 0 and np.array_equal(l_g.view(np.uint32), l_c.view(np.uint32)))
    return dict(pixels=int(same.size), mismatch=mismatch, max_linear_err=max_dl, exact=exact)


def assert_parity(results, require_exact=True):
    total = sum(r["pixels"] for r in results)
    bad = sum(r["mismatch"] for r in results)
    worst = max(r["max_linear_err"] for r in results)
    assert bad <= MISMATCH_FRAC * total, f"{bad} of {total} pixels won by a different triangle"
    assert worst <= DEPTH_TOL_M, f"linear depth error {worst} m"
    if require_exact:
        assert all(r["exact"] for r in results), results
