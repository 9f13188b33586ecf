"""The batch renderer's golden scenarios, runnable on any renderer object.

Each scenario restates one test of habitat-sim's
``src/tests/GfxBatchRendererTest.cpp`` (cited per function): the same
files, tile layout, cameras, hierarchies and transforms.  A scenario takes a
factory ``make(tile_size, tile_count, flags)`` returning an object with the
reference call surface (``addFile``, ``updateCamera``, ``addNodeHierarchy``,
``transformations``, ``draw``, ``colorImage``, ``depthImage``, ...) -- the
CPU oracle or the CUDA renderer -- and returns a list of checks.
"""
import math
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SCENES = os.path.join(GOLDEN, "scenes")
SHOTS = os.path.join(GOLDEN, "screenshots")

WHOLE = 1
GENERATE_MIPMAP = 2
NO_TEXTURES = 1

f32 = np.float32


# ------------------------------------------------------------- matrices
def identity():
    return np.eye(4, dtype=f32)


def translation(x, y, z):
    m = identity()
    m[3, :3] = [x, y, z]
    return m


def scaling(s):
    m = identity()
    m[0, 0] = m[1, 1] = m[2, 2] = f32(s)
    return m


def mul(a, b):
    """Column-major product in float32, summed left to right."""
    out = np.empty((4, 4), f32)
    for c in range(4):
        for r in range(4):
            s = f32(a[0, r]) * f32(b[c, 0])
            for k in range(1, 4):
                s = f32(s + f32(f32(a[k, r]) * f32(b[c, k])))
            out[c, r] = s
    return out


def orthographic(size_x, size_y, near, far):
    """Magnum ``Matrix4::orthographicProjection(size, near, far)``."""
    m = np.zeros((4, 4), f32)
    m[0, 0] = f32(2.0) / f32(size_x)
    m[1, 1] = f32(2.0) / f32(size_y)
    zs = f32(2.0) / (f32(near) - f32(far))
    m[2, 2] = zs
    m[3, 2] = f32(near) * zs - f32(1.0)
    m[3, 3] = 1.0
    return m


def perspective_size(size_x, size_y, near, far):
    """Magnum ``Matrix4::perspectiveProjection(size, near, far)``."""
    m = np.zeros((4, 4), f32)
    n, fa = f32(near), f32(far)
    m[0, 0] = f32(2.0) * n / f32(size_x)
    m[1, 1] = f32(2.0) * n / f32(size_y)
    zs = f32(1.0) / (n - fa)
    m[2, 2] = (fa + n) * zs
    m[2, 3] = -1.0
    m[3, 2] = f32(2.0) * fa * n * zs
    return m


def perspective(fov_deg, aspect, near, far):
    """Magnum ``Matrix4::perspectiveProjection(fov, aspectRatio, near, far)``."""
    xy = f32(2.0) * f32(math.tan(math.radians(fov_deg) / 2.0)) * f32(near)
    return perspective_size(xy, xy / f32(aspect), near, far)


def ortho_43():
    """The tests' ``orthographicProjection(2*{4/3, 1}, 0.1, 10)``."""
    return orthographic(f32(2.0) * (f32(4.0) / f32(3.0)), 2.0, 0.1, 10.0)


def ortho_34():
    return orthographic(2.0, f32(2.0) * (f32(4.0) / f32(3.0)), 0.1, 10.0)


def camera_at_z(z):
    return translation(0.0, 0.0, -z)  # translation(zAxis(z)).inverted()


def look_at(eye, target, up):
    """Magnum ``Matrix4::lookAt(eye, target, up)``: -Z towards the target."""
    eye, target, up = (np.asarray(v, f32) for v in (eye, target, up))
    b = eye - target
    b = b / f32(np.sqrt((b * b).sum()))
    r = np.cross(up, b).astype(f32)
    r = r / f32(np.sqrt((r * r).sum()))
    u = np.cross(b, r).astype(f32)
    m = identity()
    m[0, :3], m[1, :3], m[2, :3], m[3, :3] = r, u, b, eye
    return m


def rotation_y(deg):
    """Magnum ``Matrix4::rotationY(angle)`` (float sine and cosine)."""
    a = f32(math.radians(deg))
    c, s = f32(math.cos(a)), f32(math.sin(a))
    m = identity()
    m[0, 0], m[0, 2], m[2, 0], m[2, 2] = c, -s, s, c
    return m


def rgb_hex(v, scale=1.0):
    """``0xRRGGBB_rgbf * scale``."""
    return np.array([(v >> 16) & 255, (v >> 8) & 255, v & 255], f32) / f32(255.0) * f32(scale)


# ---------------------------------------------------------------- data
# (name, [(file, flags, name)], singleSceneBatchCount, multipleScenesBatchCount,
#  maxThreshold, meanThreshold) -- GfxBatchRendererTest.cpp:100-165
FILE_DATA = [
    ("", [("batch.gltf", 0, None)], 1, [1, 1, 0, 1], 0.0, 0.0),
    ("generate mipmap", [("batch.gltf", GENERATE_MIPMAP, None)], 1, [1, 1, 0, 1], 0.0, 0.0),
    ("multiple meshes", [("batch-multiple-meshes.gltf", 0, None)], 3, [4, 2, 0, 1], 0.0, 0.0),
    ("multiple textures", [("batch-multiple-textures.gltf", 0, None)], 3, [4, 2, 0, 1], 0.0, 0.0),
    ("multiple textures, generate mipmap",
     [("batch-multiple-textures.gltf", GENERATE_MIPMAP, None)], 3, [4, 2, 0, 1], 0.0, 0.0),
    ("multiple files", [("batch-square-circle-triangle.gltf", 0, None),
                        ("batch-four-squares.gltf", 0, None)], 2, [4, 2, 0, 1], 0.0, 0.0),
    ("multiple files, compressed textures",
     [("batch-square-circle-triangle-compressed.gltf", 0, None),
      ("batch-four-squares-compressed.gltf", 0, None)], 2, [4, 2, 0, 1], 1.5, 0.5),
    ("multiple files, compressed textures, generate mipmap",
     [("batch-square-circle-triangle-compressed.gltf", GENERATE_MIPMAP, None),
      ("batch-four-squares-compressed.gltf", GENERATE_MIPMAP, None)], 2, [4, 2, 0, 1], 1.5, 0.5),
    ("multiple files, some whole-file",
     [("batch-square-circle-triangle.gltf", 0, None),
      ("batch-four-squares-deep-hierarchy-whole-file.gltf", WHOLE, "four squares")],
     2, [4, 2, 0, 1], 0.0, 0.0),
]

# (name, files, renderer flags, nodeCount, drawCount, batchCount, textureMultiplier,
#  golden) -- GfxBatchRendererTest.cpp:167-220
MESH_HIERARCHY_DATA = [
    ("", [("batch.gltf", 0, None)], 0, 5, 4, 1, 0xcc / 255.0,
     "GfxBatchRendererTestMeshHierarchy.png"),
    ("multiple meshes", [("batch-multiple-meshes.gltf", 0, None)], 0, 5, 4, 4, 0xcc / 255.0,
     "GfxBatchRendererTestMeshHierarchy.png"),
    ("multiple textures", [("batch-multiple-textures.gltf", 0, None)], 0, 5, 4, 4, 0xcc / 255.0,
     "GfxBatchRendererTestMeshHierarchy.png"),
    ("multiple files", [("batch-square-circle-triangle.gltf", 0, None),
                        ("batch-four-squares.gltf", 0, None)], 0, 5, 4, 4, 0xcc / 255.0,
     "GfxBatchRendererTestMeshHierarchy.png"),
    ("multiple files with deep hierarchy as a whole",
     [("batch-square-circle-triangle.gltf", WHOLE, None),
      ("batch-four-squares-deep-hierarchy-whole-file.gltf", WHOLE, "four squares")],
     0, 5, 4, 4, 0xcc / 255.0, "GfxBatchRendererTestMeshHierarchy.png"),
    ("multiple files, no materials", [("batch-square-circle-triangle.gltf", 0, None),
                                      ("batch-four-squares-no-materials.gltf", 0, None)],
     0, 5, 4, 4, 1.0, "GfxBatchRendererTestMeshHierarchyNoTextures.png"),
    ("no textures", [("batch.gltf", 0, None)], NO_TEXTURES, 5, 4, 1, 1.0,
     "GfxBatchRendererTestMeshHierarchyNoTextures.png"),
    ("multiple meshes, no textures", [("batch-multiple-meshes.gltf", 0, None)], NO_TEXTURES,
     5, 4, 4, 1.0, "GfxBatchRendererTestMeshHierarchyNoTextures.png"),
    ("multiple files, scene-less, as a whole",
     [("batch-square-circle-triangle.gltf", WHOLE, None),
      ("batch-four-squares-no-scene.gltf", WHOLE, "four squares")],
     0, 2, 1, 1, 1.0, "GfxBatchRendererTestMeshHierarchyNoTextures.png"),
]


def load_png(name):
    from oracle.gltf import decode_png
    with open(os.path.join(SHOTS, name), "rb") as f:
        return decode_png(f.read())


def add_files(r, files):
    for (fname, fflags, nm) in files:
        assert r.addFile(os.path.join(SCENES, fname), fflags, nm)


class Check:
    """One assertion a scenario wants made on a renderer's output."""

    def __init__(self, kind, **kw):
        self.kind = kind
        self.__dict__.update(kw)


# ------------------------------------------------------------ scenarios
def defaults(make, data):
    """GfxBatchRendererTest::defaults (:1460-1522)."""
    name, files, *_ = data
    r = make((48, 32), (2, 3), 0)
    checks = [Check("eq", what="sceneCount", got=r.sceneCount(), want=6)]
    for i in range(6):
        st = r.sceneStats(i)
        checks.append(Check("eq", what=f"stats{i}", got=(st.nodeCount, st.drawCount,
                                                         st.drawBatchCount), want=(0, 0, 0)))
        checks.append(Check("eq", what=f"camera{i}", got=np.asarray(r.camera(i)).tolist(),
                            want=identity().tolist()))
    add_files(r, files)
    r.draw()
    color = r.colorImage()
    depth = r.depthImage()
    checks.append(Check("image", image=color, golden="GfxBatchRendererTestDefaults.png",
                        max=0.0, mean=0.0))
    checks.append(Check("eq", what="px", got=color[48, 48].tolist(), want=[31, 31, 31, 255]))
    checks.append(Check("eq", what="depth", got=float(depth[48, 48]), want=1.0))
    return checks


def single_mesh(make, data):
    """GfxBatchRendererTest::singleMesh (:1524-1600)."""
    name, files, _, _, mx, mean = data
    r = make((128, 96), (1, 1), 0)
    add_files(r, files)
    r.updateCamera(0, ortho_43(), camera_at_z(1.0))
    checks = [Check("eq", what="has square", got=r.hasNodeHierarchy("square"), want=True),
              Check("eq", what="has squares", got=r.hasNodeHierarchy("squares"), want=False),
              Check("eq", what="has ''", got=r.hasNodeHierarchy(""), want=False)]
    checks.append(Check("eq", what="id", got=r.addNodeHierarchy(0, "square", scaling(0.4)),
                        want=0))
    st = r.sceneStats(0)
    checks.append(Check("eq", what="stats", got=(st.nodeCount, st.drawCount, st.drawBatchCount),
                        want=(2, 1, 1)))
    checks.append(Check("eq", what="t0", got=np.asarray(r.transformations(0)[0]).tolist(),
                        want=identity().tolist()))
    r.transformations(0)[0] = scaling(2.0)
    r.draw()
    color = r.colorImage()
    depth = r.depthImage()
    checks.append(Check("image", image=color, golden="GfxBatchRendererTestSingleMesh.png",
                        max=mx, mean=mean))
    if mx == 0.0:
        checks.append(Check("eq", what="[75][35]", got=color[75, 35, :3].tolist(),
                            want=[0xcc, 0xcc, 0xcc]))
        checks.append(Check("eq", what="[20][38]", got=color[20, 38, :3].tolist(),
                            want=[0x99, 0, 0]))
    checks.append(Check("close", what="d[0][0]", got=float(depth[0, 0]), want=1.0, tol=1e-6))
    checks.append(Check("close", what="d[95][127]", got=float(depth[95, 127]), want=1.0,
                        tol=1e-6))
    checks.append(Check("close", what="d[64][48]", got=float(depth[64, 48]), want=0.0909091,
                        tol=1e-6))
    return checks


def mesh_hierarchy(make, data):
    """GfxBatchRendererTest::meshHierarchy (:1602-1660)."""
    name, files, rflags, nodes, draws, batches, mult, golden = data
    r = make((128, 96), (1, 1), rflags)
    add_files(r, files)
    r.updateCamera(0, ortho_43(), camera_at_z(1.0))
    checks = [Check("eq", what="id", got=r.addNodeHierarchy(0, "four squares"), want=0)]
    st = r.sceneStats(0)
    checks.append(Check("eq", what="stats", got=(st.nodeCount, st.drawCount, st.drawBatchCount),
                        want=(nodes, draws, batches)))
    checks.append(Check("eq", what="len", got=len(r.transformations(0)), want=nodes))
    r.transformations(0)[0] = scaling(0.8)
    r.draw()
    color = r.colorImage()
    checks.append(Check("image", image=color, golden=golden, max=0.0, mean=0.0))
    # Color3ub * float, truncated back to bytes (GfxBatchRendererTest.cpp:1654-1659)
    want = lambda rgb: [int(np.float32(v / 255.0) * np.float32(mult) * 255.0 + 0.5) for v in rgb]
    checks.append(Check("eq", what="[29][87]", got=color[29, 87, :3].tolist(),
                        want=want([0, 255, 255])))
    checks.append(Check("eq", what="[68][50]", got=color[68, 50, :3].tolist(),
                        want=want([255, 0, 255])))
    checks.append(Check("eq", what="[67][78]", got=color[67, 78, :3].tolist(),
                        want=want([255, 255, 0])))
    return checks


def multiple_meshes(make, data):
    """GfxBatchRendererTest::multipleMeshes (:1662-1722)."""
    name, files, single_batches, _, mx, mean = data
    r = make((128, 96), (1, 1), 0)
    add_files(r, files)
    r.updateCamera(0, ortho_43(), camera_at_z(1.0))
    checks = [Check("eq", what="square", got=r.addNodeHierarchy(0, "square"), want=0)]
    r.transformations(0)[0] = mul(translation(0.0, 0.5, 0.0), scaling(0.4))
    checks.append(Check("eq", what="circle", got=r.addNodeHierarchy(0, "circle"), want=2))
    r.transformations(0)[2] = mul(translation(-0.5, -0.5, 0.0), scaling(0.4))
    checks.append(Check("eq", what="triangle", got=r.addNodeHierarchy(0, "triangle"), want=4))
    r.transformations(0)[4] = mul(translation(0.5, -0.5, 0.0), scaling(0.4))
    st = r.sceneStats(0)
    checks.append(Check("eq", what="stats", got=(st.nodeCount, st.drawCount, st.drawBatchCount),
                        want=(6, 3, single_batches)))
    r.draw()
    color = r.colorImage()
    checks.append(Check("image", image=color, golden="GfxBatchRendererTestMultipleMeshes.png",
                        max=mx, mean=mean))
    checks.append(Check("eq", what="[18][44]", got=color[18, 44, :3].tolist(),
                        want=[0, 0xcc, 0xcc]))
    checks.append(Check("eq", what="[24][88]", got=color[24, 88, :3].tolist(),
                        want=[0xcc, 0, 0xcc]))
    return checks


def _multiple_scenes_setup(r, checks, batch_counts):
    checks.append(Check("eq", what="s0", got=r.addNodeHierarchy(0, "four squares"), want=0))
    checks.append(Check("eq", what="s1a", got=r.addNodeHierarchy(1, "circle"), want=0))
    checks.append(Check("eq", what="s1b", got=r.addNodeHierarchy(1, "square"), want=2))
    checks.append(Check("eq", what="s3", got=r.addNodeHierarchy(3, "triangle"), want=0))
    want_stats = [(5, 4), (4, 2), (0, 0), (2, 1)]
    for i in range(4):
        st = r.sceneStats(i)
        checks.append(Check("eq", what=f"stats{i}",
                            got=(st.nodeCount, st.drawCount, st.drawBatchCount),
                            want=want_stats[i] + (batch_counts[i],)))


def multiple_scenes(make, data):
    """GfxBatchRendererTest::multipleScenes (:1737-1813)."""
    name, files, _, batch_counts, mx, mean = data
    r = make((64, 48), (2, 2), 0)
    add_files(r, files)
    r.updateCamera(0, ortho_34(), camera_at_z(1.0))
    checks = []
    _multiple_scenes_setup(r, checks, batch_counts)
    ident = identity()
    r.updateCamera(0, ident, translation(0.0, 0.0, 1.0 * -1))
    r.transformations(0)[0] = translation(0.0, 0.0, 0.0)
    r.updateCamera(1, ident, translation(-0.0, -0.5, -1.0))
    r.transformations(1)[0] = mul(translation(0.5, 0.0, 0.0), scaling(0.5))
    r.transformations(1)[2] = mul(translation(-0.5, 1.0, 0.0), scaling(0.5))
    r.updateCamera(3, ident, translation(-0.0, 0.5, -1.0))
    r.transformations(3)[0] = mul(translation(0.5, 0.0, 0.0), scaling(0.5))
    r.draw()
    checks.append(Check("image", image=r.colorImage(),
                        golden="GfxBatchRendererTestMultipleScenes.png", max=mx, mean=mean))
    return checks


def clear_scene(make, data):
    """GfxBatchRendererTest::clearScene (:1815-1906)."""
    name, files, _, batch_counts, mx, mean = data
    r = make((64, 48), (2, 2), 0)
    add_files(r, files)
    r.updateCamera(0, ortho_34(), camera_at_z(1.0))
    checks = []
    checks.append(Check("eq", what="a", got=r.addNodeHierarchy(3, "triangle"), want=0))
    checks.append(Check("eq", what="b", got=r.addNodeHierarchy(1, "square"), want=0))
    checks.append(Check("eq", what="c", got=r.addNodeHierarchy(1, "circle"), want=2))
    checks.append(Check("eq", what="d", got=r.addNodeHierarchy(1, "triangle"), want=4))
    checks.append(Check("eq", what="e", got=r.addNodeHierarchy(0, "four squares"), want=0))
    ident = identity()
    r.updateCamera(0, ident, translation(0.0, 0.0, -1.0))
    r.transformations(0)[0] = translation(0.0, 0.0, 0.0)
    r.updateCamera(1, ident, translation(-0.0, -0.5, -1.0))
    r.updateCamera(3, ident, translation(-0.0, 0.5, -1.0))
    r.transformations(3)[0] = mul(translation(0.5, 0.0, 0.0), scaling(0.5))
    r.clear(1)
    st = r.sceneStats(1)
    checks.append(Check("eq", what="cleared", got=(st.nodeCount, st.drawCount), want=(0, 0)))
    r.draw()
    checks.append(Check("image", image=r.colorImage(),
                        golden="GfxBatchRendererTestMultipleScenesClearScene1.png",
                        max=mx, mean=mean))
    checks.append(Check("eq", what="f", got=r.addNodeHierarchy(1, "circle"), want=0))
    checks.append(Check("eq", what="g", got=r.addNodeHierarchy(1, "square"), want=2))
    r.transformations(1)[0] = mul(translation(0.5, 0.0, 0.0), scaling(0.5))
    r.transformations(1)[2] = mul(translation(-0.5, 1.0, 0.0), scaling(0.5))
    r.draw()
    checks.append(Check("image", image=r.colorImage(),
                        golden="GfxBatchRendererTestMultipleScenes.png", max=mx, mean=mean))
    return checks


def depth_unprojection(make, unproject):
    """GfxBatchRendererTest::depthUnprojection (:2175-2246)."""
    r = make((64, 64), (2, 2), 0)
    add_files(r, [("batch.gltf", 0, None)])
    proj = perspective(60.0, 1.0, 0.001, 10.0)
    for s, z in enumerate([2.5, 5.0, 7.5, 20.0]):
        r.updateCamera(s, proj, camera_at_z(z))
    checks = [Check("eq", what="has", got=r.hasNodeHierarchy("square"), want=True)]
    for i in range(4):
        checks.append(Check("eq", what=f"add{i}", got=r.addNodeHierarchy(i, "square"), want=0))
    r.draw()
    depth = np.array(r.depthImage(), np.float32, copy=True)
    for y in range(2):
        for x in range(2):
            s = y * 2 + x
            tile = np.ascontiguousarray(depth[y * 64:(y + 1) * 64, x * 64:(x + 1) * 64])
            unproject(r.cameraDepthUnprojection(s), tile)
            depth[y * 64:(y + 1) * 64, x * 64:(x + 1) * 64] = tile
    checks.append(Check("close", what="2.5", got=float(depth[32, 32]), want=2.5, tol=0.01))
    checks.append(Check("close", what="5.0", got=float(depth[32, 96]), want=5.0, tol=0.01))
    checks.append(Check("close", what="7.5", got=float(depth[96, 32]), want=7.5, tol=0.01))
    checks.append(Check("eq", what="far", got=float(depth[96, 96]), want=0.0))
    return checks


# DepthUnprojectionTest.cpp:46-67: (name, depth, expected, fov, near, far)
UNPROJECT_DATA = [
    ("z=4, near=0.01, far=100", 4.0, 4.0, 0.01, 100.0),
    ("z=4, near=1.0, far=100", 4.0, 4.0, 1.0, 100.0),
    ("z=4, near=0.01, far=10", 4.0, 4.0, 0.01, 10.0),
    ("z=0.015, near=0.015, far=100", 0.015, 0.015, 0.01, 100.0),
    ("z=10, near=0.01, far=100", 10.0, 10.0, 0.01, 100.0),
    ("z=95, near=0.01, far=100", 95.0, 95.0, 0.01, 100.0),
    ("z=near", 0.01, 0.01, 0.01, 100.0),
    ("z=far", 100.0, 0.0, 0.01, 100.0),
]


LIGHT_DATA = [
    # name, max lights, scene lights, rotation, three objects, golden
    ("no lights enabled", 0, 0, 0.0, "flat checkerboard sphere", "shaded yellow sphere",
     "shaded checkerboard sphere", "GfxBatchRendererTestLightsDisabled.png"),
    ("no lights added", 2, 0, 0.0, "flat checkerboard sphere", "shaded yellow sphere",
     "shaded checkerboard sphere", "GfxBatchRendererTestLightsNone.png"),
    ("two lights", 2, 2, 0.0, "flat checkerboard sphere", "shaded yellow sphere",
     "shaded checkerboard sphere", "GfxBatchRendererTestLights.png"),
    ("two lights, rotated", 2, 2, 180.0, "flat checkerboard sphere", "shaded yellow sphere",
     "shaded checkerboard sphere", "GfxBatchRendererTestLights.png"),
    ("four lights used but two max", 2, 4, 0.0, "flat checkerboard sphere",
     "shaded yellow sphere", "shaded checkerboard sphere", "GfxBatchRendererTestLights.png"),
    ("two lights used but four max", 4, 2, 0.0, "flat checkerboard sphere",
     "shaded yellow sphere", "shaded checkerboard sphere", "GfxBatchRendererTestLights.png"),
    ("two lights but everything flat-shaded", 2, 2, 0.0, "flat checkerboard sphere",
     "flat yellow sphere", "flat checkerboard sphere", "GfxBatchRendererTestLightsDisabled.png"),
]

DIRECTIONAL, POINT = 0, 1


def _light_scene(r, objects, up):
    checks = []
    for want, obj in zip((0, 2, 4), objects):
        checks.append(Check("eq", what=f"node {obj}", got=r.addNodeHierarchy(0, obj), want=want))
    t = r.transformations(0)
    t[0] = translation(-1.5, -1.0, 0.0)
    t[2] = translation(0.0, 1.0, 0.0)
    t[4] = translation(1.5, -1.0, 0.0)
    return checks


def _add_lights(r, count, up):
    checks = [Check("eq", what="empty node 6", got=r.addEmptyNode(0), want=6),
              Check("eq", what="empty node 7", got=r.addEmptyNode(0), want=7)]
    t = r.transformations(0)
    t[6] = translation(-1.0, 1.5, 1.0)
    t[7] = look_at([0, 0, 0], [3, 1, 3], up)
    for i in range(count):
        checks.append(Check("eq", what=f"light {i}",
                            got=r.addLight(0, 6 + i % 2, DIRECTIONAL if i % 2 else POINT), want=i))
        r.lightColors(0)[i] = rgb_hex(0xccffff, 1.0) if i % 2 else rgb_hex(0x3333ff, 3.0)
        r.lightRanges(0)[i] = np.inf if i % 2 else 1.0
    return checks


def lights(make_lit, data):
    """GfxBatchRendererTest::lights (:1908-1993)."""
    name, max_lights, count, rot, a, b, c, golden = data
    r = make_lit((128, 96), (1, 1), 0, max_lights)
    add_files(r, [("batch.gltf", 0, None)])
    r.updateCamera(0, perspective(60.0, f32(4.0) / f32(3.0), 0.1, 10.0), camera_at_z(5.0))
    checks = _light_scene(r, (a, b, c), None)
    if count:
        checks += _add_lights(r, count, [1, 0, 0])
    st = r.sceneStats(0)
    checks.append(Check("eq", what="stats", got=(st.nodeCount, st.drawCount, st.drawBatchCount),
                        want=(8 if count else 6, 3, 2)))
    r.draw()
    checks.append(Check("image", image=r.colorImage().copy(), golden=golden, max=0.75, mean=0.005))
    t = r.transformations(0)
    for n in (0, 2, 4):
        t[n] = mul(t[n], rotation_y(rot))
    r.draw()
    checks.append(Check("image", image=r.colorImage().copy(), golden=golden, max=95.0, mean=0.07))
    return checks


def clear_lights(make_lit, data=None):
    """GfxBatchRendererTest::clearLights (:1995-2117)."""
    objects = ("flat checkerboard sphere", "shaded yellow sphere", "shaded checkerboard sphere")
    r = make_lit((128, 96), (1, 1), 0, 2)
    add_files(r, [("batch.gltf", 0, None)])
    r.updateCamera(0, perspective(60.0, f32(4.0) / f32(3.0), 0.1, 10.0), camera_at_z(5.0))
    checks = _light_scene(r, objects, None) + _add_lights(r, 2, [0, 1, 0])
    r.draw()
    checks.append(Check("image", image=r.colorImage().copy(),
                        golden="GfxBatchRendererTestLights.png", max=0.75, mean=0.005))
    checks.append(Check("eq", what="nodes", got=len(r.transformations(0)), want=8))
    checks.append(Check("eq", what="lights", got=len(r.lightColors(0)), want=2))
    r.clearLights(0)
    checks.append(Check("eq", what="nodes after clearLights", got=len(r.transformations(0)),
                        want=8))
    checks.append(Check("eq", what="lights after clearLights", got=len(r.lightColors(0)), want=0))
    r.draw()
    checks.append(Check("image", image=r.colorImage().copy(),
                        golden="GfxBatchRendererTestLightsNone.png", max=0.75, mean=0.005))
    r.addLight(0, 6, POINT)
    r.addLight(0, 7, DIRECTIONAL)
    checks.append(Check("eq", what="lights re-added", got=len(r.lightColors(0)), want=2))
    r.clear(0)
    checks.append(Check("eq", what="nodes after clear", got=len(r.transformations(0)), want=0))
    checks.append(Check("eq", what="lights after clear", got=len(r.lightColors(0)), want=0))
    checks += _light_scene(r, objects, None) + _add_lights(r, 2, [1, 0, 0])
    r.draw()
    checks.append(Check("image", image=r.colorImage().copy(),
                        golden="GfxBatchRendererTestLights.png", max=0.75, mean=0.005))
    return checks


def image_delta(image, golden):
    """Magnum's image-comparison delta: per pixel the mean of the absolute
    channel differences; returns (max over pixels, mean over pixels)."""
    d = np.abs(image.astype(np.float64) - golden.astype(np.float64)).mean(axis=-1)
    return float(d.max()), float(d.mean())


def evaluate(checks):
    """Return a list of failure strings."""
    fails = []
    for c in checks:
        if c.kind == "eq":
            if c.got != c.want:
                fails.append(f"{c.what}: got {c.got}, want {c.want}")
        elif c.kind == "close":
            if not abs(c.got - c.want) <= c.tol:
                fails.append(f"{c.what}: got {c.got}, want {c.want} +- {c.tol}")
        elif c.kind == "image":
            gold = load_png(c.golden)
            if c.image.shape != gold.shape:
                fails.append(f"{c.golden}: shape {c.image.shape} vs {gold.shape}")
                continue
            mx, mean = image_delta(c.image, gold)
            if mx > c.max or mean > c.mean:
                n = int((np.abs(c.image.astype(int) - gold.astype(int)).max(-1) > 0).sum())
                fails.append(f"{c.golden}: max {mx} mean {mean:.4f} ({n} px differ) "
                             f"> {c.max}/{c.mean}")
    return fails


ALL = ([("defaults", defaults, d) for d in FILE_DATA] +
       [("singleMesh", single_mesh, d) for d in FILE_DATA] +
       [("meshHierarchy", mesh_hierarchy, d) for d in MESH_HIERARCHY_DATA] +
       [("multipleMeshes", multiple_meshes, d) for d in FILE_DATA] +
       [("multipleScenes", multiple_scenes, d) for d in FILE_DATA] +
       [("clearScene", clear_scene, d) for d in FILE_DATA])


def ids():
    return [f"{n}[{d[0] or 'default'}]" for (n, _, d) in ALL]


LIT = ([("lights", lights, d) for d in LIGHT_DATA] + [("clearLights", clear_lights, None)])


def lit_ids():
    return [n if d is None else f"{n}[{d[0]}]" for (n, _, d) in LIT]
