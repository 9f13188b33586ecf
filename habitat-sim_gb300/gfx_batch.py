"""Python mirror of habitat-sim's ``esp::gfx_batch`` batch renderer API.

Same names, argument meaning and error behaviour as the C++ classes in
``src/esp/gfx_batch/Renderer.h`` / ``RendererStandalone.h`` (the reference
binds them to Python only through its replay renderer,
``src/esp/bindings/SimBindings.cpp:467-545``).  Calls go through the C ABI
of ``libgbr.so``; framebuffer planes can be handed out as CUDA torch
tensors through DLPack without a copy.

Conventions: matrices are numpy float32 ``[4, 4]`` arrays indexed
``[column, row]`` (Magnum's column-major ``Matrix4``); images have row 0 at
the bottom (GL window origin).  Out-of-range ids raise ``GbrError`` (the
reference asserts, or raises in Python through ``ESP_CHECK``);
``addFile`` returns ``False`` and prints a message like the reference
(``Renderer.cpp:405-427``).
"""
import ctypes
import enum
import sys

import numpy as np

from . import _lib
from ._lib import GbrError, check


class RendererFlags(enum.IntFlag):
    """``RendererFlag`` (Renderer.h:21-30)."""
    NoTextures = 1


class RendererFileFlags(enum.IntFlag):
    """``RendererFileFlag`` (Renderer.h:120-154)."""
    Whole = 1
    GenerateMipmap = 2


class RendererStandaloneFlags(enum.IntFlag):
    """``RendererStandaloneFlag`` (RendererStandalone.h:21-36), plus
    ``DoubleBuffer``: two sets of output planes, alternated by the draws, so
    that an asynchronous readback of one draw overlaps the next draw."""
    QuietLog = 1
    DoubleBuffer = 2


class Plane(enum.IntFlag):
    Color = 1
    Depth = 2
    LinearDepth = 4
    Semantic = 8
    All = 15


class RendererLightType(enum.IntEnum):
    """``RendererLightType`` (Renderer.h:170-173)."""
    Directional = 0
    Point = 1


class DrawMode(enum.IntEnum):
    PerScene = 0
    Batched = 1


def _f32(m, shape=None):
    a = np.ascontiguousarray(m, dtype=np.float32)
    if shape is not None:
        a = a.reshape(shape)
    return a


def _fptr(a):
    return a.ctypes.data_as(_lib.c_float_p)


class RendererConfiguration:
    """``RendererConfiguration`` (Renderer.h:45-113, Renderer.cpp:58-92) plus
    per-scene viewports, output planes and the default draw mode."""

    def __init__(self):
        self.flags = RendererFlags(0)
        self.tile_size = (128, 128)
        self.tile_count = (1, 1)
        self.max_light_count = 0
        self.ambient_factor = 0.1
        self.viewports = None
        self.planes = Plane.All
        self.draw_mode = DrawMode.PerScene

    def setFlags(self, flags):
        self.flags = RendererFlags(flags)
        return self

    def setTileSizeCount(self, tile_size, tile_count):
        self.tile_size = (int(tile_size[0]), int(tile_size[1]))
        self.tile_count = (int(tile_count[0]), int(tile_count[1]))
        return self

    def setMaxLightCount(self, count):
        self.max_light_count = int(count)
        return self

    def setAmbientFactor(self, factor):
        self.ambient_factor = float(factor)
        return self

    def setViewports(self, viewports):
        """One (width, height) per scene: a ragged framebuffer instead of the
        tile grid, for batches whose scenes differ in resolution."""
        self.viewports = [(int(w), int(h)) for (w, h) in viewports]
        return self

    def setPlanes(self, planes):
        self.planes = Plane(planes)
        return self

    def setDrawMode(self, mode):
        self.draw_mode = DrawMode(mode)
        return self


class RendererStandaloneConfiguration:
    """``RendererStandaloneConfiguration`` (RendererStandalone.h:47-100)."""

    def __init__(self):
        self.cuda_device = 0
        self.flags = RendererStandaloneFlags(0)

    def setCudaDevice(self, device):
        self.cuda_device = int(device)
        return self

    def setFlags(self, flags):
        self.flags = RendererStandaloneFlags(flags)
        return self


class HbaoType(enum.IntEnum):
    """``HbaoType`` (src/esp/gfx_batch/Hbao.h:135)."""
    Classic = 0
    CacheAware = 1


class HbaoConfiguration:
    """``HbaoConfiguration`` (src/esp/gfx_batch/Hbao.h:30-141): intensity,
    bias, radius (metres), blur sharpness, NoBlur, UseAoSpecialBlur; and the
    algorithm ``drawEffect`` takes (``HbaoType``)."""

    def __init__(self):
        self.intensity = 0.732
        self.bias = 0.05
        self.radius = 1.84
        self.blur_sharpness = 10.0
        self.no_blur = False
        self.special_blur = False
        self.algorithm = HbaoType.Classic

    def setAlgorithm(self, algorithm):
        self.algorithm = HbaoType(algorithm)
        return self

    def setNoBlur(self, state):
        self.no_blur = bool(state)
        if state:
            self.special_blur = False
        return self

    def setUseSpecialBlur(self, state):
        self.special_blur = bool(state)
        if state:
            self.no_blur = False
        return self

    def setIntensity(self, v):
        self.intensity = float(v)
        return self

    def setBias(self, v):
        self.bias = float(v)
        return self

    def setRadius(self, v):
        self.radius = float(v)
        return self

    def setBlurSharpness(self, v):
        self.blur_sharpness = float(v)
        return self

    def scaleIntensity(self, m):
        self.intensity *= m
        return self

    def scaleBias(self, m):
        self.bias *= m
        return self

    def scaleRadius(self, m):
        self.radius *= m
        return self

    def scaleBlurSharpness(self, m):
        self.blur_sharpness *= m
        return self

    def _c(self):
        c = _lib.HbaoConfig()
        c.intensity, c.bias, c.radius = self.intensity, self.bias, self.radius
        c.blur_sharpness = self.blur_sharpness
        c.no_blur, c.special_blur = int(self.no_blur), int(self.special_blur)
        c.algorithm = int(self.algorithm)
        return c


def hbaoApply(configuration, projection, linear_depth, color, stream=None):
    """HBAO on one caller image: ``linear_depth`` float32 [h, w] and ``color``
    uint8 [h, w, 4] CUDA torch tensors (rows contiguous; colour modified in place)."""
    lib = _lib.load()
    p = _f32(projection, (4, 4))
    h, w = linear_depth.shape
    if tuple(color.shape[:2]) != (h, w) or color.stride(0) != 4 * linear_depth.stride(0):
        raise ValueError("colour and depth must have the same size and row pitch")
    c = (configuration or HbaoConfiguration())._c()
    check(lib.gbr_hbao_apply(ctypes.byref(c), _fptr(p), linear_depth.data_ptr(), color.data_ptr(),
                             w, h, linear_depth.stride(0), _stream_handle(stream)))


class SceneStats:
    """``SceneStats`` (Renderer.h:745-779)."""

    def __init__(self, node_count, draw_count, draw_batch_count):
        self.nodeCount = node_count
        self.drawCount = draw_count
        self.drawBatchCount = draw_batch_count

    def __repr__(self):
        return (f"SceneStats(nodeCount={self.nodeCount}, drawCount={self.drawCount}, "
                f"drawBatchCount={self.drawBatchCount})")


def _stream_handle(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream or None
    handle = getattr(stream, "cuda_stream", None)
    if handle is not None:
        return handle or None
    raise TypeError("stream must be an int handle or a torch.cuda.Stream")


class RendererStandalone:
    """``RendererStandalone`` with its ``Renderer`` base, on the GPU."""

    def __init__(self, configuration=None, standalone_configuration=None):
        configuration = configuration or RendererConfiguration()
        standalone_configuration = standalone_configuration or RendererStandaloneConfiguration()
        self._lib = _lib.load()
        cfg = _lib.Config()
        self._lib.gbr_config_init(ctypes.byref(cfg))
        cfg.flags = int(configuration.flags)
        cfg.tile_size[0], cfg.tile_size[1] = configuration.tile_size
        cfg.tile_count[0], cfg.tile_count[1] = configuration.tile_count
        cfg.max_light_count = configuration.max_light_count
        cfg.ambient_factor = configuration.ambient_factor
        cfg.cuda_device = standalone_configuration.cuda_device
        cfg.standalone_flags = int(standalone_configuration.flags)
        cfg.planes = int(configuration.planes)
        cfg.draw_mode = int(configuration.draw_mode)
        self._viewports = None
        if configuration.viewports:
            vp = np.ascontiguousarray(np.array(configuration.viewports, np.int32).reshape(-1))
            self._viewports = vp
            cfg.scene_count = len(configuration.viewports)
            cfg.viewports = vp.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        handle = ctypes.c_void_p()
        check(self._lib.gbr_create(ctypes.byref(cfg), ctypes.byref(handle)))
        self._h = handle
        self._config = configuration
        self._standalone = standalone_configuration
        self._quiet = bool(standalone_configuration.flags & RendererStandaloneFlags.QuietLog)
        size = (ctypes.c_int64 * 2)()
        check(self._lib.gbr_framebuffer_size(self._h, size))
        self._fb = (int(size[0]), int(size[1]))

    @classmethod
    def _borrow(cls, handle, configuration, standalone_configuration, owner):
        """A view of a renderer that `owner` (a replay renderer) created and
        destroys: valid while the owner is open; close() only drops the view."""
        self = cls.__new__(cls)
        self._lib = _lib.load()
        self._h = ctypes.c_void_p(handle)
        self._owner = owner
        self._config = configuration
        self._standalone = standalone_configuration
        self._quiet = bool(standalone_configuration.flags & RendererStandaloneFlags.QuietLog)
        self._viewports = None
        size = (ctypes.c_int64 * 2)()
        check(self._lib.gbr_framebuffer_size(self._h, size))
        self._fb = (int(size[0]), int(size[1]))
        return self

    def close(self):
        if getattr(self, "_owner", None) is not None:
            self._h = None
            return
        if getattr(self, "_h", None):
            self._lib.gbr_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ----------------------------------------------------------- queries
    def flags(self):
        return self._config.flags

    def standaloneFlags(self):
        return self._standalone.flags

    def tileSize(self):
        return self._config.tile_size

    def tileCount(self):
        return self._config.tile_count

    def sceneCount(self):
        n = ctypes.c_uint32()
        check(self._lib.gbr_scene_count(self._h, ctypes.byref(n)))
        return n.value

    def maxLightCount(self):
        return self._config.max_light_count

    def framebufferSize(self):
        """(width, height) of the tile-grid framebuffer, or (pixels, 1) for
        the ragged layout."""
        return self._fb

    def sceneViewport(self, scene):
        """(offset, pitch, width, height) of a scene inside each plane."""
        out = (ctypes.c_int64 * 4)()
        check(self._lib.gbr_scene_viewport(self._h, scene, out))
        return tuple(int(v) for v in out)

    def sceneViewports(self):
        """Every scene's (offset, pitch, width, height) as an int64 array
        [sceneCount, 4]; the layout is fixed at creation, so it is read once."""
        if getattr(self, "_scene_layout", None) is None:
            v = np.array([self.sceneViewport(i) for i in range(self.sceneCount())], np.int64)
            self._scene_layout = v.reshape(-1, 4)
        return self._scene_layout

    # ------------------------------------------------------------- files
    def addFile(self, filename, flags=0, name=None):
        st = self._lib.gbr_add_file(self._h, str(filename).encode(), int(flags),
                                    None if name is None else name.encode())
        if st != 0:
            if not self._quiet:
                print(self._lib.gbr_last_error().decode(errors="replace"), file=sys.stderr)
            return False
        return True

    # -------------------------------------------------------- procedural
    def addMesh(self, positions, colors=None, texcoords=None, objectIds=None, indices=None,
                normals=None):
        pos = _f32(positions, (-1, 3))
        n = len(pos)
        col = None if colors is None else _f32(colors, (n, 4))
        uv = None if texcoords is None else _f32(texcoords, (n, 2))
        ids = None if objectIds is None else np.ascontiguousarray(objectIds, np.uint32).reshape(n)
        nrm = None if normals is None else _f32(normals, (n, 3))
        idx = np.ascontiguousarray(indices, np.uint32).reshape(-1)
        md = _lib.MeshData(n, pos.ctypes.data, None if col is None else col.ctypes.data,
                           None if uv is None else uv.ctypes.data,
                           None if ids is None else ids.ctypes.data, len(idx), idx.ctypes.data,
                           None if nrm is None else nrm.ctypes.data)
        out = ctypes.c_uint32()
        check(self._lib.gbr_add_mesh(self._h, ctypes.byref(md), ctypes.byref(out)))
        return out.value

    def addTexture(self, pixels, filter=1, wrapS=0, wrapT=0, minFilter=0, mipFilter=0, levels=None,
                   generateMipmap=False):
        """pixels: uint8 [layers, h, w, 4] or [h, w, 4], row 0 = bottom -- or,
        with ``levels``, a list of such arrays, level 0 first (level k is
        max(1, w >> k) x max(1, h >> k)).  ``filter`` is the magnification
        filter (0 nearest, 1 bilinear); ``minFilter`` 0 = as ``filter``,
        1 nearest, 2 linear; ``mipFilter`` 0 base level only, 1 nearest
        level, 2 linear between levels; ``generateMipmap`` derives the chain
        from a single level."""
        if levels is not None:
            chain = [np.ascontiguousarray(l, np.uint8) for l in pixels]
            chain = [c[None] if c.ndim == 3 else c for c in chain]
            p = chain[0]
            data = np.concatenate([c.reshape(-1) for c in chain])
            nlev = len(chain)
        else:
            p = np.ascontiguousarray(pixels, np.uint8)
            if p.ndim == 3:
                p = p[None]
            data, nlev = p, 1
        td = _lib.TextureData(p.shape[2], p.shape[1], p.shape[0], data.ctypes.data, int(filter),
                              int(wrapS), int(wrapT), int(minFilter), int(mipFilter), nlev,
                              1 if generateMipmap else 0)
        out = ctypes.c_uint32()
        check(self._lib.gbr_add_texture(self._h, ctypes.byref(td), ctypes.byref(out)))
        return out.value

    def addMaterial(self, color=(1, 1, 1, 1), texture=0, layer=0, matrix=None, shaded=False):
        """A flat material, or with ``shaded`` a lit one (when the renderer has lights)."""
        m = np.eye(3, dtype=np.float32) if matrix is None else _f32(matrix, (3, 3))
        md = _lib.MaterialData((ctypes.c_float * 4)(*[float(c) for c in color]), int(texture),
                               int(layer), (ctypes.c_float * 9)(*m.reshape(-1).tolist()),
                               1 if shaded else 0)
        out = ctypes.c_uint32()
        check(self._lib.gbr_add_material(self._h, ctypes.byref(md), ctypes.byref(out)))
        return out.value

    def addNodeHierarchyTemplate(self, name, views):
        """views: iterable of (mesh, index_offset, index_count, material, transform|None);
        index_offset counts indices."""
        views = list(views)
        arr = (_lib.MeshView * max(1, len(views)))()
        for i, (mesh, off, cnt, mat, tr) in enumerate(views):
            t = np.eye(4, dtype=np.float32) if tr is None else _f32(tr, (4, 4))
            arr[i] = _lib.MeshView(int(mesh), int(off), int(cnt), int(mat),
                                   (ctypes.c_float * 16)(*t.reshape(-1).tolist()))
        check(self._lib.gbr_add_node_hierarchy_template(self._h, name.encode(), len(views), arr))

    # ------------------------------------------------------------ scenes
    def hasNodeHierarchy(self, name):
        out = ctypes.c_int32()
        check(self._lib.gbr_has_node_hierarchy(self._h, name.encode(), ctypes.byref(out)))
        return bool(out.value)

    def addNodeHierarchy(self, sceneId, name, bakeTransformation=None):
        bake = None if bakeTransformation is None else _f32(bakeTransformation, (4, 4))
        out = ctypes.c_uint64()
        check(self._lib.gbr_add_node_hierarchy(self._h, sceneId, name.encode(),
                                               None if bake is None else _fptr(bake),
                                               ctypes.byref(out)))
        return out.value

    def addEmptyNode(self, sceneId):
        out = ctypes.c_uint64()
        check(self._lib.gbr_add_empty_node(self._h, sceneId, ctypes.byref(out)))
        return out.value

    def clear(self, sceneId):
        check(self._lib.gbr_clear(self._h, sceneId))

    def setSemanticId(self, sceneId, nodeId, semanticId):
        check(self._lib.gbr_set_semantic_id(self._h, sceneId, nodeId, semanticId))

    def camera(self, sceneId):
        out = np.empty((4, 4), np.float32)
        check(self._lib.gbr_camera(self._h, sceneId, _fptr(out)))
        return out

    def cameraDepthUnprojection(self, sceneId):
        out = np.empty(2, np.float32)
        check(self._lib.gbr_camera_depth_unprojection(self._h, sceneId, _fptr(out)))
        return out

    def updateCamera(self, sceneId, projection, view):
        p = _f32(projection, (4, 4))
        v = _f32(view, (4, 4))
        check(self._lib.gbr_update_camera(self._h, sceneId, _fptr(p), _fptr(v)))

    def updateCameras(self, projections, views, first=0):
        p = _f32(projections, (-1, 4, 4))
        v = _f32(views, (-1, 4, 4))
        if p.shape != v.shape:
            raise ValueError("projections and views differ in count")
        check(self._lib.gbr_update_cameras(self._h, first, len(p), _fptr(p), _fptr(v)))

    def transformations(self, sceneId):
        """Writable [nodes, 4, 4] view of the scene's node transforms; valid
        until the next add/clear on this scene (Renderer.cpp:1090-1099)."""
        ptr = _lib.c_float_p()
        n = ctypes.c_uint64()
        check(self._lib.gbr_transformations(self._h, sceneId, ctypes.byref(ptr), ctypes.byref(n)))
        if n.value == 0:
            return np.zeros((0, 4, 4), np.float32)
        return np.ctypeslib.as_array(ptr, shape=(n.value, 4, 4))

    def sceneStats(self, sceneId):
        s = _lib.SceneStatsInfo()
        check(self._lib.gbr_scene_stats(self._h, sceneId, ctypes.byref(s)))
        return SceneStats(s.node_count, s.draw_count, s.draw_batch_count)

    # ------------------------------------------------------------- lights
    def addLight(self, sceneId, nodeId, type):
        """Renderer::addLight: the light follows the node (translation for a
        point light, negative backward axis for a directional one)."""
        out = ctypes.c_uint64()
        check(self._lib.gbr_add_light(self._h, sceneId, int(nodeId), int(type), ctypes.byref(out)))
        return out.value

    def clearLights(self, sceneId):
        check(self._lib.gbr_clear_lights(self._h, sceneId))

    def lightColors(self, sceneId):
        """Writable [lights, 3] view of the scene's light colours; valid until
        the next add/clear on this scene."""
        ptr, n = _lib.c_float_p(), ctypes.c_uint64()
        check(self._lib.gbr_light_colors(self._h, sceneId, ctypes.byref(ptr), ctypes.byref(n)))
        if n.value == 0:
            return np.zeros((0, 3), np.float32)
        return np.ctypeslib.as_array(ptr, shape=(n.value, 3))

    def lightRanges(self, sceneId):
        """Writable [lights] view of the scene's light ranges."""
        ptr, n = _lib.c_float_p(), ctypes.c_uint64()
        check(self._lib.gbr_light_ranges(self._h, sceneId, ctypes.byref(ptr), ctypes.byref(n)))
        if n.value == 0:
            return np.zeros(0, np.float32)
        return np.ctypeslib.as_array(ptr, shape=(n.value,))

    # ------------------------------------------- serving extensions (new)
    def setSceneSources(self, sources, first=0):
        """Scene ``first + i`` renders the nodes and draws of scene
        ``sources[i]`` with its own camera and viewport, from the next draw."""
        src = np.ascontiguousarray(sources, np.uint32).reshape(-1)
        check(self._lib.gbr_set_scene_sources(self._h, first, len(src),
                                              src.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))))

    def setSceneEnabled(self, sceneId, enabled):
        """A disabled scene is not drawn; its framebuffer rectangle keeps its pixels."""
        check(self._lib.gbr_set_scene_enabled(self._h, sceneId, 1 if enabled else 0))

    def removeMesh(self, meshId):
        check(self._lib.gbr_remove_mesh(self._h, meshId))

    def removeTexture(self, textureId):
        check(self._lib.gbr_remove_texture(self._h, textureId))

    def removeNodeHierarchyTemplate(self, name):
        check(self._lib.gbr_remove_node_hierarchy_template(self._h, name.encode()))

    def memoryUsage(self):
        """(live, reserved) device bytes of geometry, textures and chunk boxes."""
        live, reserved = ctypes.c_uint64(), ctypes.c_uint64()
        check(self._lib.gbr_memory_usage(self._h, ctypes.byref(live), ctypes.byref(reserved)))
        return live.value, reserved.value

    # -------------------------------------------------------------- draw
    def draw(self, stream=None, mode=None, graph=False):
        """Render every scene into the framebuffer, asynchronously on
        ``stream`` (a torch.cuda.Stream or a raw handle; None = default)."""
        h = _stream_handle(stream)
        if mode is None and not graph:
            check(self._lib.gbr_draw(self._h, h))
        else:
            m = self._config.draw_mode if mode is None else DrawMode(mode)
            check(self._lib.gbr_draw_mode(self._h, h, int(m), 1 if graph else 0))

    def lastDrawStats(self):
        s = _lib.DrawStats()
        check(self._lib.gbr_last_draw_stats(self._h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in _lib.DrawStats._fields_}

    def setKernelTiming(self, enabled=True):
        """CUDA events around the prepare and raster launches of batched
        draws; read back through lastDrawStats() (prepare_ms, raster_ms)."""
        check(self._lib.gbr_set_kernel_timing(self._h, 1 if enabled else 0))

    def setDeviceMemoryLimit(self, limit_bytes):
        """Cap the device memory this renderer's buffers may hold (0: none);
        an allocation beyond it fails with GBR_ERROR_OUT_OF_MEMORY."""
        check(self._lib.gbr_set_device_memory_limit(self._h, int(limit_bytes)))

    def deviceMemory(self):
        """(bytes held by the renderer's device buffers, limit or 0)."""
        held, limit = ctypes.c_uint64(), ctypes.c_uint64()
        check(self._lib.gbr_device_memory(self._h, ctypes.byref(held), ctypes.byref(limit)))
        return held.value, limit.value

    def debugCorruptParent(self, scene, node, parent):
        """Fault injection for tests: the node's parent replaced in device
        memory only; the next draw reports GBR_ERROR_DEVICE."""
        check(self._lib.gbr_debug_corrupt_parent(self._h, int(scene), int(node), int(parent)))

    def tuning(self):
        t = _lib.Tuning()
        check(self._lib.gbr_get_tuning(self._h, ctypes.byref(t)))
        return {k: int(getattr(t, k)) for k, _ in _lib.Tuning._fields_}

    def setTuning(self, **kw):
        t = _lib.Tuning()
        check(self._lib.gbr_get_tuning(self._h, ctypes.byref(t)))
        for k, v in kw.items():
            setattr(t, k, int(v))
        check(self._lib.gbr_set_tuning(self._h, ctypes.byref(t)))

    # ------------------------------------------------------------ images
    def _image(self, plane, dtype, channels=None):
        if self._config.viewports:
            raise GbrError(7, "the ragged layout has no tile grid; use sceneImage()")
        w, h = self._fb
        shape = (h, w) if channels is None else (h, w, channels)
        out = np.empty(shape, dtype)
        rect = (ctypes.c_int32 * 4)(0, 0, w, h)
        check(self._lib.gbr_image_into(self._h, int(plane), rect, out.ctypes.data,
                                       out.strides[0]))
        return out

    def colorImage(self):
        """RGBA8 [H, W, 4] (``RendererStandalone::colorImage``, RendererStandalone.cpp:161-166)."""
        return self._image(Plane.Color, np.uint8, 4)

    def depthImage(self):
        """Window depth [H, W] float32 (``RendererStandalone::depthImage``, :182-187)."""
        return self._image(Plane.Depth, np.float32)

    def linearDepthImage(self):
        """Metres along the view axis, 0 where nothing was drawn."""
        return self._image(Plane.LinearDepth, np.float32)

    def semanticImage(self):
        return self._image(Plane.Semantic, np.uint32)

    def _image_into(self, plane, rectangle, image, asynchronous=False):
        (x0, y0), (x1, y1) = rectangle
        if image.shape[0] != y1 - y0 or image.shape[1] != x1 - x0:
            raise GbrError(1, f"expected image size of {(x1 - x0, y1 - y0)} pixels but got "
                              f"{(image.shape[1], image.shape[0])}")
        if not image.flags.c_contiguous:
            raise GbrError(1, "image must be C-contiguous")
        rect = (ctypes.c_int32 * 4)(x0, y0, x1, y1)
        fn = self._lib.gbr_image_into_async if asynchronous else self._lib.gbr_image_into
        check(fn(self._h, int(plane), rect, image.ctypes.data, image.strides[0]))

    def imageIntoAsync(self, plane, rectangle, image):
        """Start copying a rectangle of a plane of the last draw into
        ``image`` (host memory; pinned for full speed) and return at once;
        ``readbackWait()`` waits for the copies."""
        self._image_into(Plane(plane), rectangle, image, asynchronous=True)

    def readbackWait(self):
        check(self._lib.gbr_readback_wait(self._h))

    def scenesIntoAsync(self, plane, first, count, out):
        """Start packing scenes [first, first + count) of a plane of the last
        draw into ``out`` -- a C-contiguous [count, h, w(, 4)] numpy array
        (host; pinned for full speed) or CUDA torch tensor -- and return at
        once; ``readbackWait()`` waits."""
        if hasattr(out, "data_ptr"):
            if not out.is_contiguous():
                raise GbrError(1, "out must be contiguous")
            ptr = out.data_ptr()
        else:
            if not out.flags.c_contiguous:
                raise GbrError(1, "out must be C-contiguous")
            ptr = out.ctypes.data
        check(self._lib.gbr_scenes_into_async(self._h, int(plane), int(first), int(count), ptr))

    def colorImageInto(self, rectangle, image):
        """``colorImageInto`` (RendererStandalone.cpp:168-180); rectangle is
        ((x0, y0), (x1, y1)), image a uint8 [y1-y0, x1-x0, 4] array."""
        self._image_into(Plane.Color, rectangle, image)

    def depthImageInto(self, rectangle, image):
        """``depthImageInto`` (RendererStandalone.cpp:189-202)."""
        self._image_into(Plane.Depth, rectangle, image)

    def linearDepthImageInto(self, rectangle, image):
        self._image_into(Plane.LinearDepth, rectangle, image)

    def semanticImageInto(self, rectangle, image):
        self._image_into(Plane.Semantic, rectangle, image)

    def sceneImage(self, plane, sceneId):
        """One scene's rectangle of a plane (either layout), row 0 = bottom."""
        _, _, w, h = self.sceneViewport(sceneId)
        plane = Plane(plane)
        if plane == Plane.Color:
            out = np.empty((h, w, 4), np.uint8)
        elif plane == Plane.Semantic:
            out = np.empty((h, w), np.uint32)
        else:
            out = np.empty((h, w), np.float32)
        self.sceneImageInto(plane, sceneId, out)
        return out

    def sceneImageInto(self, plane, sceneId, image):
        check(self._lib.gbr_scene_image_into(self._h, int(plane), sceneId, image.ctypes.data,
                                             image.strides[0]))

    # ----------------------------------------------------- device access
    def planeDevicePointer(self, plane):
        out = ctypes.c_void_p()
        n = ctypes.c_uint64()
        check(self._lib.gbr_plane_device_pointer(self._h, int(plane), ctypes.byref(out),
                                                 ctypes.byref(n)))
        return out.value, n.value

    def colorCudaBufferDevicePointer(self):
        """RendererStandalone.cpp:205-233; the live framebuffer, no copy."""
        return self.planeDevicePointer(Plane.Color)[0]

    def depthCudaBufferDevicePointer(self):
        """RendererStandalone.cpp:235-263; returns the depth plane."""
        return self.planeDevicePointer(Plane.Depth)[0]

    def deviceTensor(self, plane):
        """A CUDA torch tensor viewing a whole plane (DLPack, no copy).  The
        tensor keeps the renderer alive; its contents change at each draw."""
        import torch

        out = ctypes.c_void_p()
        check(self._lib.gbr_plane_dlpack(self._h, int(plane), ctypes.byref(out)))
        new = ctypes.pythonapi.PyCapsule_New
        new.restype = ctypes.py_object
        new.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p]
        capsule = new(out, b"dltensor", None)
        return torch.utils.dlpack.from_dlpack(capsule)

    def colorTensor(self):
        return self.deviceTensor(Plane.Color)

    def drawHbao(self, configuration=None, stream=None, algorithm=None):
        """``Hbao::drawEffect`` on every enabled scene of the last draw:
        colour darkened in place from linear depth and each scene's
        projection; ``algorithm`` (``HbaoType``) overrides the
        configuration's; asynchronous on `stream`."""
        c = (configuration or HbaoConfiguration())._c()
        if algorithm is not None:
            c.algorithm = int(HbaoType(algorithm))
        check(self._lib.gbr_hbao_draw(self._h, ctypes.byref(c), _stream_handle(stream)))

    def depthTensor(self):
        return self.deviceTensor(Plane.Depth)

    def linearDepthTensor(self):
        return self.deviceTensor(Plane.LinearDepth)

    def semanticTensor(self):
        return self.deviceTensor(Plane.Semantic)


def calculateDepthUnprojection(projection):
    """``calculateDepthUnprojection`` (DepthUnprojection.cpp:98-101)."""
    p = _f32(projection, (4, 4))
    return np.array([(p[2, 2] - np.float32(1.0)) * np.float32(0.5),
                     p[3, 2] * np.float32(0.5)], np.float32)


def unprojectDepth(unprojection, depth):
    """``unprojectDepth`` (DepthUnprojection.cpp:107-129) in place on a
    float32 [rows, cols] array whose rows may be strided."""
    lib = _lib.load()
    u = _f32(unprojection, (2,))
    if depth.dtype != np.float32 or depth.ndim != 2 or depth.strides[1] != 4:
        raise ValueError("depth must be a float32 [rows, cols] array with contiguous rows")
    check(lib.gbr_unproject_depth(_fptr(u), depth.ctypes.data_as(_lib.c_float_p),
                                  depth.shape[0], depth.shape[1], depth.strides[0] // 4))
    return depth


def unprojectDepthDevice(unprojection, tensor, stream=None):
    """unprojectDepth on a CUDA float32 [rows, cols] torch tensor, on its GPU."""
    lib = _lib.load()
    u = _f32(unprojection, (2,))
    rows, cols = tensor.shape
    check(lib.gbr_unproject_depth_device(_fptr(u), tensor.data_ptr(), rows, cols,
                                         tensor.stride(0), _stream_handle(stream)))
    return tensor
