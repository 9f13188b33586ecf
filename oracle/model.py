"""Oracle mirror of the batch renderer's scene bookkeeping (test infrastructure).

Used only by ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline.  It restates the state that habitat-sim's
``esp::gfx_batch::Renderer`` keeps between ``addFile`` and ``draw``:

* reserved texture 0 (white) and material 0 (white, untextured)
  (``src/esp/gfx_batch/Renderer.cpp:287-304``);
* file import with texture / mesh / mesh-view / material offsets
  (``Renderer.cpp:410-415, 579-633, 700-826``);
* ``addNodeHierarchy``: a root node plus one child per mesh view whose
  transform is ``bake * view.transform``, draws filed into draw batches keyed
  by (vertex-colour flag, mesh, texture) (``Renderer.cpp:880-961``,
  ``drawBatchId`` at ``Renderer.cpp:136-152``);
* ``addEmptyNode``, ``clear``, ``updateCamera`` (stores ``P*V``) and the
  depth unprojection coefficients (``Renderer.cpp:963-1088``,
  ``DepthUnprojection.cpp:98-101``);
* draw order: stable counting sort of draws by batch id
  (``Renderer.cpp:1139-1196``).

Pixels are produced by ``raster.cpp`` through ``oracle_render``.
"""
import ctypes
import os

import numpy as np

from . import gltf as _gltf
from .build import load_library

FLAG_NO_TEXTURES = 1
FILE_WHOLE = 1
FILE_GENERATE_MIPMAP = 2
BACKGROUND = 0xFF1F1F1F


class _Tex(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("width", ctypes.c_int32), ("height", ctypes.c_int32),
                ("layers", ctypes.c_int32), ("filter", ctypes.c_int32),
                ("wrap_s", ctypes.c_int32), ("wrap_t", ctypes.c_int32),
                ("min_filter", ctypes.c_int32), ("mip_filter", ctypes.c_int32),
                ("levels", ctypes.c_int32)]


def mip_chain_levels(w, h):
    """floor(log2(min(w, h))) + 1 (Renderer.cpp:445-450, 493-498)."""
    return int(min(w, h)).bit_length()


def generate_mips(level0, levels):
    """Levels 1.. of a uint8 [layers, h, w, 4] texture: each texel the mean
    (a + b + c + d + 2) >> 2 of the 2 x 2 texels above it (indices clamped to
    the finer level).  Returns the list of levels, level 0 first."""
    out = [np.ascontiguousarray(level0, np.uint8)]
    for _ in range(1, levels):
        p = out[-1].astype(np.uint32)
        _, ph, pw, _ = p.shape
        nh, nw = max(1, ph // 2), max(1, pw // 2)
        y0 = np.minimum(2 * np.arange(nh), ph - 1)
        y1 = np.minimum(2 * np.arange(nh) + 1, ph - 1)
        x0 = np.minimum(2 * np.arange(nw), pw - 1)
        x1 = np.minimum(2 * np.arange(nw) + 1, pw - 1)
        s = (p[:, y0][:, :, x0] + p[:, y0][:, :, x1] + p[:, y1][:, :, x0] + p[:, y1][:, :, x1] + 2) >> 2
        out.append(s.astype(np.uint8))
    return out


class _Mesh(ctypes.Structure):
    _fields_ = [("positions", ctypes.c_void_p), ("colors", ctypes.c_void_p),
                ("texcoords", ctypes.c_void_p), ("object_ids", ctypes.c_void_p),
                ("indices", ctypes.c_void_p), ("vertex_count", ctypes.c_uint32),
                ("index_count", ctypes.c_uint32), ("normals", ctypes.c_void_p)]


class _Mat(ctypes.Structure):
    _fields_ = [("color", ctypes.c_float * 4), ("texture", ctypes.c_int32),
                ("layer", ctypes.c_int32), ("matrix", ctypes.c_float * 9),
                ("phong", ctypes.c_int32)]


class _Light(ctypes.Structure):
    _fields_ = [("node", ctypes.c_int32), ("type", ctypes.c_int32),
                ("color", ctypes.c_float * 3), ("range", ctypes.c_float)]


LIGHT_DIRECTIONAL = 0
LIGHT_POINT = 1


class _Draw(ctypes.Structure):
    _fields_ = [("node", ctypes.c_int32), ("mesh", ctypes.c_int32),
                ("index_offset", ctypes.c_uint32), ("index_count", ctypes.c_uint32),
                ("material", ctypes.c_int32), ("semantic_id", ctypes.c_uint32)]


class _Scene(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32),
                ("fb_offset", ctypes.c_int64), ("pitch", ctypes.c_int64),
                ("pv", ctypes.c_float * 16), ("view", ctypes.c_float * 16),
                ("node_count", ctypes.c_int32), ("parents", ctypes.c_void_p),
                ("transforms", ctypes.c_void_p), ("draw_count", ctypes.c_int32),
                ("draws", ctypes.c_void_p), ("light_count", ctypes.c_int32),
                ("lights", ctypes.c_void_p)]


class _Out(ctypes.Structure):
    _fields_ = [("color", ctypes.c_void_p), ("depth", ctypes.c_void_p),
                ("linear_depth", ctypes.c_void_p), ("semantic", ctypes.c_void_p)]


def _ptr(a):
    return None if a is None else a.ctypes.data


def matmul(a, b):
    return _gltf._matmul(a, b)


class SceneStats:
    def __init__(self, node_count, draw_count, draw_batch_count):
        self.nodeCount = node_count
        self.drawCount = draw_count
        self.drawBatchCount = draw_batch_count


class OracleRenderer:
    """CPU restatement of ``RendererStandalone`` with the same call surface.

    ``viewports`` (optional) gives each scene its own (width, height) and
    switches the framebuffer to a ragged layout: scene ``s`` occupies
    ``width*height`` consecutive pixels, rows bottom-up."""

    def __init__(self, tile_size=(128, 128), tile_count=(1, 1), flags=0, viewports=None,
                 max_light_count=0, ambient_factor=0.1):
        self.flags = flags
        self.max_light_count = int(max_light_count)
        self.ambient_factor = float(ambient_factor)
        self.tile_size = tuple(tile_size)
        self.tile_count = tuple(tile_count)
        if viewports is None:
            n = tile_count[0] * tile_count[1]
            tw, th = tile_size
            pitch = tw * tile_count[0]
            self.layout = []
            for s in range(n):
                x, y = s % tile_count[0], s // tile_count[0]
                self.layout.append((tw, th, y * th * pitch + x * tw, pitch))
            self.fb_shape = (th * tile_count[1], pitch)
        else:
            self.layout = []
            off = 0
            for (w, h) in viewports:
                self.layout.append((w, h, off, w))
                off += w * h
            self.fb_shape = (off,)
        n = len(self.layout)
        white = np.full((1, 1, 1, 4), 255, np.uint8)
        self.textures = [dict(pixels=white, filter=0, wrap_s=0, wrap_t=0)]
        self.meshes = []
        self.materials = [dict(color=np.ones(4, np.float32), texture=0, layer=0,
                               matrix=np.eye(3, dtype=np.float32), phong=False)]
        self.mesh_views = []
        self.names = {}
        self.scenes = [self._empty_scene() for _ in range(n)]
        self.pv = [np.eye(4, dtype=np.float32) for _ in range(n)]
        self.view = [np.eye(4, dtype=np.float32) for _ in range(n)]
        self.unprojection = [np.zeros(2, np.float32) for _ in range(n)]
        self._lib = load_library()
        self.color = self.depth = self.linear_depth = self.semantic = None

    @staticmethod
    def _empty_scene():
        return dict(parents=[], transforms=[], draws=[], batches=[], light_nodes=[],
                    light_types=[], light_colors=np.zeros((0, 3), np.float32),
                    light_ranges=np.zeros(0, np.float32))

    def sceneCount(self):
        return len(self.scenes)

    # ---------------------------------------------------------------- files
    def addFile(self, filename, flags=0, name=None):
        f = _gltf.load_gltf(filename, whole=bool(flags & FILE_WHOLE), name=name,
                            no_textures=bool(self.flags & FLAG_NO_TEXTURES))
        texture_offset = len(self.textures)
        mesh_offset = len(self.meshes)
        view_offset = len(self.mesh_views)
        material_offset = len(self.materials)
        for t in f.textures:
            gen = bool(flags & FILE_GENERATE_MIPMAP) and not t.get("compressed", False)
            self.add_texture(t["pixels"], t["mag"], t["wrap_s"], t["wrap_t"],
                             min_filter=t.get("min", t["mag"]) + 1, mip_filter=t.get("mip", 0),
                             generate_mipmap=gen)
        for m in f.meshes:
            self.add_mesh(m["positions"], m["colors"], m["texcoords"], m["object_ids"],
                          m["indices"], m.get("normals"))
        for m in f.materials:
            tex = 0 if m["texture"] is None else m["texture"] + texture_offset
            layer = 0 if m["texture"] is None else m["layer"]
            matrix = np.eye(3, dtype=np.float32) if m["texture"] is None else m["matrix"]
            self.materials.append(dict(color=m["color"].astype(np.float32), texture=tex,
                                       layer=layer, matrix=matrix, phong=not m["flat"]))
        for v in f.mesh_views:
            mat = 0 if v["material"] == -1 else v["material"] + material_offset
            self.mesh_views.append(dict(mesh=v["mesh"] + mesh_offset,
                                        index_offset=v["index_offset_bytes"] // 4,
                                        index_count=v["index_count"], material=mat,
                                        transform=v["transform"]))
        for (nm, b, e) in f.templates:
            if nm in self.names:
                raise KeyError(f"node name {nm} already exists")
            self.names[nm] = (b + view_offset, e + view_offset)
        return True

    # ----------------------------------------------------------- procedural
    def add_mesh(self, positions, colors=None, texcoords=None, object_ids=None, indices=None,
                 normals=None):
        self.meshes.append(dict(
            normals=None if normals is None else np.ascontiguousarray(normals, np.float32).reshape(-1, 3),
            positions=np.ascontiguousarray(positions, np.float32).reshape(-1, 3),
            colors=None if colors is None else np.ascontiguousarray(colors, np.float32).reshape(-1, 4),
            texcoords=None if texcoords is None else np.ascontiguousarray(texcoords, np.float32).reshape(-1, 2),
            object_ids=None if object_ids is None else np.ascontiguousarray(object_ids, np.uint32).reshape(-1),
            indices=np.ascontiguousarray(indices, np.uint32).reshape(-1)))
        return len(self.meshes) - 1

    def add_texture(self, pixels, filter=1, wrap_s=0, wrap_t=0, min_filter=0, mip_filter=0,
                    levels=None, generate_mipmap=False):
        """pixels: uint8 [layers, h, w, 4] (level 0), or a list of levels when
        `levels` is given; min_filter 0 = as `filter`, 1 nearest, 2 linear;
        mip_filter 0 base level, 1 nearest level, 2 linear between levels."""
        if levels is not None:
            chain = [np.ascontiguousarray(l, np.uint8) for l in pixels]
            chain = [c[None] if c.ndim == 3 else c for c in chain]
        else:
            p = np.ascontiguousarray(pixels, np.uint8)
            if p.ndim == 3:
                p = p[None]
            chain = [p]
            if generate_mipmap:
                chain = generate_mips(p, mip_chain_levels(p.shape[2], p.shape[1]))
        self.textures.append(dict(
            pixels=chain[0], data=np.concatenate([c.reshape(-1) for c in chain]),
            filter=filter, wrap_s=wrap_s, wrap_t=wrap_t,
            min_filter=filter if min_filter == 0 else min_filter - 1, mip_filter=int(mip_filter),
            levels=len(chain)))
        return len(self.textures) - 1

    def add_material(self, color=(1, 1, 1, 1), texture=0, layer=0, matrix=None, shaded=False):
        self.materials.append(dict(color=np.asarray(color, np.float32), texture=int(texture),
                                   layer=int(layer),
                                   matrix=np.eye(3, dtype=np.float32) if matrix is None
                                   else np.asarray(matrix, np.float32).reshape(3, 3),
                                   phong=bool(shaded)))
        return len(self.materials) - 1

    def add_node_hierarchy_template(self, name, views):
        """views: list of (mesh, index_offset_in_indices, index_count, material, transform)."""
        if name in self.names:
            raise KeyError(f"node name {name} already exists")
        b = len(self.mesh_views)
        for (mesh, off, cnt, mat, tr) in views:
            self.mesh_views.append(dict(mesh=mesh, index_offset=off, index_count=cnt,
                                        material=mat,
                                        transform=np.eye(4, dtype=np.float32) if tr is None
                                        else np.asarray(tr, np.float32).reshape(4, 4)))
        self.names[name] = (b, len(self.mesh_views))

    # --------------------------------------------------------------- scenes
    def hasNodeHierarchy(self, name):
        return name in self.names

    def addNodeHierarchy(self, scene, name, bake=None, semantic_id=0):
        sc = self.scenes[scene]
        b, e = self.names[name]
        top = len(sc["transforms"])
        sc["parents"].append(-1)
        sc["transforms"].append(np.eye(4, dtype=np.float32))
        bake = np.eye(4, dtype=np.float32) if bake is None else np.asarray(bake, np.float32)
        for i in range(b, e):
            v = self.mesh_views[i]
            nid = len(sc["transforms"])
            sc["parents"].append(top)
            sc["transforms"].append(matmul(bake, v["transform"]))
            mesh = self.meshes[v["mesh"]]
            key = (mesh["colors"] is not None, v["mesh"], self.materials[v["material"]]["texture"])
            if key not in sc["batches"]:
                sc["batches"].append(key)
            sc["draws"].append(dict(batch=sc["batches"].index(key), node=nid, top=top,
                                    mesh=v["mesh"], index_offset=v["index_offset"],
                                    index_count=v["index_count"], material=v["material"],
                                    semantic=semantic_id))
        return top

    def addEmptyNode(self, scene):
        sc = self.scenes[scene]
        sc["parents"].append(-1)
        sc["transforms"].append(np.eye(4, dtype=np.float32))
        return len(sc["transforms"]) - 1

    # --------------------------------------------------------------- lights
    def addLight(self, scene, node, light_type):
        """Renderer::addLight (Renderer.cpp:990-1015): white, infinite range."""
        if not self.max_light_count:
            raise ValueError("max light count is zero")
        sc = self.scenes[scene]
        if not 0 <= node < len(sc["parents"]):
            raise IndexError("node out of range")
        sc["light_nodes"].append(int(node))
        sc["light_types"].append(int(light_type))
        sc["light_colors"] = np.concatenate([sc["light_colors"], np.ones((1, 3), np.float32)])
        sc["light_ranges"] = np.concatenate([sc["light_ranges"], np.full(1, np.inf, np.float32)])
        return len(sc["light_nodes"]) - 1

    def clearLights(self, scene):
        sc = self.scenes[scene]
        fresh = self._empty_scene()
        for k in ("light_nodes", "light_types", "light_colors", "light_ranges"):
            sc[k] = fresh[k]

    def lightColors(self, scene):
        return self.scenes[scene]["light_colors"]

    def lightRanges(self, scene):
        return self.scenes[scene]["light_ranges"]

    def set_semantic_id(self, scene, node, semantic_id):
        for d in self.scenes[scene]["draws"]:
            if d["top"] == node:
                d["semantic"] = semantic_id

    def clear(self, scene):
        self.scenes[scene] = self._empty_scene()

    def transformations(self, scene):
        return self.scenes[scene]["transforms"]

    def updateCamera(self, scene, projection, view):
        projection = np.asarray(projection, np.float32)
        self.pv[scene] = matmul(projection, np.asarray(view, np.float32))
        self.view[scene] = np.asarray(view, np.float32).copy()
        self.unprojection[scene] = np.array(
            [np.float32(projection[2, 2] - np.float32(1.0)) * np.float32(0.5),
             projection[3, 2] * np.float32(0.5)], np.float32)

    def camera(self, scene):
        return self.pv[scene]

    def cameraDepthUnprojection(self, scene):
        return self.unprojection[scene]

    def sceneStats(self, scene):
        sc = self.scenes[scene]
        return SceneStats(len(sc["transforms"]), len(sc["draws"]), len(sc["batches"]))

    def sorted_draws(self, scene):
        sc = self.scenes[scene]
        return sorted(sc["draws"], key=lambda d: d["batch"])  # stable

    # ----------------------------------------------------------------- draw
    def draw(self, threads=1, window_depth=True, linear_depth=True, semantic=True):
        lib = self._lib
        keep = []
        tex = (_Tex * len(self.textures))()
        for i, t in enumerate(self.textures):
            p = t["pixels"]
            d = t.get("data", p.reshape(-1))
            keep.append(d)
            tex[i] = _Tex(d.ctypes.data, p.shape[2], p.shape[1], p.shape[0], t["filter"],
                          t["wrap_s"], t["wrap_t"], t.get("min_filter", t["filter"]),
                          t.get("mip_filter", 0), t.get("levels", 1))
        meshes = (_Mesh * max(1, len(self.meshes)))()
        for i, m in enumerate(self.meshes):
            meshes[i] = _Mesh(_ptr(m["positions"]), _ptr(m["colors"]), _ptr(m["texcoords"]),
                              _ptr(m["object_ids"]), _ptr(m["indices"]), len(m["positions"]),
                              len(m["indices"]), _ptr(m.get("normals")))
        mats = (_Mat * len(self.materials))()
        for i, m in enumerate(self.materials):
            mats[i] = _Mat((ctypes.c_float * 4)(*m["color"]), m["texture"], m["layer"],
                           (ctypes.c_float * 9)(*np.asarray(m["matrix"], np.float32).reshape(-1)),
                           1 if m.get("phong") else 0)
        scenes = (_Scene * len(self.scenes))()
        for s, sc in enumerate(self.scenes):
            w, h, off, pitch = self.layout[s]
            parents = np.asarray(sc["parents"], np.int32)
            transforms = (np.stack(sc["transforms"]).astype(np.float32) if sc["transforms"]
                          else np.zeros((0, 4, 4), np.float32))
            dl = self.sorted_draws(s)
            draws = (_Draw * max(1, len(dl)))()
            for i, d in enumerate(dl):
                draws[i] = _Draw(d["node"], d["mesh"], d["index_offset"], d["index_count"],
                                 d["material"], d["semantic"])
            nl = len(sc["light_nodes"])
            lights = (_Light * max(1, nl))()
            for j in range(nl):
                lights[j] = _Light(sc["light_nodes"][j], sc["light_types"][j],
                                   (ctypes.c_float * 3)(*sc["light_colors"][j].tolist()),
                                   float(sc["light_ranges"][j]))
            keep += [parents, transforms, draws, lights]
            scenes[s] = _Scene(w, h, off, pitch,
                               (ctypes.c_float * 16)(*self.pv[s].reshape(-1)),
                               (ctypes.c_float * 16)(*self.view[s].reshape(-1)),
                               len(parents), _ptr(parents), _ptr(transforms), len(dl),
                               ctypes.addressof(draws), nl, ctypes.addressof(lights))
        self.color = np.zeros(self.fb_shape, np.uint32)
        self.depth = np.ones(self.fb_shape, np.float32) if window_depth else None
        self.linear_depth = np.zeros(self.fb_shape, np.float32) if linear_depth else None
        self.semantic = np.zeros(self.fb_shape, np.uint32) if semantic else None
        out = _Out(_ptr(self.color), _ptr(self.depth), _ptr(self.linear_depth),
                   _ptr(self.semantic))
        lib.oracle_render(tex, len(self.textures), meshes, mats, scenes, len(self.scenes),
                          self.flags, out, threads, self.max_light_count,
                          ctypes.c_float(self.ambient_factor))

    # --------------------------------------------------------------- images
    def colorImage(self):
        """RGBA8 image [H, W, 4], row 0 = bottom (GL origin)."""
        return self.color.view(np.uint8).reshape(self.color.shape + (4,))

    def depthImage(self):
        return self.depth

    def scene_image(self, plane, scene):
        """One scene's rectangle of a plane as [h, w] (row 0 = bottom)."""
        w, h, off, pitch = self.layout[scene]
        flat = plane.reshape(-1)
        return np.stack([flat[off + y * pitch: off + y * pitch + w] for y in range(h)])


def unproject_depth(unprojection, depth):
    """In-place ``unprojectDepth`` on a float32 [rows, cols] array."""
    lib = load_library()
    a = np.ascontiguousarray(unprojection, np.float32)
    assert depth.dtype == np.float32 and depth.flags.c_contiguous
    lib.oracle_unproject_depth(a.ctypes.data, depth.ctypes.data, depth.shape[0], depth.shape[1],
                               depth.shape[1])
    return depth


# Procedural call surface shared with the GPU renderer's Python API.
OracleRenderer.addMesh = lambda self, positions, colors=None, texcoords=None, objectIds=None, \
    indices=None: self.add_mesh(positions, colors, texcoords, objectIds, indices)
OracleRenderer.addTexture = lambda self, pixels, filter=1, wrapS=0, wrapT=0, minFilter=0, \
    mipFilter=0, levels=None, generateMipmap=False: \
    self.add_texture(pixels, filter, wrapS, wrapT, minFilter, mipFilter, levels, generateMipmap)
OracleRenderer.addMaterial = lambda self, color=(1, 1, 1, 1), texture=0, layer=0, matrix=None: \
    self.add_material(color, texture, layer, matrix)
OracleRenderer.addNodeHierarchyTemplate = lambda self, name, views: \
    self.add_node_hierarchy_template(name, views)
OracleRenderer.setSemanticId = lambda self, scene, node, sid: self.set_semantic_id(scene, node, sid)


def _update_cameras(self, projections, views, first=0):
    for i, (p, v) in enumerate(zip(projections, views)):
        self.updateCamera(first + i, p, v)


OracleRenderer.updateCameras = _update_cameras
