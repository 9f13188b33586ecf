"""Batch replay renderer: habitat-sim's Python ``ReplayRenderer`` on the GB300
renderer.

Mirrors the Python binding of ``AbstractReplayRenderer``
(src/esp/bindings/SimBindings.cpp:467-545) with the batch back end
(src/esp/sim/BatchReplayRenderer.cpp): per environment, a gfx-replay
keyframe (the JSON that ``Recorder::keyframeToString`` writes,
src/esp/io/JsonEspTypes.cpp:12-99) drives the instances of one renderer
scene, a user transform of the keyframe or an explicit matrix places the
camera, and ``render`` draws every environment in one batched launch and
copies colour and depth out.  The keyframe player and the batch player run
natively (include/gbr_replay.h); this module is the Python surface.

Differences a caller can see:

* ``render`` also takes CUDA torch tensors as destinations (device-to-device
  copies), and ``color_tensor()`` / ``depth_tensor()`` view the whole
  framebuffer without a copy (DLPack).
* ``cuda_depth_buffer_device_pointer`` returns the depth plane (the
  reference's binding returns the colour pointer, SimBindings.cpp:537-539).
* ``unproject`` computes the camera ray (the reference's batch back end
  returns a placeholder, BatchReplayRenderer.cpp:169-180).
* Depth is metres along the view axis computed on the GPU, 0 where nothing
  is drawn, instead of window depth unprojected on the CPU.
* Only the batch back end exists: ``create_classic_replay_renderer`` and
  drawing into a GL framebuffer raise.
"""
import ctypes
import json
import math

import numpy as np

from . import _lib
from ._lib import check
from .gfx_batch import (DrawMode, Plane, RendererConfiguration, RendererStandalone,
                        RendererStandaloneConfiguration, RendererStandaloneFlags)


class SensorSubType:
    PINHOLE = "pinhole"
    ORTHOGRAPHIC = "orthographic"


class CameraSensorSpec:
    """The ``CameraSensorSpec`` fields the replay renderer reads
    (sensor/CameraSensor.h:14-30, sensor/VisualSensor.h:36-63)."""

    def __init__(self, uuid="rgba_camera", resolution=(128, 128), hfov=90.0, near=0.01,
                 far=1000.0, sensor_subtype=SensorSubType.PINHOLE, ortho_scale=0.1):
        self.uuid = uuid
        self.resolution = list(resolution)      # [height, width]
        self.hfov = float(hfov)                 # degrees
        self.near = float(near)
        self.far = float(far)
        self.sensor_subtype = sensor_subtype
        self.ortho_scale = float(ortho_scale)


class ReplayRendererConfiguration:
    """``ReplayRendererConfiguration`` (AbstractReplayRenderer.h:24-63) plus
    the batch renderer options the reference leaves at their defaults."""

    def __init__(self):
        self.num_environments = 1
        self.gpu_device_id = 0
        self.standalone = True
        self.force_separate_semantic_scene_graph = False
        self.leave_context_with_background_renderer = False
        self.enable_frustum_culling = True
        self.enable_hbao = False
        self.sensor_specifications = []
        self.max_light_count = 0
        self.ambient_factor = 0.1
        self.draw_mode = DrawMode.Batched
        self.quiet = False


class Ray:
    def __init__(self, origin, direction):
        self.origin = np.asarray(origin, np.float32)
        self.direction = np.asarray(direction, np.float32)

    def __repr__(self):
        return f"Ray(origin={self.origin.tolist()}, direction={self.direction.tolist()})"


def _cstr(s):
    return s.encode() if isinstance(s, str) else bytes(s)


class ReplayRenderer:
    """``ReplayRenderer`` (SimBindings.cpp:467-545), batch back end."""

    def __init__(self, cfg):
        specs = list(cfg.sensor_specifications)
        if len(specs) != 1:
            raise ValueError("BatchReplayRenderer: expecting exactly one sensor")
        spec = specs[0]
        self._lib = _lib.load()
        c = _lib.ReplayConfig()
        self._lib.gbr_replay_config_init(ctypes.byref(c))
        c.num_environments = int(cfg.num_environments)
        c.gpu_device_id = int(cfg.gpu_device_id)
        c.standalone = 1 if cfg.standalone else 0
        c.enable_frustum_culling = 1 if cfg.enable_frustum_culling else 0
        c.enable_hbao = 1 if cfg.enable_hbao else 0
        self._uuid = _cstr(spec.uuid)
        c.sensor_uuid = self._uuid
        c.resolution[0], c.resolution[1] = int(spec.resolution[0]), int(spec.resolution[1])
        c.hfov_degrees = float(getattr(spec.hfov, "degrees", spec.hfov))
        c.near_plane = float(spec.near)
        c.far_plane = float(spec.far)
        c.orthographic = 1 if str(spec.sensor_subtype).lower().endswith("orthographic") else 0
        c.ortho_scale = float(spec.ortho_scale)
        c.max_light_count = int(cfg.max_light_count)
        c.ambient_factor = float(cfg.ambient_factor)
        c.draw_mode = int(cfg.draw_mode)
        c.quiet = 1 if cfg.quiet else 0
        handle = ctypes.c_void_p()
        check(self._lib.gbr_replay_create(ctypes.byref(c), ctypes.byref(handle)))
        self._h = handle
        self._spec = spec
        self._n = int(cfg.num_environments)
        self._grid = ReplayRenderer.environment_grid_size(self._n)
        self._res = (int(spec.resolution[0]), int(spec.resolution[1]))   # (h, w)
        r = ctypes.c_void_p()
        check(self._lib.gbr_replay_renderer(self._h, ctypes.byref(r)))
        rcfg = (RendererConfiguration()
                .setTileSizeCount((self._res[1], self._res[0]), self._grid)
                .setDrawMode(cfg.draw_mode))
        rcfg.max_light_count = int(cfg.max_light_count)
        rcfg.ambient_factor = float(cfg.ambient_factor)
        scfg = RendererStandaloneConfiguration().setCudaDevice(cfg.gpu_device_id).setFlags(
            RendererStandaloneFlags.QuietLog if cfg.quiet else 0)
        self._renderer = RendererStandalone._borrow(r.value, rcfg, scfg, self)

    # ------------------------------------------------------------ factory
    @staticmethod
    def create_batch_replay_renderer(cfg):
        """Create a replay renderer using the batch render pipeline."""
        return ReplayRenderer(cfg)

    @staticmethod
    def create_classic_replay_renderer(cfg):
        raise NotImplementedError("only the batch replay renderer exists on this renderer")

    @staticmethod
    def environment_grid_size(environment_count):
        """``environmentGridSize`` (AbstractReplayRenderer.cpp:26-31)."""
        out = (ctypes.c_int32 * 2)()
        check(_lib.load().gbr_replay_environment_grid_size(int(environment_count), out))
        return (out[0], out[1])

    # ---------------------------------------------------------- lifetime
    def close(self):
        """Releases the renderer and its GPU resources; safe to repeat."""
        if getattr(self, "_h", None):
            if getattr(self, "_renderer", None) is not None:
                self._renderer.close()
                self._renderer = None
            check(self._lib.gbr_replay_close(self._h))

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                if getattr(self, "_renderer", None) is not None:
                    self._renderer.close()
                self._lib.gbr_replay_destroy(self._h)
                self._h = None
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ------------------------------------------------------------ queries
    @property
    def environment_count(self):
        n = ctypes.c_uint32()
        check(self._lib.gbr_replay_environment_count(self._h, ctypes.byref(n)))
        return n.value

    def sensor_size(self, env_index):
        """(width, height) of the environment's sensor."""
        out = (ctypes.c_int32 * 2)()
        check(self._lib.gbr_replay_sensor_size(self._h, int(env_index), out))
        return (out[0], out[1])

    @property
    def renderer(self):
        """The batch renderer (``RendererStandalone``) that draws the
        environments, environment i being scene i."""
        if self._renderer is None:
            raise RuntimeError("the replay renderer is closed")
        return self._renderer

    # ------------------------------------------------------------- scenes
    def preload_file(self, file_path):
        """Load a composite file whose hierarchies keyframe creations name."""
        check(self._lib.gbr_replay_preload_file(self._h, _cstr(str(file_path))))

    def clear_environment(self, env_index):
        check(self._lib.gbr_replay_clear_environment(self._h, int(env_index)))

    def set_environment_keyframe(self, env_index, keyframe):
        """Apply a serialized ``{"keyframe": {...}}`` to the environment."""
        data = _cstr(keyframe)
        check(self._lib.gbr_replay_set_environment_keyframe(self._h, int(env_index), data, len(data)))

    def set_environment_keyframes_batch(self, keyframes, first_env=0, sensor_prefix=None):
        """``set_environment_keyframe(first_env + i, keyframes[i])`` for every
        i in one native call, then, when ``sensor_prefix`` is given,
        ``set_sensor_transforms_from_keyframe`` for each.  Every keyframe is
        parsed before any is applied: a malformed one raises and changes
        nothing."""
        data = [_cstr(k) for k in keyframes]
        n = len(data)
        # One joined buffer and numpy-built pointer/length arrays: building
        # ctypes arrays element by element costs about a microsecond each.
        lens = np.fromiter(map(len, data), np.uint64, n)
        buf = np.frombuffer(b"".join(data), np.uint8) if n else np.zeros(1, np.uint8)
        ptrs = np.zeros(n, np.uint64)
        if n:
            np.cumsum(lens[:-1], out=ptrs[1:])
            ptrs += np.uint64(buf.ctypes.data)
        check(self._lib.gbr_replay_set_environment_keyframes(
            self._h, int(first_env), n, ptrs.ctypes.data_as(ctypes.POINTER(ctypes.c_char_p)),
            lens.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
            None if sensor_prefix is None else _cstr(sensor_prefix)))

    def set_environment_keyframe_unwrapped(self, env_index, keyframe):
        data = _cstr(keyframe)
        check(self._lib.gbr_replay_set_environment_keyframe_unwrapped(self._h, int(env_index), data,
                                                                      len(data)))

    def set_environment_keyframes(self, env_index, keyframes):
        """Give the environment's player a ``{"keyframes": [...]}`` document
        (``Player::readKeyframesFromFile``); apply with
        ``set_environment_keyframe_index``."""
        data = _cstr(keyframes)
        check(self._lib.gbr_replay_set_keyframes(self._h, int(env_index), data, len(data)))

    def set_environment_keyframe_index(self, env_index, index):
        """``Player::setKeyframeIndex``."""
        check(self._lib.gbr_replay_set_keyframe_index(self._h, int(env_index), int(index)))

    def environment_keyframe_count(self, env_index):
        """(number of keyframes, current index) of the environment's player."""
        n, i = ctypes.c_int32(), ctypes.c_int32()
        check(self._lib.gbr_replay_keyframe_count(self._h, int(env_index), ctypes.byref(n),
                                                  ctypes.byref(i)))
        return n.value, i.value

    def user_transform(self, env_index, name):
        """(translation, rotation xyzw) of a user transform, or None."""
        t = np.zeros(3, np.float32)
        q = np.zeros(4, np.float32)
        found = ctypes.c_int32()
        check(self._lib.gbr_replay_user_transform(self._h, int(env_index), _cstr(name),
                                                  t.ctypes.data_as(_lib.c_float_p),
                                                  q.ctypes.data_as(_lib.c_float_p),
                                                  ctypes.byref(found)))
        return (t, q) if found.value else None

    # ------------------------------------------------------------- camera
    def set_sensor_transform(self, env_index, sensor_name, transform):
        """Camera-to-world 4x4 (column-major, ``m[col][row]``)."""
        m = np.ascontiguousarray(np.asarray(transform, np.float32).reshape(4, 4))
        check(self._lib.gbr_replay_set_sensor_transform(self._h, int(env_index), _cstr(sensor_name),
                                                        m.ctypes.data_as(_lib.c_float_p)))

    def set_sensor_transforms_from_keyframe(self, env_index, prefix):
        check(self._lib.gbr_replay_set_sensor_transforms_from_keyframe(self._h, int(env_index),
                                                                       _cstr(prefix)))

    def unproject(self, env_index, viewport_position):
        o = np.zeros(3, np.float32)
        d = np.zeros(3, np.float32)
        check(self._lib.gbr_replay_unproject(self._h, int(env_index), int(viewport_position[0]),
                                             int(viewport_position[1]),
                                             o.ctypes.data_as(_lib.c_float_p),
                                             d.ctypes.data_as(_lib.c_float_p)))
        return Ray(o, d)

    # ------------------------------------------------------------- render
    def render(self, color_images=(), depth_images=(), stream=None):
        """Draw every environment and copy environment i's RGBA8 image to
        ``color_images[i]`` ([h, w, 4] or [h, w, 3] uint8) and its depth in
        metres to ``depth_images[i]`` ([h, w] float32).  Destinations are
        numpy arrays or CUDA torch tensors with contiguous rows; either list
        may be empty.  One packed array per output ([environments, h, w, 4]
        uint8, [environments, h, w] float32) is the fast form: one gather and
        one copy per plane.  Returns when the copies are complete."""
        h, w = self._res
        cptr, crow = self._packed(color_images, (h, w, 4), np.uint8, "color")
        dptr, drow = self._packed(depth_images, (h, w), np.float32, "depth")
        color_images = [] if cptr is not None else list(color_images or ())
        depth_images = [] if dptr is not None else list(depth_images or ())
        rgb_fixups = []
        cptr = cptr if cptr is not None else []
        for i, img in enumerate(color_images):
            ptr, row, channels = self._dst(img, h, w, (3, 4), np.uint8, "color")
            if channels == 3:
                tmp = np.empty((h, w, 4), np.uint8)
                rgb_fixups.append((img, tmp))
                ptr, row = tmp.ctypes.data, tmp.strides[0]
            if i and row != crow:
                raise ValueError("color images must share one row pitch")
            crow = row
            cptr.append(ptr)
        dptr = dptr if dptr is not None else []
        for i, img in enumerate(depth_images):
            ptr, row, _ = self._dst(img, h, w, (1,), np.float32, "depth")
            if i and row != drow:
                raise ValueError("depth images must share one row pitch")
            drow = row
            dptr.append(ptr)
        carr = (ctypes.c_void_p * max(1, len(cptr)))(*cptr)
        darr = (ctypes.c_void_p * max(1, len(dptr)))(*dptr)
        s = None
        if stream is not None:
            s = stream if isinstance(stream, int) else getattr(stream, "cuda_stream", None)
        check(self._lib.gbr_replay_render(self._h, s, len(cptr), carr, crow, len(dptr), darr, drow))
        for img, tmp in rgb_fixups:
            img[...] = tmp[..., :3]

    def _packed(self, images, shape, dtype, what):
        """Pointers of every environment's image when `images` is one packed
        [environments, ...] array or tensor (validated once), else (None, 0)."""
        if images is None or isinstance(images, (list, tuple)) or getattr(images, "ndim", 0) != len(shape) + 1:
            return None, 0
        if images.shape[0] != self._n:
            raise ValueError(f"expected {self._n} {what} images, got {images.shape[0]}")
        ptr, row, _ = self._dst(images[0], *shape[:2], (shape[2] if len(shape) == 3 else 1,), dtype, what)
        if hasattr(images, "data_ptr"):
            contiguous, base, step = images.is_contiguous(), images.data_ptr(), images.stride(0) * images.element_size()
        else:
            contiguous, base, step = images.flags.c_contiguous, images.ctypes.data, images.strides[0]
        if not contiguous:
            raise ValueError(f"packed {what} images must be contiguous")
        return [base + i * step for i in range(self._n)], row

    @staticmethod
    def _dst(img, h, w, channels, dtype, what):
        if hasattr(img, "data_ptr"):          # torch tensor
            import torch
            want = torch.uint8 if dtype == np.uint8 else torch.float32
            if img.dtype != want or not img.is_cuda:
                raise ValueError(f"{what} tensor must be a CUDA {want} tensor")
            shape = tuple(img.shape)
            ch = shape[2] if len(shape) == 3 else 1
            if shape[:2] != (h, w) or ch not in channels or ch == 3:
                raise ValueError(f"{what} tensor must be [{h}, {w}{', 4' if dtype == np.uint8 else ''}]")
            if img.stride(-1) != 1 or (len(shape) == 3 and img.stride(1) != ch):
                raise ValueError(f"{what} tensor rows must be contiguous")
            return img.data_ptr(), img.stride(0) * img.element_size(), ch
        a = img
        if not isinstance(a, np.ndarray) or a.dtype != dtype:
            raise ValueError(f"{what} image must be a {np.dtype(dtype).name} array")
        ch = a.shape[2] if a.ndim == 3 else 1
        if a.shape[:2] != (h, w) or ch not in channels:
            raise ValueError(f"{what} image must be [{h}, {w}] with {channels} channels")
        if not a.flags.writeable or a.strides[-1] != a.itemsize or (a.ndim == 3 and a.strides[1] != ch * a.itemsize):
            raise ValueError(f"{what} image rows must be contiguous and writeable")
        return a.ctypes.data, a.strides[0], ch

    # ------------------------------------------------------- device views
    def cuda_color_buffer_device_pointer(self):
        """Device address of the colour plane (the whole tiled framebuffer)."""
        return self.renderer.colorCudaBufferDevicePointer()

    def cuda_depth_buffer_device_pointer(self):
        """Device address of the depth plane (window depth)."""
        return self.renderer.depthCudaBufferDevicePointer()

    def color_tensor(self):
        """[grid_h * h, grid_w * w, 4] uint8 CUDA tensor of the framebuffer."""
        return self.renderer.colorTensor()

    def depth_tensor(self):
        """[grid_h * h, grid_w * w] float32 CUDA tensor, metres (0 = nothing)."""
        return self.renderer.linearDepthTensor()

    def environment_view(self, tensor, env_index):
        """Environment i's [h, w, ...] block of a framebuffer tensor."""
        h, w = self._res
        gx = self._grid[0]
        x, y = (env_index % gx) * w, (env_index // gx) * h
        return tensor[y:y + h, x:x + w]

    def debug_line_render(self, env_index=0):
        raise NotImplementedError("debug line rendering is not part of the batch renderer")


# ----------------------------------------------------------------- keyframes
class Keyframe:
    """Builds the JSON of a gfx-replay keyframe as ``Recorder`` serializes it
    (io/JsonEspTypes.cpp:12-99): asset loads, instance creations, deletions,
    state updates, metadata, user transforms and light setups.  Rotations are
    quaternions given as (x, y, z, w); the JSON stores [w, x, y, z]."""

    def __init__(self):
        self.loads = []
        self.creations = []
        self.deletions = []
        self.state_updates = []
        self.metadata = []
        self.user_transforms = []
        self.lights = None

    def load(self, filepath, up=(0, 1, 0), front=(0, 0, -1), origin=(0, 0, 0), type=0):
        self.loads.append({"type": type, "filepath": filepath,
                           "frame": {"up": list(up), "front": list(front), "origin": list(origin)},
                           "virtualUnitToMeters": 1.0, "forceFlatShading": True,
                           "splitInstanceMesh": True, "shaderTypeToUse": "material",
                           "overridePhongMaterial": None, "hasSemanticTextures": False})
        return self

    def create(self, instance_key, filepath, scale=None, is_static=False, is_rgbd=True,
               is_semantic=True):
        c = {"filepath": filepath, "isStatic": is_static, "isRGBD": is_rgbd,
             "isSemantic": is_semantic, "isTextureSemantic": False, "lightSetupKey": "",
             "rigId": -1}
        if scale is not None:
            c["scale"] = [float(v) for v in scale]
        self.creations.append({"instanceKey": int(instance_key), "creation": c})
        return self

    def delete(self, instance_key):
        self.deletions.append(int(instance_key))
        return self

    def update(self, instance_key, translation, rotation=(0, 0, 0, 1)):
        self.state_updates.append({"instanceKey": int(instance_key),
                                   "state": {"absTransform": _transform(translation, rotation)}})
        return self

    def set_metadata(self, instance_key, object_id, semantic_id):
        self.metadata.append({"instanceKey": int(instance_key),
                              "metadata": {"objectId": int(object_id), "semanticId": int(semantic_id)}})
        return self

    def user_transform(self, name, translation, rotation=(0, 0, 0, 1)):
        self.user_transforms.append({"name": name, "transform": _transform(translation, rotation)})
        return self

    def set_lights(self, lights):
        """lights: [(vector4, color3)], vector w = 0 directional, 1 point."""
        self.lights = [{"vector": [float(v) for v in vec], "color": [float(c) for c in col],
                        "model": "global"} for vec, col in lights]
        return self

    def to_dict(self):
        d = {"loads": self.loads}
        if self.creations:
            d["creations"] = self.creations
        d["deletions"] = self.deletions
        if self.state_updates:
            d["stateUpdates"] = self.state_updates
        if self.metadata:
            d["metadata"] = self.metadata
        if self.user_transforms:
            d["userTransforms"] = self.user_transforms
        if self.lights is not None:
            d["lightsChanged"] = True
            d["lights"] = self.lights
        return d

    def to_string(self):
        """``Recorder::keyframeToString``: {"keyframe": {...}}."""
        return json.dumps({"keyframe": self.to_dict()})


def keyframes_to_string(keyframes):
    """A {"keyframes": [...]} document (``Recorder::writeSavedKeyframesToString``)."""
    return json.dumps({"keyframes": [k.to_dict() for k in keyframes]})


def _transform(translation, rotation):
    x, y, z, w = (float(v) for v in rotation)
    return {"translation": [float(v) for v in translation], "rotation": [w, x, y, z]}


def quaternion_axis_angle(axis, degrees):
    """Unit quaternion (x, y, z, w) rotating by `degrees` about `axis`."""
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    h = math.radians(degrees) / 2.0
    s = math.sin(h)
    return (float(a[0] * s), float(a[1] * s), float(a[2] * s), float(math.cos(h)))
