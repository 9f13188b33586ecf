"""Redwood depth-sensor noise on the GPU: habitat-sim's ``RedwoodNoiseModelGPUImpl``
binding (src/esp/bindings/SensorBindings.cpp:293-326) and its Python
``RedwoodDepthNoiseModel`` (src_python/habitat_sim/sensors/noise_models/
redwood_depth_noise_model.py), over the kernel of include/gbr_noise.h.

Beyond the reference: a seed and call counter make the noise reproducible
(``set_state``), and ``simulate_tiles`` / ``apply_to_renderer`` noise every
environment of a batch renderer's linear-depth plane in one launch.
"""
import ctypes
import os

import numpy as np

from . import _lib
from ._lib import check

MODEL_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data",
                          "redwood-depth-dist-model.npy")


def load_model(path=MODEL_PATH):
    """The 80 x 400 float32 distortion table."""
    return np.ascontiguousarray(np.load(path), np.float32)


def normal_quantile_table():
    """The 4097 knots of the normal quantile function the kernel interpolates."""
    out = np.zeros(4097, np.float32)
    check(_lib.load().gbr_normal_quantile_table(out.ctypes.data_as(_lib.c_float_p), out.size))
    return out


class RedwoodNoiseModelGPUImpl:
    """``RedwoodNoiseModelGPUImpl(model, gpu_device_id, noise_multiplier)``."""

    def __init__(self, model, gpu_device_id=0, noise_multiplier=1.0, seed=0):
        m = np.ascontiguousarray(model, np.float32)
        if m.ndim != 2:
            raise ValueError("model must be a 2D array")
        self._lib = _lib.load()
        self._model = m
        h = ctypes.c_void_p()
        check(self._lib.gbr_redwood_noise_create(m.ctypes.data_as(_lib.c_float_p), m.shape[0],
                                                 m.shape[1], int(gpu_device_id),
                                                 float(noise_multiplier), int(seed), ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.gbr_redwood_noise_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, seed, counter=0):
        check(self._lib.gbr_redwood_noise_set_state(self._h, int(seed), int(counter)))

    def get_state(self):
        s, c = ctypes.c_uint64(), ctypes.c_uint64()
        check(self._lib.gbr_redwood_noise_get_state(self._h, ctypes.byref(s), ctypes.byref(c)))
        return s.value, c.value

    def simulate_from_cpu(self, depth):
        d = np.ascontiguousarray(depth, np.float32)
        if d.ndim != 2:
            raise ValueError("depth must be a 2D array")
        out = np.empty_like(d)
        check(self._lib.gbr_redwood_noise_simulate_host(self._h, d.ctypes.data_as(_lib.c_float_p),
                                                        d.shape[0], d.shape[1],
                                                        out.ctypes.data_as(_lib.c_float_p)))
        return out

    def simulate_from_gpu(self, dev_depth, rows, cols, dev_noisy_depth, stream=None):
        check(self._lib.gbr_redwood_noise_simulate_device(self._h, int(dev_depth), int(rows),
                                                          int(cols), int(dev_noisy_depth), stream))

    def simulate_tiles(self, src, dst, pitch, tile_w, tile_h, tiles_x, count, stream=None):
        """`count` images as tiles of a plane (device addresses, pitch in floats)."""
        check(self._lib.gbr_redwood_noise_simulate_tiles(self._h, int(src), int(dst), int(pitch),
                                                         int(tile_w), int(tile_h), int(tiles_x),
                                                         int(count), stream))

    def simulate_images(self, src, dst, layout, stream=None):
        """Images at any places of a plane (device addresses): `layout` holds
        one (offset, pitch, width, height) per image, in floats."""
        lay = np.ascontiguousarray(layout, np.int64).reshape(-1, 4)
        check(self._lib.gbr_redwood_noise_simulate_images(
            self._h, int(src), int(dst), lay.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
            int(lay.shape[0]), stream))

    def apply_to_renderer(self, renderer, out=None, stream=None):
        """Noise every scene of a ``RendererStandalone``'s linear-depth plane
        (tile grid or ragged layout) into `out` (a CUDA float32 tensor of the
        plane's shape, allocated if None; only the scenes' pixels are
        written), on `stream` (torch's current stream if None).  Scene i is
        image i of the batch."""
        import torch
        src = renderer.linearDepthTensor()
        if out is None:
            out = torch.empty_like(src)
        if out.shape != src.shape or out.dtype != torch.float32 or not out.is_contiguous():
            raise ValueError("out must be a contiguous float32 tensor of the plane's shape")
        s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        if src.dim() == 2 and not renderer._config.viewports:
            (tw, th), (tx, ty) = renderer.tileSize(), renderer.tileCount()
            self.simulate_tiles(src.data_ptr(), out.data_ptr(), src.shape[1], tw, th, tx,
                                renderer.sceneCount(), s)
        else:
            self.simulate_images(src.data_ptr(), out.data_ptr(), renderer.sceneViewports(), s)
        return out


class RedwoodDepthNoiseModel:
    """``RedwoodDepthNoiseModel`` (noise_multiplier, gpu_device_id): call it or
    ``simulate`` on a numpy array (host round trip) or a CUDA torch tensor."""

    def __init__(self, noise_multiplier=1.0, gpu_device_id=0, model=None, seed=0):
        self.noise_multiplier = float(noise_multiplier)
        self.gpu_device_id = int(gpu_device_id)
        self._impl = RedwoodNoiseModelGPUImpl(load_model() if model is None else model,
                                              self.gpu_device_id, self.noise_multiplier, seed)

    @staticmethod
    def is_valid_sensor_type(sensor_type):
        return str(sensor_type).lower().endswith("depth")

    def simulate(self, gt_depth):
        if isinstance(gt_depth, np.ndarray):
            return self._impl.simulate_from_cpu(gt_depth)
        import torch
        if gt_depth.dtype != torch.float32 or gt_depth.dim() != 2 or not gt_depth.is_contiguous():
            raise ValueError("depth must be a contiguous 2D float32 tensor")
        noisy = torch.empty_like(gt_depth)
        rows, cols = gt_depth.shape
        self._impl.simulate_from_gpu(gt_depth.data_ptr(), rows, cols, noisy.data_ptr(),
                                     torch.cuda.current_stream().cuda_stream)
        return noisy

    def __call__(self, gt_depth):
        return self.simulate(gt_depth)
