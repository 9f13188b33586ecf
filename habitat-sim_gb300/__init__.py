"""GB300-native batch renderer: a drop-in for habitat-sim's
``esp::gfx_batch`` draw path (C ABI in ``include/gbr.h``, CUDA kernels for
sm_103a in ``csrc/``), and the batch replay renderer driven by gfx-replay
keyframes (C ABI in ``include/gbr_replay.h``), and the Redwood depth-sensor
noise model on the GPU (``include/gbr_noise.h``)."""
from .gfx_batch import (DrawMode, GbrError, HbaoConfiguration, HbaoType, Plane, RendererConfiguration, RendererFileFlags,
                        RendererFlags, RendererLightType, RendererStandalone,
                        RendererStandaloneConfiguration, RendererStandaloneFlags, SceneStats,
                        calculateDepthUnprojection, hbaoApply, unprojectDepth,
                        unprojectDepthDevice)
from .noise import RedwoodDepthNoiseModel, RedwoodNoiseModelGPUImpl
from .replay import (CameraSensorSpec, Keyframe, Ray, ReplayRenderer, ReplayRendererConfiguration,
                     SensorSubType, keyframes_to_string)

__all__ = ["DrawMode", "GbrError", "HbaoConfiguration", "HbaoType", "hbaoApply", "Plane", "RendererConfiguration", "RendererFileFlags",
           "RendererFlags", "RendererLightType", "RendererStandalone",
           "RendererStandaloneConfiguration", "RendererStandaloneFlags", "SceneStats",
           "calculateDepthUnprojection", "unprojectDepth", "unprojectDepthDevice",
           "CameraSensorSpec", "Keyframe", "Ray", "ReplayRenderer", "ReplayRendererConfiguration",
           "SensorSubType", "keyframes_to_string", "RedwoodDepthNoiseModel",
           "RedwoodNoiseModelGPUImpl"]
