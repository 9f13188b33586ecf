"""GB300-native batch renderer: a drop-in for habitat-sim's
``esp::gfx_batch`` draw path (C ABI in ``include/gbr.h``, CUDA kernels for
sm_103a in ``csrc/``)."""
from .gfx_batch import (DrawMode, GbrError, Plane, RendererConfiguration, RendererFileFlags,
                        RendererFlags, RendererLightType, RendererStandalone,
                        RendererStandaloneConfiguration, RendererStandaloneFlags, SceneStats,
                        calculateDepthUnprojection, unprojectDepth, unprojectDepthDevice)

__all__ = ["DrawMode", "GbrError", "Plane", "RendererConfiguration", "RendererFileFlags",
           "RendererFlags", "RendererLightType", "RendererStandalone",
           "RendererStandaloneConfiguration", "RendererStandaloneFlags", "SceneStats",
           "calculateDepthUnprojection", "unprojectDepth", "unprojectDepthDevice"]
