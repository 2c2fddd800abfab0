"""GB300-native (sm_103a) back-end for SoftGLRender's software rendering pipeline.

`RendererCUDA()` returns a renderer with the reference's `Renderer` interface
(src/Render/Renderer.h:24-59) backed by the CUDA library built from csrc/ (see build.py). There is
no CPU fallback: if the library has not been built, or no GPU is visible, construction raises.
"""
from __future__ import annotations

import ctypes
import os

from . import api
from .api import *  # noqa: F401,F403  (reference enums and value types)

HERE = os.path.dirname(os.path.abspath(__file__))
LIBRARY_PATH = os.path.join(HERE, "_build", "libsoftgl_cuda.so")
_LIB = None


def load_library() -> "api.Library":
    """Load the CUDA library (once). Raises if it has not been built."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIBRARY_PATH):
            raise RuntimeError(f"softglrender_gb300 CUDA library missing at {LIBRARY_PATH}; "
                               "run `python -m softglrender_gb300.build` (there is no CPU fallback)")
        _LIB = api.Library(ctypes.CDLL(LIBRARY_PATH), "sglc_")
    return _LIB


def RendererCUDA(device: int = 0) -> "api.Renderer":
    """The sm_103a renderer on `device`."""
    return api.Renderer(load_library(), device)
