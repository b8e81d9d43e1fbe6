"""wgpu_gb300 — host side of the GB300 render-pass path (a drop-in for wgpu-cpu's render-pass
hot path).  The device work runs in libgbr.so (CUDA, sm_103a) behind the C ABI of
include/gbr.h; this package mirrors the wgpu API on top of it."""

from .api import *  # noqa: F401,F403
from .api import Device, GbrError, gpu_lib  # noqa: F401
from . import workloads  # noqa: F401

__all__ = [n for n in dir() if not n.startswith("_")]
