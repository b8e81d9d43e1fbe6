"""The oracle as a device: the same host API (wgpu_gb300.api.Device) bound to liborc.so's
`orc_` symbols.  Test infrastructure only."""

import ctypes

import oracle_lib
from wgpu_gb300 import _abi
from wgpu_gb300.api import Device, Profile

_abi_lib = None


def lib() -> _abi.Lib:
    global _abi_lib
    if _abi_lib is None:
        _abi_lib = _abi.Lib(oracle_lib.load(), "orc_")
    return _abi_lib


def device(profile: int = Profile.PARITY, threads: int = 1, raster_rule: int = 0) -> Device:
    oracle_lib.load().orc_set_threads(threads)
    return Device(lib=lib(), profile=profile, raster_rule=raster_rule)
