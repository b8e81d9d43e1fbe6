"""Loader for the oracle (oracle/_build/liborc.so): the CPU restatement of wgpu-cpu's
render-pass path used as the checker.  Builds it with `make -C oracle` when missing."""

import ctypes
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "oracle", "_build", "liborc.so")

_lib = None


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            subprocess.run(["make", "-C", os.path.join(ROOT, "oracle")], check=True,
                           stdout=subprocess.DEVNULL)
        _lib = ctypes.CDLL(LIB)
        _lib.orc_kat_f16_to_f32.restype = ctypes.c_float
        _lib.orc_kat_f16_to_f32.argtypes = [ctypes.c_uint16]
        _lib.orc_kat_f32_to_f16.restype = ctypes.c_uint16
        _lib.orc_kat_f32_to_f16.argtypes = [ctypes.c_float]
        _lib.orc_kat_texture_byte_size.restype = ctypes.c_uint64
        _lib.orc_kat_texture_byte_size.argtypes = [ctypes.c_uint32] * 4
        _lib.orc_set_threads.argtypes = [ctypes.c_int]
    return _lib
