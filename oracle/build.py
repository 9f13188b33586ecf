"""Build recipe for the CPU oracle library (test infrastructure).

``g++ -O3 -ffp-contract=off`` keeps every float operation separately
rounded unless the source spells out ``std::fmaf``; the same rule holds on
x86-64 and on aarch64 (where GCC would otherwise contract to FMA)."""
import ctypes
import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, f"liboracle.{platform.machine()}.so")
SRC = os.path.join(HERE, "raster.cpp")

_lib = None


def build(force=False):
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    subprocess.check_call(["g++", "-O3", "-ffp-contract=off", "-fno-fast-math", "-std=c++17",
                           "-fPIC", "-shared", "-pthread", SRC, "-o", tmp])
    os.replace(tmp, LIB)
    return LIB


def load_library():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB)
        lib.oracle_render.restype = ctypes.c_int
        lib.oracle_unproject_depth.restype = None
        lib.oracle_unproject_depth.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                               ctypes.c_int64, ctypes.c_int64]
        _lib = lib
    return _lib
