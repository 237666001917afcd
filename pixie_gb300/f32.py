"""float32 scalar arithmetic with the C library's single-precision functions.

pixie computes path geometry in Nim ``float32``: ``+ - * /`` are IEEE single
precision and ``sin``/``cos``/``tan``/``arccos``/``sqrt``/``pow`` on float32
call the C library's ``sinf``/``cosf``/``tanf``/``acosf``/``sqrtf``/``powf``.
Python floats are doubles, so every builder in :mod:`pixie_gb300.paths` routes
its arithmetic through these helpers to produce the same float32 command
values as the reference.
"""
from __future__ import annotations

import ctypes
import ctypes.util
import struct

_libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
for _name in ("sinf", "cosf", "tanf", "acosf", "asinf", "sqrtf", "fmodf", "roundf", "floorf",
              "ceilf", "truncf", "atan2f"):
    _fn = getattr(_libm, _name)
    _fn.restype = ctypes.c_float
    _fn.argtypes = [ctypes.c_float] * (2 if _name in ("fmodf", "atan2f") else 1)
_libm.powf.restype = ctypes.c_float
_libm.powf.argtypes = [ctypes.c_float, ctypes.c_float]

_pack = struct.Struct("<f")


def f32(x: float) -> float:
    """Round a double to the nearest float32 (returned as a Python float)."""
    return _pack.unpack(_pack.pack(x))[0]


def add(a, b):
    return f32(a + b)


def sub(a, b):
    return f32(a - b)


def mul(a, b):
    return f32(a * b)


def div(a, b):
    if b == 0.0:
        if a == 0.0 or a != a:
            return float("nan")
        neg = (a < 0) != (str(b)[0] == "-")
        return float("-inf") if neg else float("inf")
    return f32(a / b)


def sin(x):
    return _libm.sinf(x)


def cos(x):
    return _libm.cosf(x)


def tan(x):
    return _libm.tanf(x)


def acos(x):
    return _libm.acosf(x)


def sqrt(x):
    return _libm.sqrtf(x)


def fmod(a, b):
    return _libm.fmodf(a, b)


PI = f32(3.141592653589793)       # Nim's PI where it meets float32 operands
TAU = f32(2 * 3.141592653589793)
EPSILON = f32(0.0001 * 3.141592653589793)  # paths.nim:44
