"""Seeded synthetic scenes for the tests, the benchmark and the smoke check.

``libjsbscene.so`` (built here from ``scene_build.cpp`` and the SoftBodySharedSettings mirror in
``shared_settings.cpp``) writes a scene's colliders, creation settings and every body's settings
bytes, byte-identical to what Jolt's own CreateConstraints / Optimize / SaveBinaryState write for the
same scene. It is test and benchmark infrastructure: the product library ``libjsb.so`` takes settings
bytes from its caller and never builds scenes itself.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libjsbscene.so")
SOURCES = [os.path.join(HERE, f) for f in ("scene_build.cpp", "shared_settings.cpp")]
HEADERS = [os.path.join(HERE, f) for f in ("scene_io.h", "scene_spec.h", "shared_settings.h", "fmath.h")]

_lib = None


def build() -> str:
    """Compiles libjsbscene.so (host C++ only; -ffp-contract=off like the reference's deterministic build)."""
    deps = SOURCES + HEADERS
    if not os.path.exists(LIB) or any(os.path.getmtime(d) > os.path.getmtime(LIB) for d in deps):
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared"] + SOURCES + ["-o", LIB],
                       check=True)
    return LIB


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.scene_build.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_size_t,
                                  ctypes.POINTER(ctypes.c_size_t)]
        L.scene_build.restype = ctypes.c_int
        L.scene_last_error.restype = ctypes.c_char_p
        _lib = L
    return _lib


def build_scene(name: str, **params) -> bytes:
    """Serialised seeded scene ("JSBS", see scene_io.h): colliders, and per body its position, creation
    settings, force and SaveBinaryState bytes."""
    L = lib()
    p = " ".join(f"{k}={v}" for k, v in params.items()).encode()
    n = ctypes.c_size_t(0)
    if L.scene_build(name.encode(), p, None, 0, ctypes.byref(n)) != 0:
        raise ValueError(L.scene_last_error().decode())
    buf = ctypes.create_string_buffer(n.value)
    if L.scene_build(name.encode(), p, buf, n.value, ctypes.byref(n)) != 0:
        raise ValueError(L.scene_last_error().decode())
    return buf.raw[: n.value]
