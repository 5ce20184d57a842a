"""Build and load the oracle's plain-C restatements (gcc, -ffp-contract=off).

TEST INFRASTRUCTURE ONLY. Output goes to _build/oracle/ (git-ignored).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_build", "oracle")
LIB = os.path.join(OUT, "libcsimoracle.so")
SRCS = [os.path.join(HERE, "hexmask.c")]


def build() -> str:
    os.makedirs(OUT, exist_ok=True)
    if os.path.exists(LIB) and all(os.path.getmtime(LIB) > os.path.getmtime(s) for s in SRCS):
        return LIB
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", LIB + ".tmp", *SRCS, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        P = C.c_void_p
        _lib.make_hex_array.argtypes = [P, P, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                        C.c_double, P]
        _lib.make_interpolation_data.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_double,
                                                 C.c_double, C.c_double, P, P, C.c_int]
        _lib.make_interpolation_data.restype = C.c_int
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def hex_design_array(hex_x, hex_y, n_rings, A, fpm_scale_factor, hex_gap, pitch):
    hx = np.ascontiguousarray(hex_x, np.float64)
    hy = np.ascontiguousarray(hex_y, np.float64)
    d = np.empty((A, A), np.int32)
    lib().make_hex_array(_p(hx), _p(hy), hx.size, n_rings, A, fpm_scale_factor, hex_gap, pitch,
                         _p(d))
    return d


def interpolation_tables(design, S, n_sub, pixel_scale, fpm_radius, fpm_scale_factor,
                         stale=False):
    """make_interpolation_data (complexHexMaskFPM.cpp:372-469); stale: the
    reference's row check as its loop runs on one OpenMP thread."""
    design = np.ascontiguousarray(design, np.int32)
    ids = np.empty((3, S, S), np.int16)
    cnt = np.empty((3, S, S), np.uint16)
    over = lib().make_interpolation_data(_p(design), design.shape[0], S, n_sub, pixel_scale,
                                         fpm_radius, fpm_scale_factor, _p(ids), _p(cnt),
                                         int(bool(stale)))
    return ids, cnt, over
