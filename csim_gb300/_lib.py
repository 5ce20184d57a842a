"""ctypes binding of libcsimgpu.so (the C ABI declared in include/csimgpu.h).

The library is the only compute path: importing this module fails loudly if
the shared object is missing, and every call raises CsgError on a non-zero
status. There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcsimgpu.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "csimgpu.h")

P = C.c_void_p
I = C.c_int
D = C.c_double
SZ = C.c_size_t
U64 = C.c_uint64

CSG_LAYOUT_COLMAJOR = 0
CSG_LAYOUT_ROWMAJOR = 1
CSG_PREC_BF16X6 = 6
CSG_PREC_BF16X3 = 3
CSG_PREC_HIGH = 16

STATUS = {0: "CSG_OK", -1: "CSG_E_ARG", -2: "CSG_E_SHAPE", -3: "CSG_E_CUDA", -4: "CSG_E_TIMEOUT",
          -5: "CSG_E_NOMEM", -6: "CSG_E_NAN", -7: "CSG_E_STATE"}


class CsgError(RuntimeError):
    def __init__(self, code: int, fn: str, msg: str):
        super().__init__(f"{fn}: {STATUS.get(code, code)}: {msg}")
        self.code = code


# name -> (argtypes, restype); restype None means "int status"
SIGNATURES = {
    "csg_create": ([C.POINTER(P), I], None),
    "csg_destroy": ([P], None),
    "csg_last_error": ([], C.c_char_p),
    "csg_sync": ([P], None),
    "csg_set_stream": ([P, P], None),
    "csg_set_wait_budget": ([P, C.c_longlong], None),
    "csg_get_stream": ([P], P),
    "csg_alloc": ([P, SZ, C.POINTER(P)], None),
    "csg_free": ([P, P], None),
    "csg_memcpy_h2d": ([P, P, P, SZ], None),
    "csg_memcpy_d2h": ([P, P, P, SZ], None),
    "csg_readout_d2h": ([P, P, P, SZ], None),
    "csg_contrast_curve": ([P, P, I, D, D, D, P, I, P, P], None),
    "csg_fd_jacobian": ([P, P, I, I, I, P, I, D, P], None),
    "csg_memset": ([P, P, I, SZ], None),
    "csg_version": ([], C.c_char_p),
    "csg_launch_count": ([], C.c_ulonglong),
    "csg_profile": ([P, I], None),
    "csg_profile_report": ([P, C.c_char_p, SZ], None),
    "csg_field_upload": ([P, P, I, I, I, I, P, P], None),
    "csg_field_download": ([P, P, I, I, I, P, P, I], None),
    "csg_point_source": ([P, P, I, I, I, D, D, P, P, P], None),
    "csg_mask_real": ([P, P, I, I, I, P, I], None),
    "csg_phase_screen": ([P, P, I, I, I, P, P, D], None),
    "csg_complex_mask": ([P, P, I, I, I, P, P, I, I], None),
    "csg_fft2d": ([P, P, I, I, I], None),
    "csg_fresnel": ([P, P, I, I, P, D, D], None),
    "csg_fresnel_prec": ([P, P, I, I, P, D, D, I], None),
    "csg_fft2d_prec": ([P, P, I, I, I, I], None),
    "csg_mft_create": ([P, C.POINTER(P), I, I, I, I, P, P, P, P, I, P, P, D, I], None),
    "csg_mft_destroy": ([P], None),
    "csg_mft_execute": ([P, P, P, P, I, P, I, P, P], None),
    "csg_mft_execute_lo": ([P, P, P, P, P, I, P], None),
    "csg_mft_workspace_bytes": ([P, I], SZ),
    "csg_hex_mask": ([P, P, P, I, I, P, I, I, P, P, D, I, D, I, P], None),
    "csg_hex_mask_noalloc": ([P, P, P, I, I, P, I, I, P, P, D, I, D, I, P], None),
    "csg_hex_tables": ([P, P, P, I, I, I, D, D, D, I, I, D, D, P, P, P, I], None),
    "csg_chain_create": ([P, C.POINTER(P), I, D, I, P, I], None),
    "csg_chain_destroy": ([P], None),
    "csg_chain_add_mask": ([P, P, I, I], None),
    "csg_chain_add_mirror": ([P, P, D], None),
    "csg_chain_add_fresnel": ([P, D, D], None),
    "csg_chain_add_fresnel_padded": ([P, D, D, D], None),
    "csg_chain_add_complex_mask": ([P, P, P, I, I, I], None),
    "csg_chain_add_fpm_hex": ([P, P, P, I, I, I, D, D, D, D, D, D, I], None),
    "csg_chain_add_fpm_hex_double": ([P, P, P, I, I, I, D, D, D, D, I], None),
    "csg_chain_add_fpm_mask": ([P, P, P, I, I, I, I, D, P, D, D, I, P, P, I], None),
    "csg_chain_set_reference_calibration": ([P, I], None),
    "csg_chain_add_fpm_double_mask": ([P, P, P, I, I, P, D, D, I], None),
    "csg_chain_add_fraunhofer": ([P, I, D, D], None),
    "csg_chain_add_fft_fpm": ([P, I, P, P, I], None),
    "csg_mlp_create": ([P, C.POINTER(P), I, I, P, I, C.c_ulonglong], None),
    "csg_mlp_destroy": ([P], None),
    "csg_de_generate_draw": ([P, I, D, D, I], None),
    "csg_mlp_features": ([P, P, I, P, D, D, D, I, I], None),
    "csg_mlp_set_input": ([P, P, I], None),
    "csg_mlp_forward": ([P, I, P], None),
    "csg_mlp_train_step": ([P, I, P, C.c_float, P], None),
    "csg_mlp_param": ([P, I, C.POINTER(P), C.POINTER(P), C.POINTER(P), C.POINTER(P)], None),
    "csg_chain_response": ([P, I, P, I, P, P], None),
    "csg_chain_batch_buffers": ([P, C.POINTER(P), C.POINTER(P), C.POINTER(P)], None),
    "csg_chain_add_fraunhofer_ragged": ([P, P, D, D], None),
    "csg_mft_create_ragged": ([P, C.POINTER(P), I, I, I, P, P, P, P, P, I, P, P, D, I], None),
    "csg_dm_create": ([P, C.POINTER(P), I, I, D], None),
    "csg_dm_destroy": ([P], None),
    "csg_dm_surface": ([P, P, P], None),
    "csg_chain_set_support_crop": ([P, I], None),
    "csg_chain_set_fft_fpm_babinet": ([P, I], None),
    "csg_chain_fpm_region": ([P, I, C.POINTER(I), C.POINTER(I), C.POINTER(I), C.POINTER(I)], None),
    "csg_chain_set_batch": ([P, I, P, P, P, P, P], None),
    "csg_chain_sags": ([P, I, I, C.POINTER(P)], None),
    "csg_chain_execute": ([P, I, I], None),
    "csg_chain_image": ([P, C.POINTER(P), C.POINTER(I)], None),
    "csg_chain_image_lo": ([P, C.POINTER(P)], None),
    "csg_chain_field": ([P, C.POINTER(P)], None),
    "csg_mft_reserve": ([P, I], None),
    "csg_mft_set_tile": ([P, I], None),
    "csg_mft_tuning": ([P, C.POINTER(I), C.POINTER(C.c_float), C.POINTER(C.c_float)], None),
    "csg_mft_tuning_log": ([C.c_char_p, SZ], None),
    "csg_region_reduce": ([P, P, I, I, I, I, P, I, I, D, P], None),
    "csg_intensity": ([P, P, I, I, I, P, P], None),
    "csg_respobj_create": ([P, C.POINTER(P), P, I, I, I, P, D, D, I], None),
    "csg_respobj_destroy": ([P], None),
    "csg_respobj_execute": ([P, P, I, P], None),
    "csg_de_create": ([P, C.POINTER(P), I, I, U64], None),
    "csg_de_destroy": ([P], None),
    "csg_de_set_bounds": ([P, P, P, P, P], None),
    "csg_de_init": ([P, P, D, I], None),
    "csg_de_buffers": ([P, C.POINTER(P), C.POINTER(P), C.POINTER(P), C.POINTER(P)], None),
    "csg_de_set_trial_buffer": ([P, P], None),
    "csg_de_generate": ([P, I, D, D], None),
    "csg_de_select": ([P, I], None),
    "csg_de_reset_best": ([P], None),
    "csg_de_stats": ([P, P, P, P, P, P], None),
}


def header_symbols() -> list[str]:
    """Every function the public header declares."""
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(csg_\w+)\s*\(", txt, re.M)))


def _load() -> C.CDLL:
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with csim_gb300.build.build() "
                          "(there is no CPU fallback)")
    return C.CDLL(LIB_PATH)


lib = _load()


class _Fn:
    def __init__(self, name: str, argtypes, restype):
        self.name = name
        self.fn = getattr(lib, name)
        self.fn.argtypes = argtypes
        self.status = restype is None
        self.fn.restype = I if restype is None else restype

    def __call__(self, *args):
        r = self.fn(*args)
        if self.status and r != 0:
            msg = lib.csg_last_error()
            raise CsgError(r, self.name, msg.decode() if msg else "")
        return r


lib.csg_last_error.restype = C.c_char_p
lib.csg_last_error.argtypes = []
api = {name: _Fn(name, a, r) for name, (a, r) in SIGNATURES.items() if hasattr(lib, name)}


def call(name: str, *args):
    return api[name](*args)


def version() -> str:
    return api["csg_version"]().decode()
