"""ctypes binding of libcpt.so (include/cpt.h).

The library is built in-tree by cudapathtracing_gb300/build.py.  Loading fails loudly when
it is missing: there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libcpt.so")

_lib = None


class CptError(RuntimeError):
    def __init__(self, status: int, where: str, message: str):
        self.status = status
        super().__init__(f"{where}: {abi.STATUS_NAMES.get(status, status)}: {message}")


def lib():
    """The loaded libcpt.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"libcpt.so is not built ({LIB_PATH}); run __graft_entry__.build() "
                              "or python cudapathtracing_gb300/build.py")
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        S = C.c_int
        sigs = {
            "cpt_abi_version": (C.c_int, []),
            "cpt_launch_count": (C.c_uint64, []),
            "cpt_last_error_string": (C.c_char_p, []),
            "cpt_context_create": (S, [C.c_int, C.POINTER(P)]),
            "cpt_context_destroy": (S, [P]),
            "cpt_context_set_render_block": (S, [P, C.c_int, C.c_int]),
            "cpt_context_set_wavefront": (S, [P, C.c_int, C.c_int, C.c_int, C.c_int]),
            "cpt_context_set_bvh_width": (S, [P, C.c_int]),
            "cpt_context_set_short_stack": (S, [P, C.c_int]),
            "cpt_context_set_loop_limits": (S, [P, C.c_int32, C.c_int32]),
            "cpt_context_set_material_sort": (S, [P, C.c_int]),
            "cpt_context_set_bvh_compression": (S, [P, C.c_int]),
            "cpt_filter_bilateral": (S, [P, P, P, P, C.c_int32, C.c_int32, C.POINTER(abi.cpt_filter_params), P]),
            "cpt_pick": (S, [P, C.c_int32, C.c_int32, C.POINTER(C.c_int32)]),
            "cpt_scene_set_material": (S, [P, C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_int32]),
            "cpt_denoiser_create": (S, [C.c_int, C.c_uint64, C.POINTER(P)]),
            "cpt_denoiser_destroy": (S, [P]),
            "cpt_denoiser_num_params": (C.c_uint64, [P]),
            "cpt_denoiser_get_params": (S, [P, P]),
            "cpt_denoiser_set_params": (S, [P, P]),
            "cpt_denoiser_get_grads": (S, [P, P]),
            "cpt_denoiser_export": (S, [P, C.c_char_p, P, C.c_uint64, C.POINTER(C.c_uint64)]),
            "cpt_denoiser_train_step": (S, [P, C.c_int32, C.c_int32, C.c_int32, P, P, P, C.c_float, C.c_int32,
                                            C.POINTER(C.c_float), P]),
            "cpt_denoise": (S, [P, C.c_int32, C.c_int32, C.c_int32, P, P, P, P]),
            "cpt_denoiser_set_backend": (S, [P, C.c_int32]),
            "cpt_denoiser_check": (S, [P]),
            "cpt_denoiser_wait_selftest": (S, [P]),
            "cpt_filter_temporal": (S, [P, P, P, P, C.POINTER(abi.cpt_camera), C.POINTER(abi.cpt_camera), C.c_float, P]),
            "cpt_ini_load": (S, [C.c_char_p, C.POINTER(P)]),
            "cpt_ini_describe": (S, [P, C.POINTER(abi.cpt_scene_desc)]),
            "cpt_ini_free": (S, [P]),
            "cpt_scene_create": (S, [P, C.POINTER(abi.cpt_scene_desc), C.POINTER(P)]),
            "cpt_scene_load_ini": (S, [P, C.c_char_p, C.POINTER(P)]),
            "cpt_scene_destroy": (S, [P]),
            "cpt_scene_info": (S, [P, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                   C.POINTER(abi.cpt_camera)]),
            "cpt_scene_update_triangles": (S, [P, P, C.c_uint32, C.c_uint32, P]),
            "cpt_lbvh_build": (S, [P, P, C.POINTER(abi.cpt_bvh_stats)]),
            "cpt_lbvh_refit": (S, [P, P, C.POINTER(abi.cpt_bvh_stats)]),
            "cpt_lbvh_export": (S, [P, P, P, P, P, P, P]),
            "cpt_lbvh_scratch_bytes": (C.c_size_t, [C.c_uint32]),
            "cpt_lbvh_build_device": (S, [C.c_uint32, P, P, C.c_uint32, P, C.POINTER(C.c_double),
                                          C.POINTER(C.c_double), P, P, P, P, P, P, P, C.c_size_t, P]),
            "cpt_trace_closest": (S, [P, P, C.c_uint64, P, C.c_int, P]),
            "cpt_render": (S, [P, C.POINTER(abi.cpt_render_params), C.POINTER(abi.cpt_render_output), P,
                               C.POINTER(abi.cpt_render_stats)]),
            "cpt_render_batch": (S, [P, C.POINTER(abi.cpt_render_job), C.c_uint32, P, C.POINTER(abi.cpt_render_stats)]),
        }
        for name, (res, args) in sigs.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status: int, where: str) -> None:
    if status != abi.CPT_OK:
        msg = lib().cpt_last_error_string()
        raise CptError(status, where, msg.decode() if msg else "")


def declared_symbols(header: str | None = None) -> list[str]:
    """Names of the functions include/cpt.h declares."""
    import re
    header = header or os.path.join(os.path.dirname(HERE), "include", "cpt.h")
    text = open(header).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\*?\s+\*?(cpt_[a-z_0-9]+)\(", text, re.M)))
