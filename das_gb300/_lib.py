"""ctypes binding of libwave2d_cuda.so (C ABI declared in include/wave2d_cuda.h).

The library is built in-tree by ``das_gb300.build``.  Loading fails loudly: there
is no CPU fallback on the product path.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

_LIB = None
_LOCK = threading.Lock()

c_int, c_float, c_void_p = ctypes.c_int, ctypes.c_float, ctypes.c_void_p
c_ll, c_ull = ctypes.c_longlong, ctypes.c_ulonglong


class W2DError(RuntimeError):
    """A non-zero status from the CUDA engine."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"wave2d_cuda error {code}: {msg}")
        self.code = code


# name -> (restype, argtypes)
_SIGS = {
    # reference-compatible symbols (wave2d.c)
    "acoustic_2d_step": (None, [c_void_p] * 5 + [c_int, c_int, c_float, c_float, c_float, c_int]),
    "elastic_2d_step": (None, [c_void_p] * 10 + [c_int, c_int, c_float, c_float, c_float, c_int]),
    "correlate_imaging_condition": (None, [c_void_p] * 3 + [c_int, c_int, c_float]),
    "build_cerjan_sponge": (None, [c_void_p, c_int, c_int, c_int, c_float, c_int]),
    "w2d_acoustic_2d_step_status": (c_int, [c_void_p] * 5 + [c_int, c_int, c_float, c_float,
                                                              c_float, c_int]),
    "w2d_elastic_2d_step_status": (c_int, [c_void_p] * 10 + [c_int, c_int, c_float, c_float,
                                                              c_float, c_int]),
    "w2d_correlate_status": (c_int, [c_void_p] * 3 + [c_int, c_int, c_float]),
    # engine
    "w2d_last_error": (ctypes.c_char_p, []),
    "w2d_version": (c_int, []),
    "w2d_sponge_lut": (c_int, [c_void_p, c_int, c_float]),
    "w2d_engine_create": (c_int, [ctypes.POINTER(c_void_p), c_int, c_int, c_float, c_float,
                                  ctypes.c_double, c_void_p, c_int]),
    "w2d_engine_destroy": (None, [c_void_p]),
    "w2d_engine_set_velocity": (c_int, [c_void_p, c_int, c_void_p]),
    "w2d_engine_set_tile": (c_int, [c_void_p, c_int, c_int]),
    "w2d_engine_set_memory_budget": (c_int, [c_void_p, c_ull]),
    "w2d_engine_set_l2_hints": (c_int, [c_void_p, c_int]),
    "w2d_engine_set_launch": (c_int, [c_void_p, c_int, c_int]),
    "w2d_engine_set_two_step": (c_int, [c_void_p, c_int]),
    "w2d_engine_set_graphs": (c_int, [c_void_p, c_int]),
    "w2d_forward": (c_int, [c_void_p, c_int, c_void_p, c_int, c_int, c_int, c_void_p, c_int, c_int,
                            c_void_p, c_void_p, c_int]),
    "w2d_backward_correlate": (c_int, [c_void_p, c_int, c_void_p, c_int, c_void_p, c_int, c_int,
                                       c_void_p, c_int, c_void_p, c_int]),
    "w2d_migrate_shot": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_void_p, c_void_p,
                                 c_int, c_int, c_int, c_int, c_void_p, c_void_p]),
    "w2d_stack_reset": (c_int, [c_void_p]),
    "w2d_stack_read": (c_int, [c_void_p, c_void_p, c_void_p]),
    "w2d_stack_add": (c_int, [c_void_p, c_void_p, c_void_p]),
    "w2d_device_memory": (c_int, [ctypes.POINTER(c_ull), ctypes.POINTER(c_ull)]),
    "w2d_post_stack": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_void_p]),
    "w2d_shot_stage": (c_int, [c_void_p, c_int, c_void_p, c_int, c_void_p, c_int]),
    "w2d_migrate_staged": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_int, c_int, c_int,
                                   c_int, c_void_p, c_void_p]),
    "w2d_engine_timer_start": (c_int, [c_void_p]),
    "w2d_engine_timer_stop": (c_int, [c_void_p, ctypes.POINTER(c_float)]),
    "w2d_set_device": (c_int, [c_int]),
    "w2d_device_pci_bus_id": (c_int, [ctypes.c_char_p, c_int]),
    "w2d_host_alloc": (c_int, [ctypes.POINTER(c_void_p), c_ull]),
    "w2d_host_free": (None, [c_void_p]),
    "w2d_fwi_forward": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_void_p, c_int,
                                c_int, c_void_p]),
    "w2d_fwi_gradient": (c_int, [c_void_p, c_void_p, c_void_p]),
    "w2d_fwi_set_segment": (c_int, [c_void_p, c_int]),
    "w2d_fwi_set_adjoint_form": (c_int, [c_void_p, c_int]),
    "w2d_flood_models": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_int, ctypes.c_double,
                                 ctypes.c_double, c_void_p, c_void_p, c_void_p, c_void_p]),
    "w2d_engine_synchronize": (c_int, [c_void_p]),
    "w2d_elastic_create": (c_int, [ctypes.POINTER(c_void_p), c_int, c_int, c_float, c_float,
                                   ctypes.c_double, c_int, c_float, c_int]),
    "w2d_elastic_destroy": (None, [c_void_p]),
    "w2d_elastic_forward": (c_int, [c_void_p] * 6 + [c_int, c_int, c_int, c_void_p, c_int, c_int,
                                                      c_void_p]),
    "w2d_elastic_gradient": (c_int, [c_void_p] * 6),
    "w2d_elastic_last_ms": (c_float, [c_void_p]),
    "w2d_elastic_forward_batch": (c_int, [c_void_p, c_int] + [c_void_p] * 5 + [c_int, c_void_p,
                                                                              c_void_p, c_void_p,
                                                                              c_int, c_int,
                                                                              c_void_p]),
    "w2d_elastic_gradient_batch": (c_int, [c_void_p] * 6),
    "w2d_elastic_shot_bytes": (c_ull, [c_int, c_int, c_int, c_int]),
    "w2d_elastic_set_adjoint": (c_int, [c_void_p, c_int]),
    "w2d_elastic_set_tiles": (c_int, [c_void_p, c_int, c_int, c_int, c_int]),
    "w2d_elastic_set_pdl": (c_int, [c_void_p, c_int]),
    "w2d_elastic_share_model": (c_int, [c_void_p, c_int]),
    "w2d_batch_create": (c_int, [ctypes.POINTER(c_void_p), c_ull, c_int]),
    "w2d_batch_destroy": (None, [c_void_p]),
    "w2d_batch_set_config": (c_int, [c_void_p, c_int, c_int, c_int, c_int]),
    "w2d_batch_set_form": (c_int, [c_void_p, c_int]),
    "w2d_batch_shot_bytes": (c_ull, [c_void_p]),
    "w2d_batch_free_bytes": (c_ull, [c_void_p]),
    "w2d_batch_submit": (c_int, [c_void_p, c_void_p, ctypes.POINTER(c_int)]),
    "w2d_batch_model_bytes": (c_ull, [c_void_p]),
    "w2d_batch_submit_modelling": (c_int, [c_void_p, c_void_p, ctypes.POINTER(c_int)]),
    "w2d_batch_fetch_traces": (c_int, [c_void_p, c_int, c_void_p]),
    "w2d_batch_step": (c_int, [c_void_p, ctypes.POINTER(c_int)]),
    "w2d_batch_launch": (c_int, [c_void_p]),
    "w2d_batch_wait": (c_int, [c_void_p, ctypes.POINTER(c_int)]),
    "w2d_batch_is_finished": (c_int, [c_void_p, c_int]),
    "w2d_batch_fetch": (c_int, [c_void_p, c_int, c_void_p, c_void_p]),
    "w2d_batch_cancel": (c_int, [c_void_p, c_int]),
    "w2d_batch_stats": (c_int, [c_void_p, ctypes.POINTER(c_int), ctypes.POINTER(c_float),
                                ctypes.POINTER(ctypes.c_double), ctypes.POINTER(c_ll)]),
    "w2d_engine_last_stats": (c_int, [c_void_p, ctypes.POINTER(c_int), ctypes.POINTER(c_ll),
                                      ctypes.POINTER(c_ll), ctypes.POINTER(c_float)]),
    # virtual-source gathers
    "w2d_xcorr_rows": (c_int, [c_int, c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int)]),
    "w2d_xcorr_create": (c_int, [ctypes.POINTER(c_void_p), c_int, c_int, c_void_p, c_int,
                                 c_void_p, c_int, c_int]),
    "w2d_xcorr_destroy": (None, [c_void_p]),
    "w2d_xcorr_shape": (c_int, [c_void_p, ctypes.POINTER(c_int), ctypes.POINTER(c_int)]),
    "w2d_xcorr_add": (c_int, [c_void_p, c_void_p, c_int]),
    "w2d_xcorr_add_device": (c_int, [c_void_p, c_void_p, c_int]),
    "w2d_xcorr_read": (c_int, [c_void_p, c_void_p, c_int]),
    "w2d_time_derivative": (c_int, [c_void_p, c_int, c_int, ctypes.c_double, c_int, c_void_p]),
    "w2d_virtual_branch": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_void_p,
                                   ctypes.POINTER(c_int)]),
    "w2d_resample_linear": (c_int, [c_void_p, c_int, c_int, ctypes.c_double, ctypes.c_double,
                                    c_int, c_void_p]),
}


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load (building first if needed) the CUDA engine library."""
    global _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        path = lib_path()
        if build_if_missing and not _build.up_to_date():
            _build.build()
        if not os.path.exists(path):
            raise RuntimeError(f"CUDA engine library missing: {path}")
        lib = ctypes.CDLL(path)
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
        return lib


def exported_symbols():
    return list(_SIGS)


def check(rc: int) -> None:
    if rc != 0:
        msg = _LIB.w2d_last_error() if _LIB is not None else b""
        raise W2DError(rc, (msg or b"").decode(errors="replace"))


def device_memory():
    """(free, total) bytes of device memory."""
    f, t = c_ull(), c_ull()
    check(load().w2d_device_memory(ctypes.byref(f), ctypes.byref(t)))
    return int(f.value), int(t.value)
