"""ctypes handle on libcontract.so with the argument types of every entry point.

The library is the product: a plain C ABI (``include/contract.h`` and
``include/contract_gb300.h``).  There is no CPU fallback -- if the shared
object is missing, every call raises.
"""
import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libcontract.so")

_lock = threading.Lock()
_lib = None

c_void_p = ctypes.c_void_p
c_int = ctypes.c_int
c_size_t = ctypes.c_size_t
c_ulong = ctypes.c_ulong
c_char_p = ctypes.c_char_p
c_int_p = ctypes.POINTER(ctypes.c_int)

# name -> (restype, argtypes)
SIGNATURES = {
    # contract.h (drop-in)
    "init": (None, [c_int]),
    "meson_two_point": (None, [c_void_p, c_void_p, c_void_p, c_ulong, c_int, c_int]),
    "meson_all_source_two_point": (None, [ctypes.POINTER(c_void_p), c_void_p, c_void_p, c_ulong, c_int]),
    "meson_all_sink_two_point": (None, [ctypes.POINTER(c_void_p), c_void_p, c_void_p, c_ulong, c_int]),
    "baryon_diquark": (None, [c_void_p, c_void_p, c_void_p, c_size_t, c_int, c_int]),
    "baryon_two_point": (None, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_ulong, c_int, c_int, c_int]),
    "baryon_general_two_point": (None, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_size_t, c_int, c_int,
                                        c_void_p]),
    "baryon_sequential_two_point": (None, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_size_t, c_int, c_int,
                                           c_int]),
    # contract_gb300.h (extensions)
    "contract_set_error_mode": (None, [c_int]),
    "contract_get_error_mode": (c_int, []),
    "contract_last_error": (c_int, []),
    "contract_last_error_message": (c_char_p, []),
    "contract_clear_error": (None, []),
    "contract_check_device": (c_int, []),
    "contract_set_wait_limit": (None, [ctypes.c_ulonglong]),
    "contract_test_withhold_chunk": (None, [c_int]),
    "contract_set_stream": (None, [c_void_p]),
    "contract_get_stream": (c_void_p, []),
    "contract_set_autotune": (None, [c_int]),
    "contract_autotune_report": (c_int, [c_void_p, c_size_t]),
    "contract_variant_names": (c_int, [c_int, c_int, c_int, c_void_p, c_size_t]),
    "contract_workspace_reserve": (c_int, [c_size_t]),
    "contract_workspace_bytes": (c_size_t, [c_int_p, c_int]),
    "contract_gamma_table": (None, [c_int_p, c_int_p]),
    "contract_projector_rank": (c_int, [c_void_p]),
    "contract_convert_precision": (None, [c_void_p, c_void_p, c_size_t, c_int]),
    "contract_convert_layout": (None, [c_void_p, c_void_p, c_int_p, c_int, c_int]),
    "contract_convert_from_quda": (None, [c_void_p, ctypes.POINTER(c_void_p), c_int_p, c_size_t, c_int]),
    "contract_convert_to_quda": (None, [ctypes.POINTER(c_void_p), c_void_p, c_int_p, c_size_t, c_int]),
    "contract_rotate_spin_basis": (None, [c_void_p, c_size_t, c_void_p, c_int]),
    "contract_meson": (None, [c_void_p, c_void_p, c_void_p, c_size_t, c_int, c_int, c_int, c_int_p]),
    "contract_meson_all": (None, [ctypes.POINTER(c_void_p), c_void_p, c_void_p, c_size_t, c_int, c_int, c_int,
                                  c_int_p]),
    "contract_baryon": (None, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_size_t, c_int, c_int, c_int, c_void_p,
                               c_int, c_int_p]),
    "contract_baryon_all_types": (None, [c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_int, c_int, c_int,
                                         c_void_p, c_int, c_int_p]),
    "contract_baryon_all_types_host": (None, [c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_int, c_int, c_int,
                                         c_void_p, c_int, c_int_p]),
    "contract_baryon_all_types_noalloc": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_int, c_int,
                                                  c_int, c_void_p, c_int, c_int_p]),
    "contract_baryon_all_types_batch": (None, [c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_int]),
    "contract_meson_all_gamma_momentum": (None, [c_void_p, c_void_p, c_void_p, c_size_t, c_int_p, c_int_p, c_int,
                                                 c_int]),
    "contract_meson_all_gamma_momentum_batch": (None, [c_void_p, c_int, c_int_p, c_int, c_int]),
    "contract_batch_mixed": (None, [c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_int, c_int_p, c_int,
                                    c_int]),
    "contract_diquark": (None, [c_void_p, c_void_p, c_void_p, c_size_t, c_int, c_int, c_int]),
    "contract_sequential_sink": (None, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_size_t, c_int_p, c_int, c_int,
                                        c_int, c_int, c_int]),
    "contract_sequential": (None, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_size_t, c_int, c_int, c_int,
                                   c_int]),
}

DROP_IN = ("init", "meson_two_point", "meson_all_source_two_point", "meson_all_sink_two_point", "baryon_diquark",
           "baryon_two_point", "baryon_general_two_point", "baryon_sequential_two_point")


def lib():
    """Load libcontract.so once (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m contract_gb300.build`")
            handle = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(handle, name)
                fn.restype = res
                fn.argtypes = args
            _lib = handle
    return _lib
