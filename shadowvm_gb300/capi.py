"""ctypes binding of include/svm_capi.h (the data plane's C ABI).

This is the same boundary a cgo / JNI / C++ caller binds; the Python host code
(service, batching loop, tests, bench) goes through it like any other caller.
There is no Python or CPU fallback: when the library is missing, load() raises.
"""
from __future__ import annotations

import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
# SVM_LIB overrides the library path (an alternate build of the same ABI).
LIB_PATH = os.environ.get("SVM_LIB") or os.path.join(HERE, "_build", "libshadowvm_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "svm_capi.h")

STATUS = {0: "SVM_OK", 1: "SVM_E_INVALID_ARG", 2: "SVM_E_UNSUPPORTED", 3: "SVM_E_OOM_BUDGET",
          4: "SVM_E_TIMEOUT", 5: "SVM_E_CUDA", 6: "SVM_E_NOT_FOUND", 7: "SVM_E_DEVICE"}
OK, E_INVALID_ARG, E_UNSUPPORTED, E_OOM_BUDGET, E_TIMEOUT, E_CUDA, E_NOT_FOUND, E_DEVICE = range(8)
JOIN_REF_COMPAT, JOIN_EXACT = 0, 1
K_STAR, K_SELECT, K_BUILD, K_FINALIZE, K_BATCH, K_OTHER, K_LOAD, K_COUNT = range(8)


class svm_config(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("hbm_budget_bytes", ctypes.c_ulonglong),
                ("tuple_per_bulk", ctypes.c_ulonglong), ("join_mode", ctypes.c_int),
                ("hash_char_signed", ctypes.c_int), ("batch_policy", ctypes.c_int),
                ("autotune", ctypes.c_int)]


class svm_arg(ctypes.Structure):
    _fields_ = [("key", ctypes.c_char_p), ("value", ctypes.c_char_p)]


class svm_column_desc(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int), ("val_size", ctypes.c_longlong)]


class svm_operator(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int), ("nargs", ctypes.c_int), ("args", ctypes.POINTER(svm_arg)),
                ("ncols", ctypes.c_int), ("output", ctypes.POINTER(svm_column_desc))]


class svm_pipeline(ctypes.Structure):
    _fields_ = [("id", ctypes.c_char_p), ("nops", ctypes.c_int), ("ops", ctypes.POINTER(svm_operator)),
                ("npre", ctypes.c_int), ("pre_pipeline_id", ctypes.POINTER(ctypes.c_char_p))]


class svm_noalloc_scan(ctypes.Structure):
    _fields_ = [("ncols", ctypes.c_int), ("cols", ctypes.POINTER(ctypes.c_void_p)),
                ("nrows", ctypes.c_ulonglong),
                ("nranges", ctypes.c_int), ("range_col", ctypes.POINTER(ctypes.c_int)),
                ("range_lo", ctypes.POINTER(ctypes.c_int)), ("range_hi", ctypes.POINTER(ctypes.c_int)),
                ("nkeys", ctypes.c_int), ("key_col", ctypes.POINTER(ctypes.c_int)),
                ("key_min", ctypes.POINTER(ctypes.c_int)), ("key_max", ctypes.POINTER(ctypes.c_int)),
                ("nmetrics", ctypes.c_int), ("metric_op", ctypes.POINTER(ctypes.c_int)),
                ("metric_a", ctypes.POINTER(ctypes.c_int)), ("metric_b", ctypes.POINTER(ctypes.c_int))]


METRIC_COL, METRIC_ADD, METRIC_SUB, METRIC_MUL = range(4)
NOALLOC_SCRATCH_WORDS = 1 << 17


class SvmError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status
        self.message = message


def declared_functions() -> list[str]:
    """Every function name include/svm_capi.h declares."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(svm_[a-z0-9_]+)\s*\(", text)) - {"svm_status"})


_lib = None


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"shadowvm_gb300: CUDA library {path} is not built "
                          "(run `python -c \"import __graft_entry__ as g; g.build()\"`)")
    lib = ctypes.CDLL(path)
    P, I, U64, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_ulonglong, ctypes.c_double
    cp = ctypes.c_char_p
    sig = {
        "svm_config_default": (None, [ctypes.POINTER(svm_config)]),
        "svm_init": (I, [ctypes.POINTER(svm_config), ctypes.POINTER(P)]),
        "svm_destroy": (None, [P]),
        "svm_last_error": (cp, [P]),
        "svm_abi_version": (I, []),
        "svm_stream": (P, [P]),
        "svm_bytes_in_use": (U64, [P]),
        "svm_object_put": (I, [P, cp, I, ctypes.POINTER(I), U64, ctypes.POINTER(P), I]),
        "svm_object_put_host": (I, [P, cp, I, ctypes.POINTER(I), U64, ctypes.POINTER(P)]),
        "svm_object_put_columns": (I, [P, cp, I, ctypes.POINTER(svm_column_desc), U64, ctypes.POINTER(P), I]),
        "svm_object_columns": (I, [P, cp, ctypes.POINTER(svm_column_desc), I]),
        "svm_object_gen_uniform": (I, [P, cp, I, U64, U64, U64, I, I, ctypes.POINTER(I)]),
        "svm_object_view": (I, [P, cp, cp, U64, U64]),
        "svm_object_info": (I, [P, cp, ctypes.POINTER(I), ctypes.POINTER(U64)]),
        "svm_object_types": (I, [P, cp, ctypes.POINTER(I), I]),
        "svm_object_read": (I, [P, cp, I, U64, U64, P]),
        "svm_object_device_ptr": (I, [P, cp, I, ctypes.POINTER(P)]),
        "svm_object_drop": (I, [P, cp]),
        "svm_object_load_text": (I, [P, cp, I, ctypes.POINTER(I), P, U64, I, ctypes.c_char, ctypes.c_char,
                                     ctypes.POINTER(U64)]),
        "svm_objects_read": (I, [P, I, ctypes.POINTER(cp), P, U64, ctypes.POINTER(U64), ctypes.POINTER(U64)]),
        "svm_run_pipeline": (I, [P, ctypes.POINTER(svm_pipeline)]),
        "svm_run_batch": (I, [P, I, ctypes.POINTER(svm_pipeline)]),
        "svm_pipeline_footprint": (I, [P, ctypes.POINTER(svm_pipeline), ctypes.POINTER(U64)]),
        "svm_batch_begin": (I, [P, I, ctypes.POINTER(svm_pipeline), I, ctypes.POINTER(P)]),
        "svm_batch_wait": (I, [P, P, ctypes.POINTER(U64), ctypes.POINTER(U64)]),
        "svm_batch_release": (I, [P, P, P, U64]),
        "svm_profile_enable": (I, [P, I]),
        "svm_profile_reset": (I, [P]),
        "svm_profile_read": (I, [P, I, ctypes.POINTER(U64), ctypes.POINTER(D)]),
        "svm_kernel_launches": (U64, []),
        "svm_test_device_wait": (I, [P, ctypes.c_uint, I]),
        "svm_last_launch": (I, [P, ctypes.c_char_p, U64]),
        "svm_pin_launch": (I, [P, I, I, I, I]),
        "svm_pin_list_after": (I, [P, I]),
        "svm_pin_batch_launch": (I, [P, I, I]),
        "svm_scan_aggregate_noalloc": (I, [P, ctypes.POINTER(svm_noalloc_scan), ctypes.POINTER(P),
                                           ctypes.POINTER(P), U64, ctypes.POINTER(U64)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib
