"""ctypes binding of ``libck_gb300.so`` (the C ABI of ``include/commkit_gb300.h``).

The library is built in-tree (``python -m commkit_gb300.build``).  There is
no fallback: if it is missing, :func:`lib` raises ``ImportError`` and every
device function of the package fails with it.
"""

from __future__ import annotations

import ctypes
import os
import sysconfig
import threading
import warnings
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_lib" / "libck_gb300.so"
# The per-call extension (csrc/python/ck_calls.cpp), built beside the library.
CALLS_PATH = _PKG / "_lib" / ("ck_calls" + (sysconfig.get_config_var("EXT_SUFFIX") or ".so"))

CK_OK = 0
CK_ERR_INVALID_ARGUMENT = 1
CK_ERR_UNSUPPORTED = 2
CK_ERR_CUDA = 3
CK_ERR_OUT_OF_MEMORY = 4
CK_ERR_DEVICE_TIMEOUT = 5

CK_LLR_MAX_K = 16
CK_GMI_CHUNK = 4096
CK_LDPC_MIN_SUM = 0
CK_LDPC_SUM_PRODUCT = 1
CK_LDPC_PLACE_AUTO = 0
CK_LDPC_PLACE_SHARED = 1
CK_LDPC_PLACE_GLOBAL = 2
CK_LDPC_PLACE_EDGES = 3
CK_LDPC_SPECIALISE_AUTO = 0
CK_LDPC_SPECIALISE_OFF = 1
CK_LDPC_SPECIALISE_ON = 2
CK_LDPC_MAX_MIXED = 12
CK_LDPC_FEED_OLDEST = 0
CK_LDPC_FEED_SHORT_FIRST = 1
CK_LDPC_STATIC_SCRATCH_BYTES = 64 * 1024 * 1024

# Every symbol the header declares; tests check the library exports them.
EXPORTS = (
    "ck_last_error",
    "ck_status_string",
    "ck_version",
    "ck_llr_separable_maxlog",
    "ck_llr_separable",
    "ck_llr_separable_maxlog_frames",
    "ck_llr_separable_frames",
    "ck_llr_points",
    "ck_llr_points_frames",
    "ck_random_bits",
    "ck_ldpc_encode",
    "ck_ldpc_encode_generator",
    "ck_ldpc_column_signs",
    "ck_map_awgn",
    "ck_count_errors",
    "ck_gmi_loss",
    "ck_gather",
    "ck_host_acquire",
    "ck_ldpc_schedule",
    "ck_ldpc_plan_create",
    "ck_ldpc_plan_destroy",
    "ck_ldpc_plan_get_info",
    "ck_ldpc_plan_set_launch",
    "ck_ldpc_plan_get_launch",
    "ck_ldpc_plan_resolved_launch",
    "ck_ldpc_plan_set_specialise",
    "ck_ldpc_plan_get_specialise",
    "ck_ldpc_specialised_source",
    "ck_ldpc_workspace_size",
    "ck_ldpc_decode",
    "ck_ldpc_workspace_status",
    "ck_ldpc_decode_static",
    "ck_ldpc_mixed_workspace_size",
    "ck_ldpc_decode_mixed",
    "ck_host_publish",
    "ck_ldpc_feed_workspace_size",
    "ck_ldpc_feed_reset",
    "ck_ldpc_feed_launch",
    "ck_ldpc_feed_publish",
)


class AxisMaxlog(ctypes.Structure):
    _fields_ = [
        ("levels", ctypes.c_void_p),
        ("labels", ctypes.c_void_p),
        ("lo", ctypes.c_void_p),
        ("hi", ctypes.c_void_p),
        ("pos", ctypes.c_void_p),
        ("L", ctypes.c_int32),
        ("k", ctypes.c_int32),
    ]


class AxisLevels(ctypes.Structure):
    _fields_ = [
        ("levels", ctypes.c_void_p),
        ("logp", ctypes.c_void_p),
        ("labels", ctypes.c_void_p),
        ("pos", ctypes.c_void_p),
        ("L", ctypes.c_int32),
        ("k", ctypes.c_int32),
    ]


class PlanInfo(ctypes.Structure):
    _fields_ = [
        (name, ctypes.c_int32)
        for name in (
            "quasi_cyclic", "lifting", "base_rows", "base_cols", "blocks", "num_checks",
            "num_variables", "num_edges", "num_layers", "max_row_degree", "device",
        )
    ]  # fmt: skip


class Batch(ctypes.Structure):
    _fields_ = [
        ("plan", ctypes.c_void_p),
        ("llr_in", ctypes.c_void_p),
        ("llr_out", ctypes.c_void_p),
        ("B", ctypes.c_int64),
        ("n_in", ctypes.c_int32),
        ("rule", ctypes.c_int32),
        ("scale", ctypes.c_float),
        ("offset", ctypes.c_float),
        ("max_iterations", ctypes.c_int32),
        ("early_stop", ctypes.c_int32),
        ("iters", ctypes.c_void_p),
        ("valid", ctypes.c_void_p),
        ("bits", ctypes.c_void_p),
        ("k_bits", ctypes.c_int32),
        ("order", ctypes.c_void_p),
        ("symbols", ctypes.c_void_p),
        ("inv_s2", ctypes.c_void_p),
        ("axis_re", ctypes.POINTER(AxisMaxlog)),
        ("axis_im", ctypes.POINTER(AxisMaxlog)),
        ("frames_per_block", ctypes.c_int32),
        ("threads_per_frame", ctypes.c_int32),
    ]


class FeedFrame(ctypes.Structure):
    """ck_ldpc_feed_frame: one frame of a continuous feed."""

    _fields_ = [
        ("symbols", ctypes.c_void_p),
        ("llr_out", ctypes.c_void_p),
        ("bits", ctypes.c_void_p),
        ("iters", ctypes.c_void_p),
        ("valid", ctypes.c_void_p),
        ("inv_s2", ctypes.c_float),
        ("seq", ctypes.c_uint32),
    ]


class FeedRing(ctypes.Structure):
    """ck_ldpc_feed_ring: a feed queue's descriptors and published count."""

    _fields_ = [
        ("frames", ctypes.c_void_p),
        ("published", ctypes.c_void_p),
        ("capacity", ctypes.c_uint32),
    ]


class Launch(ctypes.Structure):
    _fields_ = [
        ("threads_per_frame", ctypes.c_int32),
        ("frames_per_block", ctypes.c_int32),
        ("placement", ctypes.c_int32),
    ]


_lib: ctypes.CDLL | None = None
_lock = threading.Lock()


def _declare(lib: ctypes.CDLL) -> None:
    p, i32, i64, f32 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_float
    size_p = ctypes.POINTER(ctypes.c_size_t)
    sigs = {
        "ck_last_error": ([], ctypes.c_char_p),
        "ck_status_string": ([ctypes.c_int], ctypes.c_char_p),
        "ck_version": ([], ctypes.c_char_p),
        "ck_llr_separable_maxlog": (
            [p, i64, ctypes.POINTER(AxisMaxlog), ctypes.POINTER(AxisMaxlog), f32, p, p], ctypes.c_int),
        "ck_llr_separable": (
            [p, i64, ctypes.POINTER(AxisLevels), ctypes.POINTER(AxisLevels), f32, i32, p, p],
            ctypes.c_int),
        "ck_llr_separable_maxlog_frames": (
            [p, i64, i64, p, ctypes.POINTER(AxisMaxlog), ctypes.POINTER(AxisMaxlog), p, p],
            ctypes.c_int),
        "ck_llr_separable_frames": (
            [p, i64, i64, p, ctypes.POINTER(AxisLevels), ctypes.POINTER(AxisLevels), i32, p, p],
            ctypes.c_int),
        "ck_llr_points": ([p, i64, p, p, p, i32, i32, ctypes.c_float, i32, p, p], ctypes.c_int),
        "ck_llr_points_frames": ([p, i64, i64, p, p, p, p, i32, i32, i32, p, p], ctypes.c_int),
        "ck_random_bits": ([p, i64, ctypes.c_uint64, ctypes.c_uint64, p], ctypes.c_int),
        "ck_ldpc_encode": ([p, i64, i32, i32, i32, p, p, i32, p, p, ctypes.c_size_t, p, p], ctypes.c_int),
        "ck_ldpc_encode_generator": ([p, i64, i32, i32, i32, p, p, p, p, ctypes.c_size_t, p, p], ctypes.c_int),
        "ck_ldpc_column_signs": ([p, i64, i32, p, i32, p, p], ctypes.c_int),
        "ck_map_awgn": ([p, i64, i32, p, ctypes.c_float, ctypes.c_float, ctypes.c_uint64, ctypes.c_uint64, p, p],
                        ctypes.c_int),
        "ck_count_errors": ([p, p, p, p, i64, i32, i32, p, p, p, p], ctypes.c_int),
        "ck_gmi_loss": ([p, p, i64, i64, p, p], ctypes.c_int),
        "ck_gather": ([p, i32, p], ctypes.c_int),
        "ck_host_acquire": ([], None),
        "ck_ldpc_schedule": ([p, p, i64, i32, i32, p, p, p, ctypes.POINTER(i32)], ctypes.c_int),
        "ck_ldpc_plan_create": ([p, p, p, i32, i32, i32, ctypes.POINTER(p)], ctypes.c_int),
        "ck_ldpc_plan_destroy": ([p], ctypes.c_int),
        "ck_ldpc_plan_get_info": ([p, ctypes.POINTER(PlanInfo)], ctypes.c_int),
        "ck_ldpc_plan_set_launch": ([p, ctypes.POINTER(Launch)], ctypes.c_int),
        "ck_ldpc_plan_get_launch": ([p, ctypes.POINTER(Launch)], ctypes.c_int),
        "ck_ldpc_plan_resolved_launch": ([p, i32, ctypes.POINTER(Launch)], ctypes.c_int),
        "ck_ldpc_plan_set_specialise": ([p, i32], ctypes.c_int),
        "ck_ldpc_plan_get_specialise": ([p, ctypes.POINTER(i32), ctypes.POINTER(i32)], ctypes.c_int),
        "ck_ldpc_specialised_source": ([p, p, p, i32, i32, i32, i32, ctypes.c_char_p, ctypes.c_size_t,
                                        ctypes.POINTER(ctypes.c_size_t)], ctypes.c_int),
        "ck_ldpc_workspace_size": ([p, i64, i32, size_p], ctypes.c_int),
        "ck_ldpc_decode": (
            [p, p, p, i64, i32, i32, f32, f32, i32, i32, p, p, p, i32, p, ctypes.c_size_t, p],
            ctypes.c_int),
        "ck_ldpc_workspace_status": ([p, p], ctypes.c_int),
        "ck_ldpc_mixed_workspace_size": ([ctypes.POINTER(Batch), i32, size_p], ctypes.c_int),
        "ck_ldpc_decode_mixed": ([ctypes.POINTER(Batch), i32, p, ctypes.c_size_t, p], ctypes.c_int),
        "ck_ldpc_decode_static": (
            [p, p, p, i64, i32, i32, f32, f32, i32, i32, p, p, p, i32, p], ctypes.c_int),
        "ck_host_publish": ([p, ctypes.c_uint32], None),
        "ck_ldpc_feed_workspace_size": ([ctypes.POINTER(Batch), i32, size_p], ctypes.c_int),
        "ck_ldpc_feed_reset": ([p, p], ctypes.c_int),
        "ck_ldpc_feed_launch": ([ctypes.POINTER(Batch), ctypes.POINTER(FeedRing), i32, p, ctypes.c_uint32, i32, p,
                                 ctypes.c_size_t, p], ctypes.c_int),
        "ck_ldpc_feed_publish": ([p, ctypes.c_uint32, p, p, ctypes.c_uint32, i32, p, i64, p, i32, p, i32, p, f32,
                                  ctypes.c_uint32], ctypes.c_int),
    }  # fmt: skip
    for name, (args, res) in sigs.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res


def lib() -> ctypes.CDLL:
    """The loaded library; ``ImportError`` if it has not been built."""
    global _lib
    if _lib is None:
        with _lock:
            if _lib is None:
                if not LIB_PATH.exists():
                    raise ImportError(
                        f"{LIB_PATH} is missing: build it with `python -m commkit_gb300.build` "
                        "(commkit_gb300 has no CPU fallback)"
                    )
                # torch first: the library then binds to the CUDA runtime torch
                # already loaded (same soname), so both share the current device.
                import torch  # noqa: F401

                handle = ctypes.CDLL(str(LIB_PATH))
                _declare(handle)
                _lib = handle
    return _lib


_calls = None  # the loaded extension; False once found missing or turned off


def calls():
    """The per-call extension over the library, initialised; None where it was
    not built or ``COMMKIT_GB300_CALLS=0``.  It serves ``compute_llr`` and
    ``decode`` of torch CUDA tensors without a ctypes call or a Python-level
    allocation; both functions run the same kernels through ctypes without it.
    """
    global _calls
    if _calls is None:
        handle = lib()  # imports torch first, whose types the extension uses
        with _lock:
            if _calls is None:
                _calls = _load_calls(handle) or False
    return _calls or None


def _load_calls(handle: ctypes.CDLL):
    if os.environ.get("COMMKIT_GB300_CALLS", "1") == "0" or not CALLS_PATH.exists():
        return None
    import importlib.machinery
    import importlib.util

    try:
        loader = importlib.machinery.ExtensionFileLoader("commkit_gb300.ck_calls", str(CALLS_PATH))
        spec = importlib.util.spec_from_file_location("commkit_gb300.ck_calls", CALLS_PATH, loader=loader)
        mod = importlib.util.module_from_spec(spec)
        loader.exec_module(mod)
    except ImportError as e:  # built against another torch: the ctypes calls serve
        warnings.warn(f"{CALLS_PATH.name} does not load ({e}); rebuild with `python -m commkit_gb300.build`",
                      RuntimeWarning, stacklevel=3)  # fmt: skip
        return None
    from .coding import DecodeResult

    def addr(f):
        return ctypes.cast(f, ctypes.c_void_p).value

    mod.init(addr(handle.ck_ldpc_decode), addr(handle.ck_ldpc_workspace_size),
             addr(handle.ck_llr_separable_maxlog), addr(handle.ck_llr_separable), addr(handle.ck_llr_points),
             DecodeResult)  # fmt: skip
    return mod


def last_error() -> str:
    msg = lib().ck_last_error()
    return msg.decode() if msg else ""


def check(status: int, what: str) -> None:
    """Raise the Python exception of a non-zero status."""
    if status == CK_OK:
        return
    msg = f"{what}: {last_error() or lib().ck_status_string(status).decode()}"
    if status in (CK_ERR_INVALID_ARGUMENT, CK_ERR_UNSUPPORTED):
        raise ValueError(msg)
    if status == CK_ERR_OUT_OF_MEMORY:
        raise MemoryError(msg)
    raise RuntimeError(msg)
