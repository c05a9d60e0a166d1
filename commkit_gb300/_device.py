"""Device arrays at the ctypes boundary: pointers, shapes, dtypes, streams.

The reference's launchers take CuPy arrays.  Here any CUDA array works:
a ``torch.Tensor`` on a CUDA device, or an object exposing
``__cuda_array_interface__`` (CuPy, Numba).  Outputs are allocated by the
input's own library on the input's device, so the device follows the data
as in the reference (``commkit/backend.py:290-333``), and work is queued on
that library's current stream.  Host arrays are rejected: this package has
no CPU path.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Any

import numpy as np

_TORCH_TO_NP = None
_NP_TO_TORCH = None
_TORCH = None


def _torch():
    global _TORCH
    if _TORCH is None:
        import torch

        _TORCH = torch
    return _TORCH


def _torch_dtypes() -> dict:
    global _TORCH_TO_NP
    if _TORCH_TO_NP is None:
        t = _torch()
        _TORCH_TO_NP = {
            t.float32: np.dtype(np.float32),
            t.float64: np.dtype(np.float64),
            t.complex64: np.dtype(np.complex64),
            t.complex128: np.dtype(np.complex128),
            t.int32: np.dtype(np.int32),
            t.int64: np.dtype(np.int64),
            t.int8: np.dtype(np.int8),
            t.uint8: np.dtype(np.uint8),
            t.bool: np.dtype(np.bool_),
            t.int16: np.dtype(np.int16),
        }
    return _TORCH_TO_NP


def _np_to_torch(dt: np.dtype):
    global _NP_TO_TORCH
    if _NP_TO_TORCH is None:
        _NP_TO_TORCH = {v: k for k, v in _torch_dtypes().items()}
    return _NP_TO_TORCH[dt]


@dataclass
class DeviceArray:
    """A CUDA buffer seen by the library: base pointer, shape, dtype, device."""

    obj: Any
    ptr: int
    shape: tuple[int, ...]
    dtype: np.dtype
    contiguous: bool
    device: int
    kind: str  # "torch" or "cai"

    @property
    def size(self) -> int:
        n = 1
        for d in self.shape:
            n *= int(d)
        return n

    @property
    def ndim(self) -> int:
        return len(self.shape)


def is_device_array(obj: Any) -> bool:
    t = _torch()
    if isinstance(obj, t.Tensor):
        return obj.is_cuda
    return hasattr(obj, "__cuda_array_interface__")


def wrap(obj: Any, name: str = "array") -> DeviceArray:
    """Describe a CUDA array; ``TypeError`` for host or foreign data."""
    t = _torch()
    if isinstance(obj, t.Tensor):
        if not obj.is_cuda:
            raise TypeError(
                f"{name} must be on a CUDA device (commkit_gb300 has no CPU path), got a "
                f"{obj.device} tensor"
            )
        dt = _torch_dtypes().get(obj.dtype)
        if dt is None:
            raise TypeError(f"{name}: unsupported dtype {obj.dtype}")
        return DeviceArray(obj, obj.data_ptr(), tuple(obj.shape), dt, obj.is_contiguous(),
                           obj.device.index, "torch")  # fmt: skip
    cai = getattr(obj, "__cuda_array_interface__", None)
    if cai is None:
        raise TypeError(
            f"{name} must be a CUDA array (torch tensor or __cuda_array_interface__), "
            f"got {type(obj).__name__}"
        )
    shape = tuple(int(s) for s in cai["shape"])
    dt = np.dtype(cai["typestr"])
    strides = cai.get("strides")
    contiguous = True
    if strides is not None:
        expect = []
        acc = dt.itemsize
        for s in reversed(shape):
            expect.append(acc)
            acc *= s
        contiguous = tuple(strides) == tuple(reversed(expect)) or int(np.prod(shape)) <= 1
    ptr = int(cai["data"][0])
    device = _cai_device(obj)
    return DeviceArray(obj, ptr, shape, dt, contiguous, device, "cai")


def _cai_device(obj: Any) -> int:
    dev = getattr(obj, "device", None)
    idx = getattr(dev, "id", None)
    return int(idx) if idx is not None else current_device()


def current_device() -> int:
    return int(_torch().cuda.current_device())


def check(arr: DeviceArray, label: str, dtype: Any, shape: tuple[int | None, ...]) -> None:
    """The reference's ``check_arrays`` contract (``commkit/_cuda/compiler.py:97-120``):
    wrong dtype -> ``TypeError``; wrong shape or not C-contiguous -> ``ValueError``."""
    want = np.dtype(dtype)
    if arr.dtype != want:
        raise TypeError(f"{label} must be {want}, got {arr.dtype}")
    if len(arr.shape) != len(shape) or any(
        w is not None and w != g for w, g in zip(shape, arr.shape, strict=False)
    ):
        dims = ", ".join("n" if s is None else str(s) for s in shape)
        dims += "," if len(shape) == 1 else ""
        raise ValueError(f"{label} must have shape ({dims}), got {arr.shape}")
    if not arr.contiguous:
        raise ValueError(f"{label} must be C-contiguous")


def empty(like: DeviceArray, shape: tuple[int, ...], dtype: Any) -> Any:
    """A new array of the input's library on the input's device."""
    dt = np.dtype(dtype)
    if like.kind == "torch":
        return _torch().empty(shape, dtype=_np_to_torch(dt), device=like.obj.device)
    import cupy  # an __cuda_array_interface__ producer other than torch

    with cupy.cuda.Device(like.device):
        return cupy.empty(shape, dtype=dt)


def zeros(like: DeviceArray, shape: tuple[int, ...], dtype: Any) -> Any:
    if like.kind == "torch":
        return _torch().zeros(shape, dtype=_np_to_torch(np.dtype(dtype)), device=like.obj.device)
    import cupy

    with cupy.cuda.Device(like.device):
        return cupy.zeros(shape, dtype=np.dtype(dtype))


def to_device(like: DeviceArray, host: np.ndarray) -> Any:
    """Copy a host table to the input's device, in the input's library."""
    host = np.ascontiguousarray(host)
    if like.kind == "torch":
        t = _torch()
        return t.from_numpy(host.copy()).to(like.obj.device)
    import cupy

    with cupy.cuda.Device(like.device):
        return cupy.asarray(host)


def stream_of(arr: DeviceArray) -> int:
    """The cudaStream_t handle work on ``arr`` is queued on (0: legacy default)."""
    if arr.kind == "torch":
        t = _torch()
        raw = getattr(t._C, "_cuda_getCurrentRawStream", None)
        if raw is not None:
            return int(raw(arr.device))
        return int(t.cuda.current_stream(arr.obj.device).cuda_stream)
    try:
        import cupy

        return int(cupy.cuda.get_current_stream().ptr)
    except ImportError:
        return 0


class on_device:
    """Context manager making ``arr``'s device current for the library calls."""

    def __init__(self, arr: DeviceArray):
        self.dev = arr.device
        self.prev: int | None = None

    def __enter__(self):
        t = _torch()
        # torch's own getter without the Python wrapper's lazy-init checks
        # (a CUDA tensor exists, so CUDA is initialised).
        get = getattr(t._C, "_cuda_getDevice", None)
        cur = get() if get is not None else t.cuda.current_device()
        if cur != self.dev:
            self.prev = cur
            t.cuda.set_device(self.dev)
        return self

    def __exit__(self, *exc):
        if self.prev is not None:
            _torch().cuda.set_device(self.prev)
        return False
