"""Loader of libkiyosi_gpu.so, the CUDA library behind include/kgpu.h.

There is no fallback: when the library or a GPU is missing, pricing raises DeviceError.
"""
import ctypes as C
import os
import threading

from . import abi
from .errors import DeviceError, raise_for_status

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libkiyosi_gpu.so")
_lib = None
_lock = threading.Lock()
_local = threading.local()


def library():
    """The loaded CUDA library (building it in-tree first if it is absent)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                from . import build
                build.build()
            try:
                _lib = abi.declare(C.CDLL(LIB_PATH))
            except OSError as exc:
                raise DeviceError(f"cannot load {LIB_PATH}: {exc}") from exc
        return _lib


class Context:
    """Owns one kgpu_context (a CUDA stream and its device buffers) on one device."""

    def __init__(self, device: int = 0):
        self.lib = library()
        handle = C.c_void_p()
        status = self.lib.kgpu_context_create(int(device), C.byref(handle))
        if status != 0:
            raise_for_status(status, self.lib.kgpu_last_error_message(None).decode())
        self.handle = handle
        self.device = device

    def check(self, status: int) -> None:
        if status != 0:
            raise_for_status(status, self.lib.kgpu_last_error_message(self.handle).decode())

    @property
    def last_kernel_ms(self) -> float:
        return self.lib.kgpu_context_last_kernel_ms(self.handle)

    @property
    def last_path_kernel_ms(self) -> float:
        return self.lib.kgpu_context_last_path_kernel_ms(self.handle)

    @property
    def last_launches(self) -> int:
        return self.lib.kgpu_context_last_launches(self.handle)

    @property
    def last_graph(self) -> int:
        """0: the last book call launched directly; 1: captured its sequence; 2: replayed it."""
        return self.lib.kgpu_context_last_graph(self.handle)

    def close(self):
        if self.handle:
            self.lib.kgpu_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def context(device: int = 0) -> Context:
    """The calling thread's context on `device` (a context serves one thread at a time)."""
    cache = getattr(_local, "contexts", None)
    if cache is None:
        cache = _local.contexts = {}
    ctx = cache.get(device)
    if ctx is None:
        ctx = cache[device] = Context(device)
    return ctx
