"""Loader of the in-tree CUDA library libqdg.so (the engine's C ABI).

There is no fallback: if the library is missing or fails to load, every
engine call raises.  Build it with ``python -m qdng_gb300.build``.
"""
import ctypes as C
import os

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libqdg.so")
_lib = None


class QDGError(RuntimeError):
    def __init__(self, status, msg):
        self.status = status
        super().__init__(f"{abi.STATUS_NAMES.get(status, status)}: {msg}")


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"libqdg.so is not built ({LIB_PATH}); run `python -m qdng_gb300.build`")
        L = C.CDLL(LIB_PATH)
        for name, res, args in abi.SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status):
    if status != abi.QDG_OK:
        raise QDGError(status, load().qdg_last_error().decode())
