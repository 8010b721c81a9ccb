"""cosmosis module of threepoint_gb300: ``setup`` / ``execute`` / ``cleanup``.

Drop-in for the reference's cosmosis module (cuda_version/interface.cu:16-257,
referenced from ``[threepoint] file = ...`` in cosmosis/pipeline_gpu.ini:50-60):
same section, keys and outputs. cosmosis loads a Python module through these
three functions; each forwards to the C entry points ``tp_module_setup``,
``tp_module_execute`` and ``tp_module_cleanup`` of the shared library
(include/threepoint_gb300_module.h), handing them a callback table over the
data block. The block needs the cosmosis DataBlock methods ``get_double``,
``get_int`` / ``get_bool``, ``get_string``, ``get_double_array_1d`` or
``get_double_array_nd``, and ``put_double_array_1d``.

One extra option, not in the reference: ``[threepoint] precision = fp32``
selects the FP32 integrand (FP64 by default).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import FP32, FP64, ThreepointError, lib

_GET_D = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_char_p, C.c_char_p, C.POINTER(C.c_double))
_GET_I = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_char_p, C.c_char_p, C.POINTER(C.c_int))
_GET_S = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_char_p, C.c_char_p, C.c_void_p, C.c_int)
_GET_A = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_char_p, C.c_char_p, C.POINTER(C.c_double), C.c_int,
                     C.POINTER(C.c_int))
_PUT_A = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_char_p, C.c_char_p, C.POINTER(C.c_double), C.c_int)


class _DataBlock(C.Structure):
    _fields_ = [("handle", C.c_void_p), ("get_double", _GET_D), ("get_int", _GET_I), ("get_string", _GET_S),
                ("get_double_array", _GET_A), ("put_double_array", _PUT_A)]


def _bind(L):
    if getattr(L, "_module_bound", False):
        return
    pb = C.POINTER(_DataBlock)
    L.tp_module_setup.argtypes = [pb, C.c_int, C.POINTER(C.c_void_p)]
    L.tp_module_execute.argtypes = [C.c_void_p, pb]
    L.tp_module_cleanup.argtypes = [C.c_void_p]
    L.tp_module_set_precision.argtypes = [C.c_void_p, C.c_int]
    L.tp_module_n_triplets.argtypes = [C.c_void_p]
    L.tp_module_triplets.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
    L.tp_module_last_error.argtypes = [C.c_void_p]
    L.tp_module_last_error.restype = C.c_char_p
    L._module_bound = True


def _array(block, section, key):
    """A float64 array of the block, flattened row-major (p_k is 2-D)."""
    for name in ("get_double_array_nd", "get_double_array_1d"):
        f = getattr(block, name, None)
        if f is not None:
            try:
                return np.ascontiguousarray(f(section, key), dtype=np.float64).reshape(-1)
            except Exception:
                continue
    return np.ascontiguousarray(block[section, key], dtype=np.float64).reshape(-1)


class BlockAdapter:
    """tp_datablock callback table over a cosmosis-style DataBlock object.
    Keeps the ctypes callbacks alive for as long as the adapter lives."""

    def __init__(self, block):
        self.block = block
        self._cb = []

        def guard(fn):
            def wrapped(*a):
                try:
                    return fn(*a)
                except Exception:
                    return 1
            return wrapped

        def get_double(_, sec, key, out):
            out[0] = float(self.block.get_double(sec.decode(), key.decode()))
            return 0

        def get_int(_, sec, key, out):
            s, k = sec.decode(), key.decode()
            try:
                v = self.block.get_int(s, k)
            except Exception:
                v = self.block.get_bool(s, k)
            out[0] = int(v)
            return 0

        def get_string(_, sec, key, buf, cap):
            b = str(self.block.get_string(sec.decode(), key.decode())).encode()
            if len(b) + 1 > cap:
                return 1
            C.memmove(buf, b + b"\0", len(b) + 1)
            return 0

        def get_array(_, sec, key, buf, cap, n):
            a = _array(self.block, sec.decode(), key.decode())
            n[0] = a.size
            if buf:
                m = min(cap, a.size)
                C.memmove(buf, a.ctypes.data, 8 * m)
            return 0

        def put_array(_, sec, key, vals, n):
            a = np.ctypeslib.as_array(vals, shape=(n,)).copy() if n > 0 else np.zeros(0)
            self.block.put_double_array_1d(sec.decode(), key.decode(), a)
            return 0

        cbs = (_GET_D(guard(get_double)), _GET_I(guard(get_int)), _GET_S(guard(get_string)),
               _GET_A(guard(get_array)), _PUT_A(guard(put_array)))
        self._cb = cbs
        self.table = _DataBlock(None, *cbs)


class Module:
    """The module object ``setup`` returns (the reference's ``data`` class)."""

    def __init__(self, options, device=0):
        L = lib()
        _bind(L)
        self._L = L
        self._h = C.c_void_p(0)
        st = L.tp_module_setup(C.byref(BlockAdapter(options).table), device, C.byref(self._h))
        if st:
            raise ThreepointError(st, "threepoint_gb300 setup failed (see stderr)")
        prec = "fp64"
        try:
            prec = str(options.get_string("threepoint", "precision")).lower()
        except Exception:
            pass
        if prec not in ("fp64", "fp32"):
            raise ValueError("[threepoint] precision must be fp64 or fp32")
        L.tp_module_set_precision(self._h, FP32 if prec == "fp32" else FP64)

    @property
    def thetas(self):
        """The aperture-radius triplets [n, 3] (rad) built by setup."""
        n = self._L.tp_module_n_triplets(self._h)
        out = np.zeros(3 * n)
        self._L.tp_module_triplets(self._h, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out.reshape(n, 3)

    def execute(self, block):
        ad = BlockAdapter(block)
        st = self._L.tp_module_execute(self._h, C.byref(ad.table))
        if st:
            raise ThreepointError(st, self._L.tp_module_last_error(self._h).decode())
        return 0

    def close(self):
        if self._h:
            self._L.tp_module_cleanup(self._h)
            self._h = C.c_void_p(0)


# ---- the cosmosis entry points -------------------------------------------
def setup(options):
    return Module(options)


def execute(block, config):
    return config.execute(block)


def cleanup(config):
    config.close()
