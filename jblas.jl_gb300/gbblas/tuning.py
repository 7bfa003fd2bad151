"""Tensor-core engine tuning: the measured replacement of jBLAS's micro-tile choice and block options.

jBLAS picks its register tile from a register-count formula (pick_kernel_size,
src/kernel_structure.jl:76-99) and fixed block sizes (BLASOptions, src/blas_options.jl:2-7).
Here the launch configuration of the tensor-core engine (engine, L2 band, TMA stores of FP32
outputs) is chosen per kind of product and output-size class by timing the candidates on the
device (gb_autotune_tc), installed in the library (gb_set_tc_tuning) and persisted in a JSON
cache keyed by the device name, so later processes load it instead of tuning again.

    kinds: "ozaki_slices", "ozaki_crt", "f32", "adjoint"
    size classes by max(M, N): 0 up to 2048, 1 up to 8192, 2 beyond
"""
import ctypes
import json
import os

import torch

from . import _lib
from ._lib import TC_KINDS, TcTuning, check


def _kind(kind):
    return TC_KINDS[kind] if isinstance(kind, str) else int(kind)


def size_class(M, N):
    rc = _lib.lib().gb_tc_size_class(int(M), int(N))
    check(rc if rc < 0 else 0, "gb_tc_size_class")
    return rc


def default_tuning(kind, cls=1):
    t = TcTuning()
    check(_lib.lib().gb_tc_default_tuning(_kind(kind), int(cls), ctypes.byref(t)), "gb_tc_default_tuning")
    return t


def get_tuning(kind, cls):
    t = TcTuning()
    check(_lib.lib().gb_get_tc_tuning(_kind(kind), int(cls), ctypes.byref(t)), "gb_get_tc_tuning")
    return t


def set_tuning(kind, cls, tuning):
    """Installs `tuning` (a TcTuning or a dict with engine / band / tma_store; None = the default)."""
    if isinstance(tuning, dict):
        tuning = TcTuning.from_dict(tuning)
    ptr = ctypes.byref(tuning) if tuning is not None else None
    check(_lib.lib().gb_set_tc_tuning(_kind(kind), int(cls), ptr), "gb_set_tc_tuning")


def _key(kind, cls):
    return "%s|%s|%d" % (torch.cuda.get_device_name(), kind if isinstance(kind, str) else str(kind), int(cls))


def _read(cache):
    if cache and os.path.exists(cache):
        try:
            with open(cache) as f:
                return json.load(f)
        except (OSError, ValueError):
            pass
    return {}


def autotune(kind, M, N, K, reps=3, cache=None, install=True):
    """(TcTuning, ms per call) for `kind` at M x N x K: from the cache when it holds this device,
    kind and size class, else measured by gb_autotune_tc (and stored).  install=True also sets it
    in the library for later calls of that kind and class."""
    cls = size_class(M, N)
    key = _key(kind, cls)
    data = _read(cache)
    if key in data:
        t, ms = TcTuning.from_dict(data[key]["tuning"]), data[key].get("ms")
    else:
        t = TcTuning()
        ms = ctypes.c_float(0.0)
        rc = _lib.lib().gb_autotune_tc(_kind(kind), int(M), int(N), int(K), int(reps), ctypes.byref(t),
                                       ctypes.byref(ms), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        check(rc, "gb_autotune_tc")
        ms = float(ms.value)
        if cache:
            data = _read(cache)
            data[key] = {"tuning": t.as_dict(), "ms": ms, "shape": [int(M), int(N), int(K)]}
            os.makedirs(os.path.dirname(os.path.abspath(cache)), exist_ok=True)
            with open(cache, "w") as f:
                json.dump(data, f, indent=1, sort_keys=True)
    if install:
        set_tuning(kind, cls, t)
    return t, ms


def load_cache(cache):
    """Installs every cached tuning of this device; returns how many were installed."""
    dev = torch.cuda.get_device_name()
    n = 0
    for key, val in _read(cache).items():
        name, kind, cls = key.rsplit("|", 2)
        if name == dev and kind in TC_KINDS:
            set_tuning(kind, int(cls), val["tuning"])
            n += 1
    return n
