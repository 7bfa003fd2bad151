"""ctypes binding of libgbblas.so (the C ABI declared in include/gbblas.h).

The library is built in-tree by ``build_lib.py``; if it is missing this module raises
instead of falling back to any CPU or PyTorch computation.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "lib", "libgbblas.so")

GB_OK = 0
GB_ERR_INVALID_VALUE = -1
GB_ERR_UNSUPPORTED = -2
GB_ERR_PIPELINE_TIMEOUT = -3
GB_ERR_CUDA = -4
GB_ERR_ALLOC = -5
GB_ERR_NO_DEVICE = -6

MODE_NATIVE = 0
MODE_OZAKI_BF16 = 1
MODE_OZAKI_INT8 = 2
MODE_OZAKI_CRT = 3
MODE_BF16X3 = 4
MODE_BF16X6 = 5

SEMIRINGS = {"min_plus": 0, "max_plus": 1, "max_min": 2, "min_max": 3, "max_times": 4}

c_i64 = ctypes.c_int64
c_int = ctypes.c_int
c_vp = ctypes.c_void_p
c_double = ctypes.c_double
c_float = ctypes.c_float


class OzakiPlan(ctypes.Structure):
    _fields_ = [("slices", ctypes.c_int32), ("bits", ctypes.c_int32), ("k_chunk", ctypes.c_int32),
                ("products", ctypes.c_int32), ("groups", ctypes.c_int32),
                ("flops_tensor", ctypes.c_double)]


GROUPED_CLASSES = 6


class Problem(ctypes.Structure):
    """gb_problem_t: one product of a grouped call."""
    _fields_ = [("m", ctypes.c_int64), ("n", ctypes.c_int64), ("k", ctypes.c_int64),
                ("lda", ctypes.c_int64), ("ldb", ctypes.c_int64), ("ldc", ctypes.c_int64),
                ("A", ctypes.c_void_p), ("B", ctypes.c_void_p), ("C", ctypes.c_void_p),
                ("alpha", ctypes.c_double), ("beta", ctypes.c_double)]


TC_KINDS = {"ozaki_slices": 0, "ozaki_crt": 1, "f32": 2, "adjoint": 3}
TC_SIZE_CLASSES = 3


class TcTuning(ctypes.Structure):
    """gb_tc_tuning_t: tensor-core engine, L2 band, TMA-store choice and (CRT) column panels of
    one kind and size class."""
    _fields_ = [("engine", ctypes.c_int32), ("band", ctypes.c_int32), ("tma_store", ctypes.c_int32),
                ("panels", ctypes.c_int32)]

    def as_dict(self):
        return {"engine": self.engine, "band": self.band, "tma_store": self.tma_store, "panels": self.panels}

    @classmethod
    def from_dict(cls, d):
        return cls(int(d["engine"]), int(d["band"]), int(d.get("tma_store", 0)), int(d.get("panels", 0)))


class Tuning(ctypes.Structure):
    """gb_grouped_tuning_t: tile configuration per size class."""
    _fields_ = [("config", ctypes.c_int32 * GROUPED_CLASSES)]

    def as_list(self):
        return list(self.config)

    @classmethod
    def from_list(cls, cfg):
        t = cls()
        for i, c in enumerate(cfg):
            t.config[i] = int(c)
        return t


# name -> (restype, argtypes)
SIGNATURES = {
    "gb_status_string": (ctypes.c_char_p, [c_int]),
    "gb_version": (c_int, []),
    "gb_set_wait_limit_ns": (c_int, [ctypes.c_uint64]),
    "gb_set_ozaki_tolerance": (c_int, [c_double]),
    "gb_set_ozaki_min_chunks": (c_int, [c_int]),
    "gb_set_tc_engine": (c_int, [c_int]),
    "gb_check_status": (c_int, [c_vp]),
    "gb_release_workspace": (c_int, []),
    "gb_jmul_f64": (c_int, [c_vp, c_vp, c_vp, c_i64, c_i64, c_i64, c_vp]),
    "gb_jmul_f32": (c_int, [c_vp, c_vp, c_vp, c_i64, c_i64, c_i64, c_vp]),
    "gb_gemm_f64": (c_int, [c_int, c_int, c_i64, c_i64, c_i64, c_double, c_vp, c_i64, c_vp, c_i64,
                            c_double, c_vp, c_i64, c_int, c_int, ctypes.POINTER(c_double), c_vp]),
    "gb_gemm_f32": (c_int, [c_int, c_int, c_i64, c_i64, c_i64, c_float, c_vp, c_i64, c_vp, c_i64,
                            c_float, c_vp, c_i64, c_vp]),
    "gb_measure_fma_peaks": (c_int, [ctypes.POINTER(c_double), ctypes.POINTER(c_double)]),
    "gb_tc_size_class": (c_int, [c_i64, c_i64]),
    "gb_tc_default_tuning": (c_int, [c_int, c_int, ctypes.POINTER(TcTuning)]),
    "gb_get_tc_tuning": (c_int, [c_int, c_int, ctypes.POINTER(TcTuning)]),
    "gb_set_tc_tuning": (c_int, [c_int, c_int, ctypes.POINTER(TcTuning)]),
    "gb_autotune_tc": (c_int, [c_int, c_i64, c_i64, c_i64, c_int, ctypes.POINTER(TcTuning),
                               ctypes.POINTER(c_float), c_vp]),
    "gb_gemm_f32_ex": (c_int, [c_int, c_int, c_i64, c_i64, c_i64, c_float, c_vp, c_i64, c_vp, c_i64,
                               c_float, c_vp, c_i64, c_int, c_vp]),
    "gb_plan_ozaki": (c_int, [c_i64, c_i64, c_i64, c_int, ctypes.POINTER(OzakiPlan)]),
    "gb_plan_ozaki_crt": (c_int, [c_i64, c_i64, c_i64, c_int, ctypes.POINTER(OzakiPlan)]),
    "gb_crt_blocks": (c_int, [c_i64, c_i64, c_int, c_int, c_int, ctypes.POINTER(c_i64), ctypes.POINTER(c_int),
                              ctypes.POINTER(c_i64), ctypes.POINTER(c_int)]),
    "gb_gemm_adjoint_f32": (c_int, [c_i64, c_i64, c_i64, c_vp, c_i64, c_vp, c_i64, c_vp, c_i64, c_vp, c_i64,
                                    c_vp, c_i64, c_vp]),
    "gb_last_ozaki_plan": (c_int, [ctypes.POINTER(OzakiPlan)]),
    "gb_kernel_kind_name": (ctypes.c_char_p, [c_int]),
    "gb_grouped_default_tuning": (c_int, [c_int, ctypes.POINTER(Tuning)]),
    "gb_grouped_workspace_size": (ctypes.c_size_t, [c_int]),
    "gb_gemm_strided_batched_f64": (c_int, [c_i64, c_i64, c_i64, ctypes.c_double, c_vp, c_i64, c_i64, c_vp, c_i64,
                                            c_i64, ctypes.c_double, c_vp, c_i64, c_i64, c_i64, c_vp]),
    "gb_gemm_strided_batched_f32": (c_int, [c_i64, c_i64, c_i64, ctypes.c_float, c_vp, c_i64, c_i64, c_vp, c_i64,
                                            c_i64, ctypes.c_float, c_vp, c_i64, c_i64, c_i64, c_vp]),
    "gb_gemm_f64_host": (c_int, [c_int, c_int, c_i64, c_i64, c_i64, c_double, c_vp, c_i64, c_vp, c_i64,
                                 c_double, c_vp, c_i64, c_int, c_int, ctypes.POINTER(c_double), c_vp]),
    "gb_gemm_f32_host": (c_int, [c_int, c_int, c_i64, c_i64, c_i64, c_float, c_vp, c_i64, c_vp, c_i64,
                                 c_float, c_vp, c_i64, c_vp]),
    "gb_jmul_f64_host": (c_int, [c_vp, c_vp, c_vp, c_i64, c_i64, c_i64, c_vp]),
    "gb_jmul_f32_host": (c_int, [c_vp, c_vp, c_vp, c_i64, c_i64, c_i64, c_vp]),
    "gb_kernel_f64": (c_int, [c_vp, c_vp, c_vp, c_i64, c_i64, c_i64, c_i64, c_i64, c_int, c_vp]),
    "gb_kernel_f32": (c_int, [c_vp, c_vp, c_vp, c_i64, c_i64, c_i64, c_i64, c_i64, c_int, c_vp]),
    "gb_gemm_semiring_f64": (c_int, [c_int, c_int, c_int, c_i64, c_i64, c_i64, c_vp, c_i64, c_vp, c_i64, c_int,
                                     c_vp, c_i64, c_vp]),
    "gb_gemm_semiring_f32": (c_int, [c_int, c_int, c_int, c_i64, c_i64, c_i64, c_vp, c_i64, c_vp, c_i64, c_int,
                                     c_vp, c_i64, c_vp]),
    "gb_gemm_semiring_i32": (c_int, [c_int, c_int, c_int, c_i64, c_i64, c_i64, c_vp, c_i64, c_vp, c_i64, c_int,
                                     c_vp, c_i64, c_vp]),
    "gb_gemm_grouped_f64": (c_int, [c_vp, c_int, ctypes.POINTER(Tuning), c_vp, ctypes.c_size_t, c_vp]),
    "gb_gemm_grouped_f32": (c_int, [c_vp, c_int, ctypes.POINTER(Tuning), c_vp, ctypes.c_size_t, c_vp]),
    "gb_gemm_grouped_f64_noalloc": (c_int, [c_vp, c_int, ctypes.POINTER(Tuning), c_vp]),
    "gb_autotune_grouped": (c_int, [c_int, ctypes.POINTER(Problem), c_int, c_int, ctypes.POINTER(Tuning),
                                    ctypes.POINTER(ctypes.c_float), c_vp]),
    "gb_launch_counts": (c_int, [ctypes.POINTER(ctypes.c_longlong), c_int]),
    "gb_profile_start": (c_int, []),
    "gb_profile_stop": (c_int, [ctypes.POINTER(c_double), ctypes.POINTER(ctypes.c_longlong), c_int]),
}

KERNEL_KINDS = 16

_lib = None


def lib():
    """The loaded library (ctypes.CDLL); raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libgbblas.so not built (%s); run __graft_entry__.build() or "
                               "python jblas.jl_gb300/build_lib.py" % LIB_PATH)
        l = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(l, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib


class GBError(RuntimeError):
    """A gbblas call returned a non-zero status."""

    def __init__(self, status, where=""):
        self.status = status
        msg = lib().gb_status_string(status).decode()
        super().__init__("%s%s (status %d)" % (where + ": " if where else "", msg, status))


def check(status, where=""):
    if status != GB_OK:
        raise GBError(status, where)
    return status
