"""ctypes binding of libtmvg.so (the C ABI declared in include/tmvg.h).

The library is built in-tree by tmv_gb300/build.py (or __graft_entry__.build()).
There is no fallback: if the shared library is missing, importing the binding
raises, so nothing silently runs on the CPU.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libtmvg.so"

i64 = C.c_int64
dbl = C.c_double
vp = C.c_void_p

STATUS = {
    0: "ok", 1: "singular", 2: "not converged", 3: "bad argument", 4: "out of memory",
    5: "device wait timed out", 6: "cuda error", 7: "no cuda device", 8: "unsupported",
}


class TmvgError(RuntimeError):
    """Raised for a non-OK tmvg_status; .status holds the code."""

    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class SingularError(TmvgError):
    """A zero U(j,j) was met while solving (TMV's SingularUpperTriMatrix)."""


# name -> (restype, argtypes)
class IRInfo(C.Structure):
    """tmvg_ir_info: refinement steps, convergence, backward error, ||A||_inf."""

    _fields_ = [("iterations", C.c_int32), ("converged", C.c_int32),
                ("backward_error", C.c_double), ("anorm_inf", C.c_double)]


class KernelTiming(C.Structure):
    """tmvg_kernel_timing: spans, summed event ms, algorithmic bytes and flops."""

    _fields_ = [("spans", C.c_int64), ("total_ms", C.c_double), ("bytes", C.c_double),
                ("flops", C.c_double)]


KCLASS = {"trailing_update": 0, "panel": 1, "tri_solve": 2, "residual": 3}

_SIGS = {
    "tmvg_version": (C.c_int, []),
    "tmvg_status_string": (C.c_char_p, [C.c_int]),
    "tmvg_create": (C.c_int, [C.POINTER(vp), C.c_int]),
    "tmvg_destroy": (C.c_int, [vp]),
    "tmvg_set_stream": (C.c_int, [vp, vp]),
    "tmvg_synchronize": (C.c_int, [vp]),
    "tmvg_last_error": (C.c_char_p, [vp]),
    "tmvg_launch_count": (i64, [vp]),
    "tmvg_probe_fp64_rate": (C.c_int, [vp, C.POINTER(dbl)]),
    "tmvg_test_set_wait": (C.c_int, [vp, C.c_uint32, C.c_int32]),
    "tmvg_timing_enable": (C.c_int, [vp, C.c_int]),
    "tmvg_timing_read": (C.c_int, [vp, C.c_int, C.POINTER(KernelTiming)]),
    "tmvg_multmm_f64": (C.c_int, [vp, C.c_int, dbl, i64, i64, i64, vp, i64, i64, vp, i64, i64,
                                  vp, i64, i64]),
    "tmvg_multmm_f64_host": (C.c_int, [vp, C.c_int, dbl, i64, i64, i64, vp, i64, i64, vp, i64,
                                       i64, vp, i64, i64]),
    "tmvg_gemm_f32_tf32x3": (C.c_int, [vp, i64, i64, i64, vp, i64, vp, i64, vp, i64]),
    "tmvg_lu_decompose_f64": (C.c_int, [vp, i64, vp, i64, vp]),
    "tmvg_lu_decompose_f64_host": (C.c_int, [vp, i64, vp, i64, i64, vp]),
    "tmvg_lu_decompose_f64_noalloc": (C.c_int, [i64, vp, i64, vp, vp]),
    "tmvg_lu_ldiveq_f64": (C.c_int, [vp, i64, vp, i64, vp, i64, vp, i64]),
    "tmvg_lu_decompose_z64": (C.c_int, [vp, i64, vp, i64, vp]),
    "tmvg_lu_ldiveq_z64": (C.c_int, [vp, i64, vp, i64, vp, i64, vp, i64]),
    "tmvg_lu_rdiveq_z64": (C.c_int, [vp, i64, vp, i64, vp, i64, vp, i64]),
    "tmvg_lu_inverse_z64": (C.c_int, [vp, i64, vp, i64, vp, vp, i64]),
    "tmvg_lu_det_z64": (C.c_int, [vp, i64, vp, i64, vp, vp, C.POINTER(dbl), vp]),
    "tmvg_lu_decompose_z64_host": (C.c_int, [vp, i64, vp, i64, i64, vp]),
    "tmvg_lu_ldiveq_z64_host": (C.c_int, [vp, i64, vp, i64, vp, i64, vp, i64, i64]),
    "tmvg_lu_rdiveq_z64_host": (C.c_int, [vp, i64, vp, i64, vp, i64, vp, i64, i64]),
    "tmvg_lu_inverse_z64_host": (C.c_int, [vp, i64, vp, i64, vp, vp, i64, i64]),
    "tmvg_multmm_f32_host": (C.c_int, [vp, C.c_int, C.c_float, i64, i64, i64, vp, i64, i64, vp, i64,
                                       i64, vp, i64, i64]),
    "tmvg_lu_decompose_f32_host": (C.c_int, [vp, i64, vp, i64, i64, vp]),
    "tmvg_lu_ldiveq_f32_host": (C.c_int, [vp, i64, vp, i64, vp, i64, vp, i64, i64]),
    "tmvg_lu_rdiveq_f32_host": (C.c_int, [vp, i64, vp, i64, vp, i64, vp, i64, i64]),
    "tmvg_lu_inverse_f32_host": (C.c_int, [vp, i64, vp, i64, vp, vp, i64, i64]),
    "tmvg_lu_rdiveq_f64": (C.c_int, [vp, i64, vp, i64, vp, i64, vp, i64]),
    "tmvg_lu_ldiveq_f64_host": (C.c_int, [vp, i64, vp, i64, vp, i64, vp, i64, i64]),
    "tmvg_lu_rdiveq_f64_host": (C.c_int, [vp, i64, vp, i64, vp, i64, vp, i64, i64]),
    "tmvg_divide_f64": (C.c_int, [vp, i64, vp, i64, i64, vp, i64, vp, i64, vp, vp]),
    "tmvg_divide_f64_host": (C.c_int, [vp, i64, vp, i64, vp, vp, vp, vp]),
    "tmvg_lu_det_f64": (C.c_int, [vp, i64, vp, i64, vp, C.POINTER(dbl), C.POINTER(dbl),
                                  C.POINTER(dbl)]),
    "tmvg_lu_inverse_f64": (C.c_int, [vp, i64, vp, i64, vp, vp, i64]),
    "tmvg_lu_inverse_f64_host": (C.c_int, [vp, i64, vp, i64, vp, vp, i64, i64]),
    "tmvg_lu_inverse_ata_f64": (C.c_int, [vp, i64, vp, i64, vp, i64]),
    "tmvg_lu_is_singular_f64": (C.c_int, [vp, i64, vp, i64, C.POINTER(C.c_int)]),
    "tmvg_tri_ldiveq_f64": (C.c_int, [vp, C.c_int, C.c_int, i64, vp, i64, i64, i64, vp, i64, i64]),
    "tmvg_tri_rdiveq_f64": (C.c_int, [vp, C.c_int, C.c_int, i64, vp, i64, i64, i64, vp, i64, i64]),
    "tmvg_multmv_f64": (C.c_int, [vp, C.c_int, dbl, i64, i64, vp, i64, i64, vp, i64, vp, i64]),
    "tmvg_lu_solve_mixed_f64": (C.c_int, [vp, i64, vp, i64, i64, vp, i64, vp, i64, C.c_int, dbl,
                                          C.POINTER(IRInfo)]),
    "tmvg_lu_solve_mixed_f64_host": (C.c_int, [vp, i64, vp, i64, vp, vp, C.c_int, dbl,
                                               C.POINTER(IRInfo)]),
    "tmvg_lu_solve_fwd_f64": (C.c_int, [vp, i64, vp, i64, i64, vp, i64, vp, i64, vp, vp]),
    "tmvg_lu_solve_bwd_f64": (C.c_int, [vp, i64, vp, i64, vp, i64, vp, i64, vp, i64, vp, i64,
                                        vp, i64]),
    "tmvg_batch_plan_create": (C.c_int, [vp, i64, vp, vp, vp, vp, C.c_int, C.POINTER(vp)]),
    "tmvg_batch_plan_info": (C.c_int, [vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64),
                                       C.POINTER(dbl), C.POINTER(C.c_int)]),
    "tmvg_batch_plan_set_tiles": (C.c_int, [vp, C.POINTER(C.c_int)]),
    "tmvg_batched_lu_solve_f64": (C.c_int, [vp, vp, vp, vp, vp]),
    "tmvg_batched_lu_solve_mixed_f64": (C.c_int, [vp, vp, vp, vp, vp, C.c_int, dbl, vp, vp]),
    "tmvg_batch_plan_destroy": (C.c_int, [vp]),
    "tmvg_band_lu_decompose_batched_f64": (C.c_int, [vp, i64, i64, i64, i64, C.c_int, vp, i64, i64,
                                                   vp, i64]),
    "tmvg_band_lu_ldiveq_batched_f64": (C.c_int, [vp, i64, i64, i64, i64, C.c_int, vp, i64, i64, vp,
                                                i64, i64, vp, i64, i64, vp]),
    "tmvg_band_lu_rdiveq_batched_f64": (C.c_int, [vp, i64, i64, i64, i64, C.c_int, vp, i64, i64, vp,
                                                i64, i64, vp, i64, i64, vp]),
    "tmvg_band_divide_batched_f64": (C.c_int, [vp, i64, i64, i64, i64, vp, i64, i64, vp, i64, i64, vp,
                                             i64, i64, vp, i64, i64, vp]),
    "tmvg_band_lu_solve_batched_f64": (C.c_int, [vp, i64, i64, i64, i64, C.c_int, vp, i64, i64, vp,
                                               i64, i64, vp, i64, i64, vp]),
}

_lib = None


def load() -> C.CDLL:
    """Load libtmvg.so once and attach the signatures of every entry point."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build the CUDA library first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def declared_symbols() -> list[str]:
    return list(_SIGS)


class Handle:
    """Owns one tmvg context; check() turns a status into an exception."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = vp()
        st = self.lib.tmvg_create(C.byref(h), device)
        if st != 0:
            raise TmvgError(st, "tmvg_create failed")
        self.h = h
        self.device = device

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.tmvg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr: int) -> None:
        self.check(self.lib.tmvg_set_stream(self.h, vp(stream_ptr)))

    def check(self, st: int, what: str = "") -> None:
        if st == 0:
            return
        msg = (self.lib.tmvg_last_error(self.h) or b"").decode() or what
        if st == 1:
            raise SingularError(st, msg)
        raise TmvgError(st, msg)

    def launches(self) -> int:
        return int(self.lib.tmvg_launch_count(self.h))

    def fp64_rate(self) -> float:
        """The device's FP64 FMA rate in TFLOP/s (tmvg_probe_fp64_rate)."""
        v = dbl()
        self.check(self.lib.tmvg_probe_fp64_rate(self.h, C.byref(v)), "probe_fp64_rate")
        return float(v.value)

    def call(self, name: str, *args) -> int:
        return getattr(self.lib, name)(self.h, *args)

    def timing_enable(self, on: bool) -> None:
        """Turn kernel-class timing on or off (either clears the sums)."""
        self.check(self.lib.tmvg_timing_enable(self.h, 1 if on else 0), "timing_enable")

    def timing(self, kclass: str) -> dict:
        """Summed spans, event ms, algorithmic bytes and flops of one kernel class."""
        t = KernelTiming()
        self.check(self.lib.tmvg_timing_read(self.h, KCLASS[kclass], C.byref(t)), "timing_read")
        return {"spans": int(t.spans), "total_ms": t.total_ms, "bytes": t.bytes, "flops": t.flops}
