"""ctypes binding of libbiegpu.so (the C ABI declared in include/biegpu.h).

This is the Python counterpart of the ``ccall`` glue a Julia caller uses: the
same entry points, the same plain pointers and sizes.  There is no CPU
fallback: if the library cannot be built or loaded, every call raises.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

from . import _build

BIE_OK = 0
BIE_ERR_INVALID = -1
BIE_ERR_CUDA = -2
BIE_ERR_NOT_CONVERGED = -3
BIE_ERR_TIMEOUT = -4
BIE_ERR_NOMEM = -5
BIE_ERR_UNSUPPORTED = -6

BIE_TRI_LINEAR = 1
BIE_TRI_QUADRATIC = 2

BIE_F = 1
BIE_G = 2
BIE_C = 4

BIE_PREC_FP64 = 0
BIE_PREC_MIXED = 1
BIE_PREC_FP16 = 2
BIE_PREC_BF16 = 3
BIE_PREC_FP16_SPLIT = 4
BIE_PREC_BF16_SPLIT = 5
BIE_PREC_DF64 = 6

BIE_TRI_DISC_CONSTANT = 3
BIE_TRI_DISC_LINEAR = 4
BIE_TRI_DISC_QUADRATIC = 5

KIND = {"linear": BIE_TRI_LINEAR, "quadratic": BIE_TRI_QUADRATIC, "disctriconstant": BIE_TRI_DISC_CONSTANT,
        "disctrilinear": BIE_TRI_DISC_LINEAR, "disctriquadratic": BIE_TRI_DISC_QUADRATIC}
PRECISION = {"fp64": BIE_PREC_FP64, "mixed": BIE_PREC_MIXED, "fp16": BIE_PREC_FP16, "bf16": BIE_PREC_BF16,
             "fp16_split": BIE_PREC_FP16_SPLIT, "bf16_split": BIE_PREC_BF16_SPLIT, "df64": BIE_PREC_DF64}

_ERRNAMES = {
    BIE_ERR_INVALID: "invalid argument",
    BIE_ERR_CUDA: "CUDA error",
    BIE_ERR_NOT_CONVERGED: "not converged",
    BIE_ERR_TIMEOUT: "device wait timed out",
    BIE_ERR_NOMEM: "out of memory",
    BIE_ERR_UNSUPPORTED: "unsupported",
}


class BIEError(RuntimeError):
    """A libbiegpu call returned a negative status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{_ERRNAMES.get(code, 'error')} ({code}): {message}")
        self.code = code
        self.message = message


class MeshDesc(C.Structure):
    _fields_ = [
        ("n_coordinates", C.c_int64),
        ("coordinates", C.POINTER(C.c_double)),
        ("n_elements", C.c_int64),
        ("shape_kind", C.c_int32),
        ("physics_kind", C.c_int32),
        ("topology", C.POINTER(C.c_int64)),
        ("physics_topology", C.POINTER(C.c_int64)),
        ("n_sources", C.c_int64),
        ("sources", C.POINTER(C.c_double)),
        ("quad_n", C.c_int32),
        ("quad_m", C.c_int32),
        ("physics_beta", C.c_double),
    ]


class RuleTable(C.Structure):
    _fields_ = [
        ("n_points", C.c_int64),
        ("u", C.POINTER(C.c_double)),
        ("v", C.POINTER(C.c_double)),
        ("w", C.POINTER(C.c_double)),
    ]


class Peaks(C.Structure):
    _fields_ = [("fp64_flops", C.c_double), ("fp32_flops", C.c_double)]


class Stats(C.Structure):
    _fields_ = [
        ("kernel_launches", C.c_int64),
        ("timed_launches", C.c_int64),
        ("timed_ms", C.c_double),
        ("algorithmic_flops", C.c_double),
        ("quadrature_evals", C.c_int64),
        ("tensor_launches", C.c_int64),
        ("tensor_ms", C.c_double),
        ("tensor_flops", C.c_double),
        ("tensor_flops_executed", C.c_double),
    ]


BIE_OP_DENSE = 0
BIE_OP_MATRIX_FREE = 1
BIE_OP_FAST = 2


class Operator(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("A", C.c_void_p),
        ("A32", C.c_void_p),
        ("k_re", C.c_double),
        ("k_im", C.c_double),
        ("scale_re", C.c_double),
        ("scale_im", C.c_double),
        ("diag", C.c_void_p),
        ("fast", C.c_void_p),
    ]


class GmresOpts(C.Structure):
    _fields_ = [
        ("restart", C.c_int32),
        ("maxiter", C.c_int32),
        ("reltol", C.c_double),
        ("abstol", C.c_double),
        ("precision", C.c_int32),
        ("refine", C.c_int32),
        ("inner_reltol", C.c_double),
        ("max_refine", C.c_int32),
        ("initially_nonzero", C.c_int32),
    ]


class GmresInfo(C.Structure):
    _fields_ = [
        ("iterations", C.c_int32),
        ("restarts", C.c_int32),
        ("refinements", C.c_int32),
        ("converged", C.c_int32),
        ("matvecs", C.c_int64),
        ("residual_norm", C.c_double),
        ("rhs_norm", C.c_double),
    ]


class SweepOpts(C.Structure):
    _fields_ = [("precision", C.c_int32), ("refine", C.c_int32), ("gmres", GmresOpts),
                ("eager", C.c_int32), ("target_error", C.c_double), ("sensitivity", C.c_void_p)]


class SweepInfo(C.Structure):
    _fields_ = [
        ("solves", C.c_int64),
        ("converged", C.c_int64),
        ("iterations", C.c_int64),
        ("assemble_ms", C.c_double),
        ("solve_ms", C.c_double),
        ("record_ms", C.c_double),
        ("graph_launches", C.c_int64),
        ("accurate_solves", C.c_int64),
    ]


class MultisolveOpts(C.Structure):
    _fields_ = [("precision", C.c_int32), ("restart", C.c_int32), ("maxiter", C.c_int32),
                ("max_refine", C.c_int32), ("reltol", C.c_double), ("inner_reltol", C.c_double)]


class MultisolveInfo(C.Structure):
    _fields_ = [("passes", C.c_int32), ("inner_steps", C.c_int32), ("converged", C.c_int32),
                ("tensor_products", C.c_int32), ("exact_products", C.c_int32), ("reserved", C.c_int32),
                ("max_relres", C.c_double), ("setup_ms", C.c_double), ("tensor_ms", C.c_double),
                ("exact_ms", C.c_double)]


class AdjointOpts(C.Structure):
    _fields_ = [("rho_c", C.c_double), ("dir", C.c_double * 3), ("reltol", C.c_double),
                ("precision", C.c_int32)]


class AdjointInfo(C.Structure):
    _fields_ = [("forward_iterations", C.c_int32), ("forward_converged", C.c_int32),
                ("adjoint_iterations", C.c_int32), ("adjoint_converged", C.c_int32)]


_C2 = C.c_double * 2


class LossyConstants(C.Structure):
    _fields_ = [("rho", C.c_double), ("c", C.c_double), ("kp", C.c_double),
                ("ka", _C2), ("kh", _C2), ("kv", _C2), ("tau_a", _C2), ("tau_h", _C2),
                ("phi_a", _C2), ("phi_h", _C2), ("eta", C.c_double), ("mu", C.c_double),
                ("mu_a", _C2), ("mu_h", _C2)]


class LossyOpts(C.Structure):
    _fields_ = [("S", C.c_double), ("custom_air", C.c_int32), ("pa", C.c_double), ("t", C.c_double),
                ("Hr", C.c_double), ("depth", C.c_int32), ("interior", C.c_int32), ("fmm_on", C.c_int32),
                ("n_gauss", C.c_int32), ("fmm_offset", C.c_double), ("normals", C.c_void_p),
                ("solve", GmresOpts)]


BIE_LOSSY_BLOCKS = {"outer": 0, "Ha": 1, "Ga": 2, "Hh": 3, "Gh": 4, "Hv": 5, "Gv": 6, "Dc": 7, "Dr": 8,
                    "Nd": 9, "NdT": 10, "inner": 11}


_lib = None
_lock = threading.Lock()

_P = C.c_void_p
_D = C.c_double
_I = C.c_int
_I64 = C.c_int64

# name -> (restype, argtypes)
SIGNATURES = {
    "bie_version": (C.c_char_p, []),
    "bie_last_error": (C.c_char_p, []),
    "bie_quadrature_rule": (_I, [_I, _I, _I, _P, _P, _P, _I, C.POINTER(_I)]),
    "bie_basis": (_I, [_I, _D, _I64, _P, _P, _P, _P, _P]),
    "bie_ctx_create": (_I, [C.POINTER(_P), C.POINTER(MeshDesc), _I]),
    "bie_ctx_create_rules": (_I, [C.POINTER(_P), C.POINTER(MeshDesc), C.POINTER(RuleTable), _I, _I]),
    "bie_ctx_destroy": (_I, [_P]),
    "bie_ctx_stream": (_I, [_P, C.POINTER(_P)]),
    "bie_measure_peaks": (_I, [_I, C.POINTER(Peaks)]),
    "bie_ctx_set_timing": (_I, [_P, _I]),
    "bie_ctx_set_autotune": (_I, [_P, _I]),
    "bie_ctx_stats": (_I, [_P, C.POINTER(Stats), _I]),
    "bie_assemble": (_I, [_P, _D, _D, _P, _I64, _I, _I, _P, _P, _P]),
    "bie_assemble_device": (_I, [_P, _D, _D, _P, _I64, _I, _I, _P, _P, _P]),
    "bie_matvec": (_I, [_P, _D, _D, _P, _I64, _P, _P, _P, _P, _I]),
    "bie_matvec_device": (_I, [_P, _D, _D, _P, _I64, _P, _P, _P, _P, _I]),
    "bie_matvec_device_noalloc": (_I, [_P, _D, _D, _P, _I64, _P, _P, _P, _P]),
    "bie_matvec_multi_device": (_I, [_P, _D, _D, _I64, _P, _P, _P, _P, _I, _I64]),
    "bie_matvec_multi": (_I, [_P, _D, _D, _I64, _P, _P, _P, _P, _I, _I64]),
    "bie_lowp_gemm_device": (_I, [_P, _I, _I64, _I64, _I64, _P, _P, _P]),
    "bie_ctx_set_gemm_wait": (_I, [_P, _I64, _I]),
    "bie_solve_multi_device": (_I, [_P, _D, _D, _I64, _P, _P, C.POINTER(MultisolveOpts),
                                    C.POINTER(MultisolveInfo)]),
    "bie_solve_multi": (_I, [_P, _D, _D, _I64, _P, _P, C.POINTER(MultisolveOpts), C.POINTER(MultisolveInfo)]),
    "bie_ctx_get_shape": (_I, [_P, _I, _I64, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I), C.POINTER(_I)]),
    "bie_ctx_set_shape": (_I, [_P, _I, _I64, _I, _I, _I]),
    "bie_taylor_assemble": (_I, [_P, _D, _D, _P, _I64, _I, _I, _P, _P, _P]),
    "bie_fastop_create": (_I, [_P, _D, _D, _I, _I, _I, _D, _I, C.POINTER(_P)]),
    "bie_fastop_destroy": (_I, [_P]),
    "bie_fastop_apply_device": (_I, [_P, _P, _P, _I]),
    "bie_fastop_apply": (_I, [_P, _P, _P, _I]),
    "bie_fastop_evaluate_targets": (_I, [_P, _P, _I64, _P, _P, _I]),
    "bie_singular_rule": (_I, [_I, _D, _P, _P, _P, _I, C.POINTER(_I)]),
    "bie_nearfield_pattern": (_I, [_P, _I, C.POINTER(_I64), _P, _P]),
    "bie_nearfield_assemble": (_I, [_P, _D, _D, _I, _D, _I, _I, _I, _P, _P]),
    "bie_gmres_device": (_I, [_P, C.POINTER(Operator), _P, _P, C.POINTER(GmresOpts), C.POINTER(GmresInfo)]),
    "bie_gmres": (_I, [_P, C.POINTER(Operator), _P, _P, C.POINTER(GmresOpts), C.POINTER(GmresInfo)]),
    "bie_round_c64_device": (_I, [_P, _P, _P, _I64]),
    "bie_sweep": (_I, [C.POINTER(_P), _I, _P, _I, C.POINTER(_P), C.POINTER(_P), C.POINTER(SweepOpts),
                       C.POINTER(SweepInfo), _P]),
    "bie_adjoint": (_I, [_P, _D, _D, _P, _P, _I64, C.POINTER(AdjointOpts), C.POINTER(_D), _P, _P, _P,
                         C.POINTER(AdjointInfo)]),
    "bie_read_comsol": (_I, [C.c_char_p, C.POINTER(_I64), C.POINTER(_I64), C.POINTER(C.c_int32),
                             C.POINTER(_I64), _P, _P, _P]),
    "bie_ambient_to_properties": (_I, [_D, _D, _D, _D, _P]),
    "bie_visco_thermal_constants": (_I, [_D, _D, _D, _D, _D, C.POINTER(LossyConstants)]),
    "bie_tangential_derivatives": (_I, [C.POINTER(MeshDesc), C.POINTER(_I64), _P, _P, _P, _P, _P]),
    "bie_element_slicing": (_I, [C.POINTER(MeshDesc), _I, _P, _P, _P, _P]),
    "bie_lossy_create": (_I, [_P, _D, C.POINTER(LossyOpts), C.POINTER(_P)]),
    "bie_lossy_destroy": (_I, [_P]),
    "bie_lossy_constants_of": (_I, [_P, C.POINTER(LossyConstants)]),
    "bie_lossy_apply_device": (_I, [_P, _I, _P, _P]),
    "bie_lossy_solve_device": (_I, [_P, _I, _P, _P, C.POINTER(GmresOpts), C.POINTER(GmresInfo)]),
    "bie_lossy_apply": (_I, [_P, _I, _P, _P]),
    "bie_lossy_solve": (_I, [_P, _I, _P, _P, C.POINTER(GmresOpts), C.POINTER(GmresInfo)]),
    "bie_lossy_stats": (_I, [_P, C.POINTER(_I64), C.POINTER(_I64), _I]),
    "bie_lossy_set_one_launch": (_I, [_P, _I]),
}


def library_path() -> Path:
    return _build.LIB_PATH


def lib():
    """Load libbiegpu.so (building it first if it is missing or stale)."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.build()
            L = C.CDLL(str(path))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
        return _lib


def measure_peaks(device: int = 0) -> dict:
    """Measured FP64 / FP32 FMA throughput of a device in FLOP/s."""
    p = Peaks()
    check(lib().bie_measure_peaks(int(device), C.byref(p)))
    return {"fp64_flops": p.fp64_flops, "fp32_flops": p.fp32_flops}


def check(status: int) -> None:
    if status != BIE_OK:
        msg = lib().bie_last_error().decode(errors="replace")
        raise BIEError(status, msg)


def ptr(a) -> int | None:
    """Address of a numpy array or torch tensor (None for None)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data
