"""ctypes binding of libqpgpu.so (the C-ABI declared in include/qpgpu.h).

There is no CPU fallback: if the library cannot be built or loaded, or no
CUDA device is present when a compute entry point runs, the call raises.
"""
from __future__ import annotations

import ctypes as C
import os
import re

from . import build as _build

OK = 0
ERRORS = {
    -1: "QPGPU_ERR_ARG", -2: "QPGPU_ERR_STATE", -3: "QPGPU_ERR_CUDA", -4: "QPGPU_ERR_NOMEM",
    -5: "QPGPU_ERR_DAVIDSON", -6: "QPGPU_ERR_TIMEOUT", -7: "QPGPU_ERR_NUMERIC",
}
FP64, FP32, FF = 0, 1, 2
SIGMA_AUTO, SIGMA_STORED, SIGMA_DIRECT = 0, 1, 2  # qpgpu_set_sigma_mode
KEYS_OFF = 2**63 - 1  # qpgpu_set_line_keys threshold: no deletion-key tables
ALGEBRA_FAST, ALGEBRA_FP64, ALGEBRA_TC = 0, 1, 2  # qpgpu_davidson_params.algebra

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "qpgpu.h")


class QPGPUError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Info(C.Structure):
    _fields_ = [("n_det", C.c_int64), ("n_alpha_unique", C.c_int32), ("n_beta_unique", C.c_int32),
                ("n_pairs", C.c_int64), ("n_s2_pairs", C.c_int64), ("setup_ms", C.c_double),
                ("ref_energy", C.c_double), ("device_bytes", C.c_int64),
                ("n_split_rows", C.c_int64), ("direct_sigma", C.c_int32), ("n_keyed_lines", C.c_int32)]


class DavidsonParams(C.Structure):
    _fields_ = [("n_states", C.c_int32), ("n_states_diag", C.c_int32), ("davidson_sze_max", C.c_int32),
                ("s2_eig", C.c_int32), ("threshold", C.c_double), ("precision", C.c_int32),
                ("defect_every", C.c_int32), ("preconditioner", C.c_int32), ("max_iter", C.c_int32),
                ("collect_every", C.c_int32), ("collect_max", C.c_int32), ("state_following", C.c_int32),
                ("algebra", C.c_int32), ("dressed", C.c_int32), ("reserved", C.c_int32)]


class DavidsonTrace(C.Structure):
    _fields_ = [("cap", C.c_int32), ("n", C.c_int32), ("n_sigma", C.c_int32), ("converged", C.c_int32),
                ("sigma_precision", C.c_void_p), ("energies", C.c_void_p), ("residuals", C.c_void_p),
                ("elapsed_ms", C.c_void_p), ("n_fallback", C.c_int32), ("pad", C.c_int32),
                ("n_samples", C.c_int64)]


class BatchStats(C.Structure):
    _fields_ = [("n_iter", C.c_int32), ("n_sigma_launches", C.c_int32), ("n_converged", C.c_int32),
                ("tuned_warps", C.c_int32), ("tuned_blocks_per_sm", C.c_int32), ("pad", C.c_int32),
                ("elapsed_ms", C.c_double), ("tune_ms", C.c_double), ("iters", C.c_void_p)]


MLP_NPARAM = 4801


_lib = None
vp = C.c_void_p


def declared_symbols() -> list[str]:
    """Function names declared in include/qpgpu.h."""
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*|int64_t|double)\s+(qpgpu_\w+)\s*\(", txt, re.M)))


def load():
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build()
    if not os.path.exists(path):
        raise RuntimeError("libqpgpu.so is missing; build it with quantum_package_gb300.build")
    L = C.CDLL(path)
    sig = {
        "qpgpu_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(vp)]),
        "qpgpu_destroy": (C.c_int, [vp]),
        "qpgpu_last_error": (C.c_char_p, [vp]),
        "qpgpu_get_info": (C.c_int, [vp, C.POINTER(Info)]),
        "qpgpu_set_sigma_mode": (C.c_int, [vp, C.c_int]),
        "qpgpu_set_line_keys": (C.c_int, [vp, C.c_int64, C.c_int64, C.c_int]),
        "qpgpu_u0_h_u0": (C.c_int, [vp, vp, vp, C.c_int, C.c_int64]),
        "qpgpu_set_integrals": (C.c_int, [vp, vp, vp]),
        "qpgpu_set_dets": (C.c_int, [vp, vp, C.c_int64]),
        "qpgpu_h_s2_u0": (C.c_int, [vp, vp, vp, vp, C.c_int, C.c_int64]),
        "qpgpu_h_s2_u0_work": (C.c_int, [vp, vp, vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
        "qpgpu_h_s2_u0_device": (C.c_int, [vp, vp, vp, vp, C.c_int, C.c_int64, C.c_int, vp]),
        "qpgpu_sigma_bilinear": (C.c_int, [vp, vp, vp, vp, vp, C.c_int, C.c_int, vp]),
        "qpgpu_sigma_bilinear_noalloc": (C.c_int, [vp, vp, vp, vp, vp, C.c_int, C.c_int, vp]),
        "qpgpu_bilinear_order": (C.c_int, [vp, vp]),
        "qpgpu_set_dressing": (C.c_int, [vp, C.c_int, vp, C.c_int64, vp, vp, vp, vp]),
        "qpgpu_clear_dressing": (C.c_int, [vp]),
        "qpgpu_h_s2_u0_dressed": (C.c_int, [vp, vp, vp, vp, C.c_int, C.c_int64]),
        "qpgpu_gram_tc": (C.c_int, [vp, vp, C.c_int64, C.c_int, vp, C.c_int64, C.c_int, C.c_int64, vp, vp]),
        "qpgpu_select_pt2": (C.c_int, [vp, vp, C.c_int, vp, C.c_int, C.c_int, C.c_int, vp, vp, vp,
                                       C.POINTER(C.c_int64)]),
        "qpgpu_pt2_generators": (C.c_int, [vp, vp, C.c_int, vp, C.c_int, vp, C.c_int, vp]),
        "qpgpu_lincomb_tc": (C.c_int, [vp, vp, C.c_int64, C.c_int, C.c_int, vp, vp, C.c_int64, C.c_int64, vp]),
        "qpgpu_batch_create": (C.c_int, [vp, C.c_int, C.POINTER(vp)]),
        "qpgpu_batch_destroy": (C.c_int, [vp]),
        "qpgpu_batch_last_error": (C.c_char_p, [vp]),
        "qpgpu_batch_davidson": (C.c_int, [vp, vp, vp, vp, vp, vp, C.POINTER(DavidsonParams),
                                           C.POINTER(BatchStats)]),
        "qpgpu_mlp_init": (C.c_int, [vp, C.c_uint64]),
        "qpgpu_mlp_set_weights": (C.c_int, [vp, vp]),
        "qpgpu_mlp_get_weights": (C.c_int, [vp, vp]),
        "qpgpu_mlp_add_samples": (C.c_int, [vp, vp, vp, vp, C.c_int64]),
        "qpgpu_mlp_clear_samples": (C.c_int, [vp]),
        "qpgpu_mlp_n_samples": (C.c_int64, [vp]),
        "qpgpu_mlp_gradient": (C.c_int, [vp, vp, vp, vp, C.c_int64, vp, C.POINTER(C.c_float)]),
        "qpgpu_mlp_predict": (C.c_int, [vp, vp, C.c_int64, vp]),
        "qpgpu_mlp_train": (C.c_int, [vp, C.c_int, C.c_int, C.c_float, C.c_uint64, C.POINTER(C.c_float)]),
        "qpgpu_diag": (C.c_int, [vp, vp, vp]),
        "qpgpu_connected_pairs": (C.c_int, [vp, C.POINTER(C.c_int64), vp, vp, vp, vp, vp, vp, C.c_int64]),
        "qpgpu_connected_pairs_rows": (C.c_int, [vp, vp, C.c_int64, C.POINTER(C.c_int64), vp, vp, vp, vp, vp, vp,
                                                 C.c_int64]),
    }
    optional = {}
    sig["qpgpu_davidson_hs2"] = (C.c_int, [vp, vp, C.c_int64, vp, vp, C.POINTER(DavidsonParams),
                                           C.POINTER(DavidsonTrace)])
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype, f.argtypes = res, args
    for name, (res, args) in optional.items():
        if hasattr(L, name):
            f = getattr(L, name)
            f.restype, f.argtypes = res, args
    _lib = L
    return L


def check(rc, ctx=None):
    if rc != OK:
        msg = load().qpgpu_last_error(ctx).decode() if ctx else ""
        raise QPGPUError(rc, msg)
