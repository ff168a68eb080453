"""ctypes binding of libqdfn.so (the C ABI declared in include/qdfn.h).

There is no CPU fallback: every compute entry point runs the CUDA library, and
loading fails loudly when the library has not been built.
"""
import ctypes as C
import os

from . import build as _build

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int64)
_pdp = C.POINTER(_dp)

QDFN_OK = 0
ERRORS = {
    -1: "QDFN_ERR_INVALID", -2: "QDFN_ERR_CUDA", -3: "QDFN_ERR_NOMEM", -4: "QDFN_ERR_STATE",
    -10: "QDFN_ERR_DOMAIN", -11: "QDFN_ERR_EMPTY", -12: "QDFN_ERR_RETRIES", -13: "QDFN_ERR_NO_CONVERGE",
    -14: "QDFN_ERR_TIMEOUT", -15: "QDFN_ERR_HALF_SPACE",
}
LAYOUT_ROW, LAYOUT_COL = 0, 1
FP64, FP32, BF16X2 = 0, 1, 2
PRECISIONS = {"fp64": FP64, "fp32": FP32, "bf16x2": BF16X2}

# every symbol include/qdfn.h declares
EXPORTS = [
    "qdfn_version", "qdfn_status_string", "qdfn_last_error",
    "qdfn_assemble_rect", "qdfn_assemble_rect_dev", "qdfn_assemble_tri", "qdfn_assemble_tri_dev",
    "qdfn_ctx_create", "qdfn_ctx_destroy", "qdfn_set_dense", "qdfn_set_dense_dev", "qdfn_set_hmatrix",
    "qdfn_set_external_stress", "qdfn_run", "qdfn_run_async", "qdfn_sync", "qdfn_kernels_per_run",
    "qdfn_get_counters",
    "qdfn_get_state", "qdfn_set_state", "qdfn_get_history", "qdfn_apply_operator", "qdfn_get_kself",
    "qdfn_apply_dense_noalloc", "qdfn_set_state_all", "qdfn_get_state_all", "qdfn_set_blocks",
    "qdfn_get_blocks", "qdfn_read_bulk_input", "qdfn_bulk_to_segment", "qdfn_rot_verts_unit_vectors",
    "qdfn_ensemble_create", "qdfn_ensemble_destroy", "qdfn_ensemble_get_blocks", "qdfn_ensemble_set_blocks",
    "qdfn_ensemble_balance", "qdfn_ensemble_run", "qdfn_ensemble_run_async", "qdfn_ensemble_sync",
    "qdfn_ensemble_shares", "qdfn_ensemble_set_fill", "qdfn_check_division", "qdfn_adjoint_run",
    "qdfn_assemble_tri_pairs_dev", "qdfn_set_early_cols", "qdfn_get_early_cols",
    "qdfn_ensemble_state_bytes", "qdfn_ensemble_set_state_all", "qdfn_ensemble_get_state_all",
    "qdfn_hstruct_build", "qdfn_hstruct_sizes", "qdfn_hstruct_get", "qdfn_hstruct_destroy",
]


class BulkInfo(C.Structure):
    """Mirror of struct qdfn_bulk_info."""
    _fields_ = [(n, C.c_double) for n in ("switch_ss_rn", "shear_modulus", "poisson_ratio", "rock_density",
                                          "drop_crit", "drop_crit_ns_multiplier", "minimum_ns")] + \
               [("is_triangle", C.c_int32), ("columns", C.c_int32), ("fault_count", C.c_int64),
                ("loading_fault_count", C.c_int64)]


class QdfnError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "QDFN_ERR"), code, msg))
        self.code = code


class Problem(C.Structure):
    """Mirror of struct qdfn_problem."""
    _fields_ = [("N", C.c_int64), ("Nload", C.c_int64), ("n_inst", C.c_int32), ("evolution_dr", C.c_int32)] + \
               [(n, _dp) for n in ("a", "b", "Dc", "theta_i", "V_i", "f_i", "sigma0", "V_const", "mass")] + \
               [(n, C.c_double) for n in ("G", "rho", "sigma_min", "switch_v", "dt_cut", "rupture_dt", "max_dt",
                                          "alpha_evo")] + \
               [("interp_at_told", C.c_int32), ("reserved", C.c_int32), ("record_step", C.c_int64),
                ("max_records", C.c_int64)]


_lib = None


def lib_path():
    return _build.LIB_PATH


def load():
    """Load libqdfn.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB_PATH
    if not os.path.exists(path):
        raise ImportError("libqdfn.so not found at %s; build it with "
                          "`python -c 'import __graft_entry__ as g; g.build()'`" % path)
    L = C.CDLL(path)
    L.qdfn_version.restype = C.c_char_p
    L.qdfn_status_string.restype = C.c_char_p
    L.qdfn_status_string.argtypes = [C.c_int]
    L.qdfn_last_error.argtypes = [C.c_char_p, C.c_size_t]
    L.qdfn_assemble_rect.argtypes = [C.c_int64, _dp, C.c_int64, _dp, C.c_double, C.c_double, _dp, _dp, C.c_int]
    L.qdfn_assemble_rect_dev.argtypes = [C.c_int64, C.c_void_p, C.c_int64, C.c_void_p, C.c_double, C.c_double,
                                         C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_void_p]
    L.qdfn_assemble_tri.argtypes = [C.c_int64, _dp, _dp, _dp, _dp, C.c_int64, _dp, _dp, _dp, C.c_double,
                                    C.c_double, _dp, _dp, C.c_int]
    L.qdfn_assemble_tri_dev.argtypes = [C.c_int64] + [C.c_void_p] * 4 + [C.c_int64] + [C.c_void_p] * 3 + \
                                       [C.c_double, C.c_double, C.c_void_p, C.c_void_p, C.c_int64, C.c_int,
                                        C.c_void_p]
    L.qdfn_ctx_create.argtypes = [C.POINTER(C.c_void_p), C.POINTER(Problem)]
    L.qdfn_ctx_destroy.argtypes = [C.c_void_p]
    L.qdfn_set_dense.argtypes = [C.c_void_p, _dp, _dp, C.c_int64, C.c_int, C.c_int]
    L.qdfn_set_dense_dev.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_void_p]
    L.qdfn_set_hmatrix.argtypes = [C.c_void_p, C.c_int64, _ip, _ip, _pdp, _pdp, _pdp, _ip, _pdp, _pdp, _pdp, C.c_int]
    L.qdfn_hstruct_build.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int, C.c_double]
    L.qdfn_hstruct_sizes.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.qdfn_hstruct_get.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.qdfn_hstruct_destroy.argtypes = [C.c_void_p]
    L.qdfn_set_external_stress.argtypes = [C.c_void_p, C.c_int64, _dp, _dp, _dp, _dp]
    L.qdfn_run.argtypes = [C.c_void_p, C.c_int64, C.c_double]
    L.qdfn_run_async.argtypes = [C.c_void_p, C.c_int64, C.c_double, C.c_void_p]
    L.qdfn_sync.argtypes = [C.c_void_p]
    L.qdfn_kernels_per_run.argtypes = [C.c_void_p]
    L.qdfn_set_blocks.argtypes = [C.c_void_p, C.c_int]
    L.qdfn_get_blocks.argtypes = [C.c_void_p]
    L.qdfn_set_early_cols.argtypes = [C.c_void_p, C.c_int]
    L.qdfn_get_early_cols.argtypes = [C.c_void_p]
    L.qdfn_get_counters.argtypes = [C.c_void_p, _ip, C.c_int]
    L.qdfn_get_state.argtypes = [C.c_void_p, C.c_int] + [_dp] * 8 + [_ip]
    L.qdfn_set_state.argtypes = [C.c_void_p, C.c_int] + [_dp] * 6 + [C.c_double, C.c_double, C.c_int64]
    L.qdfn_get_history.argtypes = [C.c_void_p, C.c_int] + [_dp] * 6 + [_ip]
    # whole-ensemble state: raw addresses, so that pinned tensors pass straight through
    L.qdfn_set_state_all.argtypes = [C.c_void_p] + [C.c_void_p] * 9 + [C.c_void_p]
    L.qdfn_get_state_all.argtypes = [C.c_void_p] + [C.c_void_p] * 9 + [C.c_void_p, C.c_int]
    L.qdfn_apply_operator.argtypes = [C.c_void_p, _dp, _dp, _dp]
    L.qdfn_get_kself.argtypes = [C.c_void_p, _dp]
    L.qdfn_apply_dense_noalloc.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_void_p]
    L.qdfn_read_bulk_input.argtypes = [C.c_char_p, C.POINTER(BulkInfo), C.c_void_p, C.c_int64]
    L.qdfn_bulk_to_segment.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]
    L.qdfn_rot_verts_unit_vectors.argtypes = [C.c_int64] + [C.c_void_p] * 11
    L.qdfn_ensemble_create.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_void_p), C.c_void_p]
    L.qdfn_ensemble_destroy.argtypes = [C.c_void_p]
    L.qdfn_ensemble_get_blocks.argtypes = [C.c_void_p, C.c_void_p]
    L.qdfn_ensemble_set_blocks.argtypes = [C.c_void_p, C.c_void_p]
    L.qdfn_ensemble_balance.argtypes = [C.c_void_p]
    L.qdfn_ensemble_run.argtypes = [C.c_void_p, C.c_int64, C.c_double]
    L.qdfn_ensemble_run_async.argtypes = [C.c_void_p, C.c_int64, C.c_double, C.c_void_p]
    L.qdfn_ensemble_sync.argtypes = [C.c_void_p]
    L.qdfn_ensemble_shares.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p]
    L.qdfn_ensemble_set_fill.argtypes = [C.c_void_p, C.c_int]
    L.qdfn_ensemble_state_bytes.argtypes = [C.c_void_p, _ip]
    L.qdfn_ensemble_set_state_all.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.qdfn_ensemble_get_state_all.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
    L.qdfn_check_division.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.qdfn_assemble_tri_pairs_dev.argtypes = [C.c_int64] + [C.c_void_p] * 9 + [C.c_double, C.c_double] + \
                                             [C.c_void_p] * 3
    L.qdfn_adjoint_run.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_void_p, C.c_int64] + [C.c_void_p] * 9 + \
                                  [C.c_double]
    _lib = L
    return L


def last_error():
    buf = C.create_string_buffer(1024)
    load().qdfn_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(rc):
    if rc != QDFN_OK:
        raise QdfnError(rc, last_error())
    return rc


def dp(a):
    """double* of a C-contiguous float64 numpy array (or NULL for None)."""
    if a is None:
        return _dp()
    return a.ctypes.data_as(_dp)
