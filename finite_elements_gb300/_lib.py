"""ctypes binding of libfe_gb300.so (declared in include/fe_gb300.h).

The library is the only compute path: importing this module without the built
library, or calling into it without a CUDA device, raises -- nothing falls back to
the CPU.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libfe_gb300.so")

FE_OK, FE_MAXITER, FE_BREAKDOWN, FE_NONFINITE, FE_BAD_INPUT, FE_CUDA_ERR, FE_NOT_READY = range(7)
FE_KIND_ELASTIC_TRI, FE_KIND_MAGNETIC_TRI, FE_KIND_ELASTIC_TET = 1, 2, 3
FE_PLANE_STRESS, FE_PLANE_STRAIN = 1, 2
FE_ASSEMBLE_K, FE_ASSEMBLE_M, FE_ASSEMBLE_F, FE_ASSEMBLE_PATTERN = 1, 2, 4, 8
FE_MAT_K_AUGMENTED, FE_MAT_K_CSC, FE_MAT_M_CSC = 1, 2, 3
FE_PREC_FP64, FE_PREC_MIXED, FE_PREC_MIXED_CG64 = 0, 1, 2
FE_MODAL_SMALLEST, FE_MODAL_LARGEST = 0, 1
FE_SOLVE_ACCEPT_STAGNATION, FE_SOLVE_RESTART_EACH_STEP, FE_SOLVE_X0_IF_BETTER = 1, 2, 4
FE_SOLVE_MULTIGRID = 8
FE_MG_PHASES = 10
MG_PHASE_NAMES = ("input", "dinv_lmax", "aggregation", "tentative_qr", "prolongator", "a_p", "restriction",
                  "galerkin", "coarsest_inverse", "cycle_prepare")

STATUS_NAMES = {FE_OK: "FE_OK", FE_MAXITER: "FE_MAXITER", FE_BREAKDOWN: "FE_BREAKDOWN",
                FE_NONFINITE: "FE_NONFINITE", FE_BAD_INPUT: "FE_BAD_INPUT",
                FE_CUDA_ERR: "FE_CUDA_ERR", FE_NOT_READY: "FE_NOT_READY"}


class FeError(RuntimeError):
    """A failing status from the C ABI, with the library's message."""

    def __init__(self, status, message):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class SolveOpts(C.Structure):
    _fields_ = [("precision", C.c_int32), ("cheb_degree", C.c_int32), ("max_iter", C.c_int32),
                ("max_outer", C.c_int32), ("tol", C.c_double), ("inner_tol", C.c_double),
                ("cheb_ratio", C.c_double), ("x0", C.c_void_p), ("x0_device", C.c_int32),
                ("lanes", C.c_int32), ("chunk", C.c_int32), ("flags", C.c_int32)]


class SolveStats(C.Structure):
    _fields_ = [("status", C.c_int32), ("iterations", C.c_int32), ("outer", C.c_int32),
                ("spmv", C.c_int32), ("relres", C.c_double), ("bnorm", C.c_double),
                ("solve_ms", C.c_double), ("assemble_ms", C.c_double), ("fp64_iterations", C.c_int32),
                ("x0_used", C.c_int32)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


_P = C.c_void_p
_I32, _I64, _D = C.c_int32, C.c_int64, C.c_double
_PD, _PI32, _PI64 = C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_int64)

_SIGNATURES = {
    "fe_modal": ([_P, _I32, _I32, _D, _I32, _I32, _P, _P, _P], C.c_int),
    "fe_set_device": ([_I32], C.c_int),
    "fe_version": ([], C.c_int),
    "fe_status_string": ([C.c_int], C.c_char_p),
    "fe_last_error": ([], C.c_char_p),
    "fe_mesh_create": ([_I32, _I64, _I64, _P, _P, C.POINTER(_P)], C.c_int),
    "fe_destroy": ([_P], C.c_int),
    "fe_set_elastic_materials": ([_P, _P, _P, _P, _P, _I32], C.c_int),
    "fe_set_mu": ([_P, _P], C.c_int),
    "fe_set_node_loads": ([_P, _I64, _P, _P, _P], C.c_int),
    "fe_set_element_loads": ([_P, _I64, _P, _P, _P, _P, _I64], C.c_int),
    "fe_set_dirichlet": ([_P, _I64, _P, _P], C.c_int),
    "fe_element_node_factors": ([_P, _I64, _P, _P], C.c_int),
    "fe_set_rhs_additions": ([_P, _I64, _P, _P], C.c_int),
    "fe_set_continuity": ([_P, _I64, _P, _P, _P], C.c_int),
    "fe_assemble": ([_P, _I32], C.c_int),
    "fe_export_sizes": ([_P, _I32, _PI64, _PI64, _PI64], C.c_int),
    "fe_export_csr": ([_P, _I32, _P, _P, _P], C.c_int),
    "fe_export_rhs": ([_P, _P], C.c_int),
    "fe_export_element_matrices": ([_P, _I32, _P], C.c_int),
    "fe_solve": ([_P, C.POINTER(SolveOpts), _P, C.POINTER(SolveStats)], C.c_int),
    "fe_get_solution": ([_P, _P], C.c_int),
    "fe_solution_device_ptr": ([_P, C.POINTER(_P)], C.c_int),
    "fe_info": ([_P, _PI64, _PI64, _PI64], C.c_int),
    "fe_set_l2_keep": ([_P, _I64], C.c_int),
    "fe_event_record": ([_P, _I32], C.c_int),
    "fe_event_elapsed_ms": ([_P, _I32, _I32, _PD], C.c_int),
    "fe_synchronize": ([_P], C.c_int),
    "fe_launch_count": ([_P, _PI64], C.c_int),
    "fe_autotune_spmv": ([_P, _I32, _PI32, _PD], C.c_int),
    "fe_time_spmv": ([_P, _I32, _I32, _I32, _PD], C.c_int),
    "fe_sell_info": ([_P, _PI64, _PI32], C.c_int),
    "fe_profile_kernels": ([_P, _I32], C.c_int),
    "fe_profile_read": ([_P, _I32, _PD, _PI64, _PD, _PI64], C.c_int),
    "fe_profile_read_multigrid": ([_P, _PD, _PI64, _PD, _PI64, _PD, _PI64], C.c_int),
    "fe_profile_read_multigrid_phases": ([_P, _PD, C.c_int32], C.c_int),
    "fe_trim_memory_pools": ([C.c_uint64], C.c_int),
    "fe_host_register": ([_P, C.c_uint64], C.c_int),
    "fe_host_unregister": ([_P], C.c_int),
    "fe_post_elastic": ([_P, _P, _P, _P, _P], C.c_int),
    "fe_post_magnetic": ([_P, _P, _P], C.c_int),
    "fe_gnn_create": ([C.POINTER(_P)], C.c_int),
    "fe_gnn_destroy": ([_P], C.c_int),
    "fe_gnn_num_params": ([_PI64], C.c_int),
    "fe_gnn_set_params": ([_P, _P, _I64], C.c_int),
    "fe_gnn_get_params": ([_P, _P, _I64], C.c_int),
    "fe_gnn_features": ([_P, _P, _P], C.c_int),
    "fe_gnn_predict": ([_P, _P, _P, C.POINTER(_P), _PD], C.c_int),
    "fe_gnn_predict_async": ([_P, _P, C.POINTER(_P)], C.c_int),
    "fe_gnn_target_energy": ([_P, _P, _PD], C.c_int),
    "fe_gnn_loss_grad": ([_P, _P, _D, _PD, _P], C.c_int),
    "fe_gnn_fit_grad": ([_P, _P, _PD, _P], C.c_int),
    "fe_gnn_adam_step": ([_P, C.c_float, C.c_float, C.c_float, C.c_float], C.c_int),
    "fe_batch_create": ([_P, _I32, _P, C.POINTER(_P)], C.c_int),
    "fe_batch_destroy": ([_P], C.c_int),
    "fe_batch_set_tiles": ([_P, _I32, _I64], C.c_int),
    "fe_batch_autotune": ([_P, _PI32, _PI64, _PD], C.c_int),
    "fe_batch_solve": ([_P, _D, _I32, _P, _P, _P, _P, _PD], C.c_int),
    "fe_batch_set_preconditioner": ([_P, _I32, _D], C.c_int),
    "fe_batch_last_run": ([_P, _PI32, _PI32, _PI32, _PI32], C.c_int),
    "fe_scan_counts_noalloc": ([_P, _P, _I64, _P], C.c_int),
    "fe_amg_build_host": ([_I64, _I32, _P, _P, _P, _I32, _P, _D, _I64, C.POINTER(_P)], C.c_int),
    "fe_amg_build_parallel_host": ([_I64, _I32, _P, _P, _P, _I32, _P, _D, _I64, C.POINTER(_P)], C.c_int),
    "fe_amg_build_device": ([_P, _D, _I64, C.POINTER(_P)], C.c_int),
    "fe_amg_levels": ([_P, _PI32], C.c_int),
    "fe_amg_level_info": ([_P, _I32, _PI64, _PI32, _PI64, _PI64, _PI64, _PI32, _PD], C.c_int),
    "fe_amg_level_matrix": ([_P, _I32, _I32, _P, _P, _P], C.c_int),
    "fe_amg_level_aggregates": ([_P, _I32, _P], C.c_int),
    "fe_amg_vcycle_host": ([_P, _I32, _P, _P], C.c_int),
    "fe_amg_vcycle_host_f32": ([_P, _I32, _P, _P], C.c_int),
    "fe_amg_pcg_host": ([_P, _I32, _P, _D, _I32, _P, _P, _P, _P], C.c_int),
    "fe_amg_destroy": ([_P], C.c_int),
}

_lib = None


def load():
    """Load libfe_gb300.so once; raise if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with "
                          "`python -m finite_elements_gb300.build` (nvcc, sm_103a)")
    lib = C.CDLL(LIB_PATH)
    for name, (args, res) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def exported_symbols():
    return list(_SIGNATURES)


def check(status, what=""):
    if status != FE_OK:
        msg = load().fe_last_error().decode(errors="replace")
        raise FeError(status, f"{what}: {msg}" if what else msg)
    return status


def ptr(a):
    """Address of a C-contiguous numpy array (None for None)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "arrays crossing the C ABI must be contiguous"
    return a.ctypes.data_as(C.c_void_p)


class Handle:
    """Owns one fe_handle (device buffers of one problem); freed on close / GC."""

    def __init__(self, kind, coords, conn):
        lib = load()
        self._lib = lib
        tet = kind == FE_KIND_ELASTIC_TET
        coords = np.ascontiguousarray(coords, dtype=np.float64).reshape(-1, 3 if tet else 2)
        conn = np.ascontiguousarray(conn, dtype=np.int32).reshape(-1, 4 if tet else 3)
        h = C.c_void_p()
        check(lib.fe_mesh_create(kind, coords.shape[0], conn.shape[0], ptr(coords), ptr(conn),
                                 C.byref(h)), "fe_mesh_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self._lib.fe_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:   # interpreter shutdown
            pass

    def call(self, name, *args):
        return check(getattr(self._lib, name)(self.h, *args), name)
