"""ctypes binding of libtopopt_gb300.so (declarations mirror include/topopt_gb300.h).

The library is the product: there is no CPU fallback.  Loading fails loudly if
the shared object has not been built.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtopopt_gb300.so")

TOG_OK, TOG_ERR_ARG, TOG_ERR_CUDA, TOG_NOT_CONVERGED, TOG_BREAKDOWN, TOG_ERR_STATE, TOG_ERR_OOM = range(7)
TOG_FP64, TOG_FP32_IR = 0, 1
TOG_PROJ_HEAVISIDE, TOG_PROJ_SIGMOID = 1, 2
TOG_ELEM_FREE, TOG_ELEM_BLACK, TOG_ELEM_WHITE = 0, 1, 2
TOG_OPT_OC, TOG_OPT_MMA = 0, 1
TOG_CONV_DEFAULT, TOG_CONV_ENERGY = 0, 1
TOG_FILTER_NONE, TOG_FILTER_DENSITY, TOG_FILTER_SENS = 0, 1, 2
TOG_FILTER_J, TOG_FILTER_JT = 0, 1


class ProblemDesc(C.Structure):
    _fields_ = [("dim", C.c_int32), ("nel", C.c_int32 * 3), ("size", C.c_double * 3),
                ("E", C.c_double), ("nu", C.c_double), ("plane_stress", C.c_int32),
                ("xmin", C.c_double), ("penalty", C.c_double)]


class SolveStats(C.Structure):
    _fields_ = [("status", C.c_int32), ("iterations", C.c_int32), ("outer_iterations", C.c_int32),
                ("reserved", C.c_int32), ("rel_residual", C.c_double), ("abs_residual", C.c_double)]


class BatchStats(C.Structure):
    _fields_ = [("steps", C.c_int32), ("pcg_loops", C.c_int32), ("failed", C.c_int32), ("reliable_updates", C.c_int32)]


class IterStats(C.Structure):
    _fields_ = [("compliance", C.c_double), ("volume", C.c_double), ("change", C.c_double),
                ("lambda_", C.c_double), ("cg_iterations", C.c_int32), ("outer_iterations", C.c_int32),
                ("oc_steps", C.c_int32), ("status", C.c_int32), ("rel_residual", C.c_double)]


_D = C.POINTER(C.c_double)
_I32 = C.POINTER(C.c_int32)
_I64 = C.POINTER(C.c_int64)
_H = C.c_void_p

# name -> (restype, argtypes); the exported symbol set of include/topopt_gb300.h
SIGNATURES = {
    "tog_version": (C.c_char_p, []),
    "tog_last_error": (C.c_char_p, []),
    "tog_launch_count": (C.c_int64, []),
    "tog_grid_counts": (C.c_int, [C.c_int32, _I32, _I64, _I64, _I64]),
    "tog_node_dofs": (C.c_int, [C.c_int32, _I32, _I32]),
    "tog_cell_dofs": (C.c_int, [C.c_int32, _I32, _I32]),
    "tog_element_stiffness": (C.c_int, [C.c_int32, _D, C.c_double, C.c_double, C.c_int32, _D]),
    "tog_create": (C.c_int, [C.POINTER(ProblemDesc), C.POINTER(_H)]),
    "tog_destroy": (C.c_int, [_H]),
    "tog_set_stream": (C.c_int, [_H, C.c_void_p]),
    "tog_set_fixed_dofs": (C.c_int, [_H, C.c_int64, _I32]),
    "tog_set_rhs": (C.c_int, [_H, _D]),
    "tog_set_penalty": (C.c_int, [_H, C.c_double]),
    "tog_set_vars": (C.c_int, [_H, _D]),
    "tog_matvec": (C.c_int, [_H, _D, _D]),
    "tog_pcg_operator": (C.c_int, [_H, C.c_int32, C.c_double, _D, _D, _D, _D, _D]),
    "tog_solve": (C.c_int, [_H, C.c_int32, C.c_double, C.c_double, C.c_int32, C.c_int32, C.POINTER(SolveStats)]),
    "tog_get_u": (C.c_int, [_H, _D]),
    "tog_set_u": (C.c_int, [_H, _D]),
    "tog_compliance": (C.c_int, [_H, _D, _D]),
    "tog_filter_setup": (C.c_int, [_H, C.c_double]),
    "tog_filter_apply": (C.c_int, [_H, C.c_int32, _D, _D]),
    "tog_oc_update": (C.c_int, [_H, _D, _D, _D, _D, C.c_double, C.c_double, _D, _D, _D]),
    "tog_simp_init": (C.c_int, [_H, C.c_int32, C.c_double, C.c_double, C.c_double, _D]),
    "tog_simp_step": (C.c_int, [_H, C.c_int32, C.c_double, C.c_int32, C.c_int32, C.POINTER(IterStats)]),
    "tog_get_design": (C.c_int, [_H, _D]),
    "tog_set_design": (C.c_int, [_H, _D]),
    "tog_get_physical": (C.c_int, [_H, _D]),
    "tog_bench_kernel": (C.c_int, [_H, C.c_int32, C.c_int32, C.c_int32]),
    "tog_kernel_bytes": (C.c_int, [_H, C.c_int32, C.c_int32, _D]),
    "tog_batch_create": (C.c_int, [C.c_int32, _I32, _I32, _I32, _D, _D, C.POINTER(ProblemDesc), C.c_double, C.c_int32,
                                   C.POINTER(_H)]),
    "tog_batch_destroy": (C.c_int, [_H]),
    "tog_batch_set_stream": (C.c_int, [_H, C.c_void_p]),
    "tog_batch_autotune": (C.c_int, [_H, _I32]),
    "tog_batch_set_tile_rows": (C.c_int, [_H, C.c_int32]),
    "tog_batch_step": (C.c_int, [_H, C.POINTER(BatchStats)]),
    "tog_batch_results": (C.c_int, [_H, _D, _D, _I32]),
    "tog_batch_get_design": (C.c_int, [_H, C.c_int32, _D]),
    "tog_batch_solve_info": (C.c_int, [_H, _D, _I32, _I32]),
    "tog_batch_bench_kernel": (C.c_int, [_H, C.c_int32, C.c_int32, C.POINTER(C.c_double)]),
    "tog_batch_kernel_bytes": (C.c_int, [_H, C.c_int32, C.POINTER(C.c_double)]),
    "tog_nn_create": (C.c_int, [C.POINTER(C.c_int32), C.c_int32, C.c_uint64, C.POINTER(C.c_void_p)]),
    "tog_nn_destroy": (C.c_int, [_H]),
    "tog_nn_set_stream": (C.c_int, [_H, C.c_void_p]),
    "tog_nn_param_count": (C.c_int, [_H, C.POINTER(C.c_int64)]),
    "tog_nn_get_params": (C.c_int, [_H, C.POINTER(C.c_float)]),
    "tog_nn_set_params": (C.c_int, [_H, C.POINTER(C.c_float)]),
    "tog_nn_forward": (C.c_int, [_H, C.c_void_p, C.c_void_p]),
    "tog_nn_gradients": (C.c_int, [_H, C.c_void_p, C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_float)]),
    "tog_nn_train_step": (C.c_int, [_H, C.c_void_p, C.c_void_p, C.c_float, C.POINTER(C.c_double)]),
    "tog_set_warm_start_net": (C.c_int, [_H, _H]),
    "tog_keep_previous_state": (C.c_int, [_H]),
    "tog_record_next_step": (C.c_int, [_H, C.c_void_p, C.c_void_p]),
    "tog_record_status": (C.c_int, [_H, _I32]),
    "tog_projection": (C.c_int, [_H, C.c_int32, C.c_double, _D, _D, _D]),
    "tog_set_fixed_elements": (C.c_int, [_H, C.c_void_p]),
    "tog_free_variable_count": (C.c_int, [_H, _I64]),
    "tog_fixed_element_project": (C.c_int, [_H, _D, C.c_int64, _D]),
    "tog_fixed_element_pullback": (C.c_int, [_H, _D, _D]),
    "tog_mma_update": (C.c_int, [_H, _D, _D, C.c_double, _D, C.c_double, _D, _D, _D]),
    "tog_mma_reset": (C.c_int, [_H]),
    "tog_set_convergence": (C.c_int, [_H, C.c_int32]),
    "tog_multiload_compliance": (C.c_int, [_H, C.c_int32, _I64, _I32, _D, C.c_int32, C.c_double, C.c_double,
                                           C.c_int32, _D, C.c_void_p]),
    "tog_multiload_gradient": (C.c_int, [_H, C.c_int32, _D, _D]),
    "tog_simp_set_optimizer": (C.c_int, [_H, C.c_int32, C.c_double]),
    "tog_oc_update_noalloc": (C.c_int, [C.c_int64, _D, _D, _D, _D, C.c_double, C.c_double, _D, _D, C.c_void_p]),
}


class TopOptError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (status %d)" % (msg, code))
        self.code = code


class NotConverged(TopOptError):
    pass


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libtopopt_gb300.so is not built (run topopt.jl_gb300/build.py); "
                              "there is no CPU fallback")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(code):
    if code != TOG_OK:
        msg = lib().tog_last_error().decode(errors="replace")
        if code == TOG_NOT_CONVERGED:
            raise NotConverged(code, msg)
        raise TopOptError(code, msg)


def dptr(a):
    """numpy float64 C-contiguous array -> double*"""
    return a.ctypes.data_as(_D)


def iptr(a):
    return a.ctypes.data_as(_I32)
