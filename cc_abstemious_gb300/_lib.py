"""ctypes binding of libbem_gb300.so (declarations mirror include/bem.h).

The library is built in-tree by ``cc_abstemious_gb300/build.py``.  There is no
fallback: if the shared library is missing the import fails loudly.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libbem_gb300.so")

BEM_OK = 0
STATUS_NAMES = {0: "OK", 1: "BAD_INPUT", 2: "SINGULAR", 3: "NOT_CONVERGED", 4: "NAN", 5: "OOM", 6: "CUDA",
                7: "TIMEOUT"}
MEM_HOST, MEM_DEVICE = 0, 1
SIDE_RHS, SIDE_LHS = 0, 1
FORM_PLAIN_FP64, FORM_MIXED, FORM_REFINED, FORM_MIXED_ROUNDED = 0, 1, 2, 3
PRECOND_NONE, PRECOND_BLOCK_JACOBI, PRECOND_LEARNED, PRECOND_LU = 0, 1, 2, 3


class BemError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), message))
        self.status = status


class Cplx(C.Structure):
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


class SolveReport(C.Structure):
    _fields_ = [("num_mv", C.c_int64), ("restarts", C.c_int64), ("iterations", C.c_int64),
                ("backward_error", C.c_double), ("rel_err_vs_lu", C.c_double), ("seconds", C.c_double),
                ("flag", C.c_int32), ("precond", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ProblemInfo(C.Structure):
    _fields_ = [("sound_speed", C.c_double), ("mass_density", C.c_double),
                ("problem_type", C.c_int32), ("method_type", C.c_int32), ("solver", C.c_int32),
                ("incident_type", C.c_int32), ("bc_type", C.c_int32), ("output_total", C.c_int32),
                ("output_pressure", C.c_int32), ("body_index", C.c_int32),
                ("tolerance", C.c_double), ("max_iterations", C.c_int64),
                ("incident_vec", C.c_double * 3), ("incident_amp", C.c_double * 2),
                ("bc_value", C.c_double * 2), ("hm_leaf", C.c_int64), ("hm_eta", C.c_double),
                ("hm_aca_tol", C.c_double), ("num_eqn", C.c_int64), ("num_field_points", C.c_int64),
                ("num_frequencies", C.c_int64), ("mesh_elements", C.c_int64), ("mesh_nodes", C.c_int64),
                ("mesh_bodies", C.c_int64), ("num_rhs", C.c_int64)]


_vp, _i64, _d, _i = C.c_void_p, C.c_int64, C.c_double, C.c_int
_PP = C.POINTER(C.c_void_p)

# name -> (restype, argtypes); every symbol declared in include/bem.h
SIGNATURES = {
    "bem_version": (C.c_char_p, []),
    "bem_ctx_create": (_i, [_i, _PP]),
    "bem_ctx_destroy": (None, [_vp]),
    "bem_last_error": (C.c_char_p, [_vp]),
    "bem_ctx_kernel_launches": (_i64, [_vp]),
    "bem_problem_from_json": (_i, [_vp, C.c_char_p, C.c_char_p, _PP]),
    "bem_problem_from_file": (_i, [_vp, C.c_char_p, _PP]),
    "bem_problem_destroy": (None, [_vp]),
    "bem_problem_get_info": (_i, [_vp, C.POINTER(ProblemInfo)]),
    "bem_problem_frequencies": (_i, [_vp, _vp]),
    "bem_problem_set_frequency_index": (_i, [_vp, _i64]),
    "bem_collocation": (_i, [_vp, _vp, _vp]),
    "bem_get_dense_surface_matrices": (_i, [_vp, _vp, _vp, _vp, _i64, _i]),
    "bem_get_dense_field_matrices": (_i, [_vp, _vp, _vp, _vp, _i64, _i]),
    "bem_get_surface_row_or_column": (_i, [_vp, _vp, _vp, _i64, _vp, _i64, _i, _vp]),
    "bem_get_system_matrix_fp32": (_i, [_vp, _vp, _vp, _i64]),
    "bem_get_incident_surface": (_i, [_vp, _vp, _vp]),
    "bem_get_incident_field": (_i, [_vp, _vp, _vp]),
    "bem_solve_for_surface": (_i, [_vp, _vp, _vp, _vp, _vp, C.POINTER(SolveReport)]),
    "bem_solve_lu": (_i, [_vp, _i64, _vp, _i64, _vp, _i]),
    "bem_gmres_solve": (_i, [_vp, _i64, _vp, _i64, _i64, _d, _vp, C.POINTER(SolveReport), _i]),
    "bem_gmres_solve_noalloc": (_i, [_vp, _i64, _vp, _i64, _i64, _d, _vp, C.POINTER(SolveReport)]),
    "bem_get_field": (_i, [_vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp, _i]),
    "bem_evaluate_field": (_i, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "bem_convert_to_pressure": (_i, [_vp, _d, _vp, _i64]),
    "bem_write_results_at_frequency": (_i, [_vp, _vp, C.c_char_p, _vp, _vp]),
    "bem_write_results_at_point": (_i, [_vp, _vp, C.c_char_p, _i64, _vp, _vp]),
    "bem_format_f64": (_i64, [_d, C.c_char_p, _i64]),
    "bem_run": (_i, [_vp, _vp, _i, _i, _vp, _vp, C.POINTER(SolveReport), _i]),
    "bem_last_surface": (_i, [_vp, _vp, _vp, _vp]),
    "bem_run_batch": (_i, [_vp, _PP, _i, _i, _PP, _PP, _PP, _i, _i64]),
    "bem_learned_train": (_i, [_vp, _vp, _i, _i, _i, _d, C.c_uint64, _vp]),
    "bem_learned_num_params": (_i64, []),
    "bem_learned_get_weights": (_i, [_vp, _vp]),
    "bem_learned_set_weights": (_i, [_vp, _vp]),
    "bem_learned_mlp_eval": (_i, [_vp, _i64, _vp, _vp, _vp, _vp]),
    "bem_learned_mlp_infer": (_i, [_vp, _i64, _vp, _vp]),
    "bem_lu32_factor_apply": (_i, [_vp, _i, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _i64, _vp, _vp, _vp]),
    "bem_assemble_operator": (_i, [_vp, _vp, _i, _i64, _i64, _vp, _i64]),
    "bem_cluster_tree": (_i, [_vp, _i, _vp, _vp, _i64, _i64, _d, _vp, _vp, _i64, _vp, _vp, _i64, _vp, _vp]),
    "bem_hmatrix_build": (_i, [_vp, _vp, _i, _PP]),
    "bem_hmatrix_destroy": (None, [_vp]),
    "bem_hmatrix_gemv": (_i, [_vp, _vp, Cplx, _vp, Cplx, _vp]),
    "bem_hmatrix_norm": (_d, [_vp]),
    "bem_hmatrix_stats": (_i, [_vp, _vp]),
    "bem_hmatrix_to_full": (_i, [_vp, _vp, _vp, _i64]),
    "bem_ctx_load_tuning": (_i, [_vp, C.c_char_p]),
    "bem_ctx_set_tuning": (_i, [_vp, C.c_char_p, C.c_char_p, _i]),
    "bem_ctx_get_tuning": (_i, [_vp, C.c_char_p, C.c_char_p, _i64, _i64]),
    "bem_ctx_tuning_source": (C.c_char_p, [_vp]),
    "bem_ctx_set_profiling": (_i, [_vp, _i]),
    "bem_ctx_stream": (_vp, [_vp]),
    "bem_ctx_profile_count": (_i64, [_vp]),
    "bem_ctx_profile_get": (_i, [_vp, _i64, C.c_char_p, _i64, C.POINTER(C.c_double), C.POINTER(C.c_int64),
                                 C.POINTER(C.c_double)]),
}

_lib = None


def load():
    """Load the in-tree library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libbem_gb300.so not found at %s: run `python -c \"import __graft_entry__ as g; "
                          "g.build()\"` (there is no CPU fallback)" % LIB_PATH)
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(status, ctx=None):
    if status != BEM_OK:
        msg = load().bem_last_error(ctx).decode() if ctx else ""
        raise BemError(status, msg)
