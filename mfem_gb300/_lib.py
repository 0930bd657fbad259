"""ctypes binding of the C ABI in include/gbpa.h (libgbpa.so, built in-tree).

Importing this module loads the CUDA library; if it is missing the import
raises -- there is no CPU fallback on the product path.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbpa.so")

P = ctypes.c_void_p
I = ctypes.c_int
I64 = ctypes.c_int64
D = ctypes.c_double

GBPA_DIFFUSION, GBPA_MASS = 0, 1
GBPA_F64, GBPA_F32, GBPA_F64X2 = 0, 1, 2
GBPA_SCATTER_CSR, GBPA_SCATTER_ATOMIC = 0, 1
GBPA_BATCH_GRAPH, GBPA_BATCH_PERSISTENT = 0, 1
GBPA_LAYOUT_SLAB2D, GBPA_LAYOUT_3D = 0, 1

STATUS = {
    0: "success", -1: "invalid argument", -2: "unsupported", -3: "CUDA error",
    -4: "not finite", -5: "zero diagonal", -6: "not converged", -7: "timeout",
    -8: "out of memory", -9: "index out of range",
}


class GbpaError(RuntimeError):
    def __init__(self, status, where):
        self.status = status
        super().__init__(f"{where}: gbpa status {status} ({STATUS.get(status, '?')})")


class OperatorDesc(ctypes.Structure):
    _fields_ = [("kind", I), ("precision", I), ("ne", I), ("ndofs", I), ("d1d", I), ("q1d", I),
                ("symm", I), ("B", P), ("G", P), ("qdata", P), ("gather_map", P),
                ("offsets", P), ("indices", P), ("ess", P), ("n_ess", I), ("scatter", I)]


class SolveInfo(ctypes.Structure):
    _fields_ = [("iterations", I), ("converged", I), ("initial_norm", D), ("final_norm", D),
                ("true_rel_residual", D), ("outer_iterations", I), ("inner_iterations", I),
                ("seconds", D)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ProblemDesc(ctypes.Structure):
    _fields_ = [("ne", I), ("ndofs", I), ("d1d", I), ("q1d", I), ("B", P), ("G", P),
                ("qdata", P), ("gather_map", P), ("offsets", P), ("indices", P), ("ess", P),
                ("n_ess", I), ("dinv", P), ("b", P), ("x", P)]


# name -> (restype, argtypes); every symbol declared in include/gbpa.h
SIGNATURES = {
    "gbpa_version": (I, []),
    "gbpa_error_string": (ctypes.c_char_p, [I]),
    "gbpa_create": (I, [ctypes.POINTER(P), I]),
    "gbpa_destroy": (I, [P]),
    "gbpa_set_stream": (I, [P, P]),
    "gbpa_get_stream": (P, [P]),
    "gbpa_synchronize": (I, [P]),
    "gbpa_get_error_flags": (I, [P, ctypes.POINTER(I)]),
    "gbpa_launch_count": (I64, [P]),
    "gbpa_restriction_build": (I, [I, I, I, P, P, P, P, P]),
    "gbpa_restriction_build_device": (I, [P, I, I, I, P, P, P, P, P]),
    "gbpa_restriction_mult": (I, [P, I, I, I, I, I, P, P, P]),
    "gbpa_restriction_abs_mult": (I, [P, I, I, I, I, I, P, P, P]),
    "gbpa_restriction_mult_transpose": (I, [P, I, I, I, I, I, P, P, P, P, I]),
    "gbpa_restriction_abs_mult_transpose": (I, [P, I, I, I, I, I, P, P, P, P]),
    "gbpa_geom_jacobians3d": (I, [P, I, I, I, P, P, P, P]),
    "gbpa_geom_determinants3d": (I, [P, I, I, I, P, P, P, P]),
    "gbpa_geom_coordinates3d": (I, [P, I, I, I, P, P, P]),
    "gbpa_coefficient_lognormal3d": (I, [P, I, I, P, I, P, P, D, P]),
    "gbpa_selftest_bounded_wait": (I, [P, I, ctypes.c_longlong]),
    "gbpa_diffusion_setup3d": (I, [P, I, I, I, P, P, P, I64, P]),
    "gbpa_diffusion_setup3d_nodes": (I, [P, I, I, I, I, P, P, P, P, P, I64, P]),
    "gbpa_diffusion_apply3d": (I, [P, I, I, I, I, P, P, P, P, P, P, P]),
    "gbpa_diffusion_apply3d_f32": (I, [P, I, I, I, I, P, P, P, P, P]),
    "gbpa_diffusion_diagonal3d": (I, [P, I, I, I, I, P, P, P, P]),
    "gbpa_mass_setup3d": (I, [P, I, I, P, P, P, I64, I, P]),
    "gbpa_mass_apply3d": (I, [P, I, I, I, P, P, P, P, P]),
    "gbpa_mass_apply3d_f32": (I, [P, I, I, I, P, P, P, P]),
    "gbpa_mass_diagonal3d": (I, [P, I, I, I, P, P, P]),
    "gbpa_operator_create": (I, [P, ctypes.POINTER(OperatorDesc), ctypes.POINTER(P)]),
    "gbpa_operator_create_host": (I, [P, ctypes.POINTER(OperatorDesc), ctypes.POINTER(P)]),
    "gbpa_operator_destroy": (I, [P]),
    "gbpa_operator_mult": (I, [P, P, P]),
    "gbpa_operator_mult_host": (I, [P, P, P]),
    "gbpa_operator_apply_element": (I, [P, P, P]),
    "gbpa_operator_assemble_diagonal": (I, [P, P]),
    "gbpa_operator_set_element_markers": (I, [P, P, P, I]),
    "gbpa_diffusion_mult_noalloc": (I, [P, I, I, I, I, I, P, P, P, P, P, P, P, P]),
    "gbpa_vec_dot": (I, [P, I64, P, P, ctypes.POINTER(D)]),
    "gbpa_vec_add": (I, [P, I64, P, D, P, P]),
    "gbpa_jacobi_setup": (I, [P, I64, P, P, I, D, P]),
    "gbpa_pcg_solve": (I, [P, P, P, P, D, D, I, I, ctypes.POINTER(SolveInfo)]),
    "gbpa_pcg_solve_mixed": (I, [P, P, P, P, P, D, D, I, I, ctypes.POINTER(SolveInfo)]),
    "gbpa_pcg_solve_mixed_reliable": (I, [P, P, P, P, P, D, D, I, ctypes.POINTER(SolveInfo)]),
    "gbpa_operator_mult_block": (I, [P, I, P, P]),
    "gbpa_pcg_solve_block": (I, [P, I, P, P, P, D, D, I, ctypes.POINTER(SolveInfo)]),
    "gbpa_pcg_solve_block_mixed": (I, [P, P, I, P, P, P, D, D, I, I, ctypes.POINTER(SolveInfo)]),
    "gbpa_pcg_solve_block_mixed_reliable": (I, [P, P, I, P, P, P, D, D, I, ctypes.POINTER(SolveInfo)]),
    "gbpa_batched_pcg_solve":(I, [P, I, ctypes.POINTER(ProblemDesc), D, D, I, P, P, P,
                                   ctypes.POINTER(D)]),
    "gbpa_batched_pcg_solve_precision": (I, [P, I, ctypes.POINTER(ProblemDesc), I, D, D, I, P, P, P,
                                             ctypes.POINTER(D)]),
    "gbpa_batched_pcg_solve_ex": (I, [P, I, ctypes.POINTER(ProblemDesc), I, I, D, D, I, P, P, P,
                                      ctypes.POINTER(D)]),
    "gbpa_vector_diffusion_setup3d": (I, [P, I, I, I, I, P, P, P, I64, P]),
    "gbpa_vector_diffusion_apply3d": (I, [P, I, I, I, I, P, P, P, P, P]),
    "gbpa_vector_diffusion_apply3d_coeff": (I, [P, I, I, I, I, I, P, P, P, P, P]),
    "gbpa_vector_mass_setup3d": (I, [P, I, I, I, I, P, P, P, I64, P]),
    "gbpa_vector_mass_apply3d": (I, [P, I, I, I, I, I, P, P, P, P]),
    "gbpa_domain_lf3d": (I, [P, I, I, I, P, P, P, P, I64, I, P, P, P]),
    "gbpa_ptransfer_create": (I, [P, I, I, I, P, P, P, I, I, P, P, P, P, I, ctypes.POINTER(P)]),
    "gbpa_ptransfer_destroy": (I, [P]),
    "gbpa_ptransfer_mult": (I, [P, P, P]),
    "gbpa_ptransfer_mult_transpose": (I, [P, P, P]),
    "gbpa_chebyshev_create": (I, [P, P, I, D, I, D, ctypes.c_ulonglong, ctypes.POINTER(P)]),
    "gbpa_chebyshev_destroy": (I, [P]),
    "gbpa_chebyshev_get_max_eig": (I, [P, ctypes.POINTER(D)]),
    "gbpa_chebyshev_mult": (I, [P, P, P]),
    "gbpa_multigrid_create": (I, [P, I, P, P, P, D, I, I, P, ctypes.POINTER(P)]),
    "gbpa_multigrid_destroy": (I, [P]),
    "gbpa_multigrid_mult": (I, [P, P, P]),
    "gbpa_pcg_solve_mg": (I, [P, P, P, P, D, D, I, ctypes.POINTER(SolveInfo)]),
    "gbpa_set_elements_per_block": (I, [I, I, I, I, I]),
    "gbpa_get_elements_per_block": (I, [I, I, I, I]),
    "gbpa_set_apply_layout": (I, [I, I, I, I, I, I]),
    "gbpa_get_apply_layout": (I, [I, I, I, I, ctypes.POINTER(I)]),
    "gbpa_set_block_apply_layout": (I, [I, I, I, I]),
    "gbpa_get_block_apply_layout": (I, [I, I, I]),
}

_lib = None


def load(path=LIB_PATH):
    """Load libgbpa.so and bind every exported symbol. Raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(
            f"libgbpa.so not found at {path}: build it first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(status, where):
    if status != 0:
        raise GbpaError(status, where)
    return status
