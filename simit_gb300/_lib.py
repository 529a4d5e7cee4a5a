"""ctypes binding of libsimit_gb300.so (the C ABI in include/simit_gb300.h).

The library is built in-tree by simit_gb300/build.py.  There is no CPU
fallback: if the library or a GPU is missing, loading fails loudly.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsimit_gb300.so")

P = ctypes.c_void_p
I32 = ctypes.c_int32
I64 = ctypes.c_int64
D = ctypes.c_double
F32, F64 = 0, 1
ERR_ARG, ERR_CUDA, ERR_UNSUPPORTED, ERR_DEVICE, ERR_STATE = -1, -2, -3, -4, -5


class SimitError(RuntimeError):
    """A negative status from the C ABI (the analogue of SimitException)."""

    def __init__(self, code, msg):
        super().__init__("simit_gb300 error %d: %s" % (code, msg))
        self.code = code


class Mesh(ctypes.Structure):
    """sg_mesh"""
    _fields_ = [("n", I32), ("card", I32), ("nE", I64), ("endpoints", P), ("ve_ptr", P),
                ("ve_idx", P), ("rowptr", P), ("colidx", P), ("nnzb", I64), ("maxrow", I32),
                ("slots", P), ("color_order", P), ("color_ptr", P), ("ncolors", I32),
                ("slot_src_ptr", P), ("slot_src", P), ("asm_tile", I32)]


class Matrix(ctypes.Structure):
    """sg_matrix"""
    _fields_ = [("n", I32), ("bs", I32), ("nnzb", I64), ("rowptr", P), ("colidx", P),
                ("dtype", ctypes.c_int), ("vals", P)]


class SolveOpts(ctypes.Structure):
    """sg_solve_opts"""
    _fields_ = [("precision", ctypes.c_int), ("precond", ctypes.c_int), ("stop", ctypes.c_int),
                ("tol", D), ("maxiters", I32), ("verify", I32), ("check_every", I32),
                ("reliable_delta", D), ("lanes", I32), ("batch", I32), ("learned_params", P),
                ("learned_form", I32), ("storage", I32), ("pdl", I32), ("learned_exec", I32)]


class SolveResult(ctypes.Structure):
    """sg_solve_result"""
    _fields_ = [("status", I32), ("iters", I32), ("checks", I32), ("fallbacks", I32),
                ("normr2", D), ("true_normr2", D), ("bnorm2", D), ("kernels", I64)]


SOLVE_F64, SOLVE_MIXED = 0, 1
MPNN_RELU, MPNN_LINEAR, MPNN_SYM = 0, 1, 2
MPNN_EXEC_FOLDED, MPNN_EXEC_LAYERED, MPNN_EXEC_FOLDED_F32 = 0, 1, 2
STORAGE_FULL, STORAGE_SYMMETRIC = 0, 1
RESIDUAL_FP64, RESIDUAL_COMPENSATED = 0, 1
INCIDENCE_EV, INCIDENCE_VE = 0, 1
PRECOND_NONE, PRECOND_JACOBI, PRECOND_BLOCK_JACOBI, PRECOND_LEARNED = 0, 1, 2, 3
STOP_NORMR2, STOP_NORMR, STOP_RELATIVE = 0, 1, 2
STATUS = {1: "converged", 2: "maxiter", 3: "breakdown", 4: "nan"}
MODEL_LINEAR, MODEL_NEOHOOKEAN = 0, 1
MAX_COLORS = 128
LANES_AUTOTUNE = 1000

_MP = ctypes.POINTER(Mesh)
_CI = ctypes.c_int

# name -> (restype, argtypes)
SIGNATURES = {
    "sg_ctx_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(P)]),
    "sg_ctx_destroy": (ctypes.c_int, [P]),
    "sg_ctx_sync": (ctypes.c_int, [P]),
    "sg_ctx_stream": (P, [P]),
    "sg_last_error": (ctypes.c_char_p, []),
    "sg_version": (ctypes.c_char_p, []),
    "sg_incidence_build": (ctypes.c_int, [P, I32, P, I64, I32, P, P]),
    "sg_pattern_count": (ctypes.c_int, [P, I32, P, I64, I32, P, P, P, ctypes.POINTER(I64)]),
    "sg_pattern_fill": (ctypes.c_int, [P, I32, P, I64, I32, P, P, P, P]),
    "sg_slots_build": (ctypes.c_int, [P, I32, P, I64, I32, P, P, P]),
    "sg_element_coloring": (ctypes.c_int, [P, ctypes.POINTER(Mesh), P, P, ctypes.POINTER(I32)]),
    "sg_slot_sources": (ctypes.c_int, [P, ctypes.POINTER(Mesh), P, P]),
    "sg_tune_spmv": (_CI, [P, ctypes.POINTER(Matrix), _CI, _CI, _CI, ctypes.POINTER(I32),
                           ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                           ctypes.POINTER(I32), P, P, I32]),
    "sg_bspmv": (ctypes.c_int, [P, I32, I32, P, P, ctypes.c_int, P, ctypes.c_int, P, P, I32]),
    "sg_dot": (ctypes.c_int, [P, I64, ctypes.c_int, P, P, ctypes.POINTER(D)]),
    "sg_fp64_fma_rate": (ctypes.c_int, [P, ctypes.POINTER(D)]),
    "sg_assemble_cloth_stretch": (ctypes.c_int, [P, P, ctypes.c_int, P, P, P, P]),
    "sg_assemble_cloth_bend": (ctypes.c_int, [P, P, ctypes.c_int, P, P, P, P, P]),
    "sg_axpy": (ctypes.c_int, [P, I64, ctypes.c_int, D, P, P]),
    "sg_residual": (_CI, [P, ctypes.POINTER(Matrix), P, P, P, ctypes.POINTER(D), _CI]),
    "sg_incidence_pattern": (_CI, [P, _CI, I32, I64, I32, P, P, P, P]),
    "sg_assemble_incidence": (_CI, [P, _CI, I64, I32, P, P, _CI, I32, P, P]),
    "sg_pattern_rect": (_CI, [P, I32, I32, I64, I32, I32, P, P, P, P, P, ctypes.POINTER(I64)]),
    "sg_assemble_rect": (_CI, [P, I32, I32, I32, P, P, P, P, P, _CI, I32, P, P]),
    "sg_jit_check_source": (_CI, [ctypes.c_char_p, I32, I32, _CI, I32, ctypes.c_char_p, I64]),
    "sg_jit_assembly_create": (_CI, [P, ctypes.c_char_p, I32, I32, _CI, I32, ctypes.POINTER(P)]),
    "sg_jit_assemble": (_CI, [P, _MP, P, I32, P]),
    "sg_jit_check_vector_source": (_CI, [ctypes.c_char_p, I32, I32, _CI, I32, ctypes.c_char_p,
                                         I64]),
    "sg_jit_vector_create": (_CI, [P, ctypes.c_char_p, I32, I32, _CI, I32, ctypes.POINTER(P)]),
    "sg_jit_assemble_vector": (_CI, [P, _MP, P, I32, P]),
    "sg_jit_assembly_destroy": (_CI, [P]),
    "sg_bsr_add_diag": (_CI, [P, I32, I32, P, P, I64, _CI, P, D, D, P, P]),
    "sg_symbsr_create": (_CI, [P, I32, P, P, I64, I32, ctypes.POINTER(P)]),
    "sg_symbsr_fill": (_CI, [P, P]),
    "sg_symbsr_spmv": (_CI, [P, P, P]),
    "sg_symbsr_destroy": (_CI, [P]),
    "sg_pattern_maxrow": (_CI, [P, I32, P, ctypes.POINTER(I32)]),
    "sg_assemble_springs": (_CI, [P, _MP, _CI, _CI, P, P, P, P, P, P, D, D, P, P, P, _CI]),
    "sg_assemble_scalar_springs": (_CI, [P, _MP, _CI, P, D, D, P, _CI]),
    "sg_assemble_blocks": (_CI, [P, _MP, _CI, _CI, P, P, _CI]),
    "sg_hilbert_order": (_CI, [_CI, P, _CI, P]),
    "sg_morton_order": (_CI, [_CI, P, _CI, P]),
    "sg_element_order": (_CI, [_CI, _CI, P, P]),
    "sg_hilbert_index": (_CI, [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _CI, P]),
    "sg_tet_precompute": (_CI, [P, _MP, _CI, P, D, P, P, P]),
    "sg_assemble_tet_stiffness": (_CI, [P, _MP, _CI, _CI, P, P, P, P, P, P, D, D, P, _CI]),
    "sg_assemble_tet_force": (_CI, [P, _MP, _CI, _CI, P, P, P, P, P, P, P, D, D, P, P, _CI]),
    "sg_assemble_heat": (_CI, [P, _MP, _CI, P, P, P, D, P, P, P, _CI]),
    "sg_solver_create": (_CI, [P, ctypes.POINTER(Matrix), ctypes.POINTER(SolveOpts),
                               ctypes.POINTER(P)]),
    "sg_solver_solve": (_CI, [P, P, P, ctypes.POINTER(SolveResult)]),
    "sg_solver_solve_ex": (_CI, [P, P, _CI, P, _CI, ctypes.POINTER(SolveResult)]),
    "sg_solver_destroy": (_CI, [P]),
    "sg_solver_refresh": (_CI, [P]),
    "sg_dot_noalloc": (_CI, [P, I64, _CI, P, P, P]),
    "sg_batched_pcg": (_CI, [P, I32, P, P, ctypes.POINTER(Matrix), P, P, D, I32, I32, P, P, P]),
    "sg_batched_configs": (_CI, []),
    "sg_mpnn_nparams": (_CI, []),
    "sg_mpnn_graph_create": (_CI, [P, ctypes.POINTER(Matrix), ctypes.POINTER(P)]),
    "sg_mpnn_graph_refresh": (_CI, [P]),
    "sg_mpnn_graph_set_form": (_CI, [P, _CI]),
    "sg_mpnn_graph_set_exec": (_CI, [P, _CI]),
    "sg_mpnn_fold_step": (_CI, [P, I32]),
    "sg_mpnn_graph_destroy": (_CI, [P]),
    "sg_mpnn_forward": (_CI, [P, P, P, P, _CI]),
    "sg_mpnn_backward": (_CI, [P, P, P, P]),
    "sg_mpnn_loss": (_CI, [P, P, P, D, P, ctypes.POINTER(D)]),
    "sg_mpnn_adam": (_CI, [P, P, P, P, P, _CI, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                           ctypes.c_float]),
    "sg_solve": (_CI, [P, ctypes.POINTER(Matrix), ctypes.POINTER(SolveOpts), P, P,
                       ctypes.POINTER(SolveResult)]),
}

_lib = None


def load(path=LIB_PATH):
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError("simit_gb300: %s is missing; run simit_gb300/build.py "
                               "(or __graft_entry__.build()) first" % path)
        L = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            if hasattr(L, name):
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
        _lib = L
    return _lib


def exported_symbols():
    """Names declared in SIGNATURES that the loaded library exports."""
    L = load()
    return [n for n in SIGNATURES if hasattr(L, n)]


def check(rc):
    if rc != 0:
        raise SimitError(rc, load().sg_last_error().decode())
    return rc


def call(name, *args):
    return check(getattr(load(), name)(*args))
