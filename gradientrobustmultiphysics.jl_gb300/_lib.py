"""ctypes binding of libgrmp_gpu.so (the C-ABI declared in include/grmp.h).

The library is built in-tree by build.py; loading fails loudly when it is
missing -- there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgrmp_gpu.so")

# status codes (grmp_status)
OK, ERR_INVALID_ARG, ERR_OUT_OF_MEMORY, ERR_DEVICE, ERR_NOT_CONVERGED = 0, 1, 2, 3, 4
ERR_UNSUPPORTED, ERR_BUDGET, ERR_TIMEOUT, ERR_NAN, ERR_NO_DEVICE = 5, 6, 7, 8, 9
ITEM_IDENTITY, ITEM_GRADIENT = 0, 1
STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "OUT_OF_MEMORY", 3: "DEVICE", 4: "NOT_CONVERGED",
                5: "UNSUPPORTED", 6: "BUDGET", 7: "TIMEOUT", 8: "NAN", 9: "NO_DEVICE"}

OP_LAPLACE, OP_MASS, OP_HOOKE, OP_RDIVRDIV, OP_STRUCTURAL, OP_JUMPGRAD = 1, 2, 3, 4, 5, 6
NL_DIFFUSION, NL_GRAD_DIFFUSION, NL_CONVECTION = 1, 2, 3
FP64, FP32, FP64_FP32 = 0, 1, 2
RHS_CONST, RHS_CELL, RHS_FOURIER, RHS_POLY = 0, 1, 2, 3
DIRICHLET_PENALTY, DIRICHLET_ELIMINATE = 0, 1
SOLVE_FP64, SOLVE_MIXED, SOLVE_DIRECT, SOLVE_MIXED_DIRECT, SOLVE_BICGSTAB = 0, 1, 2, 3, 4
NOALLOC_MAX_ROWS = 262144   # GRMP_NOALLOC_MAX_ROWS


class GrmpError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"grmp error {STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


class BilinearTerm(ctypes.Structure):
    _fields_ = [("op_kind", ctypes.c_int), ("symmetric", ctypes.c_int), ("factor", ctypes.c_double),
                ("cell_coef", ctypes.POINTER(ctypes.c_double)), ("param", ctypes.c_double * 4),
                ("bonus_quadorder", ctypes.c_int), ("coef_on_device", ctypes.c_int)]


class NonlinearTerm(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("factor", ctypes.c_double), ("param", ctypes.c_double * 4),
                ("bonus_quadorder", ctypes.c_int)]


class Rhs(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("ncomponents", ctypes.c_int), ("params", ctypes.POINTER(ctypes.c_double)),
                ("nparams", ctypes.c_int64), ("factor", ctypes.c_double), ("bonus_quadorder", ctypes.c_int),
                ("test_operator", ctypes.c_int), ("cell_group", ctypes.POINTER(ctypes.c_int32)),
                ("ngroups", ctypes.c_int32)]


class SolveParams(ctypes.Structure):
    _fields_ = [("abstol", ctypes.c_double), ("reltol", ctypes.c_double), ("maxiter", ctypes.c_int32),
                ("mode", ctypes.c_int32), ("inner_reltol", ctypes.c_double), ("max_outer", ctypes.c_int32),
                ("spmv_config", ctypes.c_int32), ("grid_blocks", ctypes.c_int32),
                ("use_initial_guess", ctypes.c_int32)]


class SolveStats(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("iterations", ctypes.c_int32), ("outer_iterations", ctypes.c_int32),
                ("spmv_config", ctypes.c_int32), ("grid_blocks", ctypes.c_int32),
                ("final_relres", ctypes.c_double), ("solve_ms", ctypes.c_double)]


class StokesBatchParams(ctypes.Structure):
    _fields_ = [("nproblems", ctypes.c_int32), ("row_offsets", ctypes.POINTER(ctypes.c_int32)),
                ("cell_offsets", ctypes.POINTER(ctypes.c_int32)), ("lam", ctypes.c_double),
                ("sweeps", ctypes.c_int32), ("sweep_tol", ctypes.c_double), ("mode", ctypes.c_int32),
                ("reltol", ctypes.c_double), ("inner_reltol", ctypes.c_double), ("maxiter", ctypes.c_int32),
                ("block_threads", ctypes.c_int32), ("split_penalty", ctypes.c_int32)]


class StokesBatchStats(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("max_iterations", ctypes.c_int32), ("total_iterations", ctypes.c_int64),
                ("max_sweeps", ctypes.c_int32), ("failed_problems", ctypes.c_int32), ("max_relres", ctypes.c_double),
                ("solve_ms", ctypes.c_double), ("fp64_fallbacks", ctypes.c_int32)]


class Request(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int), ("nverts", ctypes.c_int32), ("coords", ctypes.POINTER(ctypes.c_double)),
                ("ncells", ctypes.c_int32), ("cells", ctypes.POINTER(ctypes.c_int32)), ("fe_kind", ctypes.c_int),
                ("ncomponents", ctypes.c_int), ("ndofs", ctypes.c_int32),
                ("celldofs", ctypes.POINTER(ctypes.c_int32)), ("nterms", ctypes.c_int),
                ("terms", ctypes.POINTER(BilinearTerm)), ("rhs", Rhs), ("nfixed", ctypes.c_int32),
                ("fixed", ctypes.POINTER(ctypes.c_int32)), ("solve", SolveParams), ("mesh_key", ctypes.c_uint64)]


class RequestStats(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("slot", ctypes.c_int32), ("iterations", ctypes.c_int32),
                ("outer_iterations", ctypes.c_int32), ("final_relres", ctypes.c_double), ("queue_ms", ctypes.c_double),
                ("run_ms", ctypes.c_double), ("latency_ms", ctypes.c_double), ("solve_ms", ctypes.c_double),
                ("ndofs", ctypes.c_int32), ("resident", ctypes.c_int32)]


# every symbol of include/grmp.h with (argtypes, restype)
_vp = ctypes.c_void_p
_i32 = ctypes.c_int32
_pi32 = ctypes.POINTER(ctypes.c_int32)
_pd = ctypes.POINTER(ctypes.c_double)
SIGNATURES = {
    "grmp_version": ([], ctypes.c_int),
    "grmp_create_context": ([ctypes.c_int, ctypes.c_size_t, ctypes.POINTER(_vp)], ctypes.c_int),
    "grmp_destroy_context": ([_vp], ctypes.c_int),
    "grmp_last_error": ([_vp], ctypes.c_char_p),
    "grmp_context_stream": ([_vp, ctypes.POINTER(_vp)], ctypes.c_int),
    "grmp_synchronize": ([_vp], ctypes.c_int),
    "grmp_context_memory": ([_vp, ctypes.POINTER(ctypes.c_size_t)], ctypes.c_int),
    "grmp_context_launches": ([_vp, ctypes.POINTER(ctypes.c_uint64)], ctypes.c_int),
    "grmp_vector_device_ptr": ([_vp, ctypes.POINTER(_vp)], ctypes.c_int),
    "grmp_context_set_wait_limit": ([_vp, ctypes.c_int64], ctypes.c_int),
    "grmp_selftest_wait_timeout": ([_vp, ctypes.c_int64, _pi32, _pi32], ctypes.c_int),
    "grmp_mesh_upload": ([_vp, ctypes.c_int, _i32, _pd, _i32, _pi32, ctypes.POINTER(_vp)], ctypes.c_int),
    "grmp_mesh_set_faces": ([_vp, _i32, _pi32, _pd, _pd, ctypes.POINTER(ctypes.c_int8)], ctypes.c_int),
    "grmp_mesh_destroy": ([_vp], ctypes.c_int),
    "grmp_space_create": ([_vp, ctypes.c_int, ctypes.c_int, _pi32, _i32, ctypes.POINTER(_vp)], ctypes.c_int),
    "grmp_space_destroy": ([_vp], ctypes.c_int),
    "grmp_space_ndofs4cell": ([_vp, ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
    "grmp_space_create_on_device": ([_vp, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_vp), _pi32], ctypes.c_int),
    "grmp_mesh_build_faces": ([_vp], ctypes.c_int),
    "grmp_mesh_faces": ([_vp, _pi32, _pi32, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                         ctypes.POINTER(ctypes.c_int8)], ctypes.c_int),
    "grmp_space_celldofs": ([_vp, _pi32], ctypes.c_int),
    "grmp_space_boundary_dofs": ([_vp, _i32, _pi32, _pi32], ctypes.c_int),
    "grmp_reference_tables": ([ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                               ctypes.POINTER(ctypes.c_int), _pd, _pd, _pd, _pd], ctypes.c_int),
    "grmp_pattern_build": ([_vp, ctypes.c_int, ctypes.POINTER(BilinearTerm), ctypes.POINTER(_vp)], ctypes.c_int),
    "grmp_matrix_destroy": ([_vp], ctypes.c_int),
    "grmp_matrix_info": ([_vp, _pi32, ctypes.POINTER(ctypes.c_int64), _pi32], ctypes.c_int),
    "grmp_matrix_from_csc": ([_vp, _i32, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64), _pd,
                              ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.POINTER(_vp)], ctypes.c_int),
    "grmp_matrix_update_values": ([_vp, _pd], ctypes.c_int),
    "grmp_matrix_penalty_rows": ([_vp, _pi32], ctypes.c_int),
    "grmp_assemble_bilinear": ([_vp, ctypes.c_int, ctypes.POINTER(BilinearTerm), ctypes.c_int], ctypes.c_int),
    "grmp_assemble_nonlinear": ([_vp, _vp, _vp, ctypes.POINTER(NonlinearTerm), ctypes.c_int, ctypes.c_int],
                                ctypes.c_int),
    "grmp_item_face_jumps": ([_vp, _vp, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int, _pd, _pd],
                             ctypes.c_int),
    "grmp_matrix_download": ([_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int64), _pi32, _pd], ctypes.c_int),
    "grmp_assemble_linear": ([_vp, ctypes.POINTER(Rhs), _vp], ctypes.c_int),
    "grmp_item_l2error": ([_vp, _vp, _vp, ctypes.c_int, ctypes.POINTER(Rhs), ctypes.c_double, ctypes.c_int, _pd, _pd],
                          ctypes.c_int),
    "grmp_vector_create": ([_vp, _i32, ctypes.POINTER(_vp)], ctypes.c_int),
    "grmp_vector_destroy": ([_vp], ctypes.c_int),
    "grmp_vector_upload": ([_vp, _pd], ctypes.c_int),
    "grmp_vector_download": ([_vp, _pd], ctypes.c_int),
    "grmp_vector_fill": ([_vp, ctypes.c_double], ctypes.c_int),
    "grmp_apply_dirichlet": ([_vp, _vp, _i32, _pi32, _pd, ctypes.c_int, ctypes.c_double], ctypes.c_int),
    "grmp_solve_params_default": ([ctypes.POINTER(SolveParams)], ctypes.c_int),
    "grmp_solve": ([_vp, _vp, _vp, ctypes.POINTER(SolveParams), ctypes.POINTER(SolveStats)], ctypes.c_int),
    "grmp_spmv": ([_vp, ctypes.c_int, _vp, _vp], ctypes.c_int),
    "grmp_solve_fp64_noalloc": ([_vp, _vp, _vp, ctypes.POINTER(SolveParams), ctypes.POINTER(SolveStats)],
                                ctypes.c_int),
    "grmp_stokes_batch_solve": ([_vp, _vp, _vp, _vp, ctypes.POINTER(StokesBatchParams), _pi32,
                                 ctypes.POINTER(StokesBatchStats)], ctypes.c_int),
    "grmp_server_create": ([ctypes.c_int, ctypes.c_size_t, ctypes.c_int, ctypes.POINTER(_vp)], ctypes.c_int),
    "grmp_server_request_bytes": ([ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_size_t)], ctypes.c_int),
    "grmp_server_submit": ([_vp, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
    "grmp_server_wait": ([_vp, ctypes.c_int64, ctypes.c_double, _pd, ctypes.POINTER(RequestStats)], ctypes.c_int),
    "grmp_server_destroy": ([_vp], ctypes.c_int),
}

_lib = None


def load(path: str = LIB_PATH):
    """Load libgrmp_gpu.so and declare every C-ABI signature.  Raises when
    the library has not been built (no fallback exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libgrmp_gpu.so not built ({path}); run __graft_entry__.build() or build.py")
    lib = ctypes.CDLL(path)
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def check(rc: int, ctx=None):
    if rc != OK:
        msg = ""
        if ctx is not None and _lib is not None:
            m = _lib.grmp_last_error(ctx)
            msg = m.decode() if m else ""
        raise GrmpError(rc, msg)
