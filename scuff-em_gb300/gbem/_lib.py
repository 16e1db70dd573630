"""ctypes binding of the C ABI in include/gbem.h (libgbem.so, built in-tree).

Loading fails loudly if the CUDA library is missing: there is no CPU path.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(_HERE, "libgbem.so")

GBEM_OK, GBEM_EINVAL, GBEM_ENOMEM, GBEM_ECUDA, GBEM_ENOTSUP, GBEM_ESINGULAR, GBEM_ENOCONV, GBEM_EMESH, GBEM_ETIMEOUT = range(9)
C128, C64, F64 = 0, 1, 2
PREC_FP64, PREC_MIXED = 0, 1

STATUS_NAMES = {0: "GBEM_OK", 1: "GBEM_EINVAL", 2: "GBEM_ENOMEM", 3: "GBEM_ECUDA", 4: "GBEM_ENOTSUP",
                5: "GBEM_ESINGULAR", 6: "GBEM_ENOCONV", 7: "GBEM_EMESH", 8: "GBEM_ETIMEOUT"}

#: every symbol include/gbem.h declares
EXPORTS = [
    "gbem_vertex_vjp_region", "gbem_power_emt_grad", "gbem_solve_refined", "gbem_lu_log_abs_det", "gbem_lu_tuning", "gbem_assemble_block_packed_host", "gbem_sp_factor_host", "gbem_sp_solve_host",
    "gbem_last_error", "gbem_version", "gbem_geometry_create", "gbem_geometry_destroy", "gbem_geometry_num_bfs",
    "gbem_geometry_edges", "gbem_geometry_near_counts", "gbem_matrix_create", "gbem_matrix_destroy",
    "gbem_matrix_device_ptr", "gbem_matrix_download", "gbem_matrix_upload", "gbem_assemble", "gbem_assemble_host",
    "gbem_lu_factor", "gbem_lu_solve", "gbem_lu_factor_host", "gbem_lu_solve_host", "gbem_solve_mixed",
    "gbem_rhs_planewave", "gbem_solve_mixed_device", "gbem_stats", "gbem_geometry_set_stream",
    "gbem_lu_solve_noalloc", "gbem_assemble_block", "gbem_assemble_block_host",
    "gbem_assemble_block_gradient", "gbem_assemble_block_gradient_host", "gbem_power_emt",
    "gbem_lu_trace", "gbem_lu_trace_host", "gbem_assemble_block_dmdt", "gbem_assemble_block_dmdt_host",
    "gbem_solve_mixed_batch", "gbem_vertex_vjp_matrix", "gbem_vertex_vjp_rhs_planewave",
    "gbem_geometry_num_vertices", "gbem_cache_preload", "gbem_cache_store", "gbem_cache_clear", "gbem_cache_size",
    "gbem_cache_lookup_stats",
]


class GbemError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), msg))
        self.status = status


class SurfaceDesc(ctypes.Structure):
    _fields_ = [("num_vertices", ctypes.c_int), ("vertices", ctypes.c_void_p), ("num_panels", ctypes.c_int),
                ("panel_vertices", ctypes.c_void_p), ("exterior_region", ctypes.c_int),
                ("interior_region", ctypes.c_int), ("is_pec", ctypes.c_int)]


class BatchJob(ctypes.Structure):
    _fields_ = [("g", ctypes.c_void_p), ("omega_re", ctypes.c_double), ("omega_im", ctypes.c_double),
                ("eps", ctypes.c_void_p), ("mu", ctypes.c_void_p), ("nrhs", ctypes.c_int), ("B", ctypes.c_void_p),
                ("ldb", ctypes.c_int), ("X", ctypes.c_void_p), ("ldx", ctypes.c_int), ("tol", ctypes.c_double),
                ("max_iter", ctypes.c_int), ("iters", ctypes.c_int), ("resid", ctypes.c_double),
                ("status", ctypes.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIBPATH):
            raise ImportError("libgbem.so is not built (run __graft_entry__.build()); there is no CPU fallback")
        L = ctypes.CDLL(LIBPATH)
        P, I, D, V = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, None
        sig = {
            "gbem_last_error": ([], ctypes.c_char_p), "gbem_version": ([], ctypes.c_char_p),
            "gbem_geometry_create": ([I, P, I, I, P], I), "gbem_geometry_destroy": ([P], I),
            "gbem_geometry_num_bfs": ([P, P], I), "gbem_geometry_edges": ([P, I, P, P, P], I),
            "gbem_geometry_near_counts": ([P, P], I), "gbem_matrix_create": ([P, I, P], I),
            "gbem_matrix_destroy": ([P], I), "gbem_matrix_device_ptr": ([P, P, P], I),
            "gbem_matrix_download": ([P, P, I], I), "gbem_matrix_upload": ([P, P, I], I),
            "gbem_assemble": ([P, D, D, P, P, I, P], I), "gbem_assemble_host": ([P, D, D, P, P, P, I], I),
            "gbem_lu_factor": ([P, P, P], I), "gbem_lu_solve": ([P, ctypes.c_char, I, P, I], I),
            "gbem_lu_factor_host": ([P, I, I, P, P], I), "gbem_lu_solve_host": ([P, I, I, P, ctypes.c_char, I, P, I], I),
            "gbem_solve_mixed": ([P, D, D, P, P, I, P, I, P, I, D, I, P, P], I),
            "gbem_rhs_planewave": ([P, D, D, P, P, P, P, P], I),
            "gbem_solve_mixed_device": ([P, D, D, P, P, I, P, I, P, I, D, I, P, P], I),
            "gbem_stats": ([I, P, P], I), "gbem_geometry_set_stream": ([P, P], I),
            "gbem_lu_solve_noalloc": ([P, ctypes.c_char, I, P, I], I),
            "gbem_lu_log_abs_det": ([P, P], I),
            "gbem_lu_tuning": ([I, P, I], I),
            "gbem_solve_refined": ([P, D, D, P, P, I, P, I, P, I, D, I, P, P], I),
            "gbem_vertex_vjp_region": ([P, D, D, P, P, I, I, P, I, P, I, D, P], I),
            "gbem_power_emt_grad": ([P, D, D, P, P, I, P, I, P, I], I),
            "gbem_assemble_block_packed_host": ([P, I, D, D, P, P, P, I], I),
            "gbem_sp_factor_host": ([P, I, I, P, P], I),
            "gbem_sp_solve_host": ([P, I, I, P, I, P, I], I),
            "gbem_assemble_block": ([P, I, I, D, D, P, P, I, P, I, I, I, I], I),
            "gbem_assemble_block_host": ([P, I, I, D, D, P, P, P, I, I, I, I], I),
            "gbem_assemble_block_gradient": ([P, I, I, D, D, P, P, P, P, P, I, I, I, I], I),
            "gbem_assemble_block_gradient_host": ([P, I, I, D, D, P, P, P, P, P, I, I, I, I], I),
            "gbem_power_emt": ([P, D, D, P, P, I, I, P, I, P, I, P, P], I),
            "gbem_lu_trace": ([P, P, I, P], I),
            "gbem_solve_mixed_batch": ([I, P, I], I),
            "gbem_assemble_block_dmdt": ([P, I, I, D, D, P, P, I, P, P, I, I, I, I], I),
            "gbem_assemble_block_dmdt_host": ([P, I, I, D, D, P, P, I, P, P, I, I, I, I], I),
            "gbem_lu_trace_host": ([P, P, I, I, P], I),
            "gbem_vertex_vjp_matrix": ([P, D, D, P, P, I, P, I, P, I, D, P], I),
            "gbem_vertex_vjp_rhs_planewave": ([P, D, D, P, P, I, P, P, P, I, P], I),
            "gbem_geometry_num_vertices": ([P, P], I),
            "gbem_cache_preload": ([ctypes.c_char_p], I), "gbem_cache_store": ([ctypes.c_char_p], I),
            "gbem_cache_clear": ([], I), "gbem_cache_size": ([P], I), "gbem_cache_lookup_stats": ([P, P, P], I),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def check(status):
    if status != GBEM_OK:
        raise GbemError(status, lib().gbem_last_error().decode())
    return status
