"""ctypes binding of libnla3d_gpu.so (include/nla3d_gpu.h).

The library is built in-tree by nla3d_gb300.build (``__graft_entry__.build()``).
There is no fallback: if the shared library is missing or cannot be loaded,
every entry point raises.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("NLA3D_GPU_LIB") or os.path.join(HERE, "libnla3d_gpu.so")

NLA3D_OK = 0
ERR_NAMES = {1: "NLA3D_ERR_ARG", 2: "NLA3D_ERR_CUDA", 3: "NLA3D_ERR_PATTERN",
             4: "NLA3D_ERR_NOMEM", 5: "NLA3D_ERR_RANGE", 6: "NLA3D_ERR_ELEMENT"}
PREC_FP64 = 0
PREC_MIXED = 1

# Every symbol declared in include/nla3d_gpu.h.
EXPORTS = [
    "nla3d_create", "nla3d_destroy", "nla3d_last_error", "nla3d_set_stream", "nla3d_get_stream",
    "nla3d_add_fix", "nla3d_add_rigid_body", "nla3d_build_pattern", "nla3d_init_solution_data",
    "nla3d_slot_maps", "nla3d_info",
    "nla3d_pattern", "nla3d_eq_numbers", "nla3d_set_U", "nla3d_set_U_device",
    "nla3d_update_results", "nla3d_assemble", "nla3d_get_K", "nla3d_get_F", "nla3d_device_K",
    "nla3d_device_F", "nla3d_synchronize", "nla3d_element_status", "nla3d_kernel_launches",
    "nla3d_set_timing", "nla3d_kernel_times", "nla3d_probe_fma_peak",
    "nla3d_assemble_solid81_noalloc",
    "nla3d_create_batch", "nla3d_mesh_count", "nla3d_mesh_add_fix", "nla3d_mesh_add_rigid_body",
    "nla3d_mesh_info", "nla3d_mesh_pattern", "nla3d_mesh_eq_numbers", "nla3d_get_K_all",
    "nla3d_set_launch_shape", "nla3d_autotune", "nla3d_graph_capture", "nla3d_graph_launch",
    "nla3d_mlp_gemm", "nla3d_mlp_tanh_backward", "nla3d_mlp_column_sum", "nla3d_mlp_adam",
    "nla3d_mlp_to_bf16", "nla3d_mlp_mse_grad", "nla3d_mlp_status", "nla3d_set_contrib_layout",
    "nla3d_block_mv", "nla3d_add_mpc", "nla3d_mesh_add_mpc", "nla3d_assemble_to_host",
    "nla3d_set_pattern_builder", "nla3d_pattern_on_device", "nla3d_add_surface_lines",
    "nla3d_set_transient", "nla3d_get_C", "nla3d_get_M",
    "nla3d_ldlt_analyze", "nla3d_ldlt_create", "nla3d_ldlt_factor", "nla3d_ldlt_solve",
    "nla3d_ldlt_solve_host", "nla3d_ldlt_order",
    "nla3d_ldlt_info", "nla3d_ldlt_last_error", "nla3d_ldlt_destroy", "nla3d_ldlt_tc_check",
]

NOALLOC_MAX_ELEMS = 15252


class NoAllocArgs(ctypes.Structure):
    """nla3d_solid81_noalloc_args: every pointer is device memory owned by the caller."""
    _fields_ = [
        ("n_elems", ctypes.c_uint32),
        ("n_nodes", ctypes.c_uint32),
        ("n_eq", ctypes.c_uint32),
        ("nnz", ctypes.c_uint64),
        ("xyz", ctypes.c_void_p),
        ("conn", ctypes.c_void_p),
        ("node_eq", ctypes.c_void_p),
        ("p_eq", ctypes.c_void_p),
        ("U", ctypes.c_void_p),
        ("k_ptr", ctypes.c_void_p),
        ("k_ids", ctypes.c_void_p),
        ("f_ptr", ctypes.c_void_p),
        ("f_ids", ctypes.c_void_p),
        ("mat_id", ctypes.c_int32),
        ("mat_c", ctypes.c_double * 5),
        ("K", ctypes.c_void_p),
        ("F", ctypes.c_void_p),
    ]


class MeshDesc(ctypes.Structure):
    _fields_ = [
        ("elem_type", ctypes.c_int32),
        ("n_nodes", ctypes.c_uint32),
        ("n_elems", ctypes.c_uint32),
        ("xyz", ctypes.c_void_p),
        ("conn", ctypes.c_void_p),
        ("mat_id", ctypes.c_int32),
        ("mat_c", ctypes.c_double * 5),
        ("elem_params", ctypes.c_void_p),
        ("n_elem_params", ctypes.c_int32),
    ]


class Nla3dError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERR_NAMES.get(code, code)}: {msg}")
        self.code = code


_lib = None


def load(path: str = LIB_PATH):
    """Load the shared library once; raise if it is not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
            " (the CUDA path has no fallback)")
    lib = ctypes.CDLL(path)
    P, U32, U64, I32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int32
    I64 = ctypes.c_int64
    sig = {
        "nla3d_create": ([ctypes.POINTER(MeshDesc), ctypes.c_int, ctypes.POINTER(P)], ctypes.c_int),
        "nla3d_destroy": ([P], ctypes.c_int),
        "nla3d_last_error": ([P], ctypes.c_char_p),
        "nla3d_set_stream": ([P, P], ctypes.c_int),
        "nla3d_get_stream": ([P], P),
        "nla3d_add_fix": ([P, U32, P, P], ctypes.c_int),
        "nla3d_add_rigid_body": ([P, U32, U32, P, U32, P], ctypes.c_int),
        "nla3d_build_pattern": ([P], ctypes.c_int),
        "nla3d_init_solution_data": ([P], ctypes.c_int),
        "nla3d_slot_maps": ([P, P, P], ctypes.c_int),
        "nla3d_info": ([P, P], ctypes.c_int),
        "nla3d_pattern": ([P, ctypes.c_int, P, P], ctypes.c_int),
        "nla3d_eq_numbers": ([P, P, P], ctypes.c_int),
        "nla3d_set_U": ([P, P, U64], ctypes.c_int),
        "nla3d_set_U_device": ([P, P, U64], ctypes.c_int),
        "nla3d_update_results": ([P], ctypes.c_int),
        "nla3d_assemble": ([P], ctypes.c_int),
        "nla3d_get_K": ([P, ctypes.c_int, P], ctypes.c_int),
        "nla3d_get_F": ([P, P], ctypes.c_int),
        "nla3d_device_K": ([P, ctypes.c_int, ctypes.POINTER(P), ctypes.POINTER(U64)], ctypes.c_int),
        "nla3d_device_F": ([P, ctypes.POINTER(P), ctypes.POINTER(U64)], ctypes.c_int),
        "nla3d_synchronize": ([P], ctypes.c_int),
        "nla3d_element_status": ([P, ctypes.POINTER(U32), ctypes.POINTER(U32)], ctypes.c_int),
        "nla3d_kernel_launches": ([P], U64),
        "nla3d_set_timing": ([P, ctypes.c_int], ctypes.c_int),
        "nla3d_kernel_times": ([P, P, ctypes.POINTER(U32)], ctypes.c_int),
        "nla3d_probe_fma_peak": ([ctypes.c_int, ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
        "nla3d_assemble_solid81_noalloc": ([ctypes.POINTER(NoAllocArgs), P, ctypes.POINTER(U32)],
                                           ctypes.c_int),
        "nla3d_create_batch": ([P, U32, ctypes.c_int, ctypes.POINTER(P)], ctypes.c_int),
        "nla3d_mesh_count": ([P], U32),
        "nla3d_mesh_add_fix": ([P, U32, U32, P, P], ctypes.c_int),
        "nla3d_mesh_add_rigid_body": ([P, U32, U32, U32, P, U32, P], ctypes.c_int),
        "nla3d_mesh_info": ([P, U32, P, P], ctypes.c_int),
        "nla3d_mesh_pattern": ([P, U32, ctypes.c_int, P, P], ctypes.c_int),
        "nla3d_mesh_eq_numbers": ([P, U32, P, P], ctypes.c_int),
        "nla3d_get_K_all": ([P, P], ctypes.c_int),
        "nla3d_set_launch_shape": ([P, ctypes.c_int, ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "nla3d_autotune": ([P, ctypes.c_int, P, ctypes.POINTER(ctypes.c_float)], ctypes.c_int),
        "nla3d_set_contrib_layout": ([P, ctypes.c_int], ctypes.c_int),
        "nla3d_add_mpc": ([P, ctypes.c_uint32, P, P, P, ctypes.c_double], ctypes.c_int),
        "nla3d_mesh_add_mpc": ([P, ctypes.c_uint32, ctypes.c_uint32, P, P, P, ctypes.c_double],
                               ctypes.c_int),
        "nla3d_assemble_to_host": ([P, ctypes.c_int, P, P, P, P], ctypes.c_int),
        "nla3d_set_pattern_builder": ([P, ctypes.c_int], ctypes.c_int),
        "nla3d_add_surface_lines": ([P, ctypes.c_uint32, P, P, P, P], ctypes.c_int),
        "nla3d_set_transient": ([P, ctypes.c_int], ctypes.c_int),
        "nla3d_get_C": ([P, ctypes.c_int, P], ctypes.c_int),
        "nla3d_get_M": ([P, ctypes.c_int, P], ctypes.c_int),
        "nla3d_ldlt_analyze": ([I64, P, P, P, P, P, P, P, P], ctypes.c_int),
        "nla3d_ldlt_create": ([I64, P, P, P, ctypes.c_int, P, P], ctypes.c_int),
        "nla3d_ldlt_factor": ([P, P], ctypes.c_int),
        "nla3d_ldlt_solve": ([P, P, P, P, ctypes.c_int, ctypes.c_double, P, P], ctypes.c_int),
        "nla3d_ldlt_solve_host": ([P, P, P, P, ctypes.c_int, ctypes.c_double, P, P],
                                  ctypes.c_int),
        "nla3d_ldlt_order": ([ctypes.c_int64, P, P, P, ctypes.c_int64, P], ctypes.c_int),
        "nla3d_ldlt_info": ([P, P], ctypes.c_int),
        "nla3d_ldlt_last_error": ([P], ctypes.c_char_p),
        "nla3d_ldlt_destroy": ([P], ctypes.c_int),
        "nla3d_ldlt_tc_check": ([ctypes.c_int, P], ctypes.c_int),
        "nla3d_pattern_on_device": ([P], ctypes.c_int),
        "nla3d_block_mv": ([P, ctypes.c_uint32, ctypes.c_int, ctypes.c_int, P, ctypes.c_double, P],
                           ctypes.c_int),
        "nla3d_graph_capture": ([P], ctypes.c_int),
        "nla3d_graph_launch": ([P], ctypes.c_int),
        "nla3d_mlp_gemm": ([ctypes.c_int, ctypes.c_int, ctypes.c_int, P, ctypes.c_int, I64, I64, P,
                            ctypes.c_int, I64, I64, P, I64, P, ctypes.c_int, P], ctypes.c_int),
        "nla3d_mlp_tanh_backward": ([P, P, I64, P], ctypes.c_int),
        "nla3d_mlp_column_sum": ([P, I64, I64, P, P], ctypes.c_int),
        "nla3d_mlp_adam": ([P, P, P, P, I64, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                            ctypes.c_float, ctypes.c_int, P, P], ctypes.c_int),
        "nla3d_mlp_to_bf16": ([P, P, I64, P], ctypes.c_int),
        "nla3d_mlp_mse_grad": ([P, P, P, I64, ctypes.c_float, P], ctypes.c_int),
        "nla3d_mlp_status": ([P], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    del I32
    _lib = lib
    return lib
