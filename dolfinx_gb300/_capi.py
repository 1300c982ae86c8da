"""ctypes binding of libdfxgpu.so (the C ABI declared in include/dfx_gpu.h).

The library is built in-tree (``dolfinx_gb300/_lib``). There is no CPU
fallback: if the shared library is missing, importing this module raises.
"""

from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libdfxgpu.so")

DFX_OK = 0
DFX_ERR_INVALID = 1
DFX_ERR_CUDA = 2
DFX_ERR_NOT_IN_SPARSITY = 3
DFX_ERR_NOT_CONVERGED = 4
DFX_ERR_TIMEOUT = 5
DFX_ERR_NO_MEMORY = 6
DFX_ERR_BREAKDOWN = 7
DFX_ERR_UNSUPPORTED = 8

FORM_POISSON = 0
FORM_ELASTICITY = 1
FORM_SOURCE = 2
FORM_BODYFORCE = 3
FORM_FACET_MASS = 4
FORM_FACET_JUMP = 5

MODE_ATOMIC = 0
MODE_COLOURED = 1

F64 = 0
F32 = 1
F32X2 = 2

IR_RESTART = 0
IR_RELIABLE = 1
IR_FLEXIBLE = 2


class DfxError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


class Form(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("degree", C.c_int32),
        ("num_cells", C.c_int32),
        ("num_nodes", C.c_int32),
        ("x_dofmap", C.c_void_p),
        ("x", C.c_void_p),
        ("dofmap", C.c_void_p),
        ("kappa", C.c_void_p),
        ("kappa_const", C.c_double),
        ("k2", C.c_double),
        ("nu", C.c_double),
        ("f", C.c_void_p),
        ("f_const", C.c_double * 3),
    ]


class Csr(C.Structure):
    _fields_ = [
        ("nrows", C.c_int32),
        ("ncols", C.c_int32),
        ("bs", C.c_int32),
        ("dtype", C.c_int32),
        ("nnz", C.c_int64),
        ("row_ptr", C.c_void_p),
        ("cols", C.c_void_p),
        ("vals", C.c_void_p),
    ]


class CgInfo(C.Structure):
    _fields_ = [
        ("iterations", C.c_int32),
        ("status", C.c_int32),
        ("rnorm0_sq", C.c_double),
        ("rnorm_sq", C.c_double),
        ("kernel_launches", C.c_int64),
    ]


class IrInfo(C.Structure):
    _fields_ = [
        ("outer_iterations", C.c_int32),
        ("inner_iterations", C.c_int32),
        ("status", C.c_int32),
        ("reserved", C.c_int32),
        ("rnorm0_sq", C.c_double),
        ("rnorm_sq", C.c_double),
        ("kernel_launches", C.c_int64),
    ]


class BatchSystem(C.Structure):
    _fields_ = [
        ("op32", C.c_void_p),
        ("op64", C.c_void_p),
        ("b", C.c_void_p),
        ("x", C.c_void_p),
        ("dinv", C.c_void_p),
        ("work", C.c_void_p),
        ("rtol", C.c_double),
        ("delta", C.c_double),
        ("max_iters", C.c_int32),
        ("mode", C.c_int32),
    ]


class Q4Mesh(C.Structure):
    _fields_ = [
        ("nx", C.c_int32),
        ("ny", C.c_int32),
        ("nz", C.c_int32),
        ("verts", C.c_void_p),
        ("kappa", C.c_double),
        ("edges32", C.c_void_p),
        ("geom32", C.c_void_p),
        ("geom64", C.c_void_p),
    ]


_P = C.c_void_p
_SIGS = {
    "dfx_last_error": (C.c_char_p, []),
    "dfx_abi_version": (C.c_int, []),
    "dfx_mesh_create_box_tet": (C.c_int, [C.c_int32] * 3 + [_P, _P, C.c_int32, _P, _P]),
    "dfx_mesh_dual_graph_tet": (C.c_int, [C.c_int32, _P, C.c_int32, _P, _P]),
    "dfx_graph_reorder_rcm": (C.c_int, [C.c_int32, _P, _P, _P]),
    "dfx_mesh_dual_graph_tet_device_workspace_bytes": (C.c_size_t, [C.c_int32, C.c_int32]),
    "dfx_mesh_dual_graph_tet_device": (C.c_int, [C.c_int32, _P, C.c_int32, _P, _P, _P,
                                                 C.c_size_t, _P]),
    "dfx_graph_reorder_rcm_device_workspace_bytes": (C.c_size_t, [C.c_int32]),
    "dfx_graph_reorder_rcm_device": (C.c_int, [C.c_int32, _P, _P, _P, _P, C.c_size_t, _P]),
    "dfx_mesh_create_box_tet_device_workspace_bytes": (C.c_size_t, [C.c_int32] * 4),
    "dfx_mesh_create_box_tet_device": (C.c_int, [C.c_int32] * 3 + [_P, _P, C.c_int32, _P, _P, _P,
                                                                   C.c_size_t, _P]),
    "dfx_dofmap_create_tet": (C.c_int, [C.c_int32, _P, C.c_int32, _P, _P]),
    "dfx_sparsity_create": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, _P, _P, _P, _P]),
    "dfx_sparsity_device_workspace_bytes": (C.c_size_t, [C.c_int32, C.c_int32, C.c_int32]),
    "dfx_sparsity_create_device": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, _P, _P, _P, _P, _P,
                                             C.c_size_t, _P]),
    "dfx_colour_cells": (C.c_int, [C.c_int32, C.c_int32, _P, C.c_int32, _P, _P, C.c_int32, _P]),
    "dfx_tabulate_dof_coordinates_tet": (C.c_int, [C.c_int32, _P, C.c_int32, _P, _P, C.c_int32,
                                                   C.c_int32, _P]),
    "dfx_exterior_facets_tet": (C.c_int, [C.c_int32, _P, _P, C.POINTER(C.c_int32)]),
    "dfx_interior_facets_tet": (C.c_int, [C.c_int32, _P, _P, C.POINTER(C.c_int32)]),
    "dfx_assemble_vector_facets": (C.c_int, [C.POINTER(Form), _P, C.c_int32, _P, _P]),
    "dfx_assemble_matrix_facets": (C.c_int, [C.POINTER(Form), _P, C.c_int32, C.POINTER(Csr), _P,
                                             _P, _P]),
    "dfx_assemble_scalar_workspace_bytes": (C.c_size_t, [C.c_int32]),
    "dfx_assemble_scalar": (C.c_int, [C.POINTER(Form), _P, C.POINTER(C.c_double), _P, C.c_size_t,
                                      _P]),
    "dfx_slot_map_bytes": (C.c_size_t, [C.POINTER(Form)]),
    "dfx_slot_map_create": (C.c_int, [C.POINTER(Form), C.POINTER(Csr), _P, _P]),
    "dfx_assemble_matrix": (C.c_int, [C.POINTER(Form), C.POINTER(Csr), _P, _P, C.c_int32, _P, _P,
                                      C.c_int32, _P]),
    "dfx_assemble_vector": (C.c_int, [C.POINTER(Form), _P, C.c_int32, _P, _P, C.c_int32, _P]),
    "dfx_apply_lifting": (C.c_int, [C.POINTER(Form), _P, _P, _P, _P, C.c_double, C.c_int32, _P, _P,
                                    C.c_int32, _P]),
    "dfx_set_bc": (C.c_int, [_P, C.c_int64, _P, C.c_int32, _P, C.c_double, _P, C.c_double, _P]),
    "dfx_set_diagonal": (C.c_int, [C.POINTER(Csr), _P, C.c_int32, C.c_double, _P]),
    "dfx_spmv": (C.c_int, [C.POINTER(Csr), _P, _P, C.c_double, _P]),
    "dfx_csr_values_to_f32": (C.c_int, [C.POINTER(Csr), _P, _P]),
    "dfx_csr_expand_blocks": (C.c_int, [C.POINTER(Csr), _P, _P, _P, _P]),
    "dfx_jacobi_inverse_diagonal": (C.c_int, [C.POINTER(Csr), _P, _P]),
    "dfx_inner_product_workspace_bytes": (C.c_size_t, [C.c_int64]),
    "dfx_inner_product": (C.c_int, [_P, _P, C.c_int64, _P, C.c_size_t, C.POINTER(C.c_double), _P]),
    "dfx_cg_workspace_bytes": (C.c_size_t, [C.c_int64]),
    "dfx_cg_solve": (C.c_int, [C.POINTER(Csr), _P, _P, _P, C.c_double, C.c_int32, C.c_int32, _P,
                               C.c_size_t, C.POINTER(CgInfo), _P]),
    "dfx_cg_solve_noalloc": (C.c_int, [C.POINTER(Csr), _P, _P, _P, C.c_double, C.c_int32,
                                       C.c_int32, C.POINTER(CgInfo), _P]),
    "dfx_tune_assembly": (C.c_int, [C.POINTER(Form), C.POINTER(Csr), _P, _P, C.c_int32, _P, _P,
                                    C.c_int32, _P, C.POINTER(C.c_int32), _P, _P]),
    "dfx_set_cells_per_block": (C.c_int, [C.POINTER(Form), C.c_int32, C.c_int32]),
    "dfx_get_cells_per_block": (C.c_int, [C.POINTER(Form), C.c_int32, C.POINTER(C.c_int32)]),
    "dfx_tune_spmv": (C.c_int, [C.POINTER(Csr), _P, _P, C.POINTER(C.c_int32), _P, _P]),
    "dfx_set_spmv_lanes": (C.c_int, [C.POINTER(Csr), C.c_int32]),
    "dfx_get_spmv_lanes": (C.c_int, [C.POINTER(Csr), C.POINTER(C.c_int32)]),
    "dfx_tune_clear": (C.c_int, []),
    "dfx_tune_export": (C.c_int, [_P, C.c_int64, C.POINTER(C.c_int64)]),
    "dfx_tune_import": (C.c_int, [_P, C.c_int64]),
    "dfx_timing_record": (C.c_int, [C.c_char_p, C.c_double]),
    "dfx_timing": (C.c_int, [C.c_char_p, C.POINTER(C.c_int32), C.POINTER(C.c_double)]),
    "dfx_timing_num_tasks": (C.c_int, [C.POINTER(C.c_int32)]),
    "dfx_timing_task": (C.c_int, [C.c_int32, C.c_char_p, C.c_int32, C.POINTER(C.c_int32),
                                  C.POINTER(C.c_int32), C.POINTER(C.c_double)]),
    "dfx_timing_clear": (C.c_int, []),
    "dfx_operator_create": (C.c_int, [C.POINTER(Csr), C.c_int32, C.c_int32, C.c_int32,
                                      C.POINTER(C.c_void_p), _P]),
    "dfx_operator_create_ex": (C.c_int, [C.POINTER(Csr), C.c_int32, C.c_int32, C.c_int32,
                                         C.c_int32, C.POINTER(C.c_void_p), _P]),
    "dfx_operator_update_values": (C.c_int, [_P, C.POINTER(Csr), _P]),
    "dfx_operator_apply": (C.c_int, [_P, _P, _P, _P]),
    "dfx_operator_apply_renumbered": (C.c_int, [_P, _P, _P, _P]),
    "dfx_operator_info": (C.c_int, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int32),
                                    C.POINTER(C.c_void_p)]),
    "dfx_operator_destroy": (C.c_int, [_P]),
    "dfx_operator_device_bytes": (C.c_int, [_P, C.POINTER(C.c_size_t)]),
    "dfx_operator_release_values": (C.c_int, [_P]),
    "dfx_operator_share": (C.c_int, [_P, C.POINTER(C.c_void_p)]),
    "dfx_operator_share_async": (C.c_int, [_P, C.c_void_p, C.POINTER(C.c_void_p)]),
    "dfx_operator_destroy_async": (C.c_int, [_P, C.c_void_p]),
    "dfx_operator_pool_trim": (C.c_int, []),
    "dfx_operator_permute": (C.c_int, [_P, _P, _P, C.c_int32, _P]),
    "dfx_batch_workspace_bytes": (C.c_size_t, [C.c_int64, C.c_int32]),
    "dfx_batch_create": (C.c_int, [C.c_int32, C.POINTER(C.c_void_p)]),
    "dfx_batch_destroy": (C.c_int, [_P]),
    "dfx_batch_set": (C.c_int, [_P, C.c_int32, C.POINTER(BatchSystem), _P]),
    "dfx_batch_clear": (C.c_int, [_P, C.c_int32]),
    "dfx_batch_step": (C.c_int, [_P, C.c_int32, C.POINTER(C.c_int32), _P]),
    "dfx_batch_info": (C.c_int, [_P, C.c_int32, C.POINTER(CgInfo), C.POINTER(C.c_int32),
                                 C.POINTER(C.c_int32)]),
    "dfx_cg_op_workspace_bytes": (C.c_size_t, [C.c_int64]),
    "dfx_cg_solve_op": (C.c_int, [_P, _P, _P, _P, C.c_double, C.c_int32, C.c_int32, _P,
                                  C.c_size_t, C.POINTER(CgInfo), _P]),
    "dfx_q4_num_dofs": (C.c_int64, [C.POINTER(Q4Mesh)]),
    "dfx_q4_action": (C.c_int, [C.POINTER(Q4Mesh), C.c_int32, _P, _P, _P]),
    "dfx_q4_action_tc": (C.c_int, [C.POINTER(Q4Mesh), _P, _P, _P]),
    "dfx_operator_set_chunk": (C.c_int, [_P, C.c_int32]),
    "dfx_set_cg_fused_update": (C.c_int, [C.c_int32]),
    "dfx_get_cg_fused_update": (C.c_int, [C.POINTER(C.c_int32)]),
    "dfx_selftest_grid_barrier": (C.c_int, [C.POINTER(C.c_int32)]),
    "dfx_dofmap_device_workspace_bytes": (C.c_size_t, [C.c_int32, C.c_int32, C.c_int32]),
    "dfx_dofmap_create_tet_device": (C.c_int, [C.c_int32, _P, C.c_int32, C.c_int32, _P, _P, _P,
                                               C.c_size_t, _P]),
    "dfx_assemble_vector_interior_facets": (C.c_int, [C.POINTER(Form), _P, C.c_int32, _P, _P]),
    "dfx_assemble_matrix_interior_facets": (C.c_int, [C.POINTER(Form), _P, C.c_int32,
                                                      C.POINTER(Csr), _P, _P]),
    "dfx_apply_lifting_facets": (C.c_int, [C.POINTER(Form), _P, C.c_int32, C.c_int32, _P, _P,
                                           _P, _P, C.c_double, _P]),
    "dfx_q4_tc_check": (C.c_int, [_P]),
    "dfx_q4_edges": (C.c_int, [C.POINTER(Q4Mesh), _P, _P]),
    "dfx_q4_geometry": (C.c_int, [C.POINTER(Q4Mesh), C.c_int32, _P, _P]),
    "dfx_q4_cg_workspace_bytes": (C.c_size_t, [C.c_int64, C.c_int32]),
    "dfx_q4_cg_solve": (C.c_int, [C.POINTER(Q4Mesh), _P, _P, C.c_double, C.c_int32, C.c_int32,
                                  C.c_double, C.c_int32, _P, C.c_size_t, C.POINTER(CgInfo), _P]),
    "dfx_ir_workspace_bytes": (C.c_size_t, [C.c_int64]),
    "dfx_ir_solve": (C.c_int, [_P, _P, _P, _P, _P, C.c_double, C.c_double, C.c_int32, C.c_int32,
                               C.c_int32, C.c_int32, _P, C.c_size_t, C.POINTER(IrInfo), _P]),
}

_lib = None


def lib():
    """The loaded libdfxgpu.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build the CUDA extension first "
                "(python -c 'import __graft_entry__ as g; g.build()'); there is no CPU fallback")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != DFX_OK:
        msg = lib().dfx_last_error().decode(errors="replace")
        raise DfxError(rc, msg or f"dfx error {rc}")


def declared_symbols(header: str | None = None) -> list[str]:
    """Function names declared in include/dfx_gpu.h."""
    import re

    if header is None:
        header = os.path.join(os.path.dirname(_HERE), "include", "dfx_gpu.h")
    text = open(header).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dfx_[a-z0-9_]+)\s*\(", text)))
