"""ctypes bindings of the native libraries (include/afm.h, include/afm_problems.h).

The libraries are built in-tree by amat_gb300.build. Loading fails loudly when
they are missing: there is no Python or CPU stand-in for the operator.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIBAFM_PATH = os.path.join(HERE, "libafm.so")
LIBPROBLEMS_PATH = os.path.join(HERE, "libafm_problems.so")

# afm_status (include/afm.h)
STATUS = {
    0: "SUCCESS", 1: "INDEX_OUT_OF_BOUNDS", 2: "UNKNOWN_ELEMENT_TYPE", 3: "UNKNOWN_ELEMENT_STATUS",
    4: "NULL_L2G_MAP", 5: "GHOST_NODE_NOT_FOUND", 6: "UNKNOWN_MAT_TYPE", 7: "WRONG_COMMUNICATION",
    8: "UNKNOWN_DOF_TYPE", 9: "UNKNOWN_CONSTRAINT", 10: "UNKNOWN_BC_METH", 11: "NOT_IMPLEMENTED",
    12: "GLOBAL_DOF_ID_NOT_FOUND", 100: "ERR_CUDA", 101: "ERR_OOM", 102: "ERR_TIMEOUT", 103: "ERR_BREAKDOWN",
    104: "ERR_STATE", 105: "ERR_INVALID_ARG", 106: "ERR_MAXIT", 107: "ERR_INTERNAL",
}


class AfmInfo(C.Structure):
    _fields_ = [
        ("n_elements", C.c_uint32), ("n_dofs", C.c_uint32), ("n_colors", C.c_uint32),
        ("max_dofs_per_element", C.c_uint32), ("precision", C.c_int), ("ke_bytes", C.c_uint64),
        ("map_bytes", C.c_uint64), ("algorithmic_bytes", C.c_uint64), ("algorithmic_flops", C.c_double),
        ("n_launches", C.c_uint32), ("device", C.c_int), ("n_patches", C.c_uint32),
        ("n_patch_colors", C.c_uint32), ("patch_index_bytes", C.c_uint64), ("ke_symmetric", C.c_int),
        ("sym_available", C.c_int), ("sym_bytes", C.c_uint64), ("csr_nnz", C.c_uint64),
        ("work_bytes", C.c_uint64),
    ]


class AfmSolveStats(C.Structure):
    _fields_ = [
        ("iterations", C.c_int), ("status", C.c_int), ("rel_residual", C.c_double),
        ("residual_norm", C.c_double), ("seconds", C.c_double), ("refinements", C.c_int),
    ]


class AfmServerInfo(C.Structure):
    _fields_ = [
        ("lane_launches", C.c_uint64), ("lane_solve_launches", C.c_uint64), ("lane_max_batch", C.c_uint32),
        ("reserved", C.c_uint32), ("lane_requests", C.c_uint64), ("stream_requests", C.c_uint64),
    ]


class AfmMesh(C.Structure):
    _fields_ = [
        ("n_nodes", C.c_uint32), ("n_elem", C.c_uint32), ("nodes_per_elem", C.c_uint32),
        ("nx", C.c_uint32), ("ny", C.c_uint32), ("nz", C.c_uint32),
        ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
        ("coords", C.POINTER(C.c_double)), ("elem_nodes", C.POINTER(C.c_uint32)),
        ("lattice", C.POINTER(C.c_uint32)),
    ]




def _header_define(name):
    """Value of an integer #define of include/afm.h (the header is the one statement of such limits)."""
    import re
    with open(os.path.join(os.path.dirname(HERE), "include", "afm.h")) as f:
        m = re.search(r"^#define\s+%s\s+(\d+)u?\s*$" % name, f.read(), re.M)
    if not m:
        raise RuntimeError("include/afm.h defines no %s" % name)
    return int(m.group(1))


# largest operator of afm_solve_cg_device_noalloc
NOALLOC_MAX_DOFS = _header_define("AFM_NOALLOC_MAX_DOFS")

P = C.c_void_p
U32 = C.c_uint32
U64 = C.c_uint64
I = C.c_int
D = C.c_double

# name -> (restype, argtypes); every symbol include/afm.h declares
AFM_SIGNATURES = {
    "afm_create": (I, [C.POINTER(P), I, I]),
    "afm_destroy": (I, [P]),
    "afm_set_matfree_type": (I, [P, I]),
    "afm_set_precision": (I, [P, I]),
    "afm_set_patch_mode": (I, [P, I]),
    "afm_set_symmetric_inner": (I, [P, I]),
    "afm_set_fused_colours": (I, [P, I]),
    "afm_set_wait_limit": (I, [P, D]),
    "afm_set_wait_probe": (I, [P, I]),
    "afm_set_element_kind": (I, [P, I, D, D, U32]),
    "afm_set_element_coords": (I, [P, U32, U32, P]),
    "afm_assemble_csr_host": (I, [U32, U32, P, P, P, P, U32, I, I, P, P, P, P]),
    "afm_assemble": (I, [P, I]),
    "afm_matvec_assembled_device": (I, [P, P, P, P]),
    "afm_get_assembled_csr": (I, [P, P, P, P, P]),
    "afm_server_create": (I, [P, I, U64, U32]),
    "afm_server_submit": (I, [P, P, P, D, D, P]),
    "afm_server_poll": (I, [P, P, P]),
    "afm_server_take": (I, [P, U64, P, P, P, P]),
    "afm_server_destroy": (I, [P]),
    "afm_server_set_lane": (I, [P, U64, U32]),
    "afm_get_solve_trace": (I, [P, U32, P, P, P]),
    "afm_debug_segment_geometry": (I, [I, U32, P]),
    "afm_server_get_info": (I, [P, P]),
    "afm_server_set_inner_format": (I, [P, I]),
    "afm_server_set_priorities": (I, [P, I]),
    "afm_patch_plan_host_matvec": (I, [U32, U32, P, P, P, P, P, P, P]),
    "afm_set_map": (I, [P, U32, P, U32, P, U32, P, U64, U64, U64]),
    "afm_set_bdr_map": (I, [P, P, P, U32]),
    "afm_set_element_matrix": (I, [P, U32, P, U32, U32, U32]),
    "afm_set_element_matrices": (I, [P, U32, U32, P]),
    "afm_finalize": (I, [P]),
    "afm_matvec": (I, [P, P, P, I]),
    "afm_matvec_device": (I, [P, P, P, P]),
    "afm_matvec_device_f32": (I, [P, P, P, P]),
    "afm_matvec_inner_device": (I, [P, P, P, P]),
    "afm_matmult_bc": (I, [P, P, P]),
    "afm_matmult_bc_device": (I, [P, P, P, P]),
    "afm_get_diagonal": (I, [P, P]),
    "afm_apply_bc_rhs": (I, [P, P]),
    "afm_get_trace": (I, [P, P]),
    "afm_solve_cg": (I, [P, P, P, D, D, I, I, P]),
    "afm_solve_cg_device": (I, [P, P, P, D, D, I, I, P]),
    "afm_solve_cg_device_noalloc": (I, [P, P, P, D, D, I, I, P]),
    "afm_solve_cg_mixed": (I, [P, P, P, D, D, I, D, I, P]),
    "afm_solve_cg_mixed_device": (I, [P, P, P, D, D, I, D, I, P]),
    "afm_matmult_bc_device_f32": (I, [P, P, P, P]),
    "afm_matvec_batched_device": (I, [P, P, P, U32, U32, P]),
    "afm_matvec_batched_device_f32": (I, [P, P, P, U32, U32, P]),
    "afm_matmult_bc_batched_device": (I, [P, P, P, U32, U32, P]),
    "afm_matmult_bc_batched_device_f32": (I, [P, P, P, U32, U32, P]),
    "afm_get_batch_tuning": (I, [P, U32, U32, I, P, P, P]),
    "afm_set_batch_tuning": (I, [P, U32, U32, I, I, I]),
    "afm_solve_cg_batched_device": (I, [P, P, P, U32, D, D, I, P]),
    "afm_solve_cg_batched_mixed_device": (I, [P, P, P, U32, D, D, I, D, I, P]),
    "afm_get_info": (I, [P, P]),
    "afm_get_colors": (I, [P, P]),
    "afm_get_stream": (I, [P, C.POINTER(P)]),
    "afm_synchronize": (I, [P]),
    "afm_status_string": (C.c_char_p, [I]),
    "afm_last_error": (C.c_char_p, []),
}

PROBLEM_SIGNATURES = {
    "afm_mesh_hex8": (I, [U32, U32, U32, D, D, D, D, U64, P]),
    "afm_mesh_hex20": (I, [U32, U32, U32, D, D, D, D, U64, P]),
    "afm_mesh_tet10": (I, [U32, U32, U32, D, D, D, D, U64, P]),
    "afm_mesh_free": (None, [P]),
    "afm_element_dofs": (U32, [I]),
    "afm_element_dofs_per_node": (U32, [I]),
    "afm_element_matrices": (I, [I, P, U32, U32, D, D, U32, P]),
    "afm_element_matrix_xe": (I, [I, P, D, D, U32, P]),
    "afm_gauss_legendre": (None, [U32, P]),
    "afm_dof_map": (I, [P, U32, P]),
    "afm_load_poisson_sine": (I, [I, P, U32, P]),
    "afm_load_elastic_bar": (I, [I, P, D, U32, P]),
    "afm_bc_poisson_boundary": (U32, [P, P, P]),
    "afm_bc_elastic_bar": (U32, [P, P, P]),
    "afm_uniform01": (D, [U64, U64]),
}

_libs = {}


def _load(path, sigs):
    if path in _libs:
        return _libs[path]
    if not os.path.exists(path):
        raise RuntimeError("native library %s is not built (run amat_gb300.build.build_all())" % path)
    lib = C.CDLL(path)
    for name, (res, args) in sigs.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _libs[path] = lib
    return lib


def libafm():
    return _load(LIBAFM_PATH, AFM_SIGNATURES)


def libproblems():
    return _load(LIBPROBLEMS_PATH, PROBLEM_SIGNATURES)


class AfmError(RuntimeError):
    def __init__(self, status, where, message):
        self.status = status
        self.name = STATUS.get(status, str(status))
        super().__init__("%s failed: %s (%s)" % (where, self.name, message))


def check(status, where):
    if status != 0:
        msg = libafm().afm_last_error()
        raise AfmError(status, where, msg.decode() if msg else "")
    return status
