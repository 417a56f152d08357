"""Python mirror of the reference's operator interface over the C ABI.

`Maps` and `aMatFree` keep the names, argument meaning and call order of
par::Maps (include/maps.hpp:279-302) and par::aMatFree / par::aMat
(include/aMat.hpp:75-242, include/aMatFree.hpp:113-238), with numpy arrays in
place of jagged C arrays and PETSc Vecs. Every call goes through libafm.so
(include/afm.h); the product runs on the GB300 only.
"""
import ctypes as C
import enum

import numpy as np

from ._native import AfmInfo, AfmSolveStats, check, libafm


class BC_METH(enum.IntEnum):
    """par::BC_METH (include/enums.hpp:20-21)"""
    BC_IMATRIX = 0
    BC_PENALTY = 1


class MATFREE_TYPE(enum.IntEnum):
    """par::MATFREE_TYPE (include/enums.hpp:56); 1 and 3 run the stored-Ke device operator, 2 the matrix-free one
    (element kernels on the device from node coordinates)."""
    QUASI_FREE = 1
    FREE = 2
    GPU_PURE = 3


class PRECISION(enum.IntEnum):
    FP64 = 0
    FP64_SPLIT = 1
    FP32 = 2
    AUTO = 3


class CG_NORM(enum.IntEnum):
    UNPRECONDITIONED = 0
    PRECONDITIONED = 1


def _ptr(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


class Maps:
    """par::Maps: element -> DoF map and boundary conditions.

    With comm = a torch.distributed process group of more than one rank, the
    map is partitioned (one GPU per rank): set_map builds the scatter map of
    Maps::buildScatterMap (amat_gb300.partition.ScatterMap) and the operator
    works over the rank-local numbering [pre-ghosts | owned | post-ghosts].
    """

    def __init__(self, comm=None):
        self._map = None
        self._bdr = None
        self._comm = comm
        self.scatter = None

    def set_map(self, n_elements_on_rank, element_to_rank_map, dofs_per_element, n_all_dofs_on_rank,
                rank_to_global_map=None, owned_global_dof_range_begin=0, owned_global_dof_range_end=None,
                n_global_dofs=None):
        """Maps::set_map (include/maps.hpp:279-286, 399-451).

        element_to_rank_map: (n_elem, n) array, or a flat array with
        dofs_per_element an array of per-element counts. owned range end is
        inclusive, as in the reference.
        """
        n_global = int(n_global_dofs if n_global_dofs is not None else n_all_dofs_on_rank)
        end = int(owned_global_dof_range_end if owned_global_dof_range_end is not None else n_global - 1)
        m = np.ascontiguousarray(element_to_rank_map, dtype=np.uint32).reshape(-1)
        dpe = np.asarray(dofs_per_element)
        if dpe.ndim == 0:
            offsets = None
            n_uniform = int(dpe)
        else:
            dpe = dpe.astype(np.uint32)
            offsets = np.zeros(len(dpe) + 1, dtype=np.uint32)
            np.cumsum(dpe, out=offsets[1:])
            n_uniform = 0
            if np.all(dpe == dpe[0]):
                offsets, n_uniform = None, int(dpe[0])
        l2g = None if rank_to_global_map is None else np.ascontiguousarray(rank_to_global_map, dtype=np.uint64)
        if self._partitioned():
            from .partition import ScatterMap
            gdofs = m.astype(np.int64) if l2g is None else l2g[m].astype(np.int64)
            begin = int(owned_global_dof_range_begin)
            self.scatter = ScatterMap(self._comm, gdofs, end - begin + 1, begin, offsets, n_uniform)
            if self.scatter.n_all != int(n_all_dofs_on_rank) or self.scatter.n_global != n_global:
                raise ValueError("n_all_dofs_on_rank %d / n_global_dofs %d disagree with the scatter map (%d, %d)"
                                 % (n_all_dofs_on_rank, n_global, self.scatter.n_all, self.scatter.n_global))
            # the rank's operator: a single-rank map over the local numbering
            m, l2g, n_all = self.scatter.local_map, None, self.scatter.n_all
            self._map = dict(n_elem=int(n_elements_on_rank), offsets=offsets, n_uniform=n_uniform, map=m,
                             n_all=n_all, l2g=None, begin=0, end=n_all - 1, n_global=n_all)
            return
        self._map = dict(n_elem=int(n_elements_on_rank), offsets=offsets, n_uniform=n_uniform, map=m,
                         n_all=int(n_all_dofs_on_rank), l2g=l2g, begin=int(owned_global_dof_range_begin), end=end,
                         n_global=n_global)

    def _partitioned(self):
        if self._comm is None:
            return False
        import torch.distributed as dist
        return dist.get_world_size(self._comm) > 1

    def set_bdr_map(self, constrained_dofs, prescribed_values, num_constraints=None):
        """Maps::set_bdr_map (include/maps.hpp:829-880)."""
        c = np.ascontiguousarray(constrained_dofs, dtype=np.uint64).reshape(-1)
        v = np.ascontiguousarray(prescribed_values, dtype=np.float64).reshape(-1)
        n = len(c) if num_constraints is None else int(num_constraints)
        c, v = c[:n].copy(), v[:n].copy()
        if self.scatter is not None:
            # global ids -> this rank's local ids; constraints on DoFs this rank does not hold are dropped
            l2g = self.scatter.local2global
            order = np.argsort(l2g)
            pos = np.searchsorted(l2g[order], c.astype(np.int64))
            pos = np.minimum(pos, len(l2g) - 1)
            hit = l2g[order][pos] == c.astype(np.int64)
            c, v = order[pos[hit]].astype(np.uint64), v[hit]
        self._bdr = (c, v)

    @property
    def n_dofs(self):
        return self._map["n_global"]


class aMatFree:
    """par::aMatFree on one GB300: stored element matrices, device matvec."""

    def __init__(self, maps, bc_method=BC_METH.BC_IMATRIX, device=-1):
        lib = libafm()
        h = C.c_void_p()
        check(lib.afm_create(C.byref(h), int(bc_method), int(device)), "afm_create")
        self._h = h
        self._lib = lib
        self.maps = maps
        self.bc_method = BC_METH(bc_method)
        mp = maps._map
        if mp is None:
            raise ValueError("Maps.set_map has not been called")
        check(lib.afm_set_map(h, mp["n_elem"], _ptr(mp["offsets"]), mp["n_uniform"], _ptr(mp["map"]), mp["n_all"],
                              _ptr(mp["l2g"]), mp["begin"], mp["end"], mp["n_global"]), "afm_set_map")
        if maps._bdr is not None:
            c, v = maps._bdr
            check(lib.afm_set_bdr_map(h, _ptr(c), _ptr(v), len(c)), "afm_set_bdr_map")
        self.n_dofs = mp["n_global"]
        self._part = None
        if maps.scatter is not None:
            from .partition import PartitionedProduct
            self._part = PartitionedProduct(maps.scatter, self._local_matvec)
            self._bc_local = np.zeros(self.n_dofs, dtype=bool)
            if maps._bdr is not None:
                self._bc_local[maps._bdr[0].astype(np.int64)] = True

    def close(self):
        if getattr(self, "_h", None):
            self._lib.afm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- set-up ----------------------------------------------------------
    def set_matfree_type(self, t):
        check(self._lib.afm_set_matfree_type(self._h, int(t)), "afm_set_matfree_type")

    def set_precision(self, p):
        check(self._lib.afm_set_precision(self._h, int(p)), "afm_set_precision")

    def set_patch_mode(self, mode):
        """Small elements as shared-memory patches, in one launch plus a combine pass when the patch colours
        are small and one launch per colour otherwise (1, default), always per colour (2), always in one
        launch (3); or no patches, one launch per element colour (0)."""
        check(self._lib.afm_set_patch_mode(self._h, int(mode)), "afm_set_patch_mode")

    def set_symmetric_inner(self, fmt):
        """Inner format of FP32 products: 1 (default) symmetric copy in FP32, 2 symmetric copy in FP32 + BF16
        correction with FP64 sums, 0 the hi plane."""
        check(self._lib.afm_set_symmetric_inner(self._h, int(fmt)), "afm_set_symmetric_inner")

    def set_fused_colours(self, enable):
        """Every colour of a split product in one cooperative launch, or one launch per colour (default)."""
        check(self._lib.afm_set_fused_colours(self._h, int(bool(enable))), "afm_set_fused_colours")

    def set_wait_limit(self, seconds):
        """Limit of each wait inside the element kernels (4 s by default); past it a call reports ERR_TIMEOUT."""
        check(self._lib.afm_set_wait_limit(self._h, float(seconds)), "afm_set_wait_limit")

    def set_wait_probe(self, enable):
        """Test hook: one warp of every element kernel waits on a flag nothing sets, so that its wait
        runs out after the wait limit and calls report ERR_TIMEOUT."""
        check(self._lib.afm_set_wait_probe(self._h, int(bool(enable))), "afm_set_wait_probe")

    def set_element_kind(self, kind, E=1.0, nu=0.3, ngt=2):
        """Element kernels of the matrix-free operator (method 2), the counterpart of
        set_element_matrix_function (include/aMat.hpp:114-116); kind as problems.HEX8_POISSON etc."""
        check(self._lib.afm_set_element_kind(self._h, int(kind), float(E), float(nu), int(ngt)),
              "afm_set_element_kind")

    def set_element_coords(self, first_eid, xe):
        """Node coordinates (count x nodes x 3) of elements first_eid, first_eid + 1, ..."""
        x = np.ascontiguousarray(xe, dtype=np.float64)
        check(self._lib.afm_set_element_coords(self._h, int(first_eid), int(x.shape[0]), _ptr(x)),
              "afm_set_element_coords")

    def set_element_matrix(self, eid, e_mat, block_i=0, block_j=0, blocks_dim=1):
        """aMatFree::set_element_matrix (include/aMatFree.hpp:856-880)."""
        k = np.ascontiguousarray(e_mat, dtype=np.float64)
        check(self._lib.afm_set_element_matrix(self._h, int(eid), _ptr(k), int(block_i), int(block_j),
                                               int(blocks_dim)), "afm_set_element_matrix")

    def set_element_matrices(self, first_eid, ke):
        k = np.ascontiguousarray(ke, dtype=np.float64)
        count = k.shape[0] if k.ndim == 3 else None
        if count is None:
            raise ValueError("ke must be (count, n, n)")
        check(self._lib.afm_set_element_matrices(self._h, int(first_eid), count, _ptr(k)),
              "afm_set_element_matrices")

    def finalize(self):
        check(self._lib.afm_finalize(self._h), "afm_finalize")

    # ---- operator --------------------------------------------------------
    def _local_matvec(self, v, u):
        check(self._lib.afm_matvec(self._h, _ptr(v), _ptr(np.ascontiguousarray(u, dtype=np.float64)), 1),
              "afm_matvec")

    def matvec(self, v, u, isGhosted=True):
        """aMatFree::matvec(v, u, isGhosted): v = K u on host arrays. Partitioned maps: u, v are the rank's
        ghosted local vectors (isGhosted) or its owned entries; u's ghosts are received from their owners
        and v's ghost rows sent to theirs (matvec_ghosted, include/aMatFree.hpp:1682-1775)."""
        assert v.dtype == np.float64 and v.flags.c_contiguous
        if self._part is not None:
            u = np.array(u, dtype=np.float64, copy=True)
            return self._part.matvec(v, u, isGhosted)
        u = np.ascontiguousarray(u, dtype=np.float64)
        check(self._lib.afm_matvec(self._h, _ptr(v), _ptr(u), int(bool(isGhosted))), "afm_matvec")
        return v

    def matmult_bc(self, v, u):
        """MatMult_mf (include/aMatFree.hpp:3894-3941). Partitioned maps: ghosted local vectors; a
        constrained row keeps its owner's v_c = u_c (the ghost copies send nothing for it)."""
        u = np.ascontiguousarray(u, dtype=np.float64)
        if self._part is not None:
            s = self._part.smap
            u = u.copy()
            s.ghost_receive(u)
            check(self._lib.afm_matmult_bc(self._h, _ptr(v), _ptr(u)), "afm_matmult_bc")
            ghost_bc = self._bc_local.copy()
            ghost_bc[s.n_pre:s.n_pre + s.n_owned] = False
            v[ghost_bc] = 0.0
            s.ghost_send(v)
            return v
        check(self._lib.afm_matmult_bc(self._h, _ptr(v), _ptr(u)), "afm_matmult_bc")
        return v

    def matvec_device(self, v_ptr, u_ptr, stream=None):
        check(self._lib.afm_matvec_device(self._h, C.c_void_p(v_ptr), C.c_void_p(u_ptr),
                                          C.c_void_p(stream) if stream else None), "afm_matvec_device")

    def matvec_device_f32(self, v_ptr, u_ptr, stream=None):
        check(self._lib.afm_matvec_device_f32(self._h, C.c_void_p(v_ptr), C.c_void_p(u_ptr),
                                              C.c_void_p(stream) if stream else None), "afm_matvec_device_f32")

    def matvec_inner_device(self, v_ptr, u_ptr, stream=None):
        """v = K u on double device vectors with the double-float products of the corrected symmetric arena
        (symmetric inner format 3)."""
        check(self._lib.afm_matvec_inner_device(self._h, C.c_void_p(v_ptr), C.c_void_p(u_ptr),
                                                C.c_void_p(stream) if stream else None), "afm_matvec_inner_device")

    def matmult_bc_device(self, v_ptr, u_ptr, stream=None):
        check(self._lib.afm_matmult_bc_device(self._h, C.c_void_p(v_ptr), C.c_void_p(u_ptr),
                                              C.c_void_p(stream) if stream else None), "afm_matmult_bc_device")

    def get_diagonal(self):
        """MatGetDiagonal_mf with apply_bc_diagonal (include/aMatFree.hpp:3945-3975, 4310-4338)."""
        d = np.empty(self.n_dofs, dtype=np.float64)
        check(self._lib.afm_get_diagonal(self._h, _ptr(d)), "afm_get_diagonal")
        if self._part is not None:
            # element sums of every rank on the owned rows (mat_get_diagonal_ghosted's ghost_send), then
            # the constrained rows set wherever any rank has an element on them (apply_bc_diagonal inserts
            # the value from every rank that holds such an element)
            s = self._part.smap
            in_elem = np.zeros(s.n_all, dtype=bool)
            in_elem[s.local_map.astype(np.int64)] = True
            d[self._bc_local] = 0.0
            s.ghost_send(d)
            flag = (self._bc_local & in_elem).astype(np.float64)
            s.ghost_send(flag)
            own = np.zeros(s.n_all, dtype=bool)
            own[s.n_pre:s.n_pre + s.n_owned] = True
            set_rows = own & self._bc_local & (flag > 0)
            if self.bc_method != BC_METH.BC_IMATRIX:
                raise NotImplementedError("partitioned diagonal with the penalty method")
            d[set_rows] = 1.0
        return d

    def apply_bc(self, rhs):
        """aMatFree::apply_bc (include/aMatFree.hpp:957-969): rhs updated in place."""
        assert rhs.dtype == np.float64 and rhs.flags.c_contiguous
        check(self._lib.afm_apply_bc_rhs(self._h, _ptr(rhs)), "afm_apply_bc_rhs")
        return rhs

    def get_trace(self):
        t = C.c_double()
        check(self._lib.afm_get_trace(self._h, C.byref(t)), "afm_get_trace")
        return t.value

    def solve(self, rhs, x=None, rtol=1e-12, atol=1e-12, maxit=10000, norm=CG_NORM.UNPRECONDITIONED,
              raise_on_fail=True):
        """par::solve (examples/include/solve.hpp:75-127): Jacobi PCG on the MatMult_mf operator."""
        b = np.ascontiguousarray(rhs, dtype=np.float64)
        x = np.zeros(self.n_dofs) if x is None else np.ascontiguousarray(x, dtype=np.float64).copy()
        st = AfmSolveStats()
        s = self._lib.afm_solve_cg(self._h, _ptr(b), _ptr(x), float(rtol), float(atol), int(maxit), int(norm),
                                   C.byref(st))
        if raise_on_fail:
            check(s, "afm_solve_cg")
        return x, st

    def solve_mixed(self, rhs, x=None, rtol=1e-8, atol=0.0, max_outer=30, inner_rtol=1e-2, max_inner=10000,
                    raise_on_fail=True):
        """Mixed-precision iterative refinement: FP64 outer residual, FP32 inner Jacobi-PCG."""
        b = np.ascontiguousarray(rhs, dtype=np.float64)
        x = np.zeros(self.n_dofs) if x is None else np.ascontiguousarray(x, dtype=np.float64).copy()
        st = AfmSolveStats()
        s = self._lib.afm_solve_cg_mixed(self._h, _ptr(b), _ptr(x), float(rtol), float(atol), int(max_outer),
                                         float(inner_rtol), int(max_inner), C.byref(st))
        if raise_on_fail:
            check(s, "afm_solve_cg_mixed")
        return x, st

    def solve_trace(self):
        """The last mixed-precision solve: [(inner iterations so far, ||b - A x|| / ||b||)] at each FP64
        residual."""
        n = C.c_uint32()
        check(self._lib.afm_get_solve_trace(self._h, 0, None, None, C.byref(n)), "afm_get_solve_trace")
        it = np.zeros(n.value, dtype=np.int32)
        res = np.zeros(n.value)
        check(self._lib.afm_get_solve_trace(self._h, n.value, _ptr(it), _ptr(res), C.byref(n)),
              "afm_get_solve_trace")
        return list(zip(it.tolist(), res.tolist()))

    def matmult_bc_device_f32(self, v_ptr, u_ptr, stream=None):
        check(self._lib.afm_matmult_bc_device_f32(self._h, C.c_void_p(v_ptr), C.c_void_p(u_ptr),
                                                  C.c_void_p(stream) if stream else None), "afm_matmult_bc_device_f32")

    # ---- batched (device blocks n_dofs x ld, row-major) ------------------
    def matvec_batched_device(self, v_ptr, u_ptr, nrhs, ld=None, f32=False, bc=False, stream=None):
        ld = nrhs if ld is None else ld
        name = "afm_%s_batched_device%s" % ("matmult_bc" if bc else "matvec", "_f32" if f32 else "")
        check(getattr(self._lib, name)(self._h, C.c_void_p(v_ptr), C.c_void_p(u_ptr), int(nrhs), int(ld),
                                       C.c_void_p(stream) if stream else None), name)

    def set_batch_tuning(self, nrhs, cols_per_thread, rows_per_thread, ld=None, f32=False):
        """Pins the batched lane tile (columns, rows): (8, 2), (8, 4), (8, 6) or (4, 4)."""
        ld = nrhs if ld is None else ld
        check(self._lib.afm_set_batch_tuning(self._h, int(nrhs), int(ld), int(bool(f32)), int(cols_per_thread),
                                             int(rows_per_thread)), "afm_set_batch_tuning")

    def batch_tuning(self, nrhs, ld=None, f32=False, solve=False):
        """(columns, rows, ms) the autotuner chose; solve=True: the FP32 products of the batched mixed solve."""
        ld = nrhs if ld is None else ld
        tr, ng, ms = C.c_int(), C.c_int(), C.c_float()
        sel = 2 if solve else int(bool(f32))
        check(self._lib.afm_get_batch_tuning(self._h, int(nrhs), int(ld), sel, C.byref(tr), C.byref(ng),
                                             C.byref(ms)), "afm_get_batch_tuning")
        return tr.value, ng.value, ms.value

    def solve_batched_device(self, b_ptr, x_ptr, nrhs, rtol=1e-8, atol=0.0, maxit=100000, mixed=False,
                             max_outer=200, inner_rtol=1e-2, max_inner=64, raise_on_fail=True):
        """Block Jacobi-PCG on nrhs columns (device blocks n_dofs x nrhs). mixed: FP32 block recursion with
        FP64 reliable updates; each FP32 segment ends after max_inner iterations (or once a column's residual
        fell by inner_rtol; the block waits for its slowest column, so short segments keep every column busy)."""
        st = AfmSolveStats()
        if mixed:
            s = self._lib.afm_solve_cg_batched_mixed_device(self._h, C.c_void_p(b_ptr), C.c_void_p(x_ptr), int(nrhs),
                                                            float(rtol), float(atol), int(max_outer),
                                                            float(inner_rtol), int(max_inner), C.byref(st))
        else:
            s = self._lib.afm_solve_cg_batched_device(self._h, C.c_void_p(b_ptr), C.c_void_p(x_ptr), int(nrhs),
                                                      float(rtol), float(atol), int(maxit), C.byref(st))
        if raise_on_fail:
            check(s, "batched solve")
        return st

    def info(self):
        i = AfmInfo()
        check(self._lib.afm_get_info(self._h, C.byref(i)), "afm_get_info")
        return {f: getattr(i, f) for f, _ in AfmInfo._fields_}

    def colors(self):
        c = np.empty(self.info()["n_elements"], dtype=np.uint32)
        check(self._lib.afm_get_colors(self._h, _ptr(c)), "afm_get_colors")
        return c

    def stream(self):
        s = C.c_void_p()
        check(self._lib.afm_get_stream(self._h, C.byref(s)), "afm_get_stream")
        return s.value

    def synchronize(self):
        check(self._lib.afm_synchronize(self._h), "afm_synchronize")

    # ---- assembled operator (par::aMatBased) ----
    def assemble(self, apply_bc=True):
        """The matrix aMatBased assembles (include/aMatBased.hpp:214-352), kept on the device as CSR."""
        check(self._lib.afm_assemble(self._h, int(bool(apply_bc))), "afm_assemble")

    def matvec_assembled_device(self, v_ptr, u_ptr, stream=None):
        """aMatBased::matmult on device vectors (CSR SpMV)."""
        check(self._lib.afm_matvec_assembled_device(self._h, C.c_void_p(v_ptr), C.c_void_p(u_ptr),
                                                    C.c_void_p(stream)), "afm_matvec_assembled_device")

    def assembled_csr(self):
        """dump_mat: (row_ptr, cols, vals) of the assembled matrix."""
        nnz = C.c_uint64(0)
        check(self._lib.afm_get_assembled_csr(self._h, C.byref(nnz), None, None, None), "afm_get_assembled_csr")
        n = self.info()["n_dofs"]
        rp = np.empty(n + 1, np.uint64)
        cols = np.empty(nnz.value, np.uint32)
        vals = np.empty(nnz.value)
        check(self._lib.afm_get_assembled_csr(self._h, C.byref(nnz), _ptr(rp), _ptr(cols), _ptr(vals)),
              "afm_get_assembled_csr")
        return rp, cols, vals


def assemble_csr_host(n_dofs, offsets, dof_map, ke, constrained=(), bc_method=BC_METH.BC_IMATRIX, apply_bc=True):
    """Host-only aMatBased assembly (afm_assemble_csr_host): ke is the concatenation of the row-major element
    matrices, offsets/dof_map the flattened map. Returns (row_ptr, cols, vals)."""
    offsets = np.ascontiguousarray(offsets, dtype=np.uint32)
    dof_map = np.ascontiguousarray(dof_map, dtype=np.uint32)
    ke = np.ascontiguousarray(ke, dtype=np.float64).ravel()
    cons = np.ascontiguousarray(constrained, dtype=np.uint64)
    n_elem = len(offsets) - 1
    nnz = C.c_uint64(0)
    args = (n_elem, int(n_dofs), _ptr(offsets), _ptr(dof_map), _ptr(ke), _ptr(cons) if len(cons) else None,
            len(cons), int(bc_method), int(bool(apply_bc)))
    check(libafm().afm_assemble_csr_host(*args, C.byref(nnz), None, None, None), "afm_assemble_csr_host")
    rp = np.empty(int(n_dofs) + 1, np.uint64)
    cols = np.empty(nnz.value, np.uint32)
    vals = np.empty(nnz.value)
    check(libafm().afm_assemble_csr_host(*args, C.byref(nnz), _ptr(rp), _ptr(cols), _ptr(vals)),
          "afm_assemble_csr_host")
    return rp, cols, vals
