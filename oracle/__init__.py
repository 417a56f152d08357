"""Python access to the CPU oracle (liboracle.so) and, where it was built, the
reference itself compiled in place (_ref/libamat_ref.so).

TEST INFRASTRUCTURE. Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline / reference arms may import this package, and only as the checker or
as the timed CPU baseline. The product (amat_gb300) never imports it.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libamat_ref.so")
REF_SIMD_LIB = os.path.join(HERE, "_ref", "libamat_ref_simd.so")  # the reference's VECTORIZED_OPENMP build

P = C.c_void_p
U32 = C.c_uint32
I = C.c_int
D = C.c_double

_ORACLE_SIGS = {
    "oracle_matvec": (None, [U32, U32, P, P, P, P, P]),
    "oracle_matvec_omp": (I, [U32, U32, P, P, P, P, P, P]),
    "oracle_matvec_omp_cfg": (I, [U32, U32, P, P, P, P, P, P, I, I]),
    "oracle_coloring": (U32, [U32, U32, P, P, P]),
    "oracle_trace": (D, [U32, P, P]),
    "oracle_get_diagonal": (None, [U32, U32, P, P, P, P, U32, I, P]),
    "oracle_matmult_bc": (None, [U32, U32, P, P, P, P, U32, P, P]),
    "oracle_apply_bc_rhs": (None, [U32, U32, P, P, P, P, P, U32, I, P]),
    "oracle_pcg": (I, [U32, U32, P, P, P, P, U32, I, P, P, D, D, I, I, P]),
}

_REF_SIGS = {
    "ref_afm_create": (P, [U32, U32, P, P, P, U32, P, P, U32, I]),
    "ref_afm_matvec": (I, [P, P, P]),
    "ref_afm_matmult_bc": (I, [P, P, P]),
    "ref_afm_get_diagonal": (I, [P, P]),
    "ref_afm_apply_bc_rhs": (I, [P, P]),
    "ref_afm_destroy": (None, [P]),
    "ref_based_create": (P, [U32, U32, P, P, P, U32, P, P, U32, I]),
    "ref_based_matmult": (I, [P, P, P]),
    "ref_based_apply_bc": (I, [P, P]),
    "ref_based_destroy": (None, [P]),
    "ref_based_csr": (C.c_uint64, [P, P, P, P]),
    "ref_mesh_coloring": (I, [U32, U32, P, P, P, P]),
    "ref_gauss": (None, [U32, P]),
    "ref_ke_hex8": (None, [P, U32, P]),
    "ref_ke_tet10": (None, [P, U32, P]),
    "ref_ke_hex8_iso": (None, [P, D, D, U32, P]),
    "ref_ke_hex20_iso": (None, [P, D, D, U32, P]),
    "ref_ke_tet10_iso": (None, [P, D, D, U32, P]),
}

_cache = {}


def _bind(path, sigs):
    if path not in _cache:
        lib = C.CDLL(path)
        for k, (r, a) in sigs.items():
            f = getattr(lib, k)
            f.restype, f.argtypes = r, a
        _cache[path] = lib
    return _cache[path]


def lib():
    if not os.path.exists(ORACLE_LIB):
        from amat_gb300 import build
        build.build_oracle()
    return _bind(ORACLE_LIB, _ORACLE_SIGS)


def ref(simd=False):
    """The reference compiled in place (simd: its VECTORIZED_OPENMP build), or None where it was not built."""
    path = REF_SIMD_LIB if simd else REF_LIB
    return _bind(path, _REF_SIGS) if os.path.exists(path) else None


def _p(a):
    # Raw pointer only: the caller must keep `a` alive across the C call, so
    # never pass a temporary (np.ascontiguousarray of a strided view is a
    # fresh copy that Python may free before the call runs).
    return C.c_void_p(a.ctypes.data) if a is not None else None


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Problem:
    """Flat CSR description shared by the oracle and the reference harness."""

    def __init__(self, n_dofs, elem_dofs, ke, constrained=(), values=()):
        if isinstance(elem_dofs, np.ndarray) and elem_dofs.ndim == 2:
            n = elem_dofs.shape[1]
            self.offsets = (np.arange(elem_dofs.shape[0] + 1, dtype=np.uint64) * n).astype(np.uint32)
            self.map = np.ascontiguousarray(elem_dofs, dtype=np.uint32).reshape(-1)
            self.ke = np.ascontiguousarray(ke, dtype=np.float64).reshape(-1)
        else:
            lens = [len(e) for e in elem_dofs]
            self.offsets = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint32)
            self.map = np.concatenate([np.asarray(e, dtype=np.uint32) for e in elem_dofs])
            self.ke = np.concatenate([np.asarray(k, dtype=np.float64).reshape(-1) for k in ke])
        self.n_elem = len(self.offsets) - 1
        self.n_dofs = int(n_dofs)
        self.constrained = np.ascontiguousarray(constrained, dtype=np.uint64)
        self.values = np.ascontiguousarray(values, dtype=np.float64)

    # ---- oracle (restatement) ----
    def matvec(self, u):
        u = _f64(u)
        v = np.empty(self.n_dofs)
        lib().oracle_matvec(self.n_elem, self.n_dofs, _p(self.offsets), _p(self.map), _p(self.ke), _p(u), _p(v))
        return v

    def matvec_omp(self, u, v=None):
        u = _f64(u)
        v = np.empty(self.n_dofs) if v is None else v
        t = lib().oracle_matvec_omp(self.n_elem, self.n_dofs, _p(self.offsets), _p(self.map), _p(self.ke), None,
                                    _p(u), _p(v))
        return v, t

    def matvec_omp_cfg(self, u, v=None, threads=0, simd=False):
        """The OpenMP loop with a thread cap and, with simd, the reference's VECTORIZED_OPENMP element product
        (column-major Ke, column-by-column axpy under omp simd). Returns (v, threads used)."""
        u = _f64(u)
        v = np.empty(self.n_dofs) if v is None else v
        cm = None
        if simd:
            if getattr(self, "_ke_cm", None) is None:
                parts, k = [], 0
                for e in range(self.n_elem):
                    n = int(self.offsets[e + 1] - self.offsets[e])
                    parts.append(self.ke[k:k + n * n].reshape(n, n).T.reshape(-1))
                    k += n * n
                self._ke_cm = np.ascontiguousarray(np.concatenate(parts))
            cm = self._ke_cm
        t = lib().oracle_matvec_omp_cfg(self.n_elem, self.n_dofs, _p(self.offsets), _p(self.map), _p(self.ke),
                                        _p(cm), _p(u), _p(v), int(threads), int(bool(simd)))
        return v, t

    def coloring(self):
        c = np.empty(self.n_elem, dtype=np.uint32)
        n = lib().oracle_coloring(self.n_dofs, self.n_elem, _p(self.offsets), _p(self.map), _p(c))
        return c, n

    def trace(self):
        return lib().oracle_trace(self.n_elem, _p(self.offsets), _p(self.ke))

    def get_diagonal(self, bc_method=0):
        d = np.empty(self.n_dofs)
        lib().oracle_get_diagonal(self.n_elem, self.n_dofs, _p(self.offsets), _p(self.map), _p(self.ke),
                                  _p(self.constrained), len(self.constrained), bc_method, _p(d))
        return d

    def matmult_bc(self, u):
        u = _f64(u)
        v = np.empty(self.n_dofs)
        lib().oracle_matmult_bc(self.n_elem, self.n_dofs, _p(self.offsets), _p(self.map), _p(self.ke),
                                _p(self.constrained), len(self.constrained), _p(u), _p(v))
        return v

    def apply_bc_rhs(self, rhs, bc_method=0):
        r = np.array(rhs, dtype=np.float64, copy=True)
        lib().oracle_apply_bc_rhs(self.n_elem, self.n_dofs, _p(self.offsets), _p(self.map), _p(self.ke),
                                  _p(self.constrained), _p(self.values), len(self.constrained), bc_method, _p(r))
        return r

    def pcg(self, b, x0=None, rtol=1e-10, atol=0.0, maxit=10000, norm_type=0, bc_method=0):
        b = _f64(b)
        x = np.zeros(self.n_dofs) if x0 is None else np.array(x0, dtype=np.float64, copy=True)
        res = C.c_double()
        it = lib().oracle_pcg(self.n_elem, self.n_dofs, _p(self.offsets), _p(self.map), _p(self.ke),
                              _p(self.constrained), len(self.constrained), bc_method, _p(b), _p(x), rtol, atol,
                              maxit, norm_type,
                              C.byref(res))
        return x, it, res.value

    # ---- the reference itself (only where compiled) ----
    def ref_all(self, u, rhs, bc_method=0, blocks_dim=1):
        """Reference aMatFree outputs: matvec, MatMult_mf, diagonal, apply_bc rhs."""
        R = ref()
        h = R.ref_afm_create(self.n_elem, self.n_dofs, _p(self.offsets), _p(self.map), _p(self.ke), blocks_dim,
                             _p(self.constrained), _p(self.values), len(self.constrained), bc_method)
        u = np.ascontiguousarray(u, dtype=np.float64)
        v = np.empty(self.n_dofs)
        R.ref_afm_matvec(h, _p(v), _p(u))
        d = np.empty(self.n_dofs)
        R.ref_afm_get_diagonal(h, _p(d))
        r = np.array(rhs, dtype=np.float64, copy=True)
        R.ref_afm_apply_bc_rhs(h, _p(r))  # allocates the saved-U_c buffer MatMult_mf uses
        w = np.empty(self.n_dofs)
        R.ref_afm_matmult_bc(h, _p(w), _p(u))
        R.ref_afm_destroy(h)
        return dict(matvec=v, diag=d, rhs_bc=r, matmult_bc=w)

    def ref_assembled(self, u, rhs, bc_method=0):
        """Reference aMatBased (PETSc-assembled) K u before BCs, then K_bc u, rhs and the matrix (CSR) after
        apply_bc."""
        R = ref()
        h = R.ref_based_create(self.n_elem, self.n_dofs, _p(self.offsets), _p(self.map), _p(self.ke), 1,
                               _p(self.constrained), _p(self.values), len(self.constrained), bc_method)
        u = np.ascontiguousarray(u, dtype=np.float64)
        v = np.empty(self.n_dofs)
        R.ref_based_matmult(h, _p(v), _p(u))
        r = np.array(rhs, dtype=np.float64, copy=True)
        R.ref_based_apply_bc(h, _p(r))
        w = np.empty(self.n_dofs)
        R.ref_based_matmult(h, _p(w), _p(u))
        nnz = int(R.ref_based_csr(h, None, None, None))
        rp = np.empty(self.n_dofs + 1, np.uint64)
        cols = np.empty(nnz, np.uint32)
        vals = np.empty(nnz)
        R.ref_based_csr(h, _p(rp), _p(cols), _p(vals))
        R.ref_based_destroy(h)
        return dict(matvec=v, rhs_bc=r, matmult_bc=w, csr_row_ptr=rp, csr_cols=cols, csr_vals=vals)

    def ref_coloring(self):
        c = np.empty(self.n_elem, dtype=np.uint32)
        n = C.c_uint32()
        ref().ref_mesh_coloring(self.n_dofs, self.n_elem, _p(self.offsets), _p(self.map), _p(c), C.byref(n))
        return c, n.value


def ref_element_matrix(kind, xe, E=1.0, nu=0.3, ngt=2):
    """Reference element kernels (examples/src/ke_matrix.cpp); kind numbering of afm_problems.h."""
    R = ref()
    xe = np.ascontiguousarray(xe, dtype=np.float64)
    n = {0: 8, 1: 24, 2: 60, 3: 10, 4: 30}[kind]
    ke = np.empty((n, n))
    if kind == 0:
        R.ref_ke_hex8(_p(xe), ngt, _p(ke))
    elif kind == 1:
        R.ref_ke_hex8_iso(_p(xe), E, nu, ngt, _p(ke))
    elif kind == 2:
        R.ref_ke_hex20_iso(_p(xe), E, nu, ngt, _p(ke))
    elif kind == 3:
        R.ref_ke_tet10(_p(xe), ngt, _p(ke))
    else:
        R.ref_ke_tet10_iso(_p(xe), E, nu, ngt, _p(ke))
    return ke


def ref_gauss(n):
    xw = np.empty(2 * n)
    ref().ref_gauss(n, _p(xw))
    return xw
