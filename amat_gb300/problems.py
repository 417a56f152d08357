"""Example problems (include/afm_problems.h) as numpy arrays.

The structured meshes, element matrices, loads and boundary conditions of the
reference's example drivers (examples/src/example03a.cpp, example05a.cpp,
example07a.cpp, examples/src/ke_matrix.cpp). Host-side input generation only.
"""
import ctypes as C

import numpy as np

from ._native import AfmMesh, libproblems

HEX8_POISSON, HEX8_ELASTIC, HEX20_ELASTIC, TET10_POISSON, TET10_ELASTIC = range(5)
KIND_NODES = {HEX8_POISSON: 8, HEX8_ELASTIC: 8, HEX20_ELASTIC: 20, TET10_POISSON: 10, TET10_ELASTIC: 10}
KIND_DPN = {HEX8_POISSON: 1, HEX8_ELASTIC: 3, HEX20_ELASTIC: 3, TET10_POISSON: 1, TET10_ELASTIC: 3}


def _p(a):
    return C.c_void_p(a.ctypes.data)


class Mesh:
    """A structured mesh owned by the native library (freed with the object)."""

    def __init__(self, kind, nx, ny=None, nz=None, L=(1.0, 1.0, 1.0), jitter=0.0, seed=0):
        ny = nx if ny is None else ny
        nz = nx if nz is None else nz
        self.kind = kind
        self._m = AfmMesh()
        lib = libproblems()
        fn = {8: lib.afm_mesh_hex8, 20: lib.afm_mesh_hex20, 10: lib.afm_mesh_tet10}[KIND_NODES[kind]]
        if fn(nx, ny, nz, float(L[0]), float(L[1]), float(L[2]), float(jitter), int(seed), C.byref(self._m)) != 0:
            raise RuntimeError("mesh generation failed")
        m = self._m
        self.n_nodes, self.n_elem, self.npe = m.n_nodes, m.n_elem, m.nodes_per_elem
        self.dpn = KIND_DPN[kind]
        self.n_dofs = self.n_nodes * self.dpn
        self.ndpe = self.npe * self.dpn

    def __del__(self):
        try:
            libproblems().afm_mesh_free(C.byref(self._m))
        except Exception:
            pass

    @property
    def coords(self):
        return np.ctypeslib.as_array(self._m.coords, shape=(self.n_nodes, 3)).copy()

    @property
    def elem_nodes(self):
        return np.ctypeslib.as_array(self._m.elem_nodes, shape=(self.n_elem, self.npe)).copy()

    @property
    def lattice(self):
        return np.ctypeslib.as_array(self._m.lattice, shape=(self.n_nodes, 3)).copy()

    def dof_map(self):
        out = np.empty((self.n_elem, self.ndpe), dtype=np.uint32)
        libproblems().afm_dof_map(C.byref(self._m), self.dpn, _p(out))
        return out

    def element_matrices(self, first=0, count=None, E=1.0, nu=0.3, ngt=2, out=None):
        count = self.n_elem - first if count is None else count
        n = self.ndpe
        ke = np.empty((count, n, n), dtype=np.float64) if out is None else out
        rc = libproblems().afm_element_matrices(self.kind, C.byref(self._m), first, count, float(E), float(nu), ngt,
                                                _p(ke))
        if rc != 0:
            raise RuntimeError("element matrices failed (%d): non-positive Jacobian?" % rc)
        return ke

    def load(self, ngt=2, rho_g=1.0):
        rhs = np.empty(self.n_dofs, dtype=np.float64)
        lib = libproblems()
        if self.dpn == 1:
            rc = lib.afm_load_poisson_sine(self.kind, C.byref(self._m), ngt, _p(rhs))
        else:
            rc = lib.afm_load_elastic_bar(self.kind, C.byref(self._m), float(rho_g), ngt, _p(rhs))
        if rc != 0:
            raise RuntimeError("load failed")
        return rhs

    def boundary_conditions(self):
        cap = self.n_dofs
        dofs = np.empty(cap, dtype=np.uint64)
        vals = np.empty(cap, dtype=np.float64)
        lib = libproblems()
        fn = lib.afm_bc_poisson_boundary if self.dpn == 1 else lib.afm_bc_elastic_bar
        n = fn(C.byref(self._m), _p(dofs), _p(vals))
        return dofs[:n].copy(), vals[:n].copy()


def element_matrix_xe(kind, xe, E=1.0, nu=0.3, ngt=2):
    n = KIND_NODES[kind] * KIND_DPN[kind]
    ke = np.empty((n, n), dtype=np.float64)
    xe = np.ascontiguousarray(xe, dtype=np.float64)
    if libproblems().afm_element_matrix_xe(kind, _p(xe), float(E), float(nu), ngt, _p(ke)) != 0:
        raise RuntimeError("element matrix failed")
    return ke


def gauss_legendre(n):
    xw = np.empty(2 * n, dtype=np.float64)
    libproblems().afm_gauss_legendre(n, _p(xw))
    return xw
