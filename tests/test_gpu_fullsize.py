"""Oracle parity at the configured workload sizes.

The three stored-matrix workloads at full size: 3-D Poisson on a 32^3 hex8
mesh (with CG to 1e-10 against the oracle's PCG), hex20 elasticity on a 64^3
mesh (262,144 elements, 7.5 GB of FP64 element matrices), and tet10 Poisson on
96^3 x 6 tetrahedra (5.3M elements). For each: v = K u and MatMult_mf of the
default (split) operator against the oracle's restatement of the reference's
CPU loop, and the assembled CSR product (the aMatBased baseline) against both,
all within the FP64 tolerance.
"""
import numpy as np
import pytest

import oracle
from amat_gb300 import Maps, aMatFree
from amat_gb300 import problems as P
from helpers import FP64_RTOL, rel

pytestmark = pytest.mark.gpu

CONFIGS = [
    # name, kind, edge, Gauss points per direction, vertex jitter (x h), seed
    ("hex8_poisson_32", P.HEX8_POISSON, 32, 2, 0.0, 0),
    ("hex20_elastic_64", P.HEX20_ELASTIC, 64, 3, 0.1, 1),
    ("tet10_poisson_96", P.TET10_POISSON, 96, 2, 0.15, 2),
]


@pytest.mark.parametrize("name,kind,n,ngt,jitter,seed", CONFIGS)
def test_full_size_parity(gpu, name, kind, n, ngt, jitter, seed):
    import torch
    m = P.Mesh(kind, n, jitter=jitter, seed=seed)
    ke = m.element_matrices(ngt=ngt)
    dofs, vals = m.boundary_conditions()
    dm = m.dof_map().reshape(m.n_elem, m.ndpe)
    maps = Maps()
    maps.set_map(m.n_elem, m.dof_map(), m.ndpe, m.n_dofs)
    maps.set_bdr_map(dofs, vals)
    A = aMatFree(maps)
    A.set_element_matrices(0, ke)
    A.finalize()
    pr = oracle.Problem(m.n_dofs, dm, ke, dofs, vals)
    u = np.random.default_rng(17).uniform(-1, 1, m.n_dofs)
    v = np.empty(m.n_dofs)
    A.matvec(v, u, True)
    ref, _ = pr.matvec_omp(u)
    assert rel(v, ref) < FP64_RTOL
    w = np.empty(m.n_dofs)
    A.matmult_bc(w, u)
    assert rel(w, pr.matmult_bc(u)) < FP64_RTOL
    # the assembled operator of the same element matrices (element-order sums), no BC rows
    A.assemble(apply_bc=False)
    du = torch.tensor(u, device="cuda")
    dv = torch.empty_like(du)
    torch.cuda.synchronize()
    A.matvec_assembled_device(dv.data_ptr(), du.data_ptr())
    A.synchronize()
    va = dv.cpu().numpy()
    assert rel(va, ref) < FP64_RTOL and rel(va, v) < FP64_RTOL
    if name == "hex8_poisson_32":
        # config 1: CG to 1e-10 against the oracle's Jacobi-PCG
        rhs = A.apply_bc(m.load())
        x, st = A.solve(rhs, rtol=1e-10, atol=0.0, maxit=5000)
        xo, it, _ = pr.pcg(rhs, rtol=1e-10, atol=0.0, maxit=5000)
        assert st.status == 0 and abs(st.iterations - it) <= 1
        assert rel(x, xo) < 1e-8
