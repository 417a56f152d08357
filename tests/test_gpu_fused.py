"""Every colour of a split product in one cooperative launch (afm_set_fused_colours): the same bits as one
launch per colour (each element's arithmetic and the colour order of every v entry's sums are unchanged), for
single-unit and chunked ring slots, with and without MatMult_mf's constrained columns, and within the FP64 bar
of the oracle."""
import numpy as np
import pytest

import oracle
from amat_gb300 import PRECISION, Maps, aMatFree
from amat_gb300 import problems as P
from helpers import FP64_RTOL, rel

pytestmark = pytest.mark.gpu


def operator(kind, n, bc):
    m = P.Mesh(kind, n, jitter=0.1, seed=6)
    ke = m.element_matrices(ngt=3 if kind == P.HEX20_ELASTIC else 2)
    maps = Maps()
    maps.set_map(m.n_elem, m.dof_map(), m.ndpe, m.n_dofs)
    dofs, vals = m.boundary_conditions() if bc else (np.zeros(0, np.uint64), np.zeros(0))
    maps.set_bdr_map(dofs, vals)
    A = aMatFree(maps)
    A.set_precision(PRECISION.FP64_SPLIT)
    A.set_element_matrices(0, ke)
    A.finalize()
    return m, ke, dofs, vals, A


@pytest.mark.parametrize("kind,n", [(P.HEX20_ELASTIC, 6), (P.HEX8_ELASTIC, 10), (P.TET10_ELASTIC, 4)])
@pytest.mark.parametrize("bc", [False, True])
def test_fused_equals_colour_launches(gpu, kind, n, bc):
    m, ke, dofs, vals, A = operator(kind, n, bc)
    u = np.random.default_rng(n).uniform(-1, 1, m.n_dofs)
    out = {}
    for fused in (0, 1):
        A.set_fused_colours(fused)
        v = np.empty(m.n_dofs)
        if bc:
            A.matmult_bc(v, u)
        else:
            A.matvec(v, u, True)
        out[fused] = v
    assert np.array_equal(out[0], out[1])
    pr = oracle.Problem(m.n_dofs, m.dof_map(), ke, dofs, vals)
    ref = pr.matmult_bc(u) if bc else pr.matvec(u)
    assert rel(out[1], ref) < FP64_RTOL


def test_fused_product_in_a_solve(gpu):
    """The CG solve (captured iterations keep the colour launches) and the mixed solve's FP64 residuals on a
    fused operator converge to the same FP64-checked tolerance."""
    m, ke, dofs, vals, A = operator(P.HEX20_ELASTIC, 6, True)
    b = A.apply_bc(m.load(ngt=3))
    x, st = A.solve(b, rtol=1e-8, atol=0.0, maxit=10000)
    pr = oracle.Problem(m.n_dofs, m.dof_map(), ke, dofs, vals)
    assert st.status == 0
    assert np.linalg.norm(b - pr.matmult_bc(x)) <= 1.01e-8 * np.linalg.norm(b)
    y, st2 = A.solve_mixed(b, rtol=1e-8, inner_rtol=0.1)
    assert st2.status == 0
    assert np.linalg.norm(b - pr.matmult_bc(y)) <= 1.01e-8 * np.linalg.norm(b)
