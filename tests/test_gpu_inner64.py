"""Symmetric inner formats 3 and 4: the mixed-precision solve's inner recursion
in FP64 vectors on products from the corrected symmetric arena (each symmetric
pair of Ke entries once, as FP32 + BF16: K to about 2^-32), of the FP64 u as a
double-float pair (3) or of u rounded to FP32 (4). The
product against the oracle for every kernel that reads the arena (warp-group
elements, patches), its exact power-of-two scaling, and the solve checked in
FP64 against the oracle's MatMult_mf."""
import numpy as np
import pytest

import oracle
from amat_gb300 import PRECISION, AfmError, Maps, aMatFree
from amat_gb300 import problems as P
from helpers import rel

pytestmark = pytest.mark.gpu

# the corrected arena holds each entry to ~2^-32 of itself; random u: |K||u| ~ |K u|
INNER_RTOL = 1e-8


def operator(kind, n, bc=False, seed=3, fmt=3):
    m = P.Mesh(kind, n, jitter=0.1, seed=seed)
    ke = m.element_matrices(ngt=3 if kind == P.HEX20_ELASTIC else 2)
    maps = Maps()
    maps.set_map(m.n_elem, m.dof_map(), m.ndpe, m.n_dofs)
    dofs, vals = m.boundary_conditions() if bc else (np.zeros(0, np.uint64), np.zeros(0))
    maps.set_bdr_map(dofs, vals)
    A = aMatFree(maps)
    A.set_precision(PRECISION.FP64_SPLIT)
    A.set_symmetric_inner(fmt)
    A.set_element_matrices(0, ke)
    A.finalize()
    return m, ke, dofs, vals, A


@pytest.mark.parametrize("fmt", [3, 4, 5])
@pytest.mark.parametrize("kind,n", [(P.HEX20_ELASTIC, 5), (P.HEX8_ELASTIC, 8), (P.TET10_ELASTIC, 4),
                                    (P.HEX8_POISSON, 10), (P.TET10_POISSON, 6)])
def test_inner_product_matches_oracle(gpu, kind, n, fmt):
    import torch
    m, ke, _, _, A = operator(kind, n, fmt=fmt)
    u = np.random.default_rng(n).uniform(-1, 1, m.n_dofs)
    du = torch.tensor(u, device="cuda")
    dv = torch.full_like(du, float("nan"))
    A.matvec_inner_device(dv.data_ptr(), du.data_ptr())
    A.synchronize()
    v = dv.cpu().numpy()
    ref = oracle.Problem(m.n_dofs, m.dof_map(), ke).matvec(u)
    # formats 4 and 5 round u to FP32 (2^-24 of each entry), 5 also the element row sums
    assert rel(v, ref) < (INNER_RTOL if fmt == 3 else 1e-6)
    if fmt != 3:
        return
    # u scaled by powers of two far from 1: the product scales exactly
    for k in (-600, 600):
        du2 = du * 2.0 ** k
        dv2 = torch.empty_like(du2)
        A.matvec_inner_device(dv2.data_ptr(), du2.data_ptr())
        A.synchronize()
        assert np.array_equal(dv2.cpu().numpy(), v * 2.0 ** k)


def test_inner_product_needs_format_3(gpu):
    import torch
    m, ke, _, _, A = operator(P.HEX8_ELASTIC, 4, fmt=1)
    d = torch.zeros(m.n_dofs, dtype=torch.float64, device="cuda")
    with pytest.raises(AfmError) as e:
        A.matvec_inner_device(d.data_ptr(), d.clone().data_ptr())
    assert e.value.name == "ERR_STATE"


@pytest.mark.parametrize("fmt", [3, 4, 5])
@pytest.mark.parametrize("kind,n", [(P.HEX20_ELASTIC, 8), (P.HEX8_ELASTIC, 12)])
def test_fp64_vector_mixed_solve(gpu, kind, n, fmt):
    """The FP64-vector inner recursion converges to the FP64-checked tolerance in about the FP64 CG's
    iteration count (random loads on the elastic bar with its six point constraints)."""
    rtol = 1e-8
    m, ke, dofs, vals, A = operator(kind, n, bc=True, fmt=fmt)
    b = np.random.default_rng(7).normal(size=m.n_dofs)
    b[dofs.astype(np.int64)] = vals
    _, s64 = A.solve(b, rtol=rtol, atol=0.0, maxit=100000)
    x, st = A.solve_mixed(b, rtol=rtol, inner_rtol=0.3, max_outer=200, max_inner=20000)
    assert st.status == 0 and st.rel_residual <= rtol
    pr = oracle.Problem(m.n_dofs, m.dof_map(), ke, dofs, vals)
    assert np.linalg.norm(b - pr.matmult_bc(x)) <= 1.01 * rtol * np.linalg.norm(b)
    # format 5 rounds each element row's sum to FP32: a cheaper product, more iterations
    assert st.iterations <= (1.3 if fmt != 5 else 1.6) * s64.iterations + 20, (st.iterations, s64.iterations)
    tr = A.solve_trace()
    assert len(tr) == st.refinements + 1 and tr[-1][1] <= rtol
    assert all(a[0] <= b_[0] for a, b_ in zip(tr, tr[1:]))
