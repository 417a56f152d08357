"""Device Jacobi-PCG (the example drivers' par::solve, KSPCG + PCJACOBI on the
MatMult_mf shell) against the oracle PCG and the examples' analytic solution."""
import numpy as np
import pytest

import oracle
from amat_gb300 import BC_METH, CG_NORM, PRECISION, AfmError, Maps, aMatFree
from amat_gb300 import problems as P
from helpers import load, make_operator, rel

pytestmark = pytest.mark.gpu


def poisson(n, jitter=0.0, seed=0, prec=PRECISION.AUTO, bc=BC_METH.BC_IMATRIX):
    m = P.Mesh(P.HEX8_POISSON, n, jitter=jitter, seed=seed)
    ke = m.element_matrices()
    dofs, vals = m.boundary_conditions()
    maps = Maps()
    maps.set_map(m.n_elem, m.dof_map(), m.ndpe, m.n_dofs)
    maps.set_bdr_map(dofs, vals)
    A = aMatFree(maps, bc)
    A.set_precision(prec)
    A.set_element_matrices(0, ke)
    A.finalize()
    return m, ke, dofs, vals, A


@pytest.mark.parametrize("prec", [PRECISION.FP64, PRECISION.FP64_SPLIT])
def test_cg_matches_oracle_pcg(gpu, prec):
    m, ke, dofs, vals, A = poisson(8, jitter=0.1, seed=3, prec=prec)
    rhs = A.apply_bc(m.load())
    x, st = A.solve(rhs, rtol=1e-10, atol=0.0, maxit=2000)
    pr = oracle.Problem(m.n_dofs, m.dof_map(), ke, dofs, vals)
    xo, it, res = pr.pcg(rhs, rtol=1e-10, atol=0.0, maxit=2000)
    assert st.status == 0 and st.rel_residual <= 1e-10 * 1.01
    assert abs(st.iterations - it) <= 1
    assert rel(x, xo) < 1e-8


def test_cg_poisson_analytic_solution(gpu):
    """example03a: u = sin(2 pi x) sin(2 pi y) sin(2 pi z) / (12 pi^2) on the unit cube."""
    errs = []
    for n in (8, 16):
        m, ke, dofs, vals, A = poisson(n)
        rhs = A.apply_bc(m.load(ngt=3))
        x, st = A.solve(rhs, rtol=1e-10, atol=0.0)
        c = m.coords
        exact = np.sin(2 * np.pi * c[:, 0]) * np.sin(2 * np.pi * c[:, 1]) * np.sin(2 * np.pi * c[:, 2]) / (12 * np.pi ** 2)
        errs.append(np.abs(x - exact).max() / np.abs(exact).max())
    assert errs[1] < 0.05 and errs[1] < errs[0] / 3  # second-order convergence


def test_cg_golden_problem_and_penalty(gpu):
    g = load("hex8_poisson_4")
    for bc in (BC_METH.BC_IMATRIX, BC_METH.BC_PENALTY):
        A = make_operator(g, bc, PRECISION.FP64)
        rhs = g["rhs"].copy()
        A.apply_bc(rhs)
        x, st = A.solve(rhs, rtol=1e-12, atol=0.0)
        pr = oracle.Problem(int(g["n_dofs"]), g["map"].reshape(-1, 8), g["ke"].reshape(-1, 8, 8),
                            g["constrained"], g["values"])
        xo, it, _ = pr.pcg(rhs, rtol=1e-12, atol=0.0, bc_method=int(bc))
        assert it >= 0 and rel(x, xo) < 1e-9


def test_cg_preconditioned_norm_option(gpu):
    m, ke, dofs, vals, A = poisson(6)
    rhs = A.apply_bc(m.load())
    x, st = A.solve(rhs, rtol=1e-10, atol=0.0, norm=CG_NORM.PRECONDITIONED)
    pr = oracle.Problem(m.n_dofs, m.dof_map(), ke, dofs, vals)
    xo, it, _ = pr.pcg(rhs, rtol=1e-10, atol=0.0, norm_type=1)
    assert abs(st.iterations - it) <= 1 and rel(x, xo) < 1e-8


def test_cg_breakdown_and_maxit_are_reported(gpu):
    m, ke, dofs, vals, A = poisson(6)
    rhs = A.apply_bc(m.load())
    bad = rhs.copy()
    bad[7] = np.nan
    with pytest.raises(AfmError) as e:
        A.solve(bad, rtol=1e-10)
    assert e.value.name == "ERR_BREAKDOWN"
    # a random load: the sine load is an eigenvector of the uniform-mesh operator
    rnd = A.apply_bc(np.random.default_rng(5).normal(size=m.n_dofs))
    x, st = A.solve(rnd, rtol=1e-14, atol=0.0, maxit=3, raise_on_fail=False)
    assert st.status == 106 and st.iterations == 3
    # the operator stays usable after both
    x, st = A.solve(rhs, rtol=1e-10, atol=0.0)
    assert st.status == 0


def test_mixed_precision_refinement(gpu):
    """FP32 inner Jacobi-PCG with FP64 outer residual reaches the FP64 tolerance."""
    m, ke, dofs, vals, A = poisson(12, jitter=0.15, seed=7, prec=PRECISION.FP64_SPLIT)
    rhs = A.apply_bc(m.load())
    x64, st64 = A.solve(rhs, rtol=1e-10, atol=0.0)
    x, st = A.solve_mixed(rhs, rtol=1e-8, atol=0.0, inner_rtol=1e-4)
    assert st.status == 0 and st.rel_residual <= 1e-8
    assert st.refinements >= 2 and st.iterations > 0
    assert rel(x, x64) < 1e-6
    pr = oracle.Problem(m.n_dofs, m.dof_map(), ke, dofs, vals)
    r = rhs - pr.matmult_bc(x)
    assert np.linalg.norm(r) <= 1.01e-8 * np.linalg.norm(rhs)


def test_mixed_precision_needs_split_arena(gpu):
    m, ke, dofs, vals, A = poisson(4, prec=PRECISION.FP64)
    with pytest.raises(AfmError) as e:
        A.solve_mixed(A.apply_bc(m.load()))
    assert e.value.name == "ERR_STATE"


def test_mixed_precision_tet10(gpu):
    """Mixed refinement on a jittered tet10 Poisson mesh (thread-per-element regime, many colours)."""
    m = P.Mesh(P.TET10_POISSON, 10, jitter=0.15, seed=2)
    ke = m.element_matrices()
    dofs, vals = m.boundary_conditions()
    maps = Maps()
    maps.set_map(m.n_elem, m.dof_map(), m.ndpe, m.n_dofs)
    maps.set_bdr_map(dofs, vals)
    A = aMatFree(maps)
    A.set_precision(PRECISION.FP64_SPLIT)
    A.set_element_matrices(0, ke)
    A.finalize()
    rhs = A.apply_bc(m.load())
    x64, st64 = A.solve(rhs, rtol=1e-10, atol=0.0)
    x, st = A.solve_mixed(rhs, rtol=1e-8, atol=0.0, inner_rtol=1e-4, raise_on_fail=False)
    assert st.status == 0, (st.refinements, st.iterations, st.rel_residual)
    assert rel(x, x64) < 1e-6


def test_mixed_precision_keeps_the_krylov_space(gpu):
    """Reliable updates continue one FP32 recursion, so the FP32 iteration
    count stays near the FP64 one instead of restarting per refinement."""
    m, ke, dofs, vals, A = poisson(16, jitter=0.15, seed=5, prec=PRECISION.FP64_SPLIT)
    rhs = A.apply_bc(m.load())
    x64, st64 = A.solve(rhs, rtol=1e-8, atol=0.0)
    x, st = A.solve_mixed(rhs, rtol=1e-8, atol=0.0, inner_rtol=0.1)
    assert st.status == 0 and st.rel_residual <= 1e-8
    assert st.refinements >= 3
    assert st.iterations <= 1.5 * st64.iterations + 10, (st.iterations, st64.iterations)
    assert rel(x, x64) < 1e-6
