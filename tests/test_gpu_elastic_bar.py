"""CG solutions of the examples' elastic bar against its exact displacement.

The bar (examples/src/example06a.cpp:9-15, example07a.cpp:938-946) hangs
under its own weight rho g with the traction rho g Lz on its top face and
rigid motions blocked at centre nodes; with x, y measured from the axis,
  u = -(nu rho g / E) x z,  v = -(nu rho g / E) y z,
  w = (rho g / 2E)(z^2 - Lz^2) + (nu rho g / 2E)(x^2 + y^2).
The field is quadratic, so on undistorted hex20 (serendipity) elements the
discrete solution is the exact one up to the solver's tolerance; hex8
elements converge at second order.
"""
import numpy as np
import pytest

from amat_gb300 import PRECISION, Maps, aMatFree
from amat_gb300 import problems as P

pytestmark = pytest.mark.gpu

E, NU, RHO_G = 1.0, 0.3, 1.0


def exact_displacement(coords, L=(1.0, 1.0, 1.0)):
    x = coords[:, 0] - L[0] / 2
    y = coords[:, 1] - L[1] / 2
    z = coords[:, 2]
    c = RHO_G / E
    u = -NU * c * x * z
    v = -NU * c * y * z
    w = 0.5 * c * (z * z - L[2] ** 2) + 0.5 * NU * c * (x * x + y * y)
    return np.stack([u, v, w], axis=1).ravel()


def bar_solution(kind, n, mixed=False):
    m = P.Mesh(kind, n)
    ngt = 3 if kind == P.HEX20_ELASTIC else 2
    dofs, vals = m.boundary_conditions()
    maps = Maps()
    maps.set_map(m.n_elem, m.dof_map(), m.ndpe, m.n_dofs)
    maps.set_bdr_map(dofs, vals)
    A = aMatFree(maps)
    A.set_precision(PRECISION.AUTO)
    A.set_element_matrices(0, m.element_matrices(E=E, nu=NU, ngt=ngt))
    A.finalize()
    rhs = A.apply_bc(m.load(ngt=ngt, rho_g=RHO_G))
    if mixed:
        x, st = A.solve_mixed(rhs, rtol=1e-10, inner_rtol=0.1)
    else:
        x, st = A.solve(rhs, rtol=1e-11, atol=0.0, maxit=20000)
    assert st.status == 0
    ex = exact_displacement(m.coords)
    return np.abs(x - ex).max() / np.abs(ex).max()


@pytest.mark.parametrize("mixed", [False, True])
def test_hex20_bar_is_exact(gpu, mixed):
    """Quadratic field in the serendipity space: the FP64 CG and the mixed-precision solve recover it
    to the solver tolerance (the mixed solve's FP64 residual is checked to 1e-10)."""
    for n in (4, 8):
        assert bar_solution(P.HEX20_ELASTIC, n, mixed) < 1e-7


def test_hex8_bar_converges_at_second_order(gpu):
    """Max-norm error of the trilinear solution: O(h^2) (ratio -> 4 per halving of h; the coarsest
    mesh is still pre-asymptotic)."""
    errs = [bar_solution(P.HEX8_ELASTIC, n) for n in (4, 8, 16)]
    assert errs[2] < 0.01
    assert errs[1] < errs[0] / 2.5 and errs[2] < errs[1] / 3
