"""Input range and error bound of the FP64-split product.

The split arithmetic stores every Ke entry as a pair of FP32 numbers (48
significant bits) and multiplies u, split the same way, with error-free FP32
transformations. FP32's exponent range is far narrower than FP64's, so each
product scales u by a power of two chosen from max|u| and max|Ke| (exact), and
the mixed-precision solve runs its FP32 recursion on the residual times a power
of two. These tests take u and the loads across the double range, use the
reference examples' Young's modulus (E = 1e6), check the error against an
exactly rounded product on near-null-space inputs (rigid-body modes of the
unconstrained elastic operator), and check that a solve's iterates scale
exactly with its load.
"""
import math

import numpy as np
import pytest

import oracle
from amat_gb300 import BC_METH, PRECISION, Maps, aMatFree
from amat_gb300 import problems as P
from helpers import FP64_RTOL, load, make_operator, rel

pytestmark = pytest.mark.gpu

# u scales of the parity sweep: from near the bottom of the normal double range to near its top
SCALES = [2.0 ** -1000, 1e-300, 1e-35, 1e-20, 1.0, 1e20, 1e35, 1e290]
CASES = [(P.HEX20_ELASTIC, 4, 3), (P.HEX8_ELASTIC, 6, 2), (P.TET10_POISSON, 6, 2), (P.HEX8_POISSON, 8, 2)]


def srel(a, b):
    """rel() of a / c and b / c, c = max|b|: the norms of vectors near the top of the double range
    would overflow."""
    c = np.abs(b).max()
    return rel(np.asarray(a) / c, np.asarray(b) / c) if c > 0 else rel(a, b)


def _operator(m, ke, prec, bc=None, bc_method=BC_METH.BC_IMATRIX):
    maps = Maps()
    maps.set_map(m.n_elem, m.dof_map(), m.ndpe, m.n_dofs)
    if bc is not None:
        maps.set_bdr_map(*bc)
    A = aMatFree(maps, bc_method)
    A.set_precision(prec)
    A.set_element_matrices(0, ke)
    A.finalize()
    return A


@pytest.mark.parametrize("E", [1.0, 1e6])
@pytest.mark.parametrize("kind,n,ngt", CASES)
def test_split_product_across_the_double_range(gpu, kind, n, ngt, E):
    """v = K u for |u| from 1e-301 to 1e290: the split product stays within
    1e-12 of the FP64 oracle (warp-group, thread-per-element and patch kernels)."""
    m = P.Mesh(kind, n, jitter=0.1, seed=5)
    ke = m.element_matrices(E=E, ngt=ngt)
    A = _operator(m, ke, PRECISION.FP64_SPLIT)
    assert A.info()["precision"] == PRECISION.FP64_SPLIT
    pr = oracle.Problem(m.n_dofs, m.dof_map(), ke)
    u0 = np.random.default_rng(8).uniform(-1, 1, m.n_dofs)
    for s in SCALES:
        u = u0 * s
        v = np.empty(m.n_dofs)
        A.matvec(v, u, True)
        ref = pr.matvec(u)
        assert np.all(np.isfinite(v)), s
        assert srel(v, ref) < FP64_RTOL, s


@pytest.mark.parametrize("name", ["mixed_random", "hex8_poisson_4", "tet10_elastic_2"])
def test_split_product_of_golden_problems_scaled(gpu, name):
    """Non-symmetric random element matrices and the reference's own problems, u scaled far from 1."""
    g = load(name)
    A = make_operator(g, 0, PRECISION.FP64_SPLIT)
    for s in (2.0 ** -600, 2.0 ** 600):
        v = np.empty(int(g["n_dofs"]))
        A.matvec(v, g["u"] * s, True)
        assert srel(v, g["matvec"] * s) < FP64_RTOL


def test_split_scale_ignores_constrained_columns(gpu):
    """MatMult_mf reads constrained columns as zero, so huge prescribed values
    there must not set the scale of the other columns."""
    m = P.Mesh(P.HEX20_ELASTIC, 4, jitter=0.1, seed=2)
    ke = m.element_matrices(ngt=3)
    dofs, vals = m.boundary_conditions()
    A = _operator(m, ke, PRECISION.FP64_SPLIT, (dofs, vals))
    pr = oracle.Problem(m.n_dofs, m.dof_map(), ke, dofs, vals)
    u = np.random.default_rng(3).uniform(-1, 1, m.n_dofs)
    con = dofs.astype(np.int64)
    u[con] = 1e300
    free = np.ones(m.n_dofs, bool)
    free[con] = False
    w = np.empty(m.n_dofs)
    A.matmult_bc(w, u)
    ref = pr.matmult_bc(u)
    assert rel(w[free], ref[free]) < FP64_RTOL
    assert np.array_equal(w[con], u[con])


def test_split_rejects_element_matrices_outside_fp32(gpu):
    m = P.Mesh(P.HEX8_POISSON, 2)
    ke = m.element_matrices() * 1e300
    from amat_gb300 import AfmError
    with pytest.raises(AfmError) as e:
        _operator(m, ke, PRECISION.FP64_SPLIT)
    assert e.value.name == "ERR_INVALID_ARG"
    A = _operator(m, ke, PRECISION.AUTO)  # AUTO keeps such an operator in FP64
    assert A.info()["precision"] == PRECISION.FP64


def _veltkamp(x):
    """x = hi + lo with hi, lo of at most 26 significant bits (products of halves are exact in FP64)."""
    c = 134217729.0 * x
    hi = c - (c - x)
    return hi, x - hi


def exact_product(n_dofs, dof_map, ke, u):
    """K u rounded once (error-free products of Veltkamp halves, math.fsum per DoF) and |K| |u|."""
    ne = ke.shape[1]
    ue = u[dof_map]
    kh, kl = _veltkamp(ke)
    uh, ul = _veltkamp(ue)
    terms = np.stack([kh * uh[:, None, :], kh * ul[:, None, :], kl * uh[:, None, :], kl * ul[:, None, :]])
    rows = np.broadcast_to(dof_map[None, :, :, None], terms.shape).ravel()
    t = terms.ravel()
    order = np.argsort(rows, kind="stable")
    rows, t = rows[order], t[order]
    cut = np.flatnonzero(np.diff(rows)) + 1
    v = np.zeros(n_dofs)
    for idx, part in zip(np.split(rows, cut), np.split(t, cut)):
        v[idx[0]] = math.fsum(part.tolist())
    mag = np.zeros(n_dofs)
    np.add.at(mag, dof_map, np.einsum("erc,ec->er", np.abs(ke), np.abs(ue)))
    return v, mag


def rigid_modes(coords):
    """The six rigid-body displacements of a 3-D body (three translations, three rotations)."""
    x, y, z = coords[:, 0], coords[:, 1], coords[:, 2]
    one, zero = np.ones_like(x), np.zeros_like(x)
    fields = [(one, zero, zero), (zero, one, zero), (zero, zero, one),
              (-y, x, zero), (zero, -z, y), (z, zero, -x)]
    return [np.stack(f, axis=1).ravel() for f in fields]


@pytest.mark.parametrize("kind,n,ngt", [(P.HEX20_ELASTIC, 4, 3), (P.HEX8_ELASTIC, 6, 2), (P.TET10_ELASTIC, 3, 2)])
def test_split_error_bound_on_rigid_body_modes(gpu, kind, n, ngt):
    """Near-null-space u: K u is ~1e-16 |K||u| (zero in exact arithmetic but for the rounding of Ke), so
    a relative error of v says nothing; both arithmetics are held to bounds in |K||u| terms instead.
    Per element row, the double-float sum of n terms is within (8 n + 10) 2^-48 |Ke||u_e| (entry and u
    splits 2 x 2^-48, cross terms 3 x 2^-48, the FP32 sum of the low parts 8 n 2^-48); the FP64 sum of
    the colours' contributions adds at most 32 x 2^-53 |K||u|. Observed errors are far below that
    (random rounding), so the test also holds them to 2^-44 |K||u|; FP64 native to 2^-46."""
    m = P.Mesh(kind, n, jitter=0.1, seed=4)
    E = 1e6
    ke = m.element_matrices(E=E, ngt=ngt)
    dm = m.dof_map().reshape(m.n_elem, m.ndpe).astype(np.int64)
    S = _operator(m, ke, PRECISION.FP64_SPLIT)
    D = _operator(m, ke, PRECISION.FP64)
    ne = m.ndpe
    bound = (8 * ne + 10) * 2.0 ** -48 + 32 * 2.0 ** -53
    rng = np.random.default_rng(9)
    modes = rigid_modes(m.coords)
    # the modes, a random combination of them, and one with a small random perturbation
    comb = sum(rng.normal() * q for q in modes)
    cases = modes + [comb, comb + 1e-9 * rng.uniform(-1, 1, m.n_dofs)]
    for u in cases:
        exact, mag = exact_product(m.n_dofs, dm, ke, u)
        vs, vd = np.empty(m.n_dofs), np.empty(m.n_dofs)
        S.matvec(vs, u, True)
        D.matvec(vd, u, True)
        mask = mag > 0
        es = np.abs(vs - exact)[mask] / mag[mask]
        ed = np.abs(vd - exact)[mask] / mag[mask]
        assert es.max() <= bound
        assert es.max() <= 2.0 ** -44
        assert ed.max() <= 2.0 ** -46
        # K u of a rigid mode is tiny next to |K||u|: the products are dominated by cancellation
        if u is modes[0]:
            assert np.linalg.norm(exact) < 1e-10 * np.linalg.norm(mag)


def _poisson(n, prec):
    m = P.Mesh(P.HEX8_POISSON, n, jitter=0.1, seed=3)
    ke = m.element_matrices()
    dofs, vals = m.boundary_conditions()
    return m, _operator(m, ke, prec, (dofs, vals))


@pytest.mark.parametrize("k", [-116, 116, -300, 300])
def test_solves_scale_exactly_with_the_load(gpu, k):
    """b -> 2^k b: the FP64 CG and the mixed solve on the split operator give 2^k x bit for bit, with the
    same iteration counts (every scale in the path is a power of two). Unscaled, 2^-116 ~ 1.2e-35 would put
    the FP32 residuals among FP32's subnormals, 2^-300 below FP32's range altogether, and 2^116 or 2^300
    would overflow FP32 dot products."""
    m, A = _poisson(10, PRECISION.FP64_SPLIT)
    rhs = A.apply_bc(m.load())
    f = 2.0 ** k
    x1, s1 = A.solve(rhs, rtol=1e-10, atol=0.0, maxit=4000)
    x2, s2 = A.solve(rhs * f, rtol=1e-10, atol=0.0, maxit=4000)
    assert s1.status == 0 and s2.status == 0 and s1.iterations == s2.iterations
    assert np.array_equal(x2, x1 * f)
    y1, t1 = A.solve_mixed(rhs, rtol=1e-8, inner_rtol=0.1)
    y2, t2 = A.solve_mixed(rhs * f, rtol=1e-8, inner_rtol=0.1)
    assert t1.status == 0 and t2.status == 0
    assert (t1.iterations, t1.refinements) == (t2.iterations, t2.refinements)
    assert np.array_equal(y2, y1 * f)
    assert rel(y2 / f, x1) < 1e-7


def test_split_accepts_tiny_entries_beside_large_ones(gpu):
    """Quadrature leaves the exact zeros of an element matrix as ~1e-35 round-off (tet10 elasticity): the
    split range is judged per element (its largest entry), so AUTO keeps the split arithmetic and the
    product stays within the FP64 bar."""
    m = P.Mesh(P.TET10_ELASTIC, 3, jitter=0.15, seed=2)
    ke = m.element_matrices(ngt=2)
    ke[0, 0, 5] = ke[0, 5, 0] = 3e-40  # a double below FP32's normal range, beside O(0.1) entries
    ke[1, 2, 7] = 1e-36
    A = _operator(m, ke, PRECISION.AUTO)
    assert A.info()["precision"] == PRECISION.FP64_SPLIT
    pr = oracle.Problem(m.n_dofs, m.dof_map(), ke)
    u = np.random.default_rng(4).uniform(-1, 1, m.n_dofs)
    v = np.empty(m.n_dofs)
    A.matvec(v, u, True)
    assert rel(v, pr.matvec(u)) < FP64_RTOL
    # an element whose largest entry is below 1e-30 keeps the operator in FP64
    ke2 = ke.copy()
    ke2[3] *= 1e-35
    assert _operator(m, ke2, PRECISION.AUTO).info()["precision"] == PRECISION.FP64
