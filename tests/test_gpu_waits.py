"""Bounded waits of the element kernels. With the wait probe on, one warp of
every element-kernel launch waits for a flag that nothing sets; its wait runs
out after the operator's (short) wait limit, the call reports ERR_TIMEOUT, and
the operator gives the same results as before once the probe is off. Nothing
here faults or hangs the GPU: every wait gives up after the limit, the
producer lets each copy it issued land before its block exits, and the
timed-out call only leaves an error flag for the host."""
import numpy as np
import pytest

import oracle
from amat_gb300 import PRECISION, AfmError, Maps, aMatFree
from amat_gb300 import problems as P
from helpers import FP64_RTOL, load, make_operator, rel

pytestmark = pytest.mark.gpu

LIMIT = 5e-3  # seconds: far above any wait of a working launch, short enough to run out quickly


def _mesh_operator(kind, n, prec, patch=1):
    m = P.Mesh(kind, n, jitter=0.1, seed=3)
    ke = m.element_matrices(ngt=3 if kind == P.HEX20_ELASTIC else 2)
    maps = Maps()
    maps.set_map(m.n_elem, m.dof_map(), m.ndpe, m.n_dofs)
    A = aMatFree(maps)
    A.set_precision(prec)
    A.set_patch_mode(patch)
    A.set_element_matrices(0, ke)
    A.finalize()
    return oracle.Problem(m.n_dofs, m.dof_map(), ke), A


def _expire(A, u):
    """One product with the probe on: it must report ERR_TIMEOUT."""
    A.set_wait_limit(LIMIT)
    A.set_wait_probe(1)
    try:
        with pytest.raises(AfmError) as e:
            A.matvec(np.empty(len(u)), u, True)
        assert e.value.name == "ERR_TIMEOUT"
    finally:
        A.set_wait_probe(0)
        A.set_wait_limit(4.0)


@pytest.mark.parametrize("kind,n,prec,patch", [
    (P.HEX20_ELASTIC, 12, PRECISION.FP64_SPLIT, 1),   # warp-group kernel
    (P.HEX20_ELASTIC, 12, PRECISION.FP64, 1),
    (P.TET10_POISSON, 12, PRECISION.FP64_SPLIT, 1),   # patch kernel
    (P.HEX8_POISSON, 24, PRECISION.FP64_SPLIT, 0),    # thread-per-element kernel
    (P.TET10_ELASTIC, 6, PRECISION.FP64, 0),          # warp-group kernel, run-time n = 30
])
def test_short_wait_limit_times_out_and_operator_recovers(gpu, kind, n, prec, patch):
    pr, A = _mesh_operator(kind, n, prec, patch)
    u = np.random.default_rng(1).uniform(-1, 1, pr.n_dofs)
    ref = pr.matvec(u)
    v0 = np.empty(pr.n_dofs)
    A.matvec(v0, u, True)
    assert rel(v0, ref) < FP64_RTOL
    _expire(A, u)
    v1 = np.empty(pr.n_dofs)
    A.matvec(v1, u, True)
    assert np.array_equal(v1, v0)


def test_short_wait_limit_warp_per_element(gpu):
    """Elements that list a DoF twice run on the warp-per-element kernel."""
    rng = np.random.default_rng(5)
    n_dofs, elems, kes = 300, [], []
    for i in range(200):
        e = rng.choice(n_dofs, size=20, replace=False).astype(np.uint32)
        e[-1] = e[0]
        elems.append(e)
        kes.append(rng.normal(size=(20, 20)))
    maps = Maps()
    maps.set_map(len(elems), np.concatenate(elems), np.full(len(elems), 20, np.uint32), n_dofs)
    A = aMatFree(maps)
    A.set_precision(PRECISION.FP64_SPLIT)
    for k, ke in enumerate(kes):
        A.set_element_matrix(k, ke)
    A.finalize()
    u = rng.uniform(-1, 1, n_dofs)
    v0 = np.empty(n_dofs)
    A.matvec(v0, u, True)
    assert rel(v0, oracle.Problem(n_dofs, elems, kes).matvec(u)) < FP64_RTOL
    _expire(A, u)
    v1 = np.empty(n_dofs)
    A.matvec(v1, u, True)
    assert np.array_equal(v1, v0)


def test_short_wait_limit_in_a_solve(gpu):
    """The captured CG iterations take the hook and the limit (they are captured again), the solve
    reports the timeout, and the next solve without the hook converges as before, bit for bit."""
    m = P.Mesh(P.HEX20_ELASTIC, 8, jitter=0.1, seed=2)
    ke = m.element_matrices(ngt=3)
    dofs, vals = m.boundary_conditions()
    maps = Maps()
    maps.set_map(m.n_elem, m.dof_map(), m.ndpe, m.n_dofs)
    maps.set_bdr_map(dofs, vals)
    A = aMatFree(maps)
    A.set_precision(PRECISION.FP64_SPLIT)
    A.set_element_matrices(0, ke)
    A.finalize()
    rhs = A.apply_bc(m.load(ngt=3))
    x0, s0 = A.solve(rhs, rtol=1e-8, atol=0.0, maxit=5000)
    A.set_wait_limit(LIMIT)
    A.set_wait_probe(1)
    with pytest.raises(AfmError) as e:
        A.solve(rhs, rtol=1e-8, atol=0.0, maxit=10)
    assert e.value.name == "ERR_TIMEOUT"
    A.set_wait_probe(0)
    A.set_wait_limit(4.0)
    x1, s1 = A.solve(rhs, rtol=1e-8, atol=0.0, maxit=5000)
    assert s1.iterations == s0.iterations and np.array_equal(x1, x0)


def test_wait_limit_arguments(gpu):
    g = load("hex8_poisson_4")
    A = make_operator(g, 0, PRECISION.FP64)
    for bad in (0.0, -1.0, 1e-12, 601.0, float("nan")):
        with pytest.raises(AfmError) as e:
            A.set_wait_limit(bad)
        assert e.value.name == "ERR_INVALID_ARG"
    assert A._lib.afm_set_wait_probe(A._h, 2) == 105  # ERR_INVALID_ARG
    A.set_wait_limit(0.5)
    v = np.empty(int(g["n_dofs"]))
    A.matvec(v, g["u"], True)
    assert rel(v, g["matvec"]) < FP64_RTOL
