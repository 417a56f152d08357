"""Batched (multi right-hand side) products and solves against column-by-column
single-vector results and the CPU oracle."""
import numpy as np
import pytest

import oracle
from amat_gb300 import PRECISION, AfmError, Maps, aMatFree
from amat_gb300 import problems as P
from helpers import FP64_RTOL, rel

pytestmark = pytest.mark.gpu


def elastic(n, prec=PRECISION.FP64_SPLIT, bc=True, kind=None, seed=3):
    kind = P.HEX8_ELASTIC if kind is None else kind
    m = P.Mesh(kind, n, jitter=0.1, seed=seed)
    ke = m.element_matrices(ngt=3 if kind == P.HEX20_ELASTIC else 2)
    maps = Maps()
    maps.set_map(m.n_elem, m.dof_map(), m.ndpe, m.n_dofs)
    if bc:
        # clamp the bottom face so the batched solves are well posed
        lat = m.lattice
        bottom = np.nonzero(lat[:, 2] == 0)[0]
        dofs = np.sort(np.concatenate([3 * bottom + d for d in range(3)])).astype(np.uint64)
        maps.set_bdr_map(dofs, np.zeros(len(dofs)))
    else:
        dofs = np.zeros(0, dtype=np.uint64)
    A = aMatFree(maps)
    A.set_precision(prec)
    A.set_element_matrices(0, ke)
    A.finalize()
    return m, ke, dofs, A


@pytest.mark.parametrize("prec", [PRECISION.FP64, PRECISION.FP64_SPLIT])
@pytest.mark.parametrize("nrhs", [8, 64])
def test_batched_matvec_matches_columns(gpu, prec, nrhs):
    import torch
    m, ke, dofs, A = elastic(5, prec, bc=False)
    rng = np.random.default_rng(nrhs)
    U = rng.uniform(-1, 1, (m.n_dofs, nrhs))
    dU = torch.tensor(U, device="cuda")
    dV = torch.empty_like(dU)
    torch.cuda.synchronize()
    A.matvec_batched_device(dV.data_ptr(), dU.data_ptr(), nrhs)
    A.synchronize()
    V = dV.cpu().numpy()
    pr = oracle.Problem(m.n_dofs, m.dof_map(), ke)
    for j in range(0, nrhs, 7):
        assert rel(V[:, j], pr.matvec(U[:, j])) < FP64_RTOL
    ct, rt, ms = A.batch_tuning(nrhs)
    assert (ct, rt) in ((8, 2), (8, 4), (8, 6), (4, 4)) and ms > 0


@pytest.mark.parametrize("prec", [PRECISION.FP64, PRECISION.FP64_SPLIT])
@pytest.mark.parametrize("f32", [False, True])
@pytest.mark.parametrize("cfg", [(8, 2), (8, 4), (8, 6), (4, 4)])
def test_batched_every_configuration(gpu, prec, f32, cfg):
    import torch
    if f32 and prec == PRECISION.FP64:
        pytest.skip("FP32 product needs the split arena")
    m, ke, dofs, A = elastic(5, prec, bc=False)
    nrhs = 16
    U = np.random.default_rng(9).uniform(-1, 1, (m.n_dofs, nrhs))
    dt = torch.float32 if f32 else torch.float64
    dU = torch.tensor(U, dtype=dt, device="cuda")
    dV = torch.empty_like(dU)
    A.set_batch_tuning(nrhs, cfg[0], cfg[1], f32=f32)
    torch.cuda.synchronize()
    A.matvec_batched_device(dV.data_ptr(), dU.data_ptr(), nrhs, f32=f32)
    A.synchronize()
    V = dV.cpu().double().numpy()
    pr = oracle.Problem(m.n_dofs, m.dof_map(), ke)
    tol = 1e-5 if f32 else FP64_RTOL
    for j in (0, 1, 5, 15):
        assert rel(V[:, j], pr.matvec(U[:, j])) < tol, j


def test_batched_f32_and_bc(gpu):
    import torch
    m, ke, dofs, A = elastic(4, PRECISION.FP64_SPLIT, bc=True)
    nrhs = 16
    rng = np.random.default_rng(1)
    U = rng.uniform(-1, 1, (m.n_dofs, nrhs))
    pr = oracle.Problem(m.n_dofs, m.dof_map(), ke, dofs, np.zeros(len(dofs)))
    dU32 = torch.tensor(U, dtype=torch.float32, device="cuda")
    dV32 = torch.empty_like(dU32)
    dU = torch.tensor(U, device="cuda")
    dV = torch.empty_like(dU)
    torch.cuda.synchronize()
    A.matvec_batched_device(dV32.data_ptr(), dU32.data_ptr(), nrhs, f32=True)
    A.matvec_batched_device(dV.data_ptr(), dU.data_ptr(), nrhs, bc=True)
    A.synchronize()
    V32, V = dV32.cpu().double().numpy(), dV.cpu().numpy()
    for j in (0, 5, 15):
        assert rel(V32[:, j], pr.matvec(U[:, j])) < 1e-5
        assert rel(V[:, j], pr.matmult_bc(U[:, j])) < FP64_RTOL


def test_batched_ld_larger_than_nrhs(gpu):
    import torch
    m, ke, dofs, A = elastic(3, PRECISION.FP64_SPLIT, bc=False)
    nrhs, ld = 8, 12
    rng = np.random.default_rng(2)
    U = rng.uniform(-1, 1, (m.n_dofs, ld))
    dU = torch.tensor(U, device="cuda")
    dV = torch.zeros_like(dU)
    torch.cuda.synchronize()
    A.matvec_batched_device(dV.data_ptr(), dU.data_ptr(), nrhs, ld)
    A.synchronize()
    V = dV.cpu().numpy()
    pr = oracle.Problem(m.n_dofs, m.dof_map(), ke)
    for j in range(nrhs):
        assert rel(V[:, j], pr.matvec(U[:, j])) < FP64_RTOL


def test_batched_rejects_small_elements(gpu):
    import torch
    m = P.Mesh(P.HEX8_POISSON, 2)
    maps = Maps()
    maps.set_map(m.n_elem, m.dof_map(), m.ndpe, m.n_dofs)
    A = aMatFree(maps)
    A.set_element_matrices(0, m.element_matrices())
    A.finalize()
    d = torch.zeros((m.n_dofs, 4), dtype=torch.float64, device="cuda")
    with pytest.raises(AfmError) as e:
        A.matvec_batched_device(d.data_ptr(), d.clone().data_ptr(), 4)
    assert e.value.name == "NOT_IMPLEMENTED"


@pytest.mark.parametrize("mixed", [False, True])
def test_batched_cg_matches_single_solves(gpu, mixed):
    import torch
    m, ke, dofs, A = elastic(4, PRECISION.FP64_SPLIT, bc=True)
    nrhs = 8
    rng = np.random.default_rng(3)
    B = rng.normal(size=(m.n_dofs, nrhs))
    B[dofs.astype(np.int64), :] = 0.0
    dB = torch.tensor(B, device="cuda")
    dX = torch.zeros_like(dB)
    torch.cuda.synchronize()
    st = A.solve_batched_device(dB.data_ptr(), dX.data_ptr(), nrhs, rtol=1e-9, mixed=mixed)
    X = dX.cpu().numpy()
    assert st.status == 0 and st.rel_residual <= 1e-9 * 1.01
    pr = oracle.Problem(m.n_dofs, m.dof_map(), ke, dofs, np.zeros(len(dofs)))
    for j in (0, 3, 7):
        x, stj = A.solve(np.ascontiguousarray(B[:, j]), rtol=1e-9, atol=0.0)
        assert rel(X[:, j], x) < 1e-7
        r = B[:, j] - pr.matmult_bc(X[:, j])
        assert np.linalg.norm(r) <= 1.01e-9 * np.linalg.norm(B[:, j])


def test_batched_mixed_reliable_updates(gpu):
    """The FP32 block recursion continues across FP64 residual updates (its
    iteration count stays near the FP64 block CG's), and columns that meet
    their tolerance early (here a zero load case) stay frozen."""
    import torch
    m, ke, dofs, A = elastic(6, PRECISION.FP64_SPLIT, bc=True)
    nrhs = 8
    B = np.random.default_rng(11).normal(size=(m.n_dofs, nrhs))
    B[:, 5] = 0.0
    B[dofs.astype(np.int64), :] = 0.0
    dB = torch.tensor(B, device="cuda")
    dX = torch.zeros_like(dB)
    st64 = A.solve_batched_device(dB.data_ptr(), dX.data_ptr(), nrhs, rtol=1e-8)
    dX.zero_()
    torch.cuda.synchronize()
    st = A.solve_batched_device(dB.data_ptr(), dX.data_ptr(), nrhs, rtol=1e-8, mixed=True, inner_rtol=1e-3,
                                max_inner=32)
    X = dX.cpu().numpy()
    assert st.status == 0 and st.rel_residual <= 1e-8
    assert st.refinements >= 3
    assert st.iterations <= 1.5 * st64.iterations + 10, (st.iterations, st64.iterations)
    assert not np.any(X[:, 5])
    pr = oracle.Problem(m.n_dofs, m.dof_map(), ke, dofs, np.zeros(len(dofs)))
    for j in (0, 7):
        r = B[:, j] - pr.matmult_bc(X[:, j])
        assert np.linalg.norm(r) <= 1.01e-8 * np.linalg.norm(B[:, j])


@pytest.mark.parametrize("f32", [False, True])
@pytest.mark.parametrize("cfg", [(8, 2), (8, 4), (8, 6), (4, 4)])
def test_batched_many_elements_per_warp(gpu, f32, cfg):
    """Enough elements per CTA (hex8 elasticity 24^3: ~11 per CTA and colour)
    that every consumer warp takes several elements and the Ke ring wraps:
    the double-buffered U staging and the slot waits at full depth."""
    import torch
    m, ke, dofs, A = elastic(24, PRECISION.FP64_SPLIT, bc=False)
    nrhs = 64
    U = np.random.default_rng(21).uniform(-1, 1, (m.n_dofs, nrhs))
    dt = torch.float32 if f32 else torch.float64
    dU = torch.tensor(U, dtype=dt, device="cuda")
    dV = torch.empty_like(dU)
    A.set_batch_tuning(nrhs, cfg[0], cfg[1], f32=f32)
    torch.cuda.synchronize()
    A.matvec_batched_device(dV.data_ptr(), dU.data_ptr(), nrhs, f32=f32)
    A.synchronize()
    V = dV.cpu().double().numpy()
    pr = oracle.Problem(m.n_dofs, m.dof_map(), ke)
    tol = 1e-5 if f32 else FP64_RTOL
    for j in (0, 31, 63):
        assert rel(V[:, j], pr.matvec(U[:, j])) < tol, j
