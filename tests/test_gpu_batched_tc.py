"""The tensor-core batched FP32 product (tcgen05, 3xTF32) against the oracle,
column by column, for every stacking of elements it uses (nrhs 32, 64, 128),
specialised and run-time element sizes, a padded leading dimension, the
MatMult_mf form, and bit-for-bit repeatability."""
import numpy as np
import pytest

import oracle
from amat_gb300 import PRECISION, Maps, aMatFree
from amat_gb300 import problems as P
from helpers import rel

pytestmark = pytest.mark.gpu

# FP32 products of the split arena's hi plane: its Ke is rounded to FP32, and the 3xTF32 products add ~2^-21
TC_RTOL = 1e-5


def operator(kind, n, bc):
    m = P.Mesh(kind, n, jitter=0.1, seed=11)
    ke = m.element_matrices(ngt=3 if kind == P.HEX20_ELASTIC else 2)
    maps = Maps()
    maps.set_map(m.n_elem, m.dof_map(), m.ndpe, m.n_dofs)
    dofs, vals = (m.boundary_conditions() if bc else (np.zeros(0, np.uint64), np.zeros(0)))
    maps.set_bdr_map(dofs, vals)
    A = aMatFree(maps)
    A.set_precision(PRECISION.FP64_SPLIT)
    A.set_element_matrices(0, ke)
    A.finalize()
    return m, ke, dofs, vals, A


@pytest.mark.parametrize("kind,n,nrhs,pad", [
    (P.HEX8_ELASTIC, 6, 64, 0), (P.HEX8_ELASTIC, 6, 32, 0), (P.HEX8_ELASTIC, 6, 128, 0),
    (P.HEX8_ELASTIC, 6, 64, 8), (P.HEX20_ELASTIC, 4, 64, 0), (P.HEX20_ELASTIC, 4, 32, 0),
    (P.TET10_ELASTIC, 4, 64, 0), (P.TET10_ELASTIC, 4, 128, 4),
])
def test_tc_product_matches_oracle(gpu, kind, n, nrhs, pad):
    import torch
    m, ke, _, _, A = operator(kind, n, False)
    ld = nrhs + pad
    U = np.random.default_rng(nrhs + n).uniform(-1, 1, (m.n_dofs, ld)).astype(np.float32)
    dU = torch.tensor(U, device="cuda")
    dV = torch.full_like(dU, float("nan"))
    A.set_batch_tuning(nrhs, 0, 0, ld=ld, f32=True)
    torch.cuda.synchronize()
    A.matvec_batched_device(dV.data_ptr(), dU.data_ptr(), nrhs, ld=ld, f32=True)
    A.synchronize()
    V = dV.cpu().double().numpy()
    pr = oracle.Problem(m.n_dofs, m.dof_map(), ke)
    for j in range(0, nrhs, 5):
        assert rel(V[:, j], pr.matvec(U[:, j].astype(np.float64))) < TC_RTOL, j
    assert A.batch_tuning(nrhs, ld=ld, f32=True)[:2] == (0, 0)
    # the same product again: bit for bit
    dW = torch.empty_like(dU)
    A.matvec_batched_device(dW.data_ptr(), dU.data_ptr(), nrhs, ld=ld, f32=True)
    A.synchronize()
    assert torch.equal(dW[:, :nrhs], dV[:, :nrhs])


def test_tc_matmult_bc(gpu):
    import torch
    m, ke, dofs, vals, A = operator(P.HEX8_ELASTIC, 6, True)
    nrhs = 64
    U = np.random.default_rng(2).uniform(-1, 1, (m.n_dofs, nrhs)).astype(np.float32)
    dU = torch.tensor(U, device="cuda")
    dV = torch.empty_like(dU)
    A.set_batch_tuning(nrhs, 0, 0, f32=True)
    torch.cuda.synchronize()
    A.matvec_batched_device(dV.data_ptr(), dU.data_ptr(), nrhs, f32=True, bc=True)
    A.synchronize()
    V = dV.cpu().double().numpy()
    pr = oracle.Problem(m.n_dofs, m.dof_map(), ke, dofs, vals)
    for j in (0, 17, 63):
        assert rel(V[:, j], pr.matmult_bc(U[:, j].astype(np.float64))) < TC_RTOL


def test_tc_agrees_with_cuda_core_kernel(gpu):
    """Both FP32 kernels of the batched product agree to FP32 precision."""
    import torch
    m, ke, _, _, A = operator(P.HEX8_ELASTIC, 8, False)
    nrhs = 64
    dU = torch.empty((m.n_dofs, nrhs), device="cuda").uniform_(-1, 1)
    out = []
    for tile in ((0, 0), (8, 4)):
        A.set_batch_tuning(nrhs, *tile, f32=True)
        dV = torch.empty_like(dU)
        A.matvec_batched_device(dV.data_ptr(), dU.data_ptr(), nrhs, f32=True)
        A.synchronize()
        out.append(dV.double().cpu().numpy())
    assert rel(out[0], out[1]) < 2e-6


def test_mixed_block_solve_keeps_cuda_core_products(gpu):
    """The batched mixed solve tunes its FP32 recursion among the CUDA-core tiles only, under its own
    key: pinning the plain FP32 product to the tensor cores leaves the solve's choice alone."""
    import torch
    m, ke, dofs, vals, A = operator(P.HEX8_ELASTIC, 6, True)
    nrhs = 64
    A.set_batch_tuning(nrhs, 0, 0, f32=True)
    B = np.random.default_rng(4).normal(size=(m.n_dofs, nrhs))
    B[dofs.astype(np.int64), :] = 0.0
    dB = torch.tensor(B, device="cuda")
    dX = torch.zeros_like(dB)
    torch.cuda.synchronize()
    st = A.solve_batched_device(dB.data_ptr(), dX.data_ptr(), nrhs, rtol=1e-8, mixed=True, inner_rtol=1e-3)
    assert st.status == 0 and st.rel_residual <= 1e-8
    assert A.batch_tuning(nrhs, solve=True)[:2] != (0, 0)
    assert A.batch_tuning(nrhs, f32=True)[:2] == (0, 0)
    X = dX.cpu().numpy()
    pr = oracle.Problem(m.n_dofs, m.dof_map(), ke, dofs, np.zeros(len(dofs)))
    for j in (0, 40):
        r = B[:, j] - pr.matmult_bc(X[:, j])
        assert np.linalg.norm(r) <= 1.01e-8 * np.linalg.norm(B[:, j])
