"""Assembled operator (par::aMatBased): the host assembly against the
reference's own assembled matrix (golden CSR written from the reference),
bit for bit, for the identity and penalty methods; and the device SpMV
against the reference's products and the assembly-free product."""
import numpy as np
import pytest
import scipy.sparse as sp

from amat_gb300 import BC_METH, PRECISION, Maps, aMatFree
from amat_gb300 import problems as P
from amat_gb300.afm import assemble_csr_host
from helpers import FP64_RTOL, golden_names, load, make_operator, rel

ASM = [n for n in golden_names() if "asm_vals" in load(n)]


@pytest.mark.parametrize("name", ASM)
def test_host_assembly_matches_reference_matrix(name):
    g = load(name)
    n = int(g["n_dofs"])
    for bc, key in [(BC_METH.BC_IMATRIX, "asm_vals"), (BC_METH.BC_PENALTY, "asm_vals_penalty")]:
        rp, cols, vals = assemble_csr_host(n, g["offsets"], g["map"], g["ke"], g["constrained"], bc, True)
        assert np.array_equal(rp, g["asm_row_ptr"]) and np.array_equal(cols, g["asm_cols"])
        assert np.array_equal(vals, g[key])  # same sums in the same order: bit for bit


@pytest.mark.parametrize("name", ASM)
def test_host_assembly_products(name):
    """K u before the boundary conditions and K_bc u after them, as the reference's MatMult gives them."""
    g = load(name)
    n = int(g["n_dofs"])
    rp, cols, vals = assemble_csr_host(n, g["offsets"], g["map"], g["ke"], g["constrained"], BC_METH.BC_IMATRIX,
                                       False)
    K = sp.csr_matrix((vals, cols.astype(np.int64), rp.astype(np.int64)), shape=(n, n))
    assert rel(K @ g["u"], g["asm_matvec"]) < FP64_RTOL
    assert rel(K @ g["u"], g["matvec"]) < FP64_RTOL  # the assembly-free product of the same matrix
    rp, cols, vals = assemble_csr_host(n, g["offsets"], g["map"], g["ke"], g["constrained"], BC_METH.BC_IMATRIX,
                                       True)
    Kb = sp.csr_matrix((vals, cols.astype(np.int64), rp.astype(np.int64)), shape=(n, n))
    assert rel(Kb @ g["u"], g["asm_matmult_bc"]) < FP64_RTOL


def test_host_assembly_rejects_bad_input():
    from amat_gb300 import AfmError
    with pytest.raises(AfmError):
        assemble_csr_host(4, [0, 2], [0, 9], np.eye(2))  # DoF out of range
    with pytest.raises(AfmError):
        assemble_csr_host(4, [0, 2], [0, 1], np.eye(2), bc_method=7)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ASM)
def test_device_assembled_matches_reference(gpu, name):
    import torch
    g = load(name)
    n = int(g["n_dofs"])
    du = torch.tensor(g["u"], device="cuda")
    dv = torch.empty_like(du)
    for bc, key, vkey in [(BC_METH.BC_IMATRIX, "asm_matmult_bc", "asm_vals"),
                          (BC_METH.BC_PENALTY, "asm_matmult_bc_penalty", "asm_vals_penalty")]:
        A = make_operator(g, bc, PRECISION.FP64_SPLIT)
        A.assemble(apply_bc=False)
        A.matvec_assembled_device(dv.data_ptr(), du.data_ptr())
        A.synchronize()
        assert rel(dv.cpu().numpy(), g["asm_matvec"]) < FP64_RTOL
        A.assemble(apply_bc=True)
        assert A.info()["csr_nnz"] == len(g["asm_cols"])
        rp, cols, vals = A.assembled_csr()
        assert np.array_equal(rp, g["asm_row_ptr"]) and np.array_equal(cols, g["asm_cols"])
        assert np.array_equal(vals, g[vkey])
        A.matvec_assembled_device(dv.data_ptr(), du.data_ptr())
        A.synchronize()
        assert rel(dv.cpu().numpy(), g[key]) < FP64_RTOL
        A.close()


@pytest.mark.gpu
@pytest.mark.parametrize("kind,n", [(P.HEX20_ELASTIC, 10), (P.TET10_POISSON, 16), (P.HEX8_POISSON, 24)])
def test_device_assembled_against_afm_at_scale(gpu, kind, n):
    """Many rows, every SpMV width: the assembled product equals the assembly-free one and repeats bit for bit."""
    import torch
    m = P.Mesh(kind, n, jitter=0.1, seed=9)
    ke = m.element_matrices(ngt=3 if kind == P.HEX20_ELASTIC else 2)
    maps = Maps()
    maps.set_map(m.n_elem, m.dof_map(), m.ndpe, m.n_dofs)
    A = aMatFree(maps)
    A.set_element_matrices(0, ke)
    A.finalize()
    A.assemble(apply_bc=False)
    u = np.random.default_rng(2).uniform(-1, 1, m.n_dofs)
    du = torch.tensor(u, device="cuda")
    v1, v2, va = torch.empty_like(du), torch.empty_like(du), torch.empty_like(du)
    A.matvec_assembled_device(v1.data_ptr(), du.data_ptr())
    A.matvec_assembled_device(v2.data_ptr(), du.data_ptr())
    A.matvec_device(va.data_ptr(), du.data_ptr())
    A.synchronize()
    assert torch.equal(v1, v2)
    assert rel(v1.cpu().numpy(), va.cpu().numpy()) < FP64_RTOL


def test_host_assembly_order_with_repeated_dofs():
    """Elements that list a DoF twice add both rows and columns into the same entry, in element, row,
    column order (MatSetValues with ADD_VALUES): the same sums as a plain loop in that order, bit for bit."""
    rng = np.random.default_rng(21)
    n_dofs, sizes = 40, [3, 5, 7, 4, 6] * 6
    maps = [rng.integers(0, n_dofs, size=s).astype(np.uint32) for s in sizes]  # repeats allowed
    kes = [rng.normal(size=(len(m), len(m))) for m in maps]
    offsets = np.concatenate([[0], np.cumsum([len(m) for m in maps])]).astype(np.uint32)
    dense = {}
    for m, k in zip(maps, kes):
        for r in range(len(m)):
            for c in range(len(m)):
                key = (int(m[r]), int(m[c]))
                dense[key] = dense.get(key, 0.0) + k[r, c]
    rp, cols, vals = assemble_csr_host(n_dofs, offsets, np.concatenate(maps), np.concatenate([k.ravel() for k in kes]),
                                       (), BC_METH.BC_IMATRIX, False)
    got = {}
    for i in range(n_dofs):
        for j in range(int(rp[i]), int(rp[i + 1])):
            got[(i, int(cols[j]))] = vals[j]
    assert got.keys() == dense.keys()
    for key, v in dense.items():
        assert got[key] == v  # bit for bit
