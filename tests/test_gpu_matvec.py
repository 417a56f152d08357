"""Parity of the GB300 AFM operator with the reference (golden vectors written
from the reference itself) and with the CPU oracle, through the C ABI.

FP64 results are compared norm-wise against the reference at FP64_RTOL
(1e-12); the colouring and the Jacobi diagonal bit for bit; FP32 at 1e-5.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from amat_gb300 import BC_METH, PRECISION, AfmError, Maps, aMatFree
from amat_gb300 import problems as P
from helpers import FP64_RTOL, element_blocks, golden_names, load, make_operator, rel

pytestmark = pytest.mark.gpu

FP32_RTOL = 1e-5
PRECS = [PRECISION.FP64, PRECISION.FP64_SPLIT]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("name", golden_names())
def test_matvec_matches_reference(gpu, name, prec):
    g = load(name)
    A = make_operator(g, 0, prec, blocks=True)
    v = np.empty(int(g["n_dofs"]))
    A.matvec(v, g["u"], True)
    assert rel(v, g["matvec"]) < FP64_RTOL
    assert rel(v, g["asm_matvec"] if "asm_matvec" in g else g["matvec"]) < FP64_RTOL
    assert np.array_equal(A.colors(), g["colors"])
    assert A.info()["n_colors"] == int(g["n_colors"])


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("name", golden_names())
def test_bc_calls_match_reference(gpu, name, prec):
    g = load(name)
    A = make_operator(g, BC_METH.BC_IMATRIX, prec, blocks=True)
    w = np.empty(int(g["n_dofs"]))
    A.matmult_bc(w, g["u"])
    assert rel(w, g["matmult_bc"]) < FP64_RTOL
    assert np.array_equal(A.get_diagonal(), g["diag"])
    if int(g["blocks_dim"]) == 1:
        rhs = g["rhs"].copy()
        A.apply_bc(rhs)
        assert rel(rhs, g["rhs_bc"]) < FP64_RTOL
    Ap = make_operator(g, BC_METH.BC_PENALTY, prec, blocks=True)
    Ap.matmult_bc(w, g["u"])
    assert rel(w, g["matmult_bc_penalty"]) < FP64_RTOL
    assert rel(Ap.get_diagonal(), g["diag_penalty"]) < FP64_RTOL
    rhs = g["rhs"].copy()
    Ap.apply_bc(rhs)
    assert rel(rhs, g["rhs_bc_penalty"]) < FP64_RTOL


@pytest.mark.parametrize("name", ["hex8_poisson_4", "mixed_random", "tet10_elastic_2", "hex20_elastic_2"])
def test_fp32_operator(gpu, name):
    import torch
    g = load(name)
    A = make_operator(g, 0, PRECISION.FP32)
    u = torch.tensor(g["u"], dtype=torch.float32, device="cuda")
    v = torch.empty_like(u)
    torch.cuda.synchronize()
    A.matvec_device_f32(v.data_ptr(), u.data_ptr())
    A.synchronize()
    assert rel(v.cpu().double().numpy(), g["matvec"]) < FP32_RTOL


@pytest.mark.parametrize("name", ["hex8_poisson_4", "mixed_random", "hex20_elastic_2", "tet10_elastic_2"])
def test_fp32_product_from_split_arena(gpu, name):
    """The hi plane of the split arena is the FP32 element matrix: FP32 product, half the bytes."""
    import torch
    g = load(name)
    A = make_operator(g, 0, PRECISION.FP64_SPLIT)
    u = torch.tensor(g["u"], dtype=torch.float32, device="cuda")
    v = torch.empty_like(u)
    torch.cuda.synchronize()
    A.matvec_device_f32(v.data_ptr(), u.data_ptr())
    A.synchronize()
    assert rel(v.cpu().double().numpy(), g["matvec"]) < FP32_RTOL
    w = torch.empty_like(u)
    A.matmult_bc_device_f32(w.data_ptr(), u.data_ptr())
    A.synchronize()
    assert rel(w.cpu().double().numpy(), g["matmult_bc"]) < FP32_RTOL


@pytest.mark.parametrize("kind,n", [(P.TET10_POISSON, 24), (P.HEX8_POISSON, 40), (P.HEX20_ELASTIC, 16)])
def test_fp32_view_at_scale(gpu, kind, n):
    """FP32 product of the split arena's hi plane against the FP64 product, many units per CTA."""
    import torch
    m = P.Mesh(kind, n, jitter=0.12, seed=4)
    ke = m.element_matrices(ngt=3 if kind == P.HEX20_ELASTIC else 2)
    maps = Maps()
    maps.set_map(m.n_elem, m.dof_map(), m.ndpe, m.n_dofs)
    A = aMatFree(maps)
    A.set_precision(PRECISION.FP64_SPLIT)
    A.set_element_matrices(0, ke)
    A.finalize()
    u = np.random.default_rng(5).uniform(-1, 1, m.n_dofs)
    v64 = np.empty(m.n_dofs)
    A.matvec(v64, u, True)
    du = torch.tensor(u, dtype=torch.float32, device="cuda")
    dv = torch.empty_like(du)
    torch.cuda.synchronize()
    A.matvec_device_f32(dv.data_ptr(), du.data_ptr())
    A.synchronize()
    assert rel(dv.cpu().double().numpy(), v64) < 1e-5


def test_device_entry_on_torch_stream(gpu):
    import torch
    g = load("hex20_elastic_2")
    A = make_operator(g, 0, PRECISION.FP64)
    s = torch.cuda.Stream()
    u = torch.tensor(g["u"], dtype=torch.float64, device="cuda")
    v = torch.empty_like(u)
    torch.cuda.synchronize()
    A.matvec_device(v.data_ptr(), u.data_ptr(), s.cuda_stream)
    s.synchronize()
    A.synchronize()
    assert rel(v.cpu().numpy(), g["matvec"]) < FP64_RTOL


@pytest.mark.parametrize("prec", PRECS)
def test_matvec_is_bitwise_reproducible(gpu, prec):
    g = load("mixed_spd")
    A = make_operator(g, 0, prec)
    outs = []
    for _ in range(5):
        v = np.empty(int(g["n_dofs"]))
        A.matvec(v, g["u"], True)
        outs.append(v)
    for v in outs[1:]:
        assert np.array_equal(v, outs[0])
    B = make_operator(g, 0, prec)  # a second operator on the same inputs
    v = np.empty(int(g["n_dofs"]))
    B.matvec(v, g["u"], True)
    assert np.array_equal(v, outs[0])


def build(n_dofs, elems, kes, constrained=(), values=(), prec=PRECISION.AUTO, bc=0):
    maps = Maps()
    dpe = np.array([len(e) for e in elems], dtype=np.uint32)
    maps.set_map(len(elems), np.concatenate(elems).astype(np.uint32), dpe, n_dofs)
    maps.set_bdr_map(np.asarray(constrained, dtype=np.uint64), np.asarray(values, dtype=np.float64))
    A = aMatFree(maps, bc)
    A.set_precision(prec)
    for e, k in enumerate(kes):
        A.set_element_matrix(e, k)
    A.finalize()
    return A


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("sizes", [[1, 2, 3], [5, 7, 9, 16], [17, 23, 31, 32], [33, 47, 64], [65, 80, 96]])
def test_generic_element_sizes(gpu, sizes, prec):
    """Element sizes without a specialised kernel (run-time n), all regimes."""
    rng = np.random.default_rng(len(sizes) * 7 + sizes[0])
    n_dofs = 400
    elems, kes = [], []
    for i in range(90):
        n = sizes[i % len(sizes)]
        elems.append(rng.choice(n_dofs, size=n, replace=False).astype(np.uint32))
        kes.append(rng.normal(size=(n, n)))
    A = build(n_dofs, elems, kes, prec=prec)
    u = rng.uniform(-1, 1, n_dofs)
    v = np.empty(n_dofs)
    A.matvec(v, u, True)
    ref = oracle.Problem(n_dofs, elems, kes).matvec(u)
    assert rel(v, ref) < FP64_RTOL


@pytest.mark.parametrize("prec", PRECS)
def test_duplicate_dof_inside_an_element(gpu, prec):
    """An element listing a DoF twice adds both rows (the reference's atomic scatter)."""
    rng = np.random.default_rng(3)
    elems = [np.array([0, 1, 1, 2], dtype=np.uint32), np.array([2, 3, 4, 5], dtype=np.uint32),
             np.array([5, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 17, 18, 19, 20, 5], dtype=np.uint32)]
    kes = [rng.normal(size=(len(e), len(e))) for e in elems]
    A = build(21, elems, kes, prec=prec)
    u = rng.uniform(-1, 1, 21)
    v = np.empty(21)
    A.matvec(v, u, True)
    assert rel(v, oracle.Problem(21, elems, kes).matvec(u)) < FP64_RTOL


def test_no_constraints_and_untouched_dofs(gpu):
    rng = np.random.default_rng(4)
    elems = [np.array([0, 2, 4, 6, 8, 10, 12, 14], dtype=np.uint32)]
    kes = [rng.normal(size=(8, 8))]
    A = build(20, elems, kes)
    u = rng.uniform(-1, 1, 20)
    v = np.full(20, np.nan)
    A.matvec(v, u, True)
    ref = oracle.Problem(20, elems, kes).matvec(u)
    assert rel(v, ref) < FP64_RTOL and np.all(v[1::2] == 0.0)
    w = np.empty(20)
    A.matmult_bc(w, u)
    assert rel(w, ref) < FP64_RTOL


def test_partial_tpe_units(gpu):
    """Colour classes whose size is not a multiple of 32 (partial thread-per-element units)."""
    m = P.Mesh(P.HEX8_POISSON, 5, 3, 7, jitter=0.1, seed=2)
    ke = m.element_matrices()
    maps = Maps()
    maps.set_map(m.n_elem, m.dof_map(), m.ndpe, m.n_dofs)
    A = aMatFree(maps)
    A.set_element_matrices(0, ke)
    A.finalize()
    u = np.random.default_rng(0).uniform(-1, 1, m.n_dofs)
    v = np.empty(m.n_dofs)
    A.matvec(v, u, True)
    assert rel(v, oracle.Problem(m.n_dofs, m.dof_map(), ke).matvec(u)) < FP64_RTOL


@pytest.mark.parametrize("prec", PRECS)
def test_hex20_32_cube_against_oracle(gpu, prec):
    """32^3 hex20 elasticity (0.94 GB of Ke): oracle parity plus K symmetry."""
    m = P.Mesh(P.HEX20_ELASTIC, 32, jitter=0.1, seed=1)
    ke = m.element_matrices(ngt=3)
    maps = Maps()
    maps.set_map(m.n_elem, m.dof_map(), m.ndpe, m.n_dofs)
    A = aMatFree(maps)
    A.set_precision(prec)
    A.set_element_matrices(0, ke)
    A.finalize()
    rng = np.random.default_rng(11)
    u, w = rng.uniform(-1, 1, m.n_dofs), rng.uniform(-1, 1, m.n_dofs)
    ku, kw = np.empty(m.n_dofs), np.empty(m.n_dofs)
    A.matvec(ku, u, True)
    A.matvec(kw, w, True)
    ref = oracle.Problem(m.n_dofs, m.dof_map(), ke).matvec_omp(u)[0]
    assert rel(ku, ref) < FP64_RTOL
    assert abs(u @ kw - w @ ku) < 1e-12 * np.linalg.norm(u) * np.linalg.norm(kw)
    # linearity
    kuw = np.empty(m.n_dofs)
    A.matvec(kuw, 2.0 * u - 3.0 * w, True)
    assert rel(kuw, 2.0 * ku - 3.0 * kw) < FP64_RTOL


def test_misuse_is_reported(gpu):
    maps = Maps()
    maps.set_map(1, np.arange(8, dtype=np.uint32), 8, 8)
    A = aMatFree(maps)
    with pytest.raises(AfmError) as e:
        A.matvec(np.empty(8), np.zeros(8), True)
    assert e.value.name == "ERR_STATE"
    with pytest.raises(AfmError) as e:
        A.set_element_matrix(3, np.eye(8))
    assert e.value.name == "INDEX_OUT_OF_BOUNDS"
    big = Maps()
    big.set_map(1, np.arange(97, dtype=np.uint32), 97, 97)
    with pytest.raises(AfmError) as e:
        aMatFree(big)
    assert e.value.name == "NOT_IMPLEMENTED"
    ghost = Maps()
    ghost.set_map(1, np.arange(8, dtype=np.uint32), 8, 8, None, 0, 7, 16)
    with pytest.raises(AfmError) as e:
        aMatFree(ghost)
    assert e.value.name == "WRONG_COMMUNICATION"


def _mesh_operator(kind, shape, jitter, prec, patch, bc=True):
    m = P.Mesh(kind, *shape, jitter=jitter, seed=2)
    ke = m.element_matrices()
    maps = Maps()
    maps.set_map(m.n_elem, m.dof_map(), m.ndpe, m.n_dofs)
    dofs, vals = m.boundary_conditions() if bc else (np.zeros(0, np.uint64), np.zeros(0))
    maps.set_bdr_map(dofs, vals)
    A = aMatFree(maps)
    A.set_precision(prec)
    A.set_patch_mode(patch)
    A.set_element_matrices(0, ke)
    A.finalize()
    return m, ke, dofs, vals, A


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("kind,shape,jitter", [
    (P.HEX8_POISSON, (12, 12, 12), 0.1),
    (P.HEX8_POISSON, (40, 1, 1), 0.0),
    (P.TET10_POISSON, (10, 10, 10), 0.15),
    (P.TET10_POISSON, (24, 24, 24), 0.15),
])
def test_patch_path_against_oracle(gpu, kind, shape, jitter, prec):
    """Small elements as shared-memory patches: v = K u and MatMult_mf against
    the oracle; one launch over every patch plus the combine pass (mode 3)
    gives the same bits as one launch per patch colour (mode 2); element
    colours (mode 0) agree within rounding; two calls in a row bit for bit."""
    import torch
    m, ke, dofs, vals, A = _mesh_operator(kind, shape, jitter, prec, 3)
    info = A.info()
    assert info["n_patches"] > 0 and info["n_launches"] <= 3
    _, _, _, _, C = _mesh_operator(kind, shape, jitter, prec, 2)
    assert C.info()["n_launches"] == C.info()["n_patch_colors"] + 1
    _, _, _, _, B = _mesh_operator(kind, shape, jitter, prec, 0)
    assert B.info()["n_patches"] == 0
    pr = oracle.Problem(m.n_dofs, m.dof_map(), ke, dofs, vals)
    u = np.random.default_rng(3).uniform(-1, 1, m.n_dofs)
    v, w, x = np.empty(m.n_dofs), np.empty(m.n_dofs), np.empty(m.n_dofs)
    A.matvec(v, u, True)
    B.matvec(w, u, True)
    C.matvec(x, u, True)
    vo = pr.matvec(u)
    assert rel(v, vo) < FP64_RTOL and rel(w, vo) < FP64_RTOL
    assert np.array_equal(v, x)
    A.matmult_bc(v, u)
    assert rel(v, pr.matmult_bc(u)) < FP64_RTOL
    du = torch.tensor(u, device="cuda")
    dv1, dv2 = torch.empty_like(du), torch.empty_like(du)
    A.matvec_device(dv1.data_ptr(), du.data_ptr())
    A.matvec_device(dv2.data_ptr(), du.data_ptr())
    A.synchronize()
    assert torch.equal(dv1, dv2)
    if prec == PRECISION.FP64_SPLIT:
        du32 = du.float()
        dv32 = torch.empty_like(du32)
        A.matvec_device_f32(dv32.data_ptr(), du32.data_ptr())
        A.synchronize()
        assert rel(dv32.double().cpu().numpy(), vo) < FP32_RTOL


@pytest.mark.parametrize("kind,n,ngt", [
    (P.HEX8_POISSON, 20, 2), (P.TET10_POISSON, 12, 2), (P.HEX8_ELASTIC, 10, 2), (P.TET10_ELASTIC, 6, 2),
    (P.HEX20_ELASTIC, 6, 3),
])
def test_symmetric_inner_arena(gpu, kind, n, ngt):
    """FP32 products of a split operator stream the symmetric copy (each pair
    of entries once) when every Ke is symmetric, in FP32 (format 1) or FP32
    with a BF16 correction plane and FP64 sums (format 2): against the FP64
    product, the hi-plane product, and themselves on a second call."""
    import torch
    m = P.Mesh(kind, n, jitter=0.12, seed=6)
    ke = m.element_matrices(ngt=ngt)
    maps = Maps()
    maps.set_map(m.n_elem, m.dof_map(), m.ndpe, m.n_dofs)
    A = aMatFree(maps)
    A.set_precision(PRECISION.FP64_SPLIT)
    A.set_element_matrices(0, ke)
    A.finalize()
    info = A.info()
    assert info["ke_symmetric"] == 1 and info["sym_available"] == 1 and info["sym_bytes"] == 0
    u = np.random.default_rng(7).uniform(-1, 1, m.n_dofs)
    v64 = np.empty(m.n_dofs)
    A.matvec(v64, u, True)
    du = torch.tensor(u, dtype=torch.float32, device="cuda")
    # v64 of the FP32-rounded u: the products' own error, apart from rounding u
    u32 = du.double().cpu().numpy()
    A.matvec(v64, u32, True)
    dh = torch.empty_like(du)
    A.set_symmetric_inner(0)
    A.matvec_device_f32(dh.data_ptr(), du.data_ptr())
    A.synchronize()
    assert A.info()["sym_available"] == 0 and A.info()["sym_bytes"] == 0
    vh = dh.double().cpu().numpy()
    assert rel(vh, v64) < FP32_RTOL
    # format: (bytes below this fraction of the split arena, error bound against FP64)
    for fmt, frac, tol in [(1, 0.29, FP32_RTOL), (2, 0.43, 3e-7)]:
        A.set_symmetric_inner(fmt)
        dv1, dv2 = torch.empty_like(du), torch.empty_like(du)
        A.matvec_device_f32(dv1.data_ptr(), du.data_ptr())
        A.matvec_device_f32(dv2.data_ptr(), du.data_ptr())
        A.synchronize()
        # the hi plane is half of the split arena; the symmetric copy about 55% (83% with the correction) of that
        assert 0 < A.info()["sym_bytes"] < frac * info["ke_bytes"]
        assert torch.equal(dv1, dv2)
        v1 = dv1.double().cpu().numpy()
        assert rel(v1, v64) < tol
        if fmt == 1:
            assert rel(v1, vh) < 2e-6


def test_symmetric_inner_needs_symmetric_ke(gpu):
    """A non-symmetric element matrix keeps FP32 products on the hi plane."""
    import torch
    g = load("mixed_random")
    A = make_operator(g, 0, PRECISION.FP64_SPLIT)
    info = A.info()
    assert info["ke_symmetric"] == 0 and info["sym_available"] == 0
    u = torch.tensor(g["u"], dtype=torch.float32, device="cuda")
    v = torch.empty_like(u)
    torch.cuda.synchronize()
    A.matvec_device_f32(v.data_ptr(), u.data_ptr())
    A.synchronize()
    assert A.info()["sym_bytes"] == 0
    assert rel(v.cpu().double().numpy(), g["matvec"]) < FP32_RTOL
