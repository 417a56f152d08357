"""Matrix-free operator (method 2, MATFREE_TYPE::FREE): element stiffness
integrated on the device from node coordinates every product. Against the
reference's method-1 products (golden vectors), the stored-Ke operator at
scale, FP32 against FP64, the Jacobi diagonal, and CG solves."""
import numpy as np
import pytest

import oracle
from amat_gb300 import BC_METH, CG_NORM, MATFREE_TYPE, PRECISION, Maps, aMatFree
from amat_gb300 import problems as P
from helpers import FP64_RTOL, load, rel

pytestmark = pytest.mark.gpu

FP32_RTOL = 1e-5
# golden mesh cases: (kind, Gauss points per direction)
GOLDEN = {"hex8_poisson_4": (P.HEX8_POISSON, 2), "hex20_elastic_2": (P.HEX20_ELASTIC, 3),
          "tet10_poisson_2": (P.TET10_POISSON, 2), "hex8_elastic_4": (P.HEX8_ELASTIC, 2),
          "tet10_elastic_2": (P.TET10_ELASTIC, 2)}


def free_operator(n_dofs, dof_map, nodes_per_elem, dpn, xe, kind, ngt, constrained=(), values=(),
                  bc=BC_METH.BC_IMATRIX):
    n_elem = xe.shape[0]
    maps = Maps()
    maps.set_map(n_elem, dof_map, nodes_per_elem * dpn, n_dofs)
    if len(constrained):
        maps.set_bdr_map(constrained, values)
    A = aMatFree(maps, bc)
    A.set_matfree_type(MATFREE_TYPE.FREE)
    A.set_element_kind(kind, E=1.0, nu=0.3, ngt=ngt)
    A.set_element_coords(0, xe)
    A.finalize()
    return A


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_free_matches_reference(gpu, name):
    import torch
    g = load(name)
    kind, ngt = GOLDEN[name]
    xe = g["coords"][g["elem_nodes"]]
    dpn = P.KIND_DPN[kind]
    A = free_operator(int(g["n_dofs"]), g["map"], g["elem_nodes"].shape[1], dpn, xe, kind, ngt, g["constrained"],
                      g["values"])
    v = np.empty(int(g["n_dofs"]))
    A.matvec(v, g["u"], True)
    assert rel(v, g["matvec"]) < FP64_RTOL
    A.matmult_bc(v, g["u"])
    assert rel(v, g["matmult_bc"]) < FP64_RTOL
    assert rel(A.get_diagonal(), g["diag"]) < 1e-14
    du = torch.tensor(g["u"], dtype=torch.float32, device="cuda")
    dv = torch.empty_like(du)
    A.matvec_device_f32(dv.data_ptr(), du.data_ptr())
    A.synchronize()
    assert rel(dv.double().cpu().numpy(), g["matvec"]) < FP32_RTOL


@pytest.mark.parametrize("kind,n", [(P.HEX20_ELASTIC, 10), (P.TET10_ELASTIC, 8), (P.HEX8_POISSON, 24),
                                    (P.TET10_POISSON, 12), (P.HEX8_ELASTIC, 12)])
def test_free_against_stored_at_scale(gpu, kind, n):
    """Many elements and colours: FP64 within 1e-12 of the stored-Ke product, bit-reproducible, FP32 within 1e-5."""
    import torch
    m = P.Mesh(kind, n, jitter=0.1, seed=11)
    ngt = 3 if kind == P.HEX20_ELASTIC else 2
    ke = m.element_matrices(ngt=ngt)
    maps = Maps()
    maps.set_map(m.n_elem, m.dof_map(), m.ndpe, m.n_dofs)
    S = aMatFree(maps)
    S.set_precision(PRECISION.FP64)
    S.set_element_matrices(0, ke)
    S.finalize()
    F = free_operator(m.n_dofs, m.dof_map(), m.elem_nodes.shape[1], m.dpn, m.coords[m.elem_nodes], kind, ngt)
    u = np.random.default_rng(4).uniform(-1, 1, m.n_dofs)
    du = torch.tensor(u, device="cuda")
    vs, v1, v2 = torch.empty_like(du), torch.empty_like(du), torch.empty_like(du)
    S.matvec_device(vs.data_ptr(), du.data_ptr())
    F.matvec_device(v1.data_ptr(), du.data_ptr())
    F.matvec_device(v2.data_ptr(), du.data_ptr())
    S.synchronize()
    F.synchronize()
    assert torch.equal(v1, v2)
    assert rel(v1.cpu().numpy(), vs.cpu().numpy()) < FP64_RTOL
    du32 = du.float()
    v32 = torch.empty_like(du32)
    F.matvec_device_f32(v32.data_ptr(), du32.data_ptr())
    F.synchronize()
    assert rel(v32.double().cpu().numpy(), vs.cpu().numpy()) < FP32_RTOL
    assert rel(F.get_diagonal(), S.get_diagonal()) < 1e-14
    assert F.info()["ke_bytes"] == 0


def test_free_solves(gpu):
    """FP64 CG and the mixed-precision solve (FP32 matrix-free inner products, FP64 matrix-free residuals)
    reach the same solution as the stored-Ke FP64 CG."""
    kind, n = P.HEX20_ELASTIC, 6
    m = P.Mesh(kind, n, jitter=0.1, seed=12)
    ke = m.element_matrices(ngt=3)
    dofs, vals = m.boundary_conditions()
    maps = Maps()
    maps.set_map(m.n_elem, m.dof_map(), m.ndpe, m.n_dofs)
    maps.set_bdr_map(dofs, vals)
    S = aMatFree(maps)
    S.set_element_matrices(0, ke)
    S.finalize()
    F = free_operator(m.n_dofs, m.dof_map(), m.elem_nodes.shape[1], m.dpn, m.coords[m.elem_nodes], kind, 3, dofs, vals)
    b = S.apply_bc(m.load(ngt=3))
    bf = F.apply_bc(m.load(ngt=3))
    assert rel(bf, b) < FP64_RTOL
    xs, st = S.solve(b, rtol=1e-10, atol=0.0, maxit=20000, norm=CG_NORM.UNPRECONDITIONED)
    xf, sf = F.solve(b, rtol=1e-10, atol=0.0, maxit=20000, norm=CG_NORM.UNPRECONDITIONED)
    assert st.status == 0 and sf.status == 0
    assert rel(xf, xs) < 1e-8
    xm, sm = F.solve_mixed(b, rtol=1e-9, atol=0.0, inner_rtol=0.1)
    assert sm.status == 0 and sm.rel_residual <= 1e-9
    assert rel(xm, xs) < 1e-6


def test_free_misuse(gpu):
    from amat_gb300 import AfmError
    maps = Maps()
    maps.set_map(1, np.arange(8, dtype=np.uint32), 8, 8)
    A = aMatFree(maps)
    A.set_matfree_type(MATFREE_TYPE.FREE)
    with pytest.raises(AfmError):
        A.finalize()  # no element kind
    with pytest.raises(AfmError):
        A.set_element_kind(9)
    with pytest.raises(AfmError):
        A.set_element_kind(P.HEX8_POISSON, ngt=4)
    A.set_element_kind(P.HEX8_POISSON)
    with pytest.raises(AfmError):
        A.finalize()  # no coordinates
    A.set_element_coords(0, np.zeros((1, 8, 3)))
    with pytest.raises(AfmError):
        A.finalize()  # degenerate element
