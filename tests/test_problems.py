"""Problem generators (include/afm_problems.h) against the reference's element
kernels and example meshes (golden element_matrices.npz)."""
import os

import numpy as np
import pytest

from amat_gb300 import problems as P
from helpers import GOLDEN


def test_element_matrices_match_reference_kernels():
    z = np.load(os.path.join(GOLDEN, "element_matrices.npz"))
    i = 0
    while "k%d_kind" % i in z.files:
        kind, ngt = int(z["k%d_kind" % i]), int(z["k%d_ngt" % i])
        E, nu = float(z["k%d_E" % i]), float(z["k%d_nu" % i])
        for xe, kref in zip(z["k%d_xe" % i], z["k%d_ke" % i]):
            k = P.element_matrix_xe(kind, xe, E=E, nu=nu, ngt=ngt)
            assert np.abs(k - kref).max() <= 1e-12 * np.abs(kref).max(), (kind, ngt)
        i += 1
    assert i == 6


def test_gauss_legendre_matches_reference():
    z = np.load(os.path.join(GOLDEN, "element_matrices.npz"))
    for n in range(1, 6):
        assert np.allclose(P.gauss_legendre(n), z["gauss"][n - 1][:2 * n], rtol=0, atol=1e-13)


@pytest.mark.parametrize("kind,n,nodes,elems", [
    (P.HEX8_POISSON, 32, 35937, 32768),     # 32^3 hex8: 35,937 nodes
    (P.HEX20_ELASTIC, 8, 2673, 512),
    (P.TET10_POISSON, 4, 729, 384),
])
def test_mesh_sizes(kind, n, nodes, elems):
    m = P.Mesh(kind, n)
    assert (m.n_nodes, m.n_elem) == (nodes, elems)


def test_hex20_node_count_formula():
    # (2N+1)^3 doubled-lattice points minus face and body centres
    for N in (1, 2, 5):
        m = P.Mesh(P.HEX20_ELASTIC, N)
        assert m.n_nodes == (2 * N + 1) ** 3 - 3 * N * N * (N + 1) - N ** 3


def test_hex20_numbering_matches_example07a():
    """Element node ids of example07a.cpp:352-386 for a 3x2x2 mesh."""
    Nex, Ney, Nez = 3, 2, 2
    m = P.Mesh(P.HEX20_ELASTIC, Nex, Ney, Nez)
    en = m.elem_nodes
    layer = (2 * Nex + 1) * (2 * Ney + 1) - Nex * Ney + (Nex + 1) * (Ney + 1)
    for k in range(Nez):
        for j in range(Ney):
            for i in range(Nex):
                e = Nex * Ney * k + Nex * j + i
                L = [0] * 20
                L[0] = 2 * i + j * (3 * Nex + 2) + k * layer
                L[1] = L[0] + 2
                L[3] = L[0] + (3 * Nex + 2)
                L[2] = L[3] + 2
                L[4] = L[0] + layer
                L[5] = L[4] + 2
                L[7] = L[4] + (3 * Nex + 2)
                L[6] = L[7] + 2
                L[8] = L[0] + 1
                L[10] = L[3] + 1
                L[11] = L[0] + (2 * Nex + 1) - i
                L[9] = L[11] + 1
                L[12] = L[4] + 1
                L[14] = L[7] + 1
                L[15] = L[4] + (2 * Nex + 1) - i
                L[13] = L[15] + 1
                L[16] = L[0] + ((2 * Nex + 1) * (2 * Ney + 1) - Nex * Ney - i) - j * (2 * Nex + 1)
                L[17] = L[16] + 1
                L[19] = L[16] + (Nex + 1)
                L[18] = L[19] + 1
                assert list(en[e]) == L


def test_hex8_numbering_matches_example03a():
    N = 3
    m = P.Mesh(P.HEX8_POISSON, N)
    en = m.elem_nodes
    e = N * N * 1 + N * 2 + 1
    b = 1 + 2 * (N + 1) + 1 * (N + 1) ** 2
    assert list(en[e]) == [b, b + 1, b + N + 2, b + N + 1, b + (N + 1) ** 2, b + (N + 1) ** 2 + 1,
                           b + (N + 1) ** 2 + N + 2, b + (N + 1) ** 2 + N + 1]


@pytest.mark.parametrize("kind", [P.HEX8_POISSON, P.HEX8_ELASTIC, P.HEX20_ELASTIC, P.TET10_POISSON, P.TET10_ELASTIC])
def test_jittered_elements_are_valid(kind):
    """Positive Jacobians at the configs' jitter, symmetric Ke, rigid modes in the kernel."""
    m = P.Mesh(kind, 3, jitter=0.15, seed=9)
    ke = m.element_matrices(ngt=3 if kind == P.HEX20_ELASTIC else 2)
    assert np.abs(ke - ke.transpose(0, 2, 1)).max() < 1e-12 * np.abs(ke).max()
    ones = np.ones(ke.shape[1]) if P.KIND_DPN[kind] == 1 else np.tile([1.0, 0.0, 0.0], ke.shape[1] // 3)
    assert np.abs(ke @ ones).max() < 1e-11 * np.abs(ke).max()


def test_jitter_is_deterministic_and_bounded():
    a = P.Mesh(P.HEX8_POISSON, 4, jitter=0.1, seed=3).coords
    b = P.Mesh(P.HEX8_POISSON, 4, jitter=0.1, seed=3).coords
    c = P.Mesh(P.HEX8_POISSON, 4, jitter=0.0).coords
    assert np.array_equal(a, b)
    assert np.abs(a - c).max() <= 0.1 * 0.25 + 1e-15
    on_face = (c == 0.0) | (c == 1.0)
    assert np.array_equal(a[on_face], c[on_face])


def test_boundary_conditions():
    m = P.Mesh(P.HEX8_POISSON, 4)
    d, v = m.boundary_conditions()
    assert len(d) == 5 ** 3 - 3 ** 3 and np.all(v == 0)
    m = P.Mesh(P.HEX20_ELASTIC, 2)
    d, v = m.boundary_conditions()
    assert len(d) == 6 and np.all(np.diff(d.astype(np.int64)) > 0)


@pytest.mark.parametrize("kind,ngt", [(P.HEX8_POISSON, 2), (P.HEX8_ELASTIC, 2), (P.HEX20_ELASTIC, 3),
                                      (P.TET10_POISSON, 2), (P.TET10_ELASTIC, 2)])
def test_element_matrices_are_symmetric(kind, ngt):
    """Every generated Ke is symmetric well inside the 1e-6 (of the largest diagonal entry) bound under which
    FP32 products may stream the symmetric copy of the element matrices."""
    m = P.Mesh(kind, 3, jitter=0.15, seed=5)
    ke = m.element_matrices(ngt=ngt)
    dmax = np.abs(np.diagonal(ke, axis1=1, axis2=2)).max(axis=1)
    asym = np.abs(ke - np.transpose(ke, (0, 2, 1))).max(axis=(1, 2))
    assert np.all(asym <= 1e-12 * dmax)
