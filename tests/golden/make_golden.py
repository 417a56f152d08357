"""Writes the golden fixtures of tests/golden/ from the reference aMat itself.

Run in a checkout where the reference tree is available (AMAT_REFERENCE,
default: a directory named reference beside the repository's root): it
builds oracle/_ref/libamat_ref.so from the reference sources in place
(oracle/build_ref.sh) and records, for small seeded
problems, the reference's own outputs:
  - aMatFree (method 1) matvec, MatMult_mf, MatGetDiagonal_mf, apply_bc rhs
    (identity and penalty), for blocks_dim 1 and 2;
  - aMatBased (assembled) K u, K_bc u and rhs, and the assembled matrix after the
    identity and penalty BCs (CSR);
  - meshGraph greedy colouring;
  - element matrices of ke_matrix.cpp for jittered elements of each kind;
  - the Gauss-Legendre rule of integration.hpp.
Inputs (maps, element matrices, vectors) are stored with the outputs, so the
fixtures are self-contained. The GPU tests read only the .npz files.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from amat_gb300 import build  # noqa: E402
from amat_gb300 import problems as P  # noqa: E402


def mesh_case(name, kind, n, jitter, seed, ngt, E=1.0, nu=0.3, bc_scale=0.5):
    m = P.Mesh(kind, n, jitter=jitter, seed=seed)
    ke = m.element_matrices(E=E, nu=nu, ngt=ngt)
    dofs, _ = m.boundary_conditions()
    rng = np.random.default_rng(seed + 100)
    vals = bc_scale * rng.uniform(-1, 1, len(dofs))  # non-zero prescribed values exercise K_fc U_c
    return dict(name=name, n_dofs=m.n_dofs, map=m.dof_map(), ke=ke, constrained=dofs, values=vals,
                coords=m.coords, elem_nodes=m.elem_nodes)


def random_case(name, seed, sizes, n_elem, n_dofs, symmetric):
    """Elements of several sizes on random DoF sets: exercises the CSR map,
    mixed regimes and non-symmetric Ke (K u, not K^T u)."""
    rng = np.random.default_rng(seed)
    maps, kes = [], []
    for _ in range(n_elem):
        n = int(rng.choice(sizes))
        maps.append(np.sort(rng.choice(n_dofs, size=n, replace=False)).astype(np.uint32)[rng.permutation(n)])
        k = rng.normal(size=(n, n))
        if symmetric:
            k = k + k.T + 2 * n * np.eye(n)
        kes.append(k)
    n_c = max(1, n_dofs // 10)
    constrained = np.sort(rng.choice(n_dofs, size=n_c, replace=False)).astype(np.uint64)
    values = rng.uniform(-1, 1, n_c)
    return dict(name=name, n_dofs=n_dofs, map_list=maps, ke_list=kes, constrained=constrained, values=values)


def blocked_case(name, seed):
    """hex8 elasticity (24x24) split into 2x2 blocks with one off-diagonal
    block zeroed, so the reference stores it as a null block."""
    m = P.Mesh(P.HEX8_ELASTIC, 2, jitter=0.1, seed=seed)
    ke = m.element_matrices()
    ke[::2, :12, 12:] = 0.0
    ke[::2, 12:, :12] = 0.0
    dofs, vals = m.boundary_conditions()
    return dict(name=name, n_dofs=m.n_dofs, map=m.dof_map(), ke=ke, constrained=dofs, values=vals, blocks_dim=2)


def record(case, out):
    if "map" in case:
        prob = oracle.Problem(case["n_dofs"], case["map"], case["ke"], case["constrained"], case["values"])
    else:
        prob = oracle.Problem(case["n_dofs"], case["map_list"], case["ke_list"], case["constrained"],
                              case["values"])
    rng = np.random.default_rng(12345)
    u = rng.uniform(-1, 1, prob.n_dofs)
    rhs = rng.normal(size=prob.n_dofs)
    bd = case.get("blocks_dim", 1)
    rid = prob.ref_all(u, rhs, bc_method=0, blocks_dim=bd)
    rpen = prob.ref_all(u, rhs, bc_method=1, blocks_dim=bd)
    col, ncol = prob.ref_coloring()
    data = dict(n_dofs=prob.n_dofs, offsets=prob.offsets, map=prob.map, ke=prob.ke, constrained=prob.constrained,
                values=prob.values, u=u, rhs=rhs, blocks_dim=bd, colors=col, n_colors=ncol,
                matvec=rid["matvec"], matmult_bc=rid["matmult_bc"], diag=rid["diag"], rhs_bc=rid["rhs_bc"],
                diag_penalty=rpen["diag"], rhs_bc_penalty=rpen["rhs_bc"], matmult_bc_penalty=rpen["matmult_bc"])
    if bd == 1:
        a = prob.ref_assembled(u, rhs, bc_method=0)
        data.update(asm_matvec=a["matvec"], asm_matmult_bc=a["matmult_bc"], asm_rhs_bc=a["rhs_bc"],
                    asm_row_ptr=a["csr_row_ptr"], asm_cols=a["csr_cols"], asm_vals=a["csr_vals"])
        a = prob.ref_assembled(u, rhs, bc_method=1)
        data.update(asm_matmult_bc_penalty=a["matmult_bc"], asm_rhs_bc_penalty=a["rhs_bc"],
                    asm_vals_penalty=a["csr_vals"])
        assert np.array_equal(a["csr_row_ptr"], data["asm_row_ptr"]) and np.array_equal(a["csr_cols"], data["asm_cols"])
    if "coords" in case:
        data.update(coords=case["coords"], elem_nodes=case["elem_nodes"])
    np.savez_compressed(out, **data)
    return out


def ke_fixture(out):
    kinds = [(P.HEX8_POISSON, 2), (P.HEX8_ELASTIC, 2), (P.HEX20_ELASTIC, 2), (P.HEX20_ELASTIC, 3),
             (P.TET10_POISSON, 2), (P.TET10_ELASTIC, 2)]
    data = {}
    for i, (kind, ngt) in enumerate(kinds):
        m = P.Mesh(kind, 2, jitter=0.15, seed=7 + i)
        xes = m.coords[m.elem_nodes[:3]]
        E, nu = (1.0, 0.3) if P.KIND_DPN[kind] == 3 else (0.0, 0.0)
        kes = np.stack([oracle.ref_element_matrix(kind, xe, E=E, nu=nu, ngt=ngt) for xe in xes])
        data["k%d_kind" % i] = kind
        data["k%d_ngt" % i] = ngt
        data["k%d_E" % i] = E
        data["k%d_nu" % i] = nu
        data["k%d_xe" % i] = xes
        data["k%d_ke" % i] = kes
    data["gauss"] = np.stack([np.pad(oracle.ref_gauss(n), (0, 2 * 5 - 2 * n)) for n in range(1, 6)])
    np.savez_compressed(out, **data)


def main():
    build.build_all()
    if build.build_reference() is None or oracle.ref() is None:
        raise SystemExit("reference tree not available: fixtures not regenerated")
    cases = [
        mesh_case("hex8_poisson_4", P.HEX8_POISSON, 4, 0.1, 0, 2),
        mesh_case("hex20_elastic_2", P.HEX20_ELASTIC, 2, 0.1, 1, 3),
        mesh_case("tet10_poisson_2", P.TET10_POISSON, 2, 0.15, 2, 2),
        # an even mesh: the bar constraints need centre nodes, and the reference
        # double-frees its saved-U_c buffer when a rank owns no constraint
        # (apply_bc deletes m_dpUc without resetting it, include/aMatFree.hpp:959-964, 495)
        mesh_case("hex8_elastic_4", P.HEX8_ELASTIC, 4, 0.1, 3, 2),
        mesh_case("tet10_elastic_2", P.TET10_ELASTIC, 2, 0.15, 4, 2),
        random_case("mixed_random", 5, [4, 8, 10, 12, 20, 24, 30, 33], 60, 300, symmetric=False),
        random_case("mixed_spd", 6, [3, 8, 17, 60, 64, 70], 40, 500, symmetric=True),
        blocked_case("hex8_elastic_blocked", 8),
    ]
    for c in cases:
        print(record(c, os.path.join(HERE, c["name"] + ".npz")))
    ke_fixture(os.path.join(HERE, "element_matrices.npz"))
    print("ok")


if __name__ == "__main__":
    main()
