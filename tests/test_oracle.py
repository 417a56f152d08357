"""The CPU oracle against the golden vectors written from the reference itself
(tests/golden/make_golden.py). Pins the restatement before it is trusted as
the checker of the GPU path."""
import numpy as np
import pytest

import oracle
from helpers import FP64_RTOL, golden_names, load, rel


def problem(g):
    return oracle.Problem(int(g["n_dofs"]), _split(g["offsets"], g["map"]), _ke_list(g), g["constrained"],
                          g["values"])


def _split(off, m):
    return [m[off[e]:off[e + 1]] for e in range(len(off) - 1)]


def _ke_list(g):
    off = g["offsets"].astype(np.int64)
    out, k = [], 0
    for e in range(len(off) - 1):
        n = int(off[e + 1] - off[e])
        out.append(g["ke"][k:k + n * n])
        k += n * n
    return out


@pytest.mark.parametrize("name", golden_names())
def test_oracle_matvec_matches_reference(name):
    g = load(name)
    p = problem(g)
    assert rel(p.matvec(g["u"]), g["matvec"]) < FP64_RTOL
    v, threads = p.matvec_omp(g["u"])
    assert threads >= 1 and rel(v, g["matvec"]) < FP64_RTOL


@pytest.mark.parametrize("name", golden_names())
def test_oracle_cpu_baseline_variants_match_reference(name):
    """Both element products the CPU baseline times (the reference's row-major GEMV and its
    VECTORIZED_OPENMP column-by-column form), on one thread and on every thread."""
    g = load(name)
    p = problem(g)
    for simd in (False, True):
        for threads in (1, 0):
            v, used = p.matvec_omp_cfg(g["u"], threads=threads, simd=simd)
            assert used >= 1 and (threads == 0 or used == threads)
            assert rel(v, g["matvec"]) < FP64_RTOL


def test_reference_vectorized_build_agrees():
    """The reference's own VECTORIZED_OPENMP build (compiled in place where the reference tree is
    available) gives the product of its default build."""
    import ctypes as C
    R = oracle.ref(simd=True)
    if R is None:
        pytest.skip("reference not compiled on this machine")
    for name in ("hex20_elastic_2", "mixed_random", "hex8_poisson_4"):
        g = load(name)
        p = problem(g)
        h = R.ref_afm_create(p.n_elem, p.n_dofs, C.c_void_p(p.offsets.ctypes.data), C.c_void_p(p.map.ctypes.data),
                             C.c_void_p(p.ke.ctypes.data), 1, None, None, 0, 0)
        u = np.ascontiguousarray(g["u"], dtype=np.float64)
        v = np.empty(p.n_dofs)
        R.ref_afm_matvec(h, C.c_void_p(v.ctypes.data), C.c_void_p(u.ctypes.data))
        R.ref_afm_destroy(h)
        assert rel(v, g["matvec"]) < FP64_RTOL


@pytest.mark.parametrize("name", golden_names())
def test_oracle_bc_matches_reference(name):
    g = load(name)
    p = problem(g)
    assert rel(p.matmult_bc(g["u"]), g["matmult_bc"]) < FP64_RTOL
    # MatMult_mf ignores the BC method (include/aMatFree.hpp:3929-3933)
    assert rel(p.matmult_bc(g["u"]), g["matmult_bc_penalty"]) < FP64_RTOL
    assert np.array_equal(p.get_diagonal(0), g["diag"])
    assert rel(p.get_diagonal(1), g["diag_penalty"]) < FP64_RTOL
    if int(g["blocks_dim"]) == 1:
        # the reference re-adds KfcUc entries once per block when blocks_dim > 1
        assert rel(p.apply_bc_rhs(g["rhs"], 0), g["rhs_bc"]) < FP64_RTOL
    assert rel(p.apply_bc_rhs(g["rhs"], 1), g["rhs_bc_penalty"]) < FP64_RTOL


@pytest.mark.parametrize("name", golden_names())
def test_oracle_coloring_matches_reference(name):
    g = load(name)
    c, n = problem(g).coloring()
    assert n == int(g["n_colors"])
    assert np.array_equal(c, g["colors"])


@pytest.mark.parametrize("name", [n for n in golden_names() if "blocked" not in n])
def test_assembled_reference_agrees(name):
    """AFM == assembled K (aMatBased, PETSc-style assembly) on the same inputs."""
    g = load(name)
    # rows of DoFs that no element touches: the assembled operator has no row
    # there (apply_bc_mat walks elements, include/aMatBased.hpp:294-352) while
    # MatMult_mf still sets v_c = u_c
    used = np.zeros(int(g["n_dofs"]), dtype=bool)
    used[g["map"]] = True
    assert rel(g["asm_matvec"], g["matvec"]) < FP64_RTOL
    assert rel(g["asm_matmult_bc"][used], g["matmult_bc"][used]) < FP64_RTOL
    assert rel(g["asm_rhs_bc"], g["rhs_bc"]) < FP64_RTOL


def test_coloring_is_proper():
    g = load("mixed_random")
    c, n = problem(g).coloring()
    off, m = g["offsets"], g["map"]
    for col in range(n):
        els = np.nonzero(c == col)[0]
        dofs = np.concatenate([m[off[e]:off[e + 1]] for e in els])
        assert len(np.unique(dofs)) == len(dofs)


def test_oracle_pcg_solves_dense_system():
    g = load("hex8_poisson_4")
    p = problem(g)
    n = p.n_dofs
    K = np.zeros((n, n))
    for j in range(n):
        e = np.zeros(n)
        e[j] = 1.0
        K[:, j] = p.matmult_bc(e)
    b = p.apply_bc_rhs(g["rhs"], 0)
    x, it, res = p.pcg(b, rtol=1e-12)
    assert it > 0 and res < 1e-11
    assert rel(x, np.linalg.solve(K, b)) < 1e-10


def test_oracle_pcg_reports_breakdown():
    """A NaN in the right-hand side is a breakdown, not a result."""
    g = load("hex8_poisson_4")
    p = problem(g)
    b = p.apply_bc_rhs(g["rhs"], 0)
    b[3] = np.nan
    _, it, _ = p.pcg(b, rtol=1e-12)
    assert it == -1


def test_oracle_accepts_strided_columns():
    """A column of a row-major block (a strided view) gives the same product
    as its contiguous copy: the wrapper keeps the converted array alive."""
    g = load("mixed_random")
    p = problem(g)
    U = np.random.default_rng(5).uniform(-1, 1, (p.n_dofs, 16))
    for j in (0, 7, 15):
        col = U[:, j]
        assert not col.flags.c_contiguous
        assert np.array_equal(p.matvec(col), p.matvec(col.copy()))
        assert np.array_equal(p.matmult_bc(col), p.matmult_bc(col.copy()))
