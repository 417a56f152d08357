"""The allocation-free CG entry point (afm_solve_cg_device_noalloc) against
the allocating one (afm_solve_cg_device), through the C ABI.

The entry point serves callers that cannot allocate device memory while they
run (an application whose allocator already holds the GPU's memory, or a loop
that must not stall on cudaMalloc/cudaFree); its CG work vectors live in a
fixed array inside libafm.so. This file is collected last so that a run that
stops at the first failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

from amat_gb300 import Maps, aMatFree, libafm
from amat_gb300 import problems as P
from amat_gb300._native import NOALLOC_MAX_DOFS, AfmSolveStats
from helpers import FP64_RTOL, rel

pytestmark = pytest.mark.gpu


def poisson_operator(n):
    m = P.Mesh(P.HEX8_POISSON, n, jitter=0.1, seed=21)
    dofs, vals = m.boundary_conditions()
    maps = Maps()
    maps.set_map(m.n_elem, m.dof_map(), m.ndpe, m.n_dofs)
    maps.set_bdr_map(dofs, vals)
    A = aMatFree(maps)
    A.set_element_matrices(0, m.element_matrices())
    A.finalize()
    return m, A


def solve(A, fn, b, rtol=1e-10):
    import torch
    lib = libafm()
    db = torch.tensor(b, dtype=torch.float64, device="cuda")
    dx = torch.zeros_like(db)
    torch.cuda.synchronize()
    st = AfmSolveStats()
    s = getattr(lib, fn)(A._h, C.c_void_p(db.data_ptr()), C.c_void_p(dx.data_ptr()), rtol, 0.0, 5000, 0,
                         C.byref(st))
    assert s == 0, lib.afm_last_error().decode()
    return dx.cpu().numpy(), st


def test_noalloc_cg_matches_allocating_cg(gpu):
    """On a fresh operator the allocation-free solve runs first: the device's free memory is the same
    before and after it and the operator has allocated no work space; then it agrees with the allocating
    solve on the same operator, on two calls in a row (the shared array keeps the previous call's
    contents)."""
    import torch
    # set-up: the first call on the device loads the module that holds the array (a one-time reservation)
    m0, A0 = poisson_operator(4)
    solve(A0, "afm_solve_cg_device_noalloc", A0.apply_bc(np.ones(m0.n_dofs)))
    m, A = poisson_operator(12)
    _, B = poisson_operator(12)  # the same system: its host calls make the loads, so A stays untouched
    rng = np.random.default_rng(0)
    bs = [B.apply_bc(rng.normal(size=m.n_dofs)) for _ in range(2)]
    assert A.info()["work_bytes"] == 0
    db = torch.tensor(bs[0], dtype=torch.float64, device="cuda")
    dx = torch.zeros_like(db)
    torch.cuda.synchronize()
    lib = libafm()
    st = AfmSolveStats()
    free0 = torch.cuda.mem_get_info()[0]
    s = lib.afm_solve_cg_device_noalloc(A._h, C.c_void_p(db.data_ptr()), C.c_void_p(dx.data_ptr()), 1e-10, 0.0,
                                        5000, 0, C.byref(st))
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert s == 0, lib.afm_last_error().decode()
    assert free1 == free0
    assert A.info()["work_bytes"] == 0
    first = dx.cpu().numpy()
    for k, b in enumerate(bs):
        x, st = solve(A, "afm_solve_cg_device_noalloc", b)
        if k == 0:
            assert np.array_equal(x, first)
        x_ref, st_ref = solve(A, "afm_solve_cg_device", b)
        assert st.status == 0 and st.iterations == st_ref.iterations
        assert rel(x, x_ref) < FP64_RTOL
        assert abs(st.rel_residual - st_ref.rel_residual) <= 1e-12


def test_noalloc_rejects_operators_beyond_its_limit(gpu):
    n = NOALLOC_MAX_DOFS + 1
    maps = Maps()
    maps.set_map(1, np.arange(8, dtype=np.uint32), 8, n)
    A = aMatFree(maps)
    A.set_element_matrix(0, np.eye(8) * 2.0)
    A.finalize()
    import torch
    db = torch.zeros(n, dtype=torch.float64, device="cuda")
    dx = torch.zeros_like(db)
    lib = libafm()
    s = lib.afm_solve_cg_device_noalloc(A._h, C.c_void_p(db.data_ptr()), C.c_void_p(dx.data_ptr()), 1e-10, 0.0,
                                        10, 0, None)
    assert s == 105
    assert b"allocation-free limit" in lib.afm_last_error()
