"""The partitioned operator with its device products: two ranks (processes)
share the one GPU, exchange ghosts through gloo on the host, and each runs its
element products through the C ABI over its local numbering. Their kernels
never wait for one another (the exchanges happen between products). Checked
against the whole-mesh oracle: v = K u, MatMult_mf with constrained DoFs on
both sides of the cut, and the Jacobi diagonal."""
import os
import socket

import numpy as np
import pytest

import oracle
from amat_gb300 import problems as P
from helpers import FP64_RTOL, rel

pytestmark = pytest.mark.gpu


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, kind, n, prec):
    import torch.distributed as dist
    from amat_gb300 import Maps, aMatFree
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        m = P.Mesh(kind, n, jitter=0.1, seed=3)
        ke = m.element_matrices(ngt=3 if kind == P.HEX20_ELASTIC else 2)
        npe = m.ndpe
        dm = m.dof_map().reshape(m.n_elem, npe).astype(np.int64)
        dofs, vals = m.boundary_conditions()
        splits = np.linspace(0, m.n_dofs, world + 1).astype(np.int64)
        owner = np.searchsorted(splits[1:], dm.max(axis=1), side="right")
        mine = np.nonzero(owner == rank)[0]
        b, e = int(splits[rank]), int(splits[rank + 1])
        # the rank's own local numbering for set_map: its DoFs in any order, mapped to global ids
        gl = np.unique(dm[mine])
        local_ids = np.searchsorted(gl, dm[mine]).astype(np.uint32)
        maps = Maps(comm=dist.group.WORLD)
        pre = int(np.sum(gl < b))
        n_all = len(np.union1d(gl, np.arange(b, e)))
        maps.set_map(len(mine), local_ids, npe, n_all, gl.astype(np.uint64), b, e - 1, m.n_dofs)
        maps.set_bdr_map(dofs, vals)
        A = aMatFree(maps)
        A.set_precision(prec)
        A.set_element_matrices(0, ke[mine])
        A.finalize()
        s = maps.scatter
        assert s.n_pre == pre
        glob = oracle.Problem(m.n_dofs, dm, ke, dofs, vals)
        u = np.random.default_rng(9).uniform(-1, 1, m.n_dofs)
        v = np.zeros(s.n_all)
        A.matvec(v, s.ghosted(u[b:e]), True)
        assert rel(s.owned(v), glob.matvec(u)[b:e]) < FP64_RTOL
        w = np.zeros(s.n_all)
        A.matmult_bc(w, s.ghosted(u[b:e]))
        assert rel(s.owned(w), glob.matmult_bc(u)[b:e]) < FP64_RTOL
        d = A.get_diagonal()
        assert rel(s.owned(d), glob.get_diagonal()[b:e]) < 1e-14
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("kind,n,prec", [(P.HEX20_ELASTIC, 4, 1), (P.HEX8_POISSON, 8, 0), (P.TET10_POISSON, 4, 1)])
def test_partitioned_device_products(gpu, kind, n, prec):
    import torch.multiprocessing as mp
    mp.spawn(_worker, args=(2, _free_port(), kind, n, prec), nprocs=2, join=True)
