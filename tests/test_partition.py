"""Element-partitioned operator on CPU ranks (gloo): the scatter map of
Maps::buildScatterMap and the ghost exchanges of aMatFree around a local
product, checked against the whole-mesh oracle. The local products are the
oracle's (the device product of each rank runs the same C ABI call as a
single-rank operator); what is under test is the partition logic: ghost lists,
owners, send lists, local numbering, and the exchange and accumulation order."""
import os
import socket

import numpy as np
import pytest

import oracle
from amat_gb300 import problems as P
from helpers import rel


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _partition(dm, n_dofs, world, scheme):
    """Contiguous owned DoF ranges and an element -> rank assignment."""
    splits = np.linspace(0, n_dofs, world + 1).astype(np.int64)
    key = dm.max(axis=1) if scheme == "max" else dm.min(axis=1)
    return splits, np.searchsorted(splits[1:], key, side="right")


def _worker(rank, world, port, kind, n, scheme):
    import torch.distributed as dist
    from amat_gb300.partition import PartitionedProduct, ScatterMap
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        m = P.Mesh(kind, n, jitter=0.1, seed=7)
        ke = m.element_matrices()
        npe = m.ndpe
        dm = m.dof_map().reshape(m.n_elem, npe).astype(np.int64)
        splits, owner = _partition(dm, m.n_dofs, world, scheme)
        mine = np.nonzero(owner == rank)[0]
        b, e = int(splits[rank]), int(splits[rank + 1])
        smap = ScatterMap(dist.group.WORLD, dm[mine], e - b, b, n_per_element=npe)
        assert smap.n_global == m.n_dofs and smap.begin == b and smap.end == e
        # every ghost lies outside the owned range, sorted and unique; local -> global is a bijection
        assert np.all(smap.pre < b) and np.all(smap.post >= e)
        assert np.all(np.diff(smap.pre) > 0) and np.all(np.diff(smap.post) > 0)
        assert len(np.unique(smap.local2global)) == smap.n_all
        lmap = smap.local_map.reshape(-1, npe).astype(np.int64)
        assert np.array_equal(smap.local2global[lmap], dm[mine])
        local = oracle.Problem(smap.n_all, lmap, ke[mine])

        def product(v, u):
            v[:] = local.matvec(u)

        part = PartitionedProduct(smap, product)
        ug_all = np.random.default_rng(5).uniform(-1, 1, m.n_dofs)  # the same global u on every rank
        glob = oracle.Problem(m.n_dofs, dm, ke)
        ref = glob.matvec(ug_all)
        # ghost receive fills exactly the owners' values
        u = smap.ghosted(ug_all[b:e])
        smap.ghost_receive(u)
        assert np.array_equal(u, ug_all[smap.local2global])
        # the partitioned product on the owned rows
        v = np.zeros(smap.n_all)
        part.matvec(v, smap.ghosted(ug_all[b:e]), True)
        assert rel(smap.owned(v), ref[b:e]) < 1e-13
        w = np.zeros(e - b)
        part.matvec(w, ug_all[b:e], False)
        assert np.array_equal(w, smap.owned(v))
        # diagonal: element sums of every rank on the owned rows
        d = part.diagonal(local.get_diagonal())
        dref = glob.get_diagonal()
        assert rel(smap.owned(d), dref[b:e]) < 1e-14
        # the exchange is reproducible: a second product gives the same bits
        v2 = np.zeros(smap.n_all)
        part.matvec(v2, smap.ghosted(ug_all[b:e]), True)
        assert np.array_equal(smap.owned(v2), smap.owned(v))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world,kind,n,scheme", [
    (2, P.HEX8_POISSON, 5, "max"),
    (3, P.HEX8_POISSON, 6, "min"),
    (2, P.HEX8_ELASTIC, 3, "min"),
    (3, P.TET10_POISSON, 3, "max"),
])
def test_partitioned_product_matches_whole_mesh(world, kind, n, scheme):
    import torch.multiprocessing as mp
    mp.spawn(_worker, args=(world, _free_port(), kind, n, scheme), nprocs=world, join=True)


def _bad_range_worker(rank, world, port):
    import torch.distributed as dist
    from amat_gb300.partition import ScatterMap
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # both ranks claim a start that the scan of owned counts (0, 4) contradicts, so both stop at
        # the same check, before any further collective
        with pytest.raises(ValueError):
            ScatterMap(dist.group.WORLD, np.array([0, 1, 2, 3], dtype=np.int64), 4, 1 if rank == 0 else 3,
                       n_per_element=4)
    finally:
        dist.destroy_process_group()


def test_scatter_map_rejects_a_gap_in_the_owned_ranges():
    import torch.multiprocessing as mp
    mp.spawn(_bad_range_worker, args=(2, _free_port()), nprocs=2, join=True)
