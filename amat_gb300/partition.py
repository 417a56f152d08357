"""Element-partitioned operators: one rank per GPU, each rank owning a
contiguous range of global DoFs and the elements it was given.

The scatter map follows par::Maps::buildScatterMap (include/maps.hpp:520-826):
the ranks' owned DoF counts are gathered and scanned into owned ranges; the
DoFs of this rank's elements below its range are pre-ghosts and those above
are post-ghosts (each sorted, unique); every ghost is owned by the rank whose
range holds it; the ghost ids are sent to their owners, which turn them into
send lists of their own local ids. The rank-local numbering is the
reference's: [pre-ghosts | owned | post-ghosts].

The exchanges follow aMatFree::ghost_receive_begin/end and
ghost_send_begin/end (include/aMatFree.hpp:1427-1679): before a product the
owners' values of u are copied into every rank's ghost slots; after it the
ghost rows of v are sent to their owners, which add them to their own rows,
rank by rank in rank order (so the sums are reproducible). Communication is
torch.distributed all_to_all_single over the given process group (gloo with
host tensors, NCCL with device tensors), with zero-sized parts for ranks that
exchange nothing.

The device product of a rank runs over its local numbering through the C ABI
(afm_matvec on an operator whose map is the rank-local one); no device kernel
waits for another rank, and the exchange happens between products.
"""
import numpy as np


def _dist():
    import torch.distributed as dist
    return dist


class ScatterMap:
    """Maps::buildScatterMap for this rank of `group`.

    element_dofs: global DoF ids of this rank's elements, flat, with
    `offsets` (n_elem + 1) or a uniform `n_per_element`. n_owned: DoFs this
    rank owns; owned_begin: the first of them (global id), which must equal
    the scan of the ranks' counts (continuous partition, as in the reference).
    """

    def __init__(self, group, element_dofs, n_owned, owned_begin, offsets=None, n_per_element=None):
        import torch
        dist = _dist()
        self.group = group
        self.size = dist.get_world_size(group)
        self.rank = dist.get_rank(group)
        g = np.ascontiguousarray(element_dofs, dtype=np.int64).reshape(-1)
        counts = torch.zeros(self.size, dtype=torch.int64)
        mine = torch.tensor([int(n_owned)], dtype=torch.int64)
        parts = [torch.zeros(1, dtype=torch.int64) for _ in range(self.size)]
        dist.all_gather(parts, mine, group=group)
        counts = np.array([int(p.item()) for p in parts], dtype=np.int64)
        scan = np.zeros(self.size + 1, dtype=np.int64)
        np.cumsum(counts, out=scan[1:])
        self.dof_counts = counts
        self.dof_scan = scan
        self.n_global = int(scan[-1])
        self.begin = int(scan[self.rank])
        self.n_owned = int(n_owned)
        self.end = self.begin + self.n_owned  # exclusive
        if int(owned_begin) != self.begin:
            raise ValueError("owned range starts at %d, the scan of owned counts gives %d" % (owned_begin, self.begin))
        if g.size and (g.min() < 0 or g.max() >= self.n_global):
            raise ValueError("element DoF id outside [0, %d)" % self.n_global)
        self.pre = np.unique(g[g < self.begin])
        self.post = np.unique(g[g >= self.end])
        self.n_pre, self.n_post = len(self.pre), len(self.post)
        self.n_all = self.n_pre + self.n_owned + self.n_post
        # local ids of the element slots: [pre | owned | post]
        loc = np.empty_like(g)
        own = (g >= self.begin) & (g < self.end)
        loc[own] = g[own] - self.begin + self.n_pre
        lo = g < self.begin
        loc[lo] = np.searchsorted(self.pre, g[lo])
        hi = g >= self.end
        loc[hi] = self.n_pre + self.n_owned + np.searchsorted(self.post, g[hi])
        self.local_map = loc.astype(np.uint32)
        self.offsets = None if offsets is None else np.asarray(offsets, dtype=np.uint32)
        self.n_per_element = n_per_element
        self.local2global = np.concatenate([self.pre, np.arange(self.begin, self.end, dtype=np.int64), self.post])
        # ghosts in the order they are received: pre-ghosts then post-ghosts, grouped by owner (ascending)
        req = np.concatenate([self.pre, self.post])
        owner = np.searchsorted(scan[1:], req, side="right")
        self.ghost_local = np.concatenate([np.arange(self.n_pre),
                                           self.n_pre + self.n_owned + np.arange(self.n_post)]).astype(np.int64)
        self.recv_counts = np.bincount(owner, minlength=self.size).astype(np.int64)  # ghosts I get from each rank
        # how many of my DoFs each rank wants
        rc = torch.tensor(self.recv_counts, dtype=torch.int64)
        sc = torch.empty(self.size, dtype=torch.int64)
        dist.all_to_all_single(sc, rc, group=group)
        self.send_counts = sc.numpy().astype(np.int64)
        # the requested global ids, turned into my local ids (the send lists)
        want = torch.empty(int(self.send_counts.sum()), dtype=torch.int64)
        dist.all_to_all_single(want, torch.tensor(req, dtype=torch.int64), self.send_counts.tolist(),
                               self.recv_counts.tolist(), group=group)
        want = want.numpy()
        if want.size and (want.min() < self.begin or want.max() >= self.end):
            raise RuntimeError("scatter map: a rank asked for a DoF this rank does not own")
        self.send_ids = (want - self.begin + self.n_pre).astype(np.int64)
        self.send_offsets = np.zeros(self.size + 1, dtype=np.int64)
        np.cumsum(self.send_counts, out=self.send_offsets[1:])

    # ---- exchanges ---------------------------------------------------------
    def ghost_receive(self, vec):
        """Owners' values into this rank's ghost slots (vec: local ghosted, n_all)."""
        import torch
        dist = _dist()
        send = torch.as_tensor(np.ascontiguousarray(vec[self.send_ids]))
        recv = torch.empty(int(self.recv_counts.sum()), dtype=send.dtype)
        dist.all_to_all_single(recv, send, self.recv_counts.tolist(), self.send_counts.tolist(), group=self.group)
        vec[self.ghost_local] = recv.numpy()
        return vec

    def ghost_send(self, vec):
        """Ghost rows of vec to their owners, which add them to their rows rank by rank (vec: n_all)."""
        import torch
        dist = _dist()
        send = torch.as_tensor(np.ascontiguousarray(vec[self.ghost_local]))
        recv = torch.empty(int(self.send_counts.sum()), dtype=send.dtype)
        dist.all_to_all_single(recv, send, self.send_counts.tolist(), self.recv_counts.tolist(), group=self.group)
        r = recv.numpy()
        for p in range(self.size):
            a, b = self.send_offsets[p], self.send_offsets[p + 1]
            if b > a:
                vec[self.send_ids[a:b]] += r[a:b]  # unique ids within one rank's part
        return vec

    # ---- vector layouts ----------------------------------------------------
    def owned(self, vec):
        return vec[self.n_pre:self.n_pre + self.n_owned]

    def ghosted(self, owned_vec):
        """A local ghosted vector with the owned entries set and zero ghosts (Maps::local_to_ghost)."""
        out = np.zeros(self.n_all, dtype=np.asarray(owned_vec).dtype)
        out[self.n_pre:self.n_pre + self.n_owned] = owned_vec
        return out


class PartitionedProduct:
    """aMatFree::matvec_ghosted across ranks: v = K u on local ghosted vectors.

    local_product(v, u) computes this rank's element products over the local
    numbering (every local row, ghost rows included); the device operator's
    afm_matvec in the library, any function of the same shape in tests.
    """

    def __init__(self, smap, local_product):
        self.smap = smap
        self.local_product = local_product

    def matvec(self, v, u, isGhosted=True):
        s = self.smap
        if not isGhosted:
            ug = s.ghosted(u)
            vg = np.zeros(s.n_all)
            self.matvec(vg, ug, True)
            v[:] = s.owned(vg)
            return v
        s.ghost_receive(u)
        self.local_product(v, u)
        s.ghost_send(v)
        return v

    def diagonal(self, local_diag):
        """The assembled diagonal on owned rows from each rank's element diagonal sums."""
        d = np.array(local_diag, dtype=np.float64, copy=True)
        self.smap.ghost_send(d)
        return d
