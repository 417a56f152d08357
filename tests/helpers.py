"""Shared helpers of the test suite: golden fixtures and operator set-up."""
import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# Relative tolerance of every FP64 parity check (norm-wise, ||x - ref|| / ||ref||).
FP64_RTOL = 1e-12


def golden_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not p.endswith("element_matrices.npz"))


def load(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / (nb if nb > 0 else 1.0)


def element_blocks(g):
    """(offsets, per-element row-major Ke views) of a fixture."""
    off = g["offsets"].astype(np.int64)
    ke = g["ke"]
    out, k = [], 0
    for e in range(len(off) - 1):
        n = int(off[e + 1] - off[e])
        out.append(ke[k:k + n * n].reshape(n, n))
        k += n * n
    return off, out


def make_operator(g, bc_method=0, precision=None, blocks=False):
    """aMatFree built from a fixture through the reference-shaped API."""
    from amat_gb300 import Maps, aMatFree
    off, kes = element_blocks(g)
    dpe = np.diff(off).astype(np.uint32)
    maps = Maps()
    maps.set_map(len(dpe), g["map"], dpe, int(g["n_dofs"]), None, 0, int(g["n_dofs"]) - 1, int(g["n_dofs"]))
    maps.set_bdr_map(g["constrained"], g["values"], len(g["constrained"]))
    A = aMatFree(maps, bc_method)
    if precision is not None:
        A.set_precision(precision)
    bd = int(g.get("blocks_dim", 1)) if blocks else 1
    for e, k in enumerate(kes):
        n = k.shape[0]
        nb = n // bd
        for bi in range(bd):
            for bj in range(bd):
                blk = k[bi * nb:(bi + 1) * nb, bj * nb:(bj + 1) * nb]
                if bi == bj or np.any(blk != 0):
                    A.set_element_matrix(e, np.ascontiguousarray(blk), bi, bj, bd)
    A.finalize()
    return A
