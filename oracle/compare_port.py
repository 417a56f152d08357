"""Times the oracle's port of the reference CPU loop against the reference
itself, compiled in place (oracle/_ref, this x86 container only), on the
same sample of the default workload: hex20 elasticity, the first --elements
elements of the 64^3 mesh. Both the reference's default build (row-major
element GEMV) and its VECTORIZED_OPENMP build (column-major element matrices,
omp simd element product) against the port of each, at one thread and at
every host thread. Test infrastructure: it says how faithfully the port,
which is what the GPU machine can run, stands in for the reference's speed.

    python oracle/compare_port.py [--elements 16384] [--seconds 3]

Each thread count runs in a child process (OMP_NUM_THREADS), so both
libraries start their OpenMP runtime with it.
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)


def sample(n_elem):
    from amat_gb300 import problems as P
    m = P.Mesh(P.HEX20_ELASTIC, 64, jitter=0.1, seed=1)
    ne = min(n_elem, m.n_elem)
    ke = m.element_matrices(0, ne, ngt=3)
    dm = np.ascontiguousarray(m.dof_map().reshape(m.n_elem, m.ndpe)[:ne])
    used = np.unique(dm).size
    return m, ke, dm, used


def timed(fn, seconds):
    fn()  # warm-up
    ts = []
    while sum(ts) < seconds or len(ts) < 3:
        t0 = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - t0)
    return float(np.median(ts))


def child(n_elem, seconds):
    import ctypes as C

    import oracle
    m, ke, dm, used = sample(n_elem)
    ne, n = dm.shape
    pr = oracle.Problem(m.n_dofs, dm, ke)
    u = np.random.default_rng(0).uniform(-1, 1, m.n_dofs)
    v = np.empty(m.n_dofs)
    nbytes = ne * (n * n * 8 + 4 * n) + 16 * used  # Ke, map, the u entries read and v entries written
    out = {"elements": ne, "bytes": nbytes, "threads": None}
    ref_v = pr.matvec(u)
    for simd in (False, True):
        tag = "simd" if simd else "rowmajor"
        R = oracle.ref(simd)
        if R is not None:
            h = R.ref_afm_create(pr.n_elem, pr.n_dofs, C.c_void_p(pr.offsets.ctypes.data),
                                 C.c_void_p(pr.map.ctypes.data), C.c_void_p(pr.ke.ctypes.data), 1, None, None, 0, 0)
            w = np.empty(m.n_dofs)
            t = timed(lambda: R.ref_afm_matvec(h, C.c_void_p(w.ctypes.data), C.c_void_p(u.ctypes.data)), seconds)
            R.ref_afm_destroy(h)
            out["reference_" + tag] = {"s": t, "gbs": nbytes / t / 1e9,
                                       "rel_diff": float(np.linalg.norm(w - ref_v) / np.linalg.norm(ref_v))}
        t = timed(lambda: pr.matvec_omp_cfg(u, v, 0, simd), seconds)
        _, th = pr.matvec_omp_cfg(u, v, 0, simd)
        out["threads"] = th
        out["port_" + tag] = {"s": t, "gbs": nbytes / t / 1e9,
                              "rel_diff": float(np.linalg.norm(v - ref_v) / np.linalg.norm(ref_v))}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--elements", type=int, default=16384)
    ap.add_argument("--seconds", type=float, default=3.0)
    ap.add_argument("--child", action="store_true")
    args = ap.parse_args()
    if args.child:
        child(args.elements, args.seconds)
        return
    rows = {}
    for nt in (1, os.cpu_count() or 1):
        env = dict(os.environ, OMP_NUM_THREADS=str(nt))
        r = subprocess.run([sys.executable, __file__, "--child", "--elements", str(args.elements), "--seconds",
                            str(args.seconds)], env=env, capture_output=True, text=True, check=True)
        rows[nt] = json.loads(r.stdout.strip().splitlines()[-1])
    print(json.dumps(rows, indent=1))


if __name__ == "__main__":
    main()
