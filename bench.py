"""Benchmark of the GB300 AFM matvec (v = K u, stored element matrices).

Workload (default): 3-D linear elasticity on a structured 64^3 mesh of 20-node
serendipity hexahedra (262,144 elements, 1,085,825 nodes, 3,257,475 DoF),
60x60 FP64 element matrices from 3x3x3 Gauss quadrature, E = 1, nu = 0.3,
vertex coordinates jittered by uniform +-0.1 h (seed 1). One step = one
matvec over the whole mesh with u resident in HBM. The inputs (7.66 GB) are
~60x the 129 MB L2, so no L2 flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`--impl reference` times the CPU implementation of the reference's method-1
loop (the oracle's port of matvec_ghosted_OMP: OpenMP parallel-for over
elements, row-major GEMV, atomic scatter) on all host cores, on a bounded
sample of the same workload. One JSON line on stdout (rank 0).

Other measurements (`--mode`, each one JSON line):
  solve      CG solves/s to --rtol: FP64 Jacobi-PCG against the mixed-precision
             solve (--free 1: on the matrix-free operator)
  batched    block CG over --nrhs load cases against one-at-a-time FP64 CG
  product    the batched multi-RHS product in FP32 and FP64-split, TFLOP/s
  serve      served solves/s and p50/p99 latency under Poisson arrivals
  assembled  the aMatBased CSR SpMV against the assembly-free product
  free       the matrix-free (method 2) products against the stored-Ke ones
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "hex20_elastic_64": dict(kind=2, n=64, ngt=3, jitter=0.1, seed=1,
                             desc="hex20 elasticity 64^3, 60x60 FP64 Ke, 3x3x3 Gauss, jitter 0.1h"),
    "hex20_elastic_32": dict(kind=2, n=32, ngt=3, jitter=0.1, seed=1,
                             desc="hex20 elasticity 32^3, 60x60 FP64 Ke, 3x3x3 Gauss, jitter 0.1h"),
    "hex8_poisson_32": dict(kind=0, n=32, ngt=2, jitter=0.0, seed=0,
                            desc="hex8 Poisson 32^3, 8x8 FP64 Ke, 2x2x2 Gauss"),
    "hex8_elastic_48": dict(kind=1, n=48, ngt=2, jitter=0.1, seed=3,
                            desc="hex8 elasticity 48^3, 24x24 FP64 Ke"),
    "tet10_poisson_96": dict(kind=3, n=96, ngt=2, jitter=0.15, seed=2,
                             desc="tet10 Poisson 96^3 x 6 (5.3M tets), 10x10 Ke"),
    "tet10_poisson_48": dict(kind=3, n=48, ngt=2, jitter=0.15, seed=2,
                             desc="tet10 Poisson 48^3 x 6 (663k tets), 10x10 Ke"),
    "tet10_poisson_64": dict(kind=3, n=64, ngt=2, jitter=0.15, seed=2,
                             desc="tet10 Poisson 64^3 x 6 (1.57M tets), 10x10 Ke"),
    "tet10_elastic_64": dict(kind=4, n=64, ngt=2, jitter=0.15, seed=2,
                             desc="tet10 elasticity 64^3 x 6 (1.57M tets), 30x30 Ke, E=1, nu=0.3"),
    "tet10_elastic_96": dict(kind=4, n=96, ngt=2, jitter=0.15, seed=2,
                             desc="tet10 elasticity 96^3 x 6 (5.3M tets), 30x30 Ke, E=1, nu=0.3"),
    "hex8_poisson_96": dict(kind=0, n=96, ngt=2, jitter=0.1, seed=0,
                            desc="hex8 Poisson 96^3, 8x8 FP64 Ke, 2x2x2 Gauss, jitter 0.1h"),
}
PREC_NAMES = {"fp64": 0, "fp64_split": 1, "fp32": 2, "auto": 3}
PREC_DTYPE = {0: "f64", 1: "f64 (Ke as hi+lo f32 pair, double-float products; <=1e-12 rel. vs FP64)", 2: "f32"}
PREC_KEYS = {0: "fp64", 1: "fp64_split", 2: "fp32"}
CHUNK = 16384  # elements per generated block


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(key):
    """DRAM bytes per matvec of the dominant kernel from the committed ncu summary, or None."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        return json.load(f).get(key)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def build_problem(w, prec, device_index, keep_ke=False):
    """Mesh, element matrices (generated in blocks straight into the operator), operator; with keep_ke, also
    the host copy of every element matrix (for the full-size parity check)."""
    from amat_gb300 import Maps, aMatFree
    from amat_gb300 import problems as P
    t0 = time.time()
    m = P.Mesh(w["kind"], w["n"], jitter=w["jitter"], seed=w["seed"])
    dmap = m.dof_map()
    maps = Maps()
    maps.set_map(m.n_elem, dmap, m.ndpe, m.n_dofs)
    A = aMatFree(maps, 0, device_index)
    A.set_precision(prec)
    ke = np.empty((m.n_elem, m.ndpe, m.ndpe)) if keep_ke else None
    buf = np.empty((CHUNK, m.ndpe, m.ndpe))
    for e0 in range(0, m.n_elem, CHUNK):
        c = min(CHUNK, m.n_elem - e0)
        blk = ke[e0:e0 + c] if keep_ke else buf[:c]
        m.element_matrices(e0, c, ngt=w["ngt"], out=blk)
        A.set_element_matrices(e0, blk)
    t1 = time.time()
    A.finalize()
    t2 = time.time()
    log("setup: mesh+Ke %.1fs finalize %.1fs, %d elements, %d DoF" % (t1 - t0, t2 - t1, m.n_elem, m.n_dofs))
    if keep_ke:
        return m, dmap, A, ke
    return m, dmap, A


def cpu_sample(w, m, dmap, max_elems):
    """Reference CPU loop on the first max_elems elements (oracle port, all host threads)."""
    import oracle
    from amat_gb300 import problems as P
    ne = min(m.n_elem, max_elems)
    ke = m.element_matrices(0, ne, ngt=w["ngt"])
    pr = oracle.Problem(m.n_dofs, dmap[:ne], ke)
    u = np.random.default_rng(0).uniform(-1, 1, m.n_dofs)
    v = np.empty(m.n_dofs)
    pr.matvec_omp(u, v)  # warm-up
    n = m.ndpe
    # Ke and map of the sample, and the u entries it reads and v entries it writes (its own DoFs only)
    sample_bytes = ne * (n * n * 8 + 4 * n) + 16 * int(np.unique(pr.map).size)
    return pr, u, v, ne, sample_bytes


def full_parity(m, dmap, ke, u, v):
    """||v - v_ref|| / ||v_ref||, v_ref = the reference CPU loop (oracle port) over every element."""
    import oracle
    pr = oracle.Problem(m.n_dofs, dmap.reshape(m.n_elem, m.ndpe), ke)
    ref, _ = pr.matvec_omp(u)
    return float(np.linalg.norm(v - ref) / np.linalg.norm(ref))


def time_cpu(pr, u, v, reps, seconds=0.0, threads=0, simd=False):
    """reps matvecs, continued until `seconds` of CPU time have been timed (threads 0: every host thread;
    simd: the port of the reference's VECTORIZED_OPENMP element product)."""
    ts = []
    used = 1
    while len(ts) < reps or sum(ts) < seconds:
        t0 = time.perf_counter()
        _, used = pr.matvec_omp_cfg(u, v, threads, simd)
        ts.append(time.perf_counter() - t0)
    return ts, used


def run_reference(args, w, rank):
    from amat_gb300 import problems as P
    if rank != 0:
        return None
    m = P.Mesh(w["kind"], w["n"], jitter=w["jitter"], seed=w["seed"])
    dmap = m.dof_map()
    pr, u, v, ne, sbytes = cpu_sample(w, m, dmap, args.cpu_sample_elems)
    # both builds of the reference's loop (row-major GEMV, VECTORIZED_OPENMP), on every host thread and on
    # one; the line reports the faster on every thread
    variants = {}
    for simd in (False, True):
        time_cpu(pr, u, v, args.warmup, simd=simd)
        ts, threads = time_cpu(pr, u, v, args.steps, simd=simd)
        t1, _ = time_cpu(pr, u, v, 2, threads=1, simd=simd)
        key = "vectorized_openmp" if simd else "rowmajor"
        variants[key] = {"all_threads_gbs": sbytes * len(ts) / sum(ts) / 1e9, "threads": threads,
                         "one_thread_gbs": sbytes * len(t1) / sum(t1) / 1e9, "ms_per_step": 1e3 * sum(ts) / len(ts)}
    best = max(variants, key=lambda k: variants[k]["all_threads_gbs"])
    t = variants[best]["ms_per_step"] * 1e-3 * args.steps
    threads = variants[best]["threads"]
    value = variants[best]["all_threads_gbs"]
    sample = "%d of %d elements (%s) per step, %d steps; %s element product" % (ne, m.n_elem, w["desc"],
                                                                                args.steps, best)
    return {
        "impl": "reference", "metric": "AFM matvec GB/s", "value": value, "unit": "GB/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": w["desc"], "method": "method 1 (QUASI_FREE), OpenMP + atomic scatter, CPU"},
        "cpu_baseline": {"value": value, "unit": "GB/s", "cores": threads, "kind": "port", "sample": sample,
                         "variants": variants},
        "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


L2_BYTES = 129 * 2 ** 20
L2_FLUSH_BYTES = 4 * L2_BYTES


def flushes_l2(info):
    """Steps whose bytes are under four L2 capacities are timed one by one after an L2 flush."""
    return info["algorithmic_bytes"] < 4 * L2_BYTES


def l2_note(info):
    alg = info["algorithmic_bytes"]
    if flushes_l2(info):
        return "flushed: %d MB written before each step (inputs %.3f GB)" % (L2_FLUSH_BYTES >> 20, alg / 1e9)
    return "no flush: inputs %.2f GB > 4 x 129 MB L2" % (alg / 1e9)


def measure_device(A, n, steps, warmup, world, dev, rank, sample_clocks):
    """Times `steps` matvecs on device-resident vectors (CUDA events on the operator's stream)."""
    import torch
    info = A.info()
    stream_ptr = A.stream()
    stream = torch.cuda.ExternalStream(stream_ptr)
    f32 = info["precision"] == 2
    u_host = np.random.default_rng(1234 + rank).uniform(-1, 1, n)
    u = torch.tensor(u_host, dtype=torch.float32 if f32 else torch.float64, device="cuda")
    v = torch.empty_like(u)
    torch.cuda.synchronize()

    def step():
        if f32:
            A.matvec_device_f32(v.data_ptr(), u.data_ptr(), stream_ptr)
        else:
            A.matvec_device(v.data_ptr(), u.data_ptr(), stream_ptr)

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    # timed region: K matvecs bracketed by barrier + synchronize
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clk = ClockSampler(dev) if sample_clocks else None
    if clk:
        clk.__enter__()
    if flushes_l2(info):
        # inputs that fit in L2 several times over: each step starts cold, after a write of L2_FLUSH_BYTES
        # on the same stream; the step alone is timed (one event pair per step)
        junk = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        with torch.cuda.stream(stream):
            for a, b in evs:
                junk.fill_(1.0)
                a.record(stream)
                step()
                b.record(stream)
        torch.cuda.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in evs)
    else:
        ev0.record(stream)
        for _ in range(steps):
            step()
        ev1.record(stream)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1)
    if clk:
        clk.__exit__(None, None, None)
    A.synchronize()
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    return info, ms, u_host, v, clk


def measure_e2e(A, u_host, v_dev, steps, world):
    """The reference-facing host call afm_matvec: u H2D and v D2H inside every step."""
    import ctypes as C
    import torch
    n = len(u_host)
    u_pin = torch.from_numpy(u_host).pin_memory()
    v_pin = torch.empty(n, dtype=torch.float64).pin_memory()
    lib = A._lib
    up, vp = C.c_void_p(u_pin.data_ptr()), C.c_void_p(v_pin.data_ptr())
    for _ in range(2):
        assert lib.afm_matvec(A._h, vp, up, 1) == 0
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(steps):
        assert lib.afm_matvec(A._h, vp, up, 1) == 0
    e2e_s = time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([e2e_s], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    # the host call and the device call agree bit for bit
    assert np.array_equal(v_pin.numpy(), v_dev.cpu().numpy())
    return e2e_s


def measure_inner_f32(A, m, steps, warmup):
    """FP32 products of the split operator (the inner matvec of the mixed-precision solve): from the
    symmetric copy (each pair of entries once) with and without its BF16 correction plane, and from the
    hi plane; GB/s over the bytes streamed."""
    import torch
    stream_ptr = A.stream()
    stream = torch.cuda.ExternalStream(stream_ptr)
    u = torch.tensor(np.random.default_rng(99).uniform(-1, 1, m.n_dofs), dtype=torch.float32, device="cuda")
    v = torch.empty_like(u)
    base = 4 * m.n_elem * m.ndpe + 8 * m.n_dofs  # map entries, u read, v written
    out = {}
    names = {5: "symmetric_copy_bf16_correction_fp64_vectors_fp32_u_fp32_rows",
             4: "symmetric_copy_bf16_correction_fp64_vectors_fp32_u",
             3: "symmetric_copy_bf16_correction_fp64_vectors", 2: "symmetric_copy_bf16_correction",
             1: "symmetric_copy", 0: "hi_plane"}
    u64 = u.double()
    v64 = torch.empty_like(u64)
    for sym in (5, 4, 3, 2, 1, 0):
        A.set_symmetric_inner(sym)

        def product():
            if sym >= 3:  # FP64 vectors (the inner products of formats 3 and 4)
                A.matvec_inner_device(v64.data_ptr(), u64.data_ptr(), stream_ptr)
            else:
                A.matvec_device_f32(v.data_ptr(), u.data_ptr(), stream_ptr)
        for _ in range(warmup):
            product()
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(steps):
            product()
        ev1.record(stream)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1) / steps
        info = A.info()
        ke = info["sym_bytes"] if sym else info["ke_bytes"] // 2
        if sym and not ke:
            continue  # no symmetric copy for this operator
        vec = base + 8 * m.n_dofs if sym >= 3 else base  # FP64 u and v
        out[names[sym]] = {
            "ms": ms, "ke_bytes": ke, "streamed_gbs": (ke + vec) / (ms * 1e-3) / 1e9}
    A.set_symmetric_inner(1)
    return out


def run_ours(args, w, rank, world, local_rank):
    import torch
    dev = local_rank
    torch.cuda.set_device(dev)
    prec = PREC_NAMES[args.precision]
    keep = args.cpu_sample_elems > 0 and rank == 0
    if keep:
        m, dmap, A, ke_host = build_problem(w, prec, dev, keep_ke=True)
    else:
        (m, dmap, A), ke_host = build_problem(w, prec, dev), None
    A.set_fused_colours(bool(args.fused))
    n = m.n_dofs
    info, ms, u_host, v, clk = measure_device(A, n, args.steps, args.warmup, world, dev, rank, True)
    ms_step = ms / args.steps
    alg = info["algorithmic_bytes"]
    value = alg * world * args.steps / (ms * 1e-3) / 1e9
    f32 = info["precision"] == 2
    e2e = None
    if not f32:
        e2e_s = measure_e2e(A, u_host, v, args.steps, world)
        e2e = {"value": alg * world * args.steps / e2e_s / 1e9, "unit": "GB/s", "h2d_bytes_per_step": 8 * n,
               "d2h_bytes_per_step": 8 * n}
    inner = measure_inner_f32(A, m, args.steps, args.warmup) if info["precision"] == 1 else None
    native = None
    if args.also_native and info["precision"] == 1:
        # the same workload in native FP64 arithmetic, for comparison
        A.close()
        from amat_gb300 import Maps, aMatFree
        m2, dmap2, A2 = build_problem(w, 0, dev)
        info2, ms2, _, _, _ = measure_device(A2, n, args.steps, args.warmup, world, dev, rank, False)
        a2 = info2["algorithmic_bytes"] / (ms2 / args.steps * 1e-3) / 1e9
        native = {"value": a2 * world, "ms_per_step": ms2 / args.steps, "dtype": "f64 (native FMA)",
                  "bound": "fp64 FMA (1.008 TFLOP/s measured)"}
        A2.close()
    if rank != 0:
        return None
    peak, peak_kind = measured_peak()
    achieved = alg / (ms_step * 1e-3) / 1e9
    key = "%s_%s" % (args.workload, PREC_KEYS[info["precision"]])
    out = {
        "metric": "AFM matvec GB/s", "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": PREC_DTYPE[info["precision"]], "data": "synthetic",
        "config": {"workload": w["desc"], "n_elements": m.n_elem, "n_dofs": n, "colors": info["n_colors"],
                   "precision": PREC_KEYS[info["precision"]], "parallelism": "replicas x%d" % world,
                   "l2": l2_note(info)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": ncu_traffic(key), "peak_kind": peak_kind,
                     "kernel": ("afm_patch_kernel, one launch per patch colour + v zero fill (%d launches/step)"
                                if info["n_patches"] else
                                "afm_wpg_kernel, one launch per colour + v zero fill (%d launches/step)")
                               % info["n_launches"],
                     "algorithmic_bytes_per_step": alg},
        "e2e": e2e,
        "gpu_launches": (info["n_launches"] - 1) * args.steps,
    }
    if native:
        out["fp64_native"] = native
    if inner:
        out["fp32_inner_products"] = inner
    clk_sum = clk.summary() if clk else None
    if clk_sum:
        out["clocks"] = clk_sum
    if args.cpu_sample_elems > 0:
        pr, uc, vc, ne, sbytes = cpu_sample(w, m, dmap, args.cpu_sample_elems)
        ts, threads = time_cpu(pr, uc, vc, 5, args.cpu_seconds)
        out["cpu_baseline"] = {"value": sbytes * len(ts) / sum(ts) / 1e9, "unit": "GB/s", "cores": threads,
                               "kind": "port",
                               "sample": "%d of %d elements, %d matvecs (%.1f s), oracle port of matvec_ghosted_OMP"
                                         % (ne, m.n_elem, len(ts), sum(ts))}
        # the same CPU loop once over the whole mesh, as the checker of the timed device product (outside every
        # timed region): norm-wise relative difference of the last timed v from the reference loop's v
        err = full_parity(m, dmap, ke_host, u_host, v.cpu().numpy())
        out["parity_rel_err"] = err
        out["cpu_baseline"]["parity"] = {"rel_err": err, "tolerance": 1e-12, "elements": m.n_elem,
                                         "against": "oracle port of matvec_ghosted_OMP, whole mesh"}
    del ke_host
    if args.with_solves and world == 1:
        A.close()
        out["solves"] = default_solves(args, dev)
    return out


def run_assembled(args, w, rank, world, local_rank):
    """The aMatBased baseline: the same operator assembled into CSR (element-order sums, as the reference's
    PETSc assembly) and multiplied by the hand-written CSR SpMV, against the assembly-free product."""
    import torch
    dev = local_rank
    torch.cuda.set_device(dev)
    prec = PREC_NAMES[args.precision]
    m, dmap, A = build_problem(w, prec, dev)
    t0 = time.time()
    A.assemble(apply_bc=False)
    t_asm = time.time() - t0
    info = A.info()
    n, nnz = m.n_dofs, info["csr_nnz"]
    stream_ptr = A.stream()
    stream = torch.cuda.ExternalStream(stream_ptr)
    du = torch.tensor(np.random.default_rng(3).uniform(-1, 1, n), device="cuda")
    va, vf = torch.empty_like(du), torch.empty_like(du)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    ms_csr = timed(lambda: A.matvec_assembled_device(va.data_ptr(), du.data_ptr(), stream_ptr))
    ms_afm = timed(lambda: A.matvec_device(vf.data_ptr(), du.data_ptr(), stream_ptr))
    diff = float(torch.linalg.norm(va - vf) / torch.linalg.norm(vf))
    csr_bytes = nnz * 12 + 8 * (n + 1) + 16 * n
    peak, peak_kind = measured_peak()
    gbs = csr_bytes / (ms_csr * 1e-3) / 1e9
    return {"metric": "assembled (CSR) matvec GB/s", "value": gbs, "unit": "GB/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_csr, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": w["desc"], "n_dofs": n, "n_elements": m.n_elem, "csr_nnz": nnz,
                       "csr_bytes": csr_bytes, "host_assembly_s": t_asm},
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                         "peak_kind": peak_kind, "kernel": "k_csr_spmv (%d threads per row)" % (
                             4 if nnz / n <= 32 else 8 if nnz / n <= 64 else 16 if nnz / n <= 128 else 32)},
            "afm": {"ms": ms_afm, "algorithmic_bytes": info["algorithmic_bytes"],
                    "precision": PREC_KEYS[info["precision"]]},
            "afm_speedup_vs_assembled": ms_csr / ms_afm, "rel_diff_vs_afm": diff} if rank == 0 else None


def run_free(args, w, rank, world, local_rank):
    """Method 2 (MATFREE_TYPE::FREE): element stiffness integrated on the device from node coordinates every
    product, FP64 and FP32, against the stored-Ke products (FP64-split, and the FP32 symmetric copy the inner CG
    uses) of the same operator; then the mixed-precision solve on each."""
    import torch
    from amat_gb300 import MATFREE_TYPE, Maps, aMatFree
    from amat_gb300 import problems as P
    dev = local_rank
    torch.cuda.set_device(dev)
    m, dmap, S = build_problem(w, PREC_NAMES["fp64_split"], dev)
    xe = m.coords[m.elem_nodes]
    maps = Maps()
    maps.set_map(m.n_elem, dmap, m.ndpe, m.n_dofs)
    F = aMatFree(maps, 0, dev)
    F.set_matfree_type(MATFREE_TYPE.FREE)
    F.set_element_kind(w["kind"], E=1.0, nu=0.3, ngt=w["ngt"])
    F.set_element_coords(0, xe)
    t0 = time.time()
    F.finalize()
    t_fin = time.time() - t0
    n = m.n_dofs
    u = np.random.default_rng(5).uniform(-1, 1, n)
    d64 = torch.tensor(u, device="cuda")
    d32 = d64.float()
    o64, o32 = torch.empty_like(d64), torch.empty_like(d32)

    def timed(A, fn):
        st = torch.cuda.ExternalStream(A.stream())
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(args.steps):
            fn()
        e1.record(st)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    fs = F.stream()
    ss = S.stream()
    ms_f64 = timed(F, lambda: F.matvec_device(o64.data_ptr(), d64.data_ptr(), fs))
    ref64 = o64.clone()
    ms_f32 = timed(F, lambda: F.matvec_device_f32(o32.data_ptr(), d32.data_ptr(), fs))
    ms_s64 = timed(S, lambda: S.matvec_device(o64.data_ptr(), d64.data_ptr(), ss))
    diff = float(torch.linalg.norm(o64 - ref64) / torch.linalg.norm(o64))
    S.set_symmetric_inner(1)
    ms_s32 = timed(S, lambda: S.matvec_device_f32(o32.data_ptr(), d32.data_ptr(), ss))
    info = S.info()
    nn = m.elem_nodes.shape[1]
    # FP32 bytes the matrix-free product moves per element: coordinates, map, u and v entries
    free_bytes = m.n_elem * (nn * 3 * 4 + m.ndpe * 4) + 8 * n
    return {"metric": "matrix-free (method 2) FP32 product ms", "value": ms_f32, "unit": "ms", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_f32, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": w["desc"], "n_dofs": n, "n_elements": m.n_elem, "free_finalize_s": t_fin},
            "free": {"fp64_ms": ms_f64, "fp32_ms": ms_f32, "fp32_bytes_per_product": free_bytes,
                     "rel_diff_fp64_vs_stored": diff, "device_ke_bytes": F.info()["ke_bytes"]},
            "stored": {"fp64_split_ms": ms_s64, "fp32_symmetric_copy_ms": ms_s32, "ke_bytes": info["ke_bytes"],
                       "symmetric_copy_bytes": info["sym_bytes"]},
            "fp32_speedup_vs_stored_fp32": ms_s32 / ms_f32, "fp64_speedup_vs_stored_fp64": ms_s64 / ms_f64} \
        if rank == 0 else None


def build_bc_problem(w, dev):
    """Operator with the workload's boundary conditions (FP64_SPLIT arena: FP64 residual + FP32 view)."""
    from amat_gb300 import Maps, aMatFree
    from amat_gb300 import problems as P
    t0 = time.time()
    m = P.Mesh(w["kind"], w["n"], jitter=w["jitter"], seed=w["seed"])
    dofs, vals = m.boundary_conditions()
    maps = Maps()
    maps.set_map(m.n_elem, m.dof_map(), m.ndpe, m.n_dofs)
    maps.set_bdr_map(dofs, vals)
    A = aMatFree(maps, 0, dev)
    A.set_precision(PREC_NAMES["fp64_split"])
    buf = np.empty((CHUNK, m.ndpe, m.ndpe))
    for e0 in range(0, m.n_elem, CHUNK):
        c = min(CHUNK, m.n_elem - e0)
        m.element_matrices(e0, c, ngt=w["ngt"], out=buf[:c])
        A.set_element_matrices(e0, buf[:c])
    A.finalize()
    log("solve setup %.1fs, %d DoF, %d constrained" % (time.time() - t0, m.n_dofs, len(dofs)))
    return m, dofs, vals, A


def solve_compare(A, m, rhs, rtol, steps, inner_rtol, M=None, nvtx=None):
    """FP64 Jacobi-PCG on A against the mixed-precision solve on M (default A) for the same system: one
    short warm-up of each (graph capture), then `steps` timed solves of each (device time per solve)."""
    M = A if M is None else M
    A.solve(rhs, rtol=rtol, atol=0.0, maxit=8, raise_on_fail=False)
    M.solve_mixed(rhs, rtol=rtol, atol=0.0, inner_rtol=inner_rtol, max_outer=1, max_inner=8, raise_on_fail=False)
    t64, tmx = [], []
    for _ in range(steps):
        if nvtx:
            nvtx.range_push("fp64_solve")  # ranges for profiler filters (ncu --nvtx-include)
        x64, st = A.solve(rhs, rtol=rtol, atol=0.0, maxit=200000)
        if nvtx:
            nvtx.range_pop()
            nvtx.range_push("mixed_solve")
        xm, stm = M.solve_mixed(rhs, rtol=rtol, atol=0.0, inner_rtol=inner_rtol, raise_on_fail=False)
        if nvtx:
            nvtx.range_pop()
        if stm.status != 0:
            raise SystemExit("mixed-precision solve did not converge (status %d)" % stm.status)
        t64.append(st.seconds)
        tmx.append(stm.seconds)
    s64, smx = steps / sum(t64), steps / sum(tmx)
    log("fp64 CG: %d iterations, %.3f s; mixed: %d refinements, %d inner iterations, %.3f s" % (
        st.iterations, t64[-1], stm.refinements, stm.iterations, tmx[-1]))
    out = {"mixed": {"solves_per_s": smx, "inner_iterations": stm.iterations, "refinements": stm.refinements,
                     "rel_residual": stm.rel_residual,
                     "rel_error_vs_fp64_solution": float(np.linalg.norm(xm - x64) / np.linalg.norm(x64))},
           "fp64": {"solves_per_s": s64, "iterations": st.iterations, "rel_residual": st.rel_residual,
                    "dtype": "f64 (split arena)"},
           "speedup_vs_fp64": smx / s64, "rtol": rtol, "inner_rtol": inner_rtol, "steps": steps}
    return out, xm, x64


def poisson_analytic_error(m, x):
    """max |x - u| / max |u| against example03a's u = sin(2 pi x) sin(2 pi y) sin(2 pi z) / (12 pi^2)."""
    c = m.coords
    exact = np.sin(2 * np.pi * c[:, 0]) * np.sin(2 * np.pi * c[:, 1]) * np.sin(2 * np.pi * c[:, 2]) / (12 * np.pi ** 2)
    return float(np.abs(x - exact).max() / np.abs(exact).max())


def default_solves(args, dev):
    """The solve half of the metric beside the default matvec line: config 3 (tet10 Poisson 96^3 x 6, mixed
    precision against FP64 CG to 1e-8) and config 2 (hex20 elasticity 64^3, CG to 1e-10)."""
    out = {}
    w3 = WORKLOADS["tet10_poisson_96"]
    m, dofs, vals, A = build_bc_problem(w3, dev)
    rhs = A.apply_bc(m.load(ngt=w3["ngt"]))
    r3, xm, _ = solve_compare(A, m, rhs, 1e-8, args.solve_steps, 0.1)
    r3["workload"] = w3["desc"]
    r3["n_dofs"] = m.n_dofs
    r3["mixed"]["analytic_rel_error_max"] = poisson_analytic_error(m, xm)
    out["config3_mixed_vs_fp64"] = r3
    A.close()
    w2 = WORKLOADS["hex20_elastic_64"]
    m, dofs, vals, A = build_bc_problem(w2, dev)
    rhs = A.apply_bc(m.load(ngt=w2["ngt"]))
    # the mixed solve of this ill-conditioned system iterates in FP64 vectors (symmetric inner format 4): its
    # FP32 recursion stalls
    A.set_symmetric_inner(4)
    r2, _, _ = solve_compare(A, m, rhs, 1e-10, 1, 0.3)
    r2["mixed"]["inner_format"] = 4
    r2["workload"] = w2["desc"] + ", elastic bar: body load and end traction, clamped end"
    r2["n_dofs"] = m.n_dofs
    out["config2_cg_1e-10"] = r2
    A.close()
    return out


def run_solve(args, w, rank, world, local_rank):
    """CG solves/s: FP64 Jacobi-PCG and mixed-precision refinement on the same system."""
    import torch
    from amat_gb300 import problems as P
    dev = local_rank
    torch.cuda.set_device(dev)
    m, dofs, vals, A = build_bc_problem(w, dev)
    if args.load == "random":  # N(0,1) per DoF, the prescribed values on constrained DoFs (the serving mix)
        rhs = np.random.default_rng(w["seed"]).normal(size=m.n_dofs)
        rhs[dofs.astype(np.int64)] = vals
    else:
        rhs = A.apply_bc(m.load(ngt=w["ngt"]))
    rtol = args.rtol
    A.set_symmetric_inner(args.sym_format)
    M = A
    if args.free:
        # the mixed solve on the matrix-free operator (method 2): no element matrix on the device
        from amat_gb300 import MATFREE_TYPE, Maps, aMatFree
        maps = Maps()
        maps.set_map(m.n_elem, m.dof_map(), m.ndpe, m.n_dofs)
        maps.set_bdr_map(dofs, vals)
        M = aMatFree(maps, 0, dev)
        M.set_matfree_type(MATFREE_TYPE.FREE)
        M.set_element_kind(w["kind"], E=1.0, nu=0.3, ngt=w["ngt"])
        M.set_element_coords(0, m.coords[m.elem_nodes])
        M.finalize()
    r, xm, _ = solve_compare(A, m, rhs, rtol, args.steps, args.inner_rtol, M, torch.cuda.nvtx)
    smx = r["mixed"]["solves_per_s"]
    # inner iterations so far and ||b - A x|| / ||b|| at each FP64 residual of the last mixed solve
    r["mixed"]["trace"] = [[i, float("%.3e" % v)] for i, v in M.solve_trace()]
    r["mixed"]["inner_ke_bytes"] = 0 if args.free else A.info()["sym_bytes"] or A.info()["ke_bytes"] // 2
    r["mixed"]["inner_arena"] = ("matrix-free (method 2): Ke integrated from coordinates" if args.free else
                                 {0: "hi plane", 1: "symmetric copy, FP32",
                                  2: "symmetric copy, FP32 + BF16 correction",
                                  3: "symmetric copy, FP32 + BF16 correction; FP64 inner vectors",
                                  4: "symmetric copy, FP32 + BF16 correction; FP64 inner vectors, FP32 u",
                                  5: "symmetric copy, FP32 + BF16 correction; FP64 inner vectors, FP32 u, "
                                     "FP32 row sums"}[
                                     A.info()["sym_available"]])
    out = {"metric": "CG solves/s at %g rel. residual" % rtol, "value": smx, "unit": "solves/s", "n_gpus": world,
           "steps": args.steps, "warmup": 1, "ms_per_step": 1e3 / smx, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32 inner / f64 residual", "data": "synthetic",
           "config": {"workload": w["desc"], "n_dofs": m.n_dofs, "n_elements": m.n_elem, "rtol": rtol,
                      "inner_rtol": args.inner_rtol, "load": args.load},
           "mixed": r["mixed"], "fp64": r["fp64"], "speedup_vs_fp64": r["speedup_vs_fp64"]}
    if P.KIND_DPN[w["kind"]] == 1:
        out["analytic_rel_error_max"] = poisson_analytic_error(m, xm)
    return out if rank == 0 else None


def run_batched(args, w, rank, world, local_rank):
    """Block CG solves/s on nrhs load cases at once (FP32 inner batched CG under FP64 refinement),
    against single-vector FP64 Jacobi-PCG on the same operator."""
    import torch
    dev = local_rank
    torch.cuda.set_device(dev)
    m, dofs, vals, A = build_bc_problem(w, dev)
    n, R, rtol = m.n_dofs, args.nrhs, args.rtol
    # R load cases N(0,1) per DoF; the constrained DoFs carry the (zero) prescribed values
    B = np.random.default_rng(w["seed"]).standard_normal((n, R))
    assert not np.any(vals)
    B[dofs.astype(np.int64), :] = 0.0
    dB = torch.tensor(B, device="cuda")
    dX = torch.zeros_like(dB)
    torch.cuda.synchronize()

    def batched(mixed):
        dX.zero_()
        torch.cuda.synchronize()
        return A.solve_batched_device(dB.data_ptr(), dX.data_ptr(), R, rtol=rtol, atol=0.0, mixed=mixed,
                                      inner_rtol=args.inner_rtol, max_inner=args.segment, maxit=200000)

    # warm-up: autotuner, graph capture
    for _ in range(max(1, args.warmup - 2)):
        stm = batched(True)
    log("batched mixed: %d refinements, %d inner iterations, worst rel residual %.3e, %.3f s" % (
        stm.refinements, stm.iterations, stm.rel_residual, stm.seconds))
    tuning = {"fp32": A.batch_tuning(R, solve=True), "fp64": A.batch_tuning(R)}
    clk = ClockSampler(dev)
    with clk:
        tm = [batched(True).seconds for _ in range(args.steps)]
    smx = R * args.steps / sum(tm)
    Xm = dX.cpu().numpy()
    # single-vector FP64 CG on a few columns (the plain GPU path)
    cols = list(range(min(R, args.single_cols)))
    t64, x64 = [], {}
    A.solve(B[:, 0], rtol=rtol, atol=0.0, maxit=200000)  # graph capture
    for j in cols:
        x, st = A.solve(B[:, j], rtol=rtol, atol=0.0, maxit=200000)
        t64.append(st.seconds)
        x64[j] = x
    s64 = len(cols) / sum(t64)
    err = max(float(np.linalg.norm(Xm[:, j] - x64[j]) / np.linalg.norm(x64[j])) for j in cols)
    out = {"metric": "CG solves/s at %g rel. residual (%d load cases per solve)" % (rtol, R), "value": smx,
           "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1e3 * sum(tm) / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32 inner (batched) / f64 residual", "data": "synthetic",
           "config": {"workload": w["desc"], "n_dofs": n, "n_elements": m.n_elem, "nrhs": R, "rtol": rtol,
                      "inner_rtol": args.inner_rtol, "segment": args.segment,
                      "loads": "N(0,1) per DoF, seed %d" % w["seed"],
                      "tuning (tile columns, tile rows, ms)": tuning},
           "batched_mixed": {"solves_per_s": smx, "inner_iterations": stm.iterations,
                             "refinements": stm.refinements, "worst_rel_residual": stm.rel_residual,
                             "max_rel_diff_vs_fp64_single": err},
           "fp64_single": {"solves_per_s": s64, "iterations": st.iterations, "rel_residual": st.rel_residual,
                           "columns_timed": len(cols)},
           "speedup_vs_fp64_single": smx / s64}
    if args.batched_fp64:
        st64 = batched(False)
        out["batched_fp64"] = {"solves_per_s": R / st64.seconds, "iterations": st64.iterations,
                               "worst_rel_residual": st64.rel_residual}
    clk_sum = clk.summary()
    if clk_sum:
        out["clocks"] = clk_sum
    return out if rank == 0 else None


def run_product(args, w, rank, world, local_rank):
    """The batched product alone (V = K U on nrhs columns, the inner kernel of the batched solves): FP32 on the
    hi plane of the split arena and FP64 (double-float) on the whole arena; autotuned or pinned lane tile,
    CUDA-event time per product."""
    import torch
    dev = local_rank
    torch.cuda.set_device(dev)
    m, dofs, vals, A = build_bc_problem(w, dev)
    R = args.nrhs
    info = A.info()
    flops = info["algorithmic_flops"] * R
    stream_ptr = A.stream()
    stream = torch.cuda.ExternalStream(stream_ptr)
    out = {}
    for f32 in (True, False):
        key = "fp32" if f32 else "fp64_split"
        dt = torch.float32 if f32 else torch.float64
        U = torch.empty((m.n_dofs, R), dtype=dt, device="cuda").uniform_(-1, 1)
        V = torch.empty_like(U)
        if args.tile:  # pin the lane tile (columns, rows) instead of the autotuner's choice
            ct, rt = (int(x) for x in args.tile.split(","))
            if f32 or (ct, rt) != (0, 0):  # (0, 0), the tensor-core kernel, computes FP32 products only
                A.set_batch_tuning(R, ct, rt, f32=f32)
        torch.cuda.synchronize()
        for _ in range(max(args.warmup, 3)):  # the first call runs the autotuner
            A.matvec_batched_device(V.data_ptr(), U.data_ptr(), R, f32=f32, stream=stream_ptr)
        A.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            A.matvec_batched_device(V.data_ptr(), U.data_ptr(), R, f32=f32, stream=stream_ptr)
        e1.record(stream)
        torch.cuda.synchronize()
        A.synchronize()  # reports any device-side error of the timed products
        ms = e0.elapsed_time(e1) / args.steps
        ke_bytes = info["ke_bytes"] // 2 if f32 else info["ke_bytes"]
        vec_bytes = 3 * m.n_dofs * R * (4 if f32 else 8)
        out[key] = {"ms": ms, "tflops": flops / (ms * 1e-3) / 1e12,
                    "tile (columns, rows)": A.batch_tuning(R, f32=f32)[:2],
                    "streamed_gbs": (ke_bytes + vec_bytes) / (ms * 1e-3) / 1e9}
        log("batched product %s: %.3f ms, %.2f TFLOP/s" % (key, ms, out[key]["tflops"]))
    best = out["fp32"]
    res = {"metric": "batched AFM product TFLOP/s (%d right-hand sides)" % R, "value": best["tflops"],
           "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps, "warmup": max(args.warmup, 3),
           "ms_per_step": best["ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32 (hi plane of the split arena)", "data": "synthetic",
           "config": {"workload": w["desc"], "n_dofs": m.n_dofs, "n_elements": m.n_elem, "nrhs": R,
                      "flops_per_product": flops},
           "products": out}
    return res if rank == 0 else None


SERVE_KINDS = [(0, "hex8 Poisson"), (1, "hex8 elasticity"), (2, "hex20 elasticity")]


def serve_requests(args, seed):
    """Seeded request set: element type uniform over SERVE_KINDS, edge log-uniform in [8, edge_max],
    coordinates jittered 0.1 h, loads N(0,1) per DoF (prescribed values on constrained DoFs)."""
    from amat_gb300 import Maps, aMatFree
    from amat_gb300 import problems as P
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(args.requests):
        kind, name = SERVE_KINDS[int(rng.integers(len(SERVE_KINDS)))]
        edge = int(round(np.exp(rng.uniform(np.log(8), np.log(args.edge_max)))))
        if kind != 0:
            edge += edge % 2  # the elastic bar's constraints sit on centre nodes (even edge)
        m = P.Mesh(kind, edge, jitter=0.1, seed=seed * 1000 + i)
        ke = m.element_matrices(ngt=3 if kind == P.HEX20_ELASTIC else 2)
        dofs, vals = m.boundary_conditions()
        maps = Maps()
        maps.set_map(m.n_elem, m.dof_map(), m.ndpe, m.n_dofs)
        maps.set_bdr_map(dofs, vals)
        A = aMatFree(maps)
        A.set_element_matrices(0, ke)
        b = rng.normal(size=m.n_dofs)
        b[dofs.astype(np.int64)] = vals
        reqs.append(dict(A=A, b=b, kind=name, edge=edge, n_dofs=m.n_dofs, n_elem=m.n_elem))
    return reqs


def new_server(dev, args):
    from amat_gb300.serve import Server
    srv = Server(dev)
    srv.set_lane(int(args.lane_mb * 2 ** 20), 32)
    srv.set_inner_format(args.serve_format)
    srv.set_priorities(bool(args.serve_prio))
    return srv


def run_serve(args, w, rank, world, local_rank):
    """Served CG solves: Poisson arrivals at each rate, admission by HBM, mixed-precision solves to rtol,
    p50/p99 latency (arrival to result) beside solves/s; against the plain path (finalize + FP64 CG, one
    request after another) on the same requests."""
    import torch
    from amat_gb300.serve import Server
    dev = local_rank
    torch.cuda.set_device(dev)
    rates = [float(r) for r in args.rates.split(",")]
    seed = 4
    # plain FP64 GPU path, sequential
    reqs = serve_requests(args, seed)
    t0 = time.perf_counter()
    its, t_fin, t_dev = 0, 0.0, 0.0
    for r in reqs:
        tf = time.perf_counter()
        r["A"].finalize()
        t_fin += time.perf_counter() - tf
        x, st = r["A"].solve(r["b"], rtol=args.rtol, atol=0.0, maxit=1000000)
        its += st.iterations
        t_dev += st.seconds
        log("  plain: %s edge %d, %d DoF: %d FP64 iterations, %.2f s" % (r["kind"], r["edge"], r["n_dofs"],
                                                                       st.iterations, st.seconds))
        r["A"].close()
    t_plain = time.perf_counter() - t0
    plain = {"solves_per_s": len(reqs) / t_plain, "total_s": t_plain, "finalize_s": t_fin, "solve_device_s": t_dev,
             "fp64_iterations": its, "dtype": "f64 (split arena)"}
    log("plain: %d solves in %.2f s" % (len(reqs), t_plain))
    # the same requests one at a time through the server (mixed precision, no overlap)
    reqs = serve_requests(args, seed)
    srv = new_server(dev, args)
    t0 = time.perf_counter()
    for r in reqs:
        rid = srv.submit(r["A"], r["b"], rtol=args.rtol, inner_rtol=args.serve_inner)
        while (res := srv.take(rid)) is None:
            time.sleep(0.0002)
        _, st, tt = res
        log("  alone: %s edge %d, %d DoF: %.2f s (solve %.2f s), %d inner iterations, %d updates, status %d" % (
            r["kind"], r["edge"], r["n_dofs"], tt[3] - tt[0], st.seconds, st.iterations, st.refinements,
            st.status))
    t_alone = time.perf_counter() - t0
    srv.close()
    alone = {"solves_per_s": len(reqs) / t_alone, "total_s": t_alone}
    log("served one at a time: %d solves in %.2f s" % (len(reqs), t_alone))
    lines = []
    clk = ClockSampler(dev)
    with clk:
        for rate in rates:
            reqs = serve_requests(args, seed)
            arr = np.cumsum(np.random.default_rng(seed + int(rate)).exponential(1.0 / rate, len(reqs)))
            srv = new_server(dev, args)
            ids, lat, res, brk = {}, [], [], []
            k = 0
            t0 = time.monotonic()
            last = t0
            while len(lat) < len(reqs):
                now = time.monotonic() - t0
                while k < len(reqs) and arr[k] <= now:
                    ids[srv.submit(reqs[k]["A"], reqs[k]["b"], rtol=args.rtol, inner_rtol=args.serve_inner)] = k
                    k += 1
                got = 0
                for rid in list(ids):
                    out = srv.take(rid)
                    if out is None:
                        continue
                    got += 1
                    j = ids.pop(rid)
                    x, st, tt = out
                    lat.append(tt[3] - (t0 + arr[j]))
                    res.append(st.rel_residual)
                    brk.append((tt[1] - tt[0], tt[2] - tt[1], tt[3] - tt[2], st.seconds))
                    last = max(last, tt[3])
                if not got:  # the server's progress thread does the work; wait a little
                    nxt = arr[k] - (time.monotonic() - t0) if k < len(reqs) else 0.0005
                    time.sleep(max(0.0, min(nxt, 0.0005)))
            lane = srv.info()
            srv.close()
            span = last - (t0 + arr[0])
            lat = np.array(lat)
            brk = np.array(brk)
            lines.append({"rate_req_s": rate, "solves_per_s": len(reqs) / span, "p50_ms": 1e3 * np.percentile(lat, 50),
                          "p99_ms": 1e3 * np.percentile(lat, 99), "max_rel_residual": float(max(res)),
                          "median_ms": {"queued": 1e3 * float(np.median(brk[:, 0])),
                                        "finalize": 1e3 * float(np.median(brk[:, 1])),
                                        "solve_wall": 1e3 * float(np.median(brk[:, 2])),
                                        "solve_device": 1e3 * float(np.median(brk[:, 3]))},
                          "lane": lane})
            log("rate %g: %.2f solves/s, p50 %.1f ms, p99 %.1f ms" % (rate, lines[-1]["solves_per_s"],
                                                                     lines[-1]["p50_ms"], lines[-1]["p99_ms"]))
    best = max(lines, key=lambda d: d["solves_per_s"])
    sizes = [r["n_dofs"] for r in reqs]
    out = {"metric": "served CG solves/s at %g rel. residual (FP64-checked)" % args.rtol,
           "value": best["solves_per_s"], "unit": "solves/s", "n_gpus": world, "steps": len(rates),
           "warmup": 0, "ms_per_step": 1e3 / best["solves_per_s"], "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32 inner / f64 reliable updates", "data": "synthetic",
           "config": {"workload": "serving: Poisson arrivals, %d requests, types %s, edge log-uniform 8..%d, "
                                  "jitter 0.1h, loads N(0,1)" % (args.requests, [k[1] for k in SERVE_KINDS],
                                                                  args.edge_max),
                      "n_dofs_range": [int(min(sizes)), int(max(sizes))], "rtol": args.rtol,
                      "inner_rtol": args.serve_inner, "admission": "lane-sized first, then arrival order, by HBM budget (85% of free), 64 slots",
                      "lane_mb": args.lane_mb, "inner_format": args.serve_format, "priorities": args.serve_prio},
           "rates": lines, "p50_ms": best["p50_ms"], "p99_ms": best["p99_ms"], "plain_fp64_sequential": plain,
           "served_one_at_a_time": alone,
           "speedup_vs_plain": best["solves_per_s"] / plain["solves_per_s"]}
    cs = clk.summary()
    if cs:
        out["clocks"] = cs
    return out if rank == 0 else None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="hex20_elastic_64", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="auto", choices=sorted(PREC_NAMES))
    ap.add_argument("--also-native", type=int, default=1, help="also time native FP64 when the split path runs")
    ap.add_argument("--cpu-sample-elems", type=int, default=65536)
    ap.add_argument("--fused", type=int, default=0, choices=[0, 1],
                    help="every colour of a split product in one cooperative launch (slower; off by default)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="CPU time the baseline sample is timed for")
    ap.add_argument("--mode", default="matvec", choices=["matvec", "solve", "batched", "product", "serve",
                                                         "assembled", "free"])
    ap.add_argument("--rates", default="10,20,50,100,200,500", help="serve: arrival rates (requests/s)")
    ap.add_argument("--requests", type=int, default=48, help="serve: requests per rate")
    ap.add_argument("--edge-max", type=int, default=96, help="serve: largest mesh edge")
    ap.add_argument("--serve-inner", type=float, default=0.3, help="serve: FP32 reduction between FP64 updates")
    ap.add_argument("--serve-format", type=int, default=4, choices=[0, 1, 2, 3, 4, 5],
                    help="serve: symmetric inner format of the requests on their own streams")
    ap.add_argument("--serve-prio", type=int, default=1, choices=[0, 1],
                    help="serve: stream priorities by request size")
    ap.add_argument("--lane-mb", type=float, default=8.0,
                    help="serve: requests with at most this many MB of FP32 element matrices share lane launches")
    ap.add_argument("--nrhs", type=int, default=64)
    ap.add_argument("--single-cols", type=int, default=2, help="columns solved one by one for the FP64 comparison")
    ap.add_argument("--batched-fp64", type=int, default=0, help="also time the FP64 batched block CG")
    ap.add_argument("--segment", type=int, default=64, help="FP32 iterations between FP64 updates (batched)")
    ap.add_argument("--tile", default="", help="product: pin the batched lane tile 'columns,rows'")
    ap.add_argument("--rtol", type=float, default=1e-8)
    ap.add_argument("--free", type=int, default=0, help="solve: mixed solve on the matrix-free operator (method 2)")
    ap.add_argument("--inner-rtol", type=float, default=1e-2)
    ap.add_argument("--sym-format", type=int, default=1, choices=[0, 1, 2, 3, 4, 5],
                    help="solve: inner arena (1 symmetric FP32, 2 with BF16 correction, 0 hi plane; 3 the arena "
                         "of 2 with FP64 inner vectors)")
    ap.add_argument("--load", default="example", choices=["example", "random"],
                    help="solve: the example's load, or N(0,1) per DoF as in the serving mix")
    ap.add_argument("--with-solves", type=int, default=1,
                    help="matvec: also record the config-3 mixed/FP64 solves and the config-2 CG to 1e-10")
    ap.add_argument("--solve-steps", type=int, default=3, help="timed solves of each kind in --with-solves")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    w = WORKLOADS[args.workload]
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        out = run_reference(args, w, rank)
    else:
        if world > 1:
            import torch
            torch.cuda.set_device(local_rank)
            torch.distributed.init_process_group("nccl")
        run = {"matvec": run_ours, "solve": run_solve, "batched": run_batched, "product": run_product,
               "assembled": run_assembled, "free": run_free,
               "serve": run_serve}[args.mode]
        out = run(args, w, rank, world, local_rank)
        if world > 1:
            import torch
            torch.distributed.destroy_process_group()
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
