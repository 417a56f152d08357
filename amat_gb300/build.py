"""Builds the native libraries in-tree.

  amat_gb300/libafm.so          the C ABI of include/afm.h (host runtime + sm_103a kernels)
  amat_gb300/libafm_problems.so the example problem generators of include/afm_problems.h
  oracle/_build/liboracle.so    the CPU oracle (test infrastructure)

Translation units compile in parallel; only `-gencode arch=compute_103a,code=sm_103a`.
Nothing is rebuilt when its outputs are newer than every source.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libafm.so")
PROBLEMS_LIB = os.path.join(HERE, "libafm_problems.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "_build", "liboracle.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fopenmp", "--expt-relaxed-constexpr"] + ARCH
CU_SOURCES = ["afm_mv_fp64.cu", "afm_mv_split.cu", "afm_mv_fp32.cu", "afm_mv_f32sym.cu", "afm_mv_f32symx.cu", "afm_mv_splitsymx.cu", "afm_mv_f32symc.cu",
              "afm_solver.cu",
              "afm_batched_solver.cu", "afm_batched_tc.cu", "afm_lane.cu", "afm_noalloc.cu", "afm_spmv.cu", "afm_free.cu", "afm_capi.cpp", "afm_server.cpp",
              "afm_assembled.cpp"]
HEADERS = ["afm_internal.hpp", "afm_matvec.cuh", "afm_batched.cuh", "afm_patch.cuh", "afm_mv_launch.inl",
           "afm_solver.hpp", "afm_batched_solver.hpp", "afm_mixed.hpp", "afm_shape.hpp"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _newer(out, srcs):
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(s) <= t for s in srcs)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build_afm(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    deps = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "afm.h")]
    objs, jobs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if not _newer(o, [s] + deps):
            xflags = ["-x", "cu"] if src.endswith(".cu") else []
            extra = ["-Xptxas", "-v"] if verbose and src.endswith(".cu") else []
            jobs.append([nvcc] + NVCC_FLAGS + extra + inc + xflags + ["-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for t in outs:
            sys.stdout.write(t)
    if not _newer(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-Xcompiler", "-fopenmp", "-o", LIB] + objs + ["-lgomp"])
    return LIB


def build_problems():
    src = os.path.join(CSRC, "afm_problems.cpp")
    hdr = os.path.join(ROOT, "include", "afm_problems.h")
    if not os.path.exists(src):
        return None
    if not _newer(PROBLEMS_LIB, [src, hdr, os.path.join(CSRC, "afm_shape.hpp")]):
        cxx = shutil.which("g++") or "g++"
        _run([cxx, "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-I" + os.path.join(ROOT, "include"),
              src, "-o", PROBLEMS_LIB])
    return PROBLEMS_LIB


def build_oracle():
    src = os.path.join(ORACLE_DIR, "afm_oracle.c")
    if not _newer(ORACLE_LIB, [src]):
        os.makedirs(os.path.dirname(ORACLE_LIB), exist_ok=True)
        cc = shutil.which("gcc") or "cc"
        _run([cc, "-O3", "-std=c99", "-fPIC", "-shared", "-fopenmp", src, "-o", ORACLE_LIB, "-lm"])
    return ORACLE_LIB


def build_reference():
    """Compiles the reference CPU path in place (x86 container only)."""
    script = os.path.join(ORACLE_DIR, "build_ref.sh")
    out = os.path.join(ORACLE_DIR, "_ref", "libamat_ref.so")
    out_simd = os.path.join(ORACLE_DIR, "_ref", "libamat_ref_simd.so")
    ref = os.environ.get("AMAT_REFERENCE", os.path.join(os.path.dirname(ROOT), "reference"))
    if not os.path.isdir(os.path.join(ref, "include")):
        return None
    if os.path.exists(out) and os.path.exists(out_simd):
        return out
    subprocess.run(["sh", script], check=True, env=dict(os.environ, REF=ref))
    return out if os.path.exists(out) else None


def build_all(verbose=False):
    with ThreadPoolExecutor(max_workers=3) as ex:
        f1 = ex.submit(build_afm, verbose)
        f2 = ex.submit(build_problems)
        f3 = ex.submit(build_oracle)
        res = [f1.result(), f2.result(), f3.result()]
    return res


if __name__ == "__main__":
    print(build_all(verbose="-v" in sys.argv))
