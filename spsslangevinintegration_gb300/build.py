"""Build libspss_gpu.so (sm_103a) in-tree with nvcc.

``python -m spsslangevinintegration_gb300.build`` or ``build_library()``.
Translation units compile in parallel; the FP64 reference-arithmetic unit is
compiled with ``--fmad=false`` so its expressions round as the reference's
``-ffp-contract=off`` build does.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libspss_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                 "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")]
PER_FILE = {"f64_path.cu": ["--fmad=false"]}
SOURCES = ["common.cu", "f64_path.cu", "fast_path.cu", "spss_gpu.cu", "surrogate.cu", "dopri5.cu"]


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _needs(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(verbose=False, force=False, ptxas_verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "spss_gpu.h"))
    jobs = []
    objs = []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(obj)
        if force or _needs(obj, [path] + headers):
            cmd = [nvcc()] + COMMON + PER_FILE.get(src, []) + (["-Xptxas", "-v"] if ptxas_verbose else [])
            cmd += ["-c", path, "-o", obj]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            for cmd, r in ex.map(run, jobs):
                if verbose or r.returncode != 0 or ptxas_verbose:
                    sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
                if r.returncode != 0:
                    raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if force or jobs or _needs(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    build_library(verbose=True, force="--force" in sys.argv, ptxas_verbose="-v" in sys.argv)
    print(LIB)
