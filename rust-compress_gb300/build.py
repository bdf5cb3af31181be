"""Build librcg.so (the CUDA library behind include/rcg.h) in-tree for sm_103a.

Each translation unit is compiled by its own nvcc process in parallel, then linked with the static CUDA runtime.
codec.cu and exact.cu are compiled with -fmad=false: the encoder and decoder reproduce the reference's f32
arithmetic bit for bit, and the exact scorer its f64 arithmetic, so neither may contract a*b+c into an FMA. Host code gets -ffp-contract=off for the same reason (the host
computes the per-quality tables that the device also computes).

Usage: python rust-compress_gb300/build.py [--verbose] [--ptxas-info]
"""

import concurrent.futures
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librcg.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ARCH + [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "--expt-relaxed-constexpr",
    "-Xcompiler",
    "-fPIC,-ffp-contract=off,-O2",
]
UNITS = {
    "codec.cu": ["-fmad=false"],
    "exact.cu": ["-fmad=false"],
    "ssim2.cu": [],
    "capi.cu": [],
    "plan.cu": [],
    "metrics.cu": [],
    "jpegdec.cu": [],
    "adjoint.cu": [],
    "perceptual.cu": [],
}


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def compile_unit(name, extra, verbose, ptxas_info):
    src = os.path.join(CSRC, name)
    obj = os.path.join(BUILD, name + ".o")
    cmd = [nvcc()] + COMMON + extra + ["-c", src, "-o", obj]
    if ptxas_info:
        cmd += ["-Xptxas", "-v"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {name}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def needs_rebuild():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(HERE, "..", "include", "rcg.h"),
        os.path.abspath(__file__),
    ]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose=False, ptxas_info=False, force=False):
    if not force and not ptxas_info and not needs_rebuild():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        futs = [ex.submit(compile_unit, n, e, verbose, ptxas_info) for n, e in UNITS.items()]
        results = [f.result() for f in futs]
    if ptxas_info:
        for _, err in results:
            sys.stderr.write(err)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-ldl", "-lrt", "-lpthread"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(verbose="--verbose" in sys.argv, ptxas_info="--ptxas-info" in sys.argv, force=True)
    print(LIB)
