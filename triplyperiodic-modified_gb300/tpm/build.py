"""Build libtpm.so in-tree with nvcc for sm_103a (GB300).

The translation units are compiled in parallel and linked into
``triplyperiodic-modified_gb300/lib/libtpm.so``.  The FP64 kernels are built
with ``--fmad=false`` so that a*b+c is never contracted: the field algebra
then rounds exactly like the reference's unfused double-precision C++.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libtpm.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["tpm_ctx.cu", "tpm_fields.cu", "tpm_fft.cu", "tpm_particles.cu", "tpm_diag.cu", "tpm_graph.cu", "tpm_pcg.cu", "tpm_adjoint.cu", "tpm_io.cpp"]
# per-source extra flags
EXTRA = {}


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags():
    return ARCH + ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-I", os.path.join(REPO, "include"), "-I", CSRC]


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(os.path.join(LIBDIR, "obj"), exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    deps = srcs + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith(".cuh")]
    deps.append(os.path.join(REPO, "include", "tpm.h"))
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) > max(os.path.getmtime(d) for d in deps)):
        return LIB
    cc = nvcc()
    objs = []

    def compile_one(src):
        obj = os.path.join(LIBDIR, "obj", os.path.basename(src) + ".o")
        cmd = [cc] + _flags() + EXTRA.get(os.path.basename(src), []) + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
