"""Builds the CUDA library libmdsc.so in-tree (mdspherocyl_gb300/_lib/).

Every translation unit is compiled for sm_103a only, in parallel, then
linked into one shared library with the C ABI of include/mdsc.h.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libmdsc.so")

SOURCES = ["k_real.cu", "k_kspace.cu", "k_int.cu", "k_wca.cu", "k_obs.cu", "k_render.cu", "k_init.cu", "api.cu",
           "gen.cpp", "noalloc.cu", "k_probe.cu"]
# files that repeat the reference's FP64 arithmetic operation by operation
NO_FMA = ("k_wca.cu", "k_init.cu")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
           "--expt-relaxed-constexpr", "-I", CSRC, "-I", INCLUDE]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmdsc")


def _digest() -> str:
    h = hashlib.sha256()
    for d in (CSRC, INCLUDE):
        for name in sorted(os.listdir(d)):
            with open(os.path.join(d, name), "rb") as f:
                h.update(name.encode())
                h.update(f.read())
    h.update(" ".join(ARCH + NVFLAGS).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> str:
    """Compile (if sources changed) and return the path of libmdsc.so."""
    os.makedirs(LIBDIR, exist_ok=True)
    stamp = os.path.join(LIBDIR, "build.stamp")
    dig = _digest()
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == dig:
                return LIB
    cc = nvcc()
    objdir = os.path.join(LIBDIR, "obj")
    os.makedirs(objdir, exist_ok=True)
    flags = NVFLAGS + (extra_flags or [])

    def one(src):
        obj = os.path.join(objdir, os.path.splitext(src)[0] + ".o")
        cmd = [cc] + ARCH + flags + ["-c", os.path.join(CSRC, src), "-o", obj]
        if src in NO_FMA:
            # the exact FP64 pair path keeps the reference's rounding: no FMA contraction
            cmd.insert(1, "-fmad=false")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(one, SOURCES))
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(dig)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
