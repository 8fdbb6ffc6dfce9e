"""Build libnls_gb300.so (the sm_103a kernels and the C ABI) in-tree with nvcc.

    python -m nls_gb300.build            # or nls_gb300.build.build()

Translation units are compiled in parallel into nls_gb300/_build/ and linked into
nls_gb300/lib/libnls_gb300.so.  One -gencode (sm_103a), no cmake: a minute or less on either
the x86_64 development container or the aarch64 GPU host.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libnls_gb300.so")

SOURCES = ["k1d.cu", "k2d.cu", "kdiag.cu", "runtime.cu", "noalloc.cu", "host_ops.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden",
          "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libnls_gb300.so")


def _obj(src: str) -> str:
    return os.path.join(BUILD, os.path.splitext(src)[0] + ".o")


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(ROOT, "include", "nls_gb300.h"))
    return hs


def _compile(src: str, extra) -> str:
    path = os.path.join(CSRC, src)
    out = _obj(src)
    if not _stale(out, [path] + _headers()):
        return out
    cmd = [nvcc()] + ARCH + COMMON + list(extra) + ["-c", path, "-o", out]
    if src.endswith(".cpp"):
        cmd = [nvcc()] + COMMON + list(extra) + ["-x", "c++", "-c", path, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip():
        sys.stderr.write(r.stderr)
    return out


def build(verbose_ptxas: bool = False, force: bool = False) -> str:
    """Compile every translation unit (in parallel) and link libnls_gb300.so; returns its path.

    NLS_GB300_NVCC_FLAGS (whitespace-separated) adds compiler flags, e.g. a -D of a kernel tuning
    macro; a change of the flags forces a rebuild."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    flags = os.environ.get("NLS_GB300_NVCC_FLAGS", "").split()
    stamp = os.path.join(BUILD, "flags.txt")
    old = open(stamp).read() if os.path.exists(stamp) else ""
    if force or old != " ".join(flags):
        for s in SOURCES:
            if os.path.exists(_obj(s)):
                os.remove(_obj(s))
        with open(stamp, "w") as f:
            f.write(" ".join(flags))
    extra = (["-Xptxas", "-v"] if verbose_ptxas else []) + flags
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    if _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-fPIC"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose_ptxas="-v" in sys.argv, force="-f" in sys.argv))
