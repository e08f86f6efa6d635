"""Build the renderer's native library in-tree: fuzzy_ellipses/_lib/libfuzzy_ellipses.so.

Every CUDA translation unit under csrc/ is compiled for sm_103a only, in parallel, then linked
into one shared library with a plain C ABI (include/fuzzy_ellipses.h). Usage:

    python fuzzy-ellipses_gb300/build.py [--debug]
"""

from __future__ import annotations

import concurrent.futures
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "fuzzy_ellipses", "_lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIBNAME = "libfuzzy_ellipses.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include")]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _digest(paths, flags):
    h = hashlib.sha256()
    for p in paths:
        with open(p, "rb") as f:
            h.update(f.read())
    h.update(" ".join(flags).encode())
    return h.hexdigest()


def build(debug: bool = False, verbose: bool = False, extra_flags=()) -> str:
    """Compile (if sources changed) and return the path of the shared library."""
    os.makedirs(OBJDIR, exist_ok=True)
    srcs = sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "fuzzy_ellipses.h"))
    flags = ARCH + COMMON + list(extra_flags) + (["-DFE_DEBUG=1"] if debug else [])
    lib = os.path.join(LIBDIR, LIBNAME)
    stamp = os.path.join(LIBDIR, "build.stamp")
    digest = _digest(srcs + sorted(headers), flags)
    if os.path.exists(lib) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == digest:
                return lib
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
        cmd = [cc, *flags, "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr, flush=True)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = lib + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    with open(stamp, "w") as f:
        f.write(digest)
    return lib


if __name__ == "__main__":
    print(build(debug="--debug" in sys.argv, verbose="-v" in sys.argv))
