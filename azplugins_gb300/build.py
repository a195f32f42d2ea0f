"""Build recipe of the native library ``libazplugins_gb300.so`` (sm_103a only).

Each ``csrc/*.cu`` is compiled by nvcc in parallel, then linked into one shared
library next to this file (in-tree, git-ignored). No CMake, no torch extension
machinery: the library is a plain C ABI loaded with ctypes.
"""

from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libazplugins_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    path = shutil.which("nvcc")
    if path:
        return path
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build azplugins_gb300")


def common_flags(debug: bool = False):
    f = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
         "--expt-relaxed-constexpr", "-I", os.path.join(HERE, "..", "include")] + ARCH
    if debug:
        f += ["-DAZP_DEBUG"]
    return f


def _compile(src: str, obj: str, flags) -> str:
    cmd = [nvcc(), "-c", src, "-o", obj] + flags
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    return r.stderr


def build(verbose: bool = False, ptxas_info: bool = False, jobs: int | None = None) -> str:
    """Compile and link; returns the library path. Rebuilds only stale objects."""
    os.makedirs(BUILD, exist_ok=True)
    flags = common_flags()
    if ptxas_info:
        flags = flags + ["-Xptxas", "-v"]
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(HERE, "..", "include", "*.h"))
    newest_header = max((os.path.getmtime(h) for h in headers), default=0.0)
    todo = []
    objs = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if ptxas_info or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), newest_header):
            todo.append((s, o))
    if todo:
        n = jobs or min(len(todo), os.cpu_count() or 4)
        with cf.ThreadPoolExecutor(max_workers=n) as ex:
            futs = {ex.submit(_compile, s, o, flags): s for s, o in todo}
            for fu in cf.as_completed(futs):
                log = fu.result()
                if verbose and log:
                    print(f"--- {os.path.basename(futs[fu])}\n{log}", file=sys.stderr)
    if todo or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        cmd = [nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-Xcompiler", "-fPIC"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="-v" in sys.argv)
    print(LIB)
