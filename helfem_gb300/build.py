"""Build libhelfem_gb300.so in-tree with nvcc for sm_103a (no cmake).

    python helfem_gb300/build.py          # incremental
    python helfem_gb300/build.py --force  # rebuild everything

(run as a script: importing the package itself requires the built library)

Translation units are compiled in parallel; the CUDA runtime is linked
statically, cuSOLVER/cuBLAS dynamically. Host code is portable C++17 (no
x86 intrinsics) so the same recipe builds on x86_64 and aarch64.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libhelfem_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources():
    out = []
    for d, _, files in os.walk(CSRC):
        for f in sorted(files):
            if f.endswith((".cu", ".cpp")):
                out.append(os.path.join(d, f))
    return sorted(out)


def headers():
    hs = [os.path.join(ROOT, "include", "helfem_gb300.h")]
    for d, _, files in os.walk(CSRC):
        hs += [os.path.join(d, f) for f in files if f.endswith((".hpp", ".cuh", ".h"))]
    return hs


def _obj_for(src):
    rel = os.path.relpath(src, CSRC).replace(os.sep, "_")
    return os.path.join(OBJ, rel + ".o")


def _compile(src, force, hdr_mtime):
    obj = _obj_for(src)
    if not force and os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), hdr_mtime):
        return obj, None
    cmd = [nvcc(), "-c", src, "-o", obj + ".tmp", "-O3", "-std=c++17", "-lineinfo",
           "-Xcompiler", "-fPIC,-fopenmp,-O3", "-I", os.path.join(ROOT, "include"), "-I", CSRC]
    if src.endswith(".cu"):
        cmd += ARCH + (["-Xptxas", "-v"] if os.environ.get("HFG_PTXAS_VERBOSE") else [])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    os.replace(obj + ".tmp", obj)
    return obj, r.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    srcs = sources()
    hdr_mtime = max(os.path.getmtime(h) for h in headers())
    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        res = list(ex.map(lambda s: _compile(s, force, hdr_mtime), srcs))
    objs = [o for o, _ in res]
    if verbose:
        for o, log in res:
            if log:
                print(log, file=sys.stderr)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = [nvcc(), "-shared", "-o", tmp] + objs + ARCH + [
            "-Xcompiler", "-fopenmp", "-lgomp", "-lcusolver", "-lcublas"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
