"""Build the sm_103a CUDA backend library in-tree: ``mpsboost_gb300/_build/libmpsb_cuda.so``.

One ``nvcc`` per translation unit, run in parallel, then one shared link. Host code is
compiled with floating-point contraction disabled so FP64 host arithmetic rounds like
the reference C++.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libmpsb_cuda.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["hist.cu", "kernels.cu", "host.cu", "node_entries.cu", "noalloc.cu", "binning.cu",
           "quantize.cpp", "model_io.cu"]


def _nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found; the CUDA backend needs the CUDA 13 toolkit")
    return path


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    lib_time = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "mpsb_cuda.h"))
    deps.append(__file__)
    return any(os.path.getmtime(d) > lib_time for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> str:
    """Compile every translation unit for sm_103a and link the shared library."""

    if not force and not _stale():
        return LIB
    nvcc = _nvcc()
    obj_dir = os.path.join(BUILD, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    common = [
        "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-Wall",
        f"-I{os.path.join(HERE, '..', 'include')}",
    ] + list(extra_flags or [])
    procs = []
    objs = []
    for src in SOURCES:
        obj = os.path.join(obj_dir, src + ".o")
        objs.append(obj)
        cmd = [nvcc] + ARCH + common + ["-c", os.path.join(CSRC, src), "-o", obj]
        if src.endswith(".cpp"):
            cmd = [nvcc] + common + ["-x", "c++", "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((src, out.decode(errors="replace")))
        elif verbose and out:
            print(out.decode(errors="replace"), file=sys.stderr)
    if failed:
        raise RuntimeError("\n".join(f"--- {s} ---\n{o}" for s, o in failed))
    tmp = LIB + ".tmp"
    link = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"]
    subprocess.run(link, check=True, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
