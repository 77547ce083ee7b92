"""The C++ adapter (include/mpsboost_cuda/cuda_backend.hpp) is a drop-in for the
reference's backend contract: it compiles against the reference's own headers, links with
the reference's training core and, where no GPU is present, fails loudly with the
reference's BackendError instead of computing anything on the CPU."""

from __future__ import annotations

import os
import subprocess

import pytest

import oracle
from mpsboost_gb300 import build as cuda_build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = oracle.REFERENCE_ROOT


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src", "core")), reason="reference sources absent")
def test_adapter_builds_against_reference_core(tmp_path):
    lib = cuda_build.build()
    sources = [os.path.join(REF, "src", "core", f) for f in sorted(os.listdir(os.path.join(REF, "src", "core")))
               if f.endswith(".cpp")]
    sources.append(os.path.join(REF, "src", "cpu", "reference_backend.cpp"))
    exe = tmp_path / "dropin"
    cmd = ["g++", "-std=c++17", "-O1", "-w", f"-I{REF}/include", f"-I{REF}/src/core", f"-I{ROOT}/include",
           os.path.join(ROOT, "tests", "dropin", "dropin_main.cpp"), *sources, lib,
           f"-Wl,-rpath,{os.path.dirname(lib)}", "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except ImportError:
        has_gpu = False
    if has_gpu:
        assert "trained 5 trees" in out.stdout
    else:
        assert "BackendError" in out.stdout
