"""The C++ drop-in adapter run on the GPU through the backend contract.

``include/mpsboost_cuda/cuda_backend.hpp`` derives from the reference's GradientComputer,
HistogramBuilder and LayerHistogramBuilder. The reference's sources are not present where
the GPU is, so ``tests/dropin/adapter_gpu_check.cpp`` is compiled against stand-in
declarations of that contract (``tests/dropin/stand_in``, same names and signatures) and
linked with the CUDA library: it checks the capability detection, the gradients, layer
and node histograms against FP64 sums, a dataset replacing the resident one, and the
contract's errors. Where the reference's sources are present, ``test_dropin.py`` also
compiles the adapter against the reference's own headers and training core.
"""

from __future__ import annotations

import os
import shutil
import subprocess

import pytest

from mpsboost_gb300 import build as cuda_build

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_adapter_on_gpu(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    lib = cuda_build.build()
    exe = tmp_path / "adapter_check"
    cmd = ["g++", "-std=c++17", "-O2", f"-I{ROOT}/tests/dropin/stand_in", f"-I{ROOT}/include",
           os.path.join(ROOT, "tests", "dropin", "adapter_gpu_check.cpp"), lib,
           f"-Wl,-rpath,{os.path.dirname(lib)}", "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "adapter ok" in out.stdout
