"""The transform pipeline's own device functions compiled for the CPU.

`tests/native/ring_emulation.cpp` runs the forward and inverse transforms of
`dm_ntt.cuh` exactly as the kernels schedule them (16 residues per thread, the
swizzled shared-memory exchanges, the last-pass twiddle order, the lazy value
bounds), the MAC, the even/odd cross terms and the Garner CRT, and compares
with schoolbook negacyclic products in Z_q for ring sizes 1 .. 4096 (the
reference's `negacyclic_multiply` contract, src/algebra/ntt.rs:112-195 and its
test `negacyclic_multiply_across_runtime_sizes`, :509-521).  It also checks
that each exchange is bank-conflict free for the kernels' block shapes, and
that the forward transform's radix-32 pass shape (32 residues per thread, the
alternative the autotuner may pick from 2^5 on) gives the same slots as the
radix-16 one within the same lazy bounds.
"""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "damascus000_gb300" / "csrc"


def _cuda_include():
    for cand in (Path("/usr/local/cuda/include"), Path("/usr/local/cuda/targets/sbsa-linux/include")):
        if (cand / "cuda_runtime.h").exists():
            return cand
    return None


def test_ring_pipeline_host_emulation(tmp_path):
    cxx = shutil.which("g++")
    inc = _cuda_include()
    if cxx is None or inc is None:
        pytest.skip("g++ or the CUDA headers are missing")
    exe = tmp_path / "ring_emulation"
    cmd = [cxx, "-O2", "-std=c++17", "-I", str(inc), "-I", str(CSRC), "-x", "c++",
           str(ROOT / "tests" / "native" / "ring_emulation.cpp"), str(CSRC / "dm_tables.cpp"), "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    assert res.stdout.strip().startswith("ok"), res.stdout
