"""The library's host protocol code compiled for the CPU (no GPU): the nonzero
challenge sampler, the fixed-width field encoding and the protocol constants
against the reference's own unit tests for them, and the verifier's one-pass
commitment update against its two-step form (`tests/native/protocol_host.cpp`)."""
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


def test_protocol_host_code(tmp_path):
    cxx = shutil.which("g++")
    inc = _cuda_include()
    if cxx is None or inc is None:
        pytest.skip("g++ or the CUDA headers are missing")
    exe = tmp_path / "protocol_host"
    cmd = [cxx, "-O2", "-std=c++17", "-pthread", "-I", str(inc), "-I", str(CSRC), "-x", "c++",
           str(ROOT / "tests" / "native" / "protocol_host.cpp"), str(CSRC / "protocol.cpp"),
           str(CSRC / "host_blake3.cpp"), "-o", str(exe)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-4000:]
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stdout + res.stderr
    assert res.stdout.strip().endswith("ok"), res.stdout
