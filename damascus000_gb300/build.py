"""In-tree build of libdamascus_gb300.so for sm_103a (GB300).

Every CUDA source is compiled with ``-gencode arch=compute_103a,code=sm_103a``;
host C++ goes through the same nvcc driver so the objects link against the
static CUDA runtime.  Objects are built in parallel and the shared library is
written to ``damascus000_gb300/_build/``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
CSRC = PKG_DIR / "csrc"
INCLUDE = PKG_DIR.parent / "include"
BUILD_DIR = PKG_DIR / "_build"
LIB_NAME = "libdamascus_gb300.so"
LIB_PATH = BUILD_DIR / LIB_NAME

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
          "-I", str(CSRC), "-I", str(INCLUDE)]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (Path(cand).exists() or cand == "nvcc"):
            return cand
    return "nvcc"


def sources():
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _headers():
    return sorted(list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h")))


def _compile(src: Path, ptxas_verbose: bool) -> Path:
    obj = BUILD_DIR / (src.name + ".o")
    cmd = [_nvcc()] + COMMON + ARCH + ["-c", str(src), "-o", str(obj)]
    if src.suffix == ".cu":
        cmd += ["-Xptxas", "-v"] if ptxas_verbose else []
    else:
        cmd += ["-x", "c++"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    log = BUILD_DIR / (src.name + ".log")
    log.write_text(res.stdout + res.stderr)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")
    return obj


def build(force: bool = False, ptxas_verbose: bool = True, jobs: int | None = None) -> Path:
    """Compile every source for sm_103a and link the shared library."""
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    srcs = sources()
    newest = max(p.stat().st_mtime for p in srcs + _headers() + [Path(__file__)])
    if not force and LIB_PATH.exists() and LIB_PATH.stat().st_mtime >= newest:
        return LIB_PATH
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, ptxas_verbose), srcs))
    tmp = BUILD_DIR / f"{LIB_NAME}.tmp{os.getpid()}"
    cmd = [_nvcc()] + ARCH + ["-shared", "-Xcompiler", "-fPIC", "-Xlinker", "--export-dynamic", "-o", str(tmp)] + \
        [str(o) for o in objs] + ["-lpthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
