"""The Rust binding (rust/damascus-gb300) against the C header it binds.

Neither this machine nor the GPU machine has cargo, so the crate is not compiled
here; this test keeps its raw declarations in step with include/damascus.h:
every C entry point has a `pub fn` of the same name and parameter count in
src/sys.rs and none is extra, and the drop-in module keeps the public names of
damascus-core's src/utils/gpu.rs."""
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
CRATE = ROOT / "rust" / "damascus-gb300"


def c_decls():
    src = (ROOT / "include" / "damascus.h").read_text()
    out = {}
    for m in re.finditer(r'^(?:int|void|const char\*|uint64_t|uint32_t|size_t)\s+(damascus_\w+)\(([^;]*)\);', src,
                         re.M):
        args = " ".join(m.group(2).split())
        out[m.group(1)] = 0 if args == "void" else args.count(",") + 1
    return out


def rust_decls():
    src = (CRATE / "src" / "sys.rs").read_text()
    out = {}
    for m in re.finditer(r'pub fn (damascus_\w+)\(([^)]*)\)', src):
        args = m.group(2).strip()
        out[m.group(1)] = 0 if not args else args.count(",") + 1
    return out


def test_sys_declares_every_c_entry_point():
    c, r = c_decls(), rust_decls()
    assert len(c) > 70
    assert set(c) == set(r), (sorted(set(c) - set(r)), sorted(set(r) - set(c)))
    assert {k: v for k, v in c.items() if r[k] != v} == {}


def test_status_codes_match_header():
    hdr = dict(re.findall(r'#define (DAMASCUS_E\w+|DAMASCUS_OK) \(?(-?\d+)\)?', (ROOT / "include" / "damascus.h")
                          .read_text()))
    rs = dict(re.findall(r'pub const (DAMASCUS_E\w+|DAMASCUS_OK): c_int = (-?\d+);', (CRATE / "src" / "sys.rs")
                         .read_text()))
    assert hdr and hdr == rs


def test_gpu_module_keeps_reference_names():
    src = (CRATE / "src" / "gpu.rs").read_text()
    for name in ("pub fn cuda_device_info", "pub fn cuda_backend_ready", "pub fn try_fold_pairs_gpu",
                 "pub fn try_ntt_batch_gpu", "pub struct CudaDeviceInfo"):
        assert name in src
    build = (CRATE / "build.rs").read_text()
    assert "cargo:rustc-cfg=damascus_cuda_available" in build and "DAMASCUS_GPU" in build
