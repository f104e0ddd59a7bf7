//! Links libdamascus_gb300.so for `damascus-core` behind DAMASCUS_GPU=1.
//!
//! The library is the in-tree build of `damascus000_gb300/build.py` (nvcc,
//! sm_103a).  With DAMASCUS_GB300_LIB_DIR set, that directory is linked as is;
//! otherwise this script runs the Python build from the repository root (two
//! levels above this crate) and links `damascus000_gb300/_build/`.  With
//! DAMASCUS_GPU=0 nothing is linked and `cfg(damascus_cuda_available)` stays
//! off, as in the reference's build.rs; there is no CPU implementation in this
//! crate, so its safe API then reports the GPU as unavailable.
use std::env;
use std::path::PathBuf;
use std::process::Command;

fn main() {
    println!("cargo:rerun-if-env-changed=DAMASCUS_GPU");
    println!("cargo:rerun-if-env-changed=DAMASCUS_GB300_LIB_DIR");
    println!("cargo:rustc-check-cfg=cfg(damascus_cuda_available)");
    if env::var("DAMASCUS_GPU").is_ok_and(|v| v == "0") {
        println!("cargo:warning=DAMASCUS_GPU=0: libdamascus_gb300 not linked");
        return;
    }
    let lib_dir = match env::var("DAMASCUS_GB300_LIB_DIR") {
        Ok(dir) => PathBuf::from(dir),
        Err(_) => {
            let manifest = PathBuf::from(env::var("CARGO_MANIFEST_DIR").expect("CARGO_MANIFEST_DIR"));
            let repo = manifest.join("..").join("..");
            let python = env::var("PYTHON").unwrap_or_else(|_| "python3".to_string());
            let out = Command::new(&python)
                .current_dir(&repo)
                .args(["-c", "from damascus000_gb300 import build as b; print(b.build())"])
                .output();
            match out {
                Ok(o) if o.status.success() => {
                    let path = String::from_utf8_lossy(&o.stdout).trim().to_string();
                    PathBuf::from(path).parent().map(|p| p.to_path_buf()).expect("library path")
                }
                Ok(o) => panic!(
                    "building libdamascus_gb300 failed:\n{}",
                    String::from_utf8_lossy(&o.stderr)
                ),
                Err(e) => panic!("cannot run {python} to build libdamascus_gb300: {e}"),
            }
        }
    };
    println!("cargo:rustc-link-search=native={}", lib_dir.display());
    println!("cargo:rustc-link-lib=dylib=damascus_gb300");
    // the shared library is found at run time without LD_LIBRARY_PATH
    println!("cargo:rustc-link-arg=-Wl,-rpath,{}", lib_dir.display());
    println!("cargo:rustc-cfg=damascus_cuda_available");
}
