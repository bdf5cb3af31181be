//! Links librcg.so. RCG_LIB_DIR names the directory that holds it (default: the package directory next to this
//! crate, where `python rust-compress_gb300/build.py` writes it). The library carries the CUDA runtime statically;
//! it needs a CUDA 13 driver and an sm_103a GPU at run time.
use std::env;
use std::path::PathBuf;

fn main() {
    let dir = env::var("RCG_LIB_DIR").map(PathBuf::from).unwrap_or_else(|_| {
        PathBuf::from(env::var("CARGO_MANIFEST_DIR").expect("cargo sets CARGO_MANIFEST_DIR")).join("..")
    });
    println!("cargo:rustc-link-search=native={}", dir.display());
    println!("cargo:rustc-link-lib=dylib=rcg");
    println!("cargo:rerun-if-env-changed=RCG_LIB_DIR");
    println!("cargo:rerun-if-changed={}", dir.join("librcg.so").display());
}
