// Builds libferiphys_gb300 (CUDA for sm_103a, no cmake) with the package's own
// build step and links it.  The library directory is found from
// FERIPHYS_GB300_DIR (the repository root), else from this crate's location
// inside the repository (rust/feriphys-gb300-sys).  Requires python3 and nvcc
// (CUDA 13) on the build machine.
use std::env;
use std::path::PathBuf;
use std::process::Command;

fn main() {
    let root = match env::var("FERIPHYS_GB300_DIR") {
        Ok(dir) => PathBuf::from(dir),
        Err(_) => PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap()).join("..").join(".."),
    };
    let pkg = root.join("feriphys_gb300");
    // feriphys_gb300/build.py compiles every .cu/.cpp of csrc/ with
    // -gencode arch=compute_103a,code=sm_103a -fmad=false and links the .so in place
    let status = Command::new("python3")
        .arg(pkg.join("build.py"))
        .status()
        .expect("python3 is required to build libferiphys_gb300");
    assert!(status.success(), "building libferiphys_gb300 failed");
    println!("cargo:rustc-link-search=native={}", pkg.display());
    println!("cargo:rustc-link-lib=dylib=feriphys_gb300");
    // the shared library is found next to the binary's rpath at run time
    println!("cargo:rustc-link-arg=-Wl,-rpath,{}", pkg.display());
    println!("cargo:rerun-if-env-changed=FERIPHYS_GB300_DIR");
    println!("cargo:rerun-if-changed={}", pkg.join("csrc").display());
    println!("cargo:rerun-if-changed={}", root.join("include").join("feriphys_gb300.h").display());
}
