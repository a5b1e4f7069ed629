//! Builds libtinytrace_cuda.so in-tree (nvcc, sm_103a) through the package's build script
//! and tells cargo where to find it.  TINYTRACE_CUDA_LIB_DIR skips the build and links the
//! library found in that directory instead.

use std::env;
use std::path::PathBuf;
use std::process::Command;

fn main() {
    println!("cargo:rerun-if-env-changed=TINYTRACE_CUDA_LIB_DIR");
    let lib_dir = match env::var("TINYTRACE_CUDA_LIB_DIR") {
        Ok(dir) => PathBuf::from(dir),
        Err(_) => {
            // rust/tinytrace_cuda_sys -> repository root
            let root = PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap()).join("../..");
            let status = Command::new("python3")
                .current_dir(&root)
                .args(["-c", "from tinytrace_gb300 import build; build.build()"])
                .status()
                .expect("python3 is needed to run the nvcc build of libtinytrace_cuda.so");
            assert!(status.success(), "building libtinytrace_cuda.so failed");
            for src in ["include/tinytrace_cuda.h", "tinytrace_gb300/csrc", "tinytrace_gb300/build.py"] {
                println!("cargo:rerun-if-changed={}", root.join(src).display());
            }
            root.join("tinytrace_gb300/_build")
        }
    };
    println!("cargo:rustc-link-search=native={}", lib_dir.display());
    println!("cargo:rustc-link-lib=dylib=tinytrace_cuda");
    println!("cargo:rustc-link-arg=-Wl,-rpath,{}", lib_dir.display());
}
