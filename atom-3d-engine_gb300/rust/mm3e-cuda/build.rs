//! Links the crate against libmm3e_cuda.so, the C ABI declared in include/mm3e_cuda.h of the
//! GB300 render-path repository. MM3E_CUDA_LIB_DIR names the directory holding the library (its
//! in-tree build location is atom-3d-engine_gb300/mm3e_cuda/_lib); the library links the CUDA
//! runtime statically, so only the NVIDIA driver is needed at run time.
use std::env;

fn main() {
    println!("cargo:rerun-if-env-changed=MM3E_CUDA_LIB_DIR");
    if let Ok(dir) = env::var("MM3E_CUDA_LIB_DIR") {
        println!("cargo:rustc-link-search=native={dir}");
        // let binaries and tests find the library without LD_LIBRARY_PATH
        println!("cargo:rustc-link-arg=-Wl,-rpath,{dir}");
    }
    println!("cargo:rustc-link-lib=dylib=mm3e_cuda");
}
