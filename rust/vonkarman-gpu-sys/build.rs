// Links the prebuilt libvonkarman_gpu.so.  Build it first with
//   python -c "import __graft_entry__ as g; g.build()"
// (nvcc, sm_103a, static CUDA runtime) and point VONKARMAN_GPU_LIB_DIR at the
// directory holding it (vonkarman_gb300/ in this repository).
fn main() {
    let dir = std::env::var("VONKARMAN_GPU_LIB_DIR")
        .expect("set VONKARMAN_GPU_LIB_DIR to the directory of libvonkarman_gpu.so");
    println!("cargo:rustc-link-search=native={dir}");
    println!("cargo:rustc-link-lib=dylib=vonkarman_gpu");
    println!("cargo:rerun-if-env-changed=VONKARMAN_GPU_LIB_DIR");
}
