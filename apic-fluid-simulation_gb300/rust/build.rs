// Links the GB300 library: build it first with
//   python -c "import __graft_entry__ as g; g.build()"
// and point APIC_GPU_LIB_DIR at apic-fluid-simulation_gb300/lib.
fn main() {
    let dir = std::env::var("APIC_GPU_LIB_DIR").expect("set APIC_GPU_LIB_DIR to the directory of libapic_gpu.so");
    println!("cargo:rustc-link-search=native={dir}");
    println!("cargo:rustc-link-lib=dylib=apic_gpu");
    println!("cargo:rerun-if-env-changed=APIC_GPU_LIB_DIR");
}
