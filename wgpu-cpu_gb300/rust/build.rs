// Links libgbr.so: GBR_LIB_DIR names its directory (by default the package's wgpu_gb300/, where
// build_lib.py writes it), and the rpath lets the binary find it at run time.
fn main() {
    let dir = std::env::var("GBR_LIB_DIR").unwrap_or_else(|_| {
        let here = std::path::PathBuf::from(std::env::var("CARGO_MANIFEST_DIR").unwrap());
        here.join("../wgpu_gb300").to_string_lossy().into_owned()
    });
    println!("cargo:rustc-link-search=native={dir}");
    println!("cargo:rustc-link-lib=dylib=gbr");
    println!("cargo:rustc-link-arg=-Wl,-rpath,{dir}");
    println!("cargo:rerun-if-env-changed=GBR_LIB_DIR");
}
