// Link step the reference crate adds for the GI stage: librc.so is built by
// the engine's own build (python -c "import __graft_entry__ as g; g.build()")
// into radiancecascade_gb300/; RC_LIB_DIR points at that folder.
fn main() {
    let dir = std::env::var("RC_LIB_DIR").unwrap_or_else(|_| "../../radiancecascade_gb300".to_string());
    println!("cargo:rustc-link-search=native={}", dir);
    println!("cargo:rustc-link-lib=dylib=rc");
    println!("cargo:rerun-if-env-changed=RC_LIB_DIR");
}
