//! Links the engine library built by `python -c "import __graft_entry__ as g; g.build()"`
//! (auto_gb300/_build/liblenia_gb300.so, sm_103a).  LENIA_GB300_LIB names its folder.

fn main() {
    let dir = std::env::var("LENIA_GB300_LIB")
        .expect("set LENIA_GB300_LIB to the folder holding liblenia_gb300.so");
    println!("cargo:rerun-if-env-changed=LENIA_GB300_LIB");
    println!("cargo:rustc-link-search=native={dir}");
    println!("cargo:rustc-link-lib=dylib=lenia_gb300");
}
