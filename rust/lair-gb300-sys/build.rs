// Links liblair_gb300.so.  Build it first with
//   python -c "import __graft_entry__ as g; g.build()"
// and point LAIR_GB300_LIB_DIR at the directory holding it (default: the
// lair_gb300/ directory of this repository, two levels up).
use std::env;
use std::path::PathBuf;

fn main() {
    let dir = env::var("LAIR_GB300_LIB_DIR").map(PathBuf::from).unwrap_or_else(|_| {
        PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap()).join("../../lair_gb300")
    });
    println!("cargo:rustc-link-search=native={}", dir.display());
    println!("cargo:rustc-link-lib=dylib=lair_gb300");
    println!("cargo:rerun-if-env-changed=LAIR_GB300_LIB_DIR");
}
