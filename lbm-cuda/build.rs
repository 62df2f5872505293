// Build script of the lbm-cuda crate.
//
// Default: compiles the library's CUDA sources (chemsim_gb300/csrc/*.cu next
// to this crate, or the directory in LBM_CUDA_SRC) with nvcc through the cc
// crate, for sm_103a only, and links them statically together with the
// static CUDA runtime; the final binary then needs only the CUDA driver.
// The flags are those of chemsim_gb300/build.py, which builds the same
// sources into liblbm_cuda.so.
//
// With LBM_CUDA_DIR set: links the prebuilt liblbm_cuda.so in that directory
// instead (the file chemsim_gb300/build.py writes to chemsim_gb300/_lib).
use std::env;
use std::path::PathBuf;

fn main() {
    println!("cargo:rerun-if-env-changed=LBM_CUDA_DIR");
    println!("cargo:rerun-if-env-changed=LBM_CUDA_SRC");
    if let Ok(dir) = env::var("LBM_CUDA_DIR") {
        println!("cargo:rustc-link-search=native={}", dir);
        println!("cargo:rustc-link-lib=dylib=lbm_cuda");
        return;
    }
    let manifest = PathBuf::from(env::var("CARGO_MANIFEST_DIR").expect("cargo sets CARGO_MANIFEST_DIR"));
    let src = env::var("LBM_CUDA_SRC")
        .map(PathBuf::from)
        .unwrap_or_else(|_| manifest.join("..").join("chemsim_gb300").join("csrc"));
    let include = manifest.join("..").join("include");

    let mut sources: Vec<PathBuf> = std::fs::read_dir(&src)
        .unwrap_or_else(|e| panic!("CUDA sources in {}: {}", src.display(), e))
        .filter_map(|entry| entry.ok().map(|e| e.path()))
        .filter(|p| p.extension().map_or(false, |x| x == "cu"))
        .collect();
    sources.sort();
    assert!(!sources.is_empty(), "no .cu files in {}", src.display());

    let mut build = cc::Build::new();
    build
        .cuda(true)
        .cudart("static")
        .flag("-gencode")
        .flag("arch=compute_103a,code=sm_103a")
        .flag("-O3")
        .flag("-lineinfo")
        .flag("-std=c++17")
        .flag("--expt-relaxed-constexpr")
        .flag("-Xcompiler")
        .flag("-ffp-contract=off")
        .include(&include);
    for f in &sources {
        build.file(f);
        println!("cargo:rerun-if-changed={}", f.display());
    }
    for dir in [&src, &include].iter() {
        for entry in std::fs::read_dir(dir).into_iter().flatten().flatten() {
            let p = entry.path();
            if p.extension().map_or(false, |x| x == "cuh" || x == "h") {
                println!("cargo:rerun-if-changed={}", p.display());
            }
        }
    }
    build.compile("lbm_cuda");
    // the host side of the .cu files is C++
    println!("cargo:rustc-link-lib=dylib=stdc++");
}
