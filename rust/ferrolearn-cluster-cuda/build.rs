//! Compiles the hand-written CUDA kernels of the KMeans back end for
//! sm_103a (GB300) with nvcc and links them as a static library.
//!
//! Environment: FERROKMEANS_ROOT (the repository holding ferrolearn_gb300/
//! and include/; default: two directories above this manifest), NVCC (default
//! "nvcc" on PATH), CUDA_HOME (default /usr/local/cuda) for cudart_static.

use std::env;
use std::fs;
use std::path::PathBuf;
use std::process::Command;

// Units whose distances and sums must match the reference bit for bit: no
// fused multiply-add is ever contracted there (they also use _rn intrinsics).
const EXACT_UNITS: [&str; 4] = ["fk_assign.cu", "fk_update.cu", "fk_kpp.cu", "fk_batched.cu"];

fn main() {
    let manifest = PathBuf::from(env::var("CARGO_MANIFEST_DIR").expect("CARGO_MANIFEST_DIR"));
    let root = env::var("FERROKMEANS_ROOT").map(PathBuf::from).unwrap_or_else(|_| manifest.join("../.."));
    let csrc = root.join("ferrolearn_gb300").join("csrc");
    let include = root.join("include");
    let out = PathBuf::from(env::var("OUT_DIR").expect("OUT_DIR"));
    let nvcc = env::var("NVCC").unwrap_or_else(|_| "nvcc".to_string());
    let cuda_home = env::var("CUDA_HOME").unwrap_or_else(|_| "/usr/local/cuda".to_string());

    let mut sources: Vec<PathBuf> = fs::read_dir(&csrc)
        .unwrap_or_else(|e| panic!("cannot read {}: {e}", csrc.display()))
        .filter_map(|e| e.ok().map(|e| e.path()))
        .filter(|p| p.extension().is_some_and(|x| x == "cu"))
        .collect();
    sources.sort();
    println!("cargo:rerun-if-changed={}", csrc.display());
    println!("cargo:rerun-if-changed={}", include.join("ferrokmeans.h").display());

    let mut objects = Vec::new();
    for src in &sources {
        let name = src.file_name().unwrap().to_string_lossy().to_string();
        let obj = out.join(name.replace(".cu", ".o"));
        let mut cmd = Command::new(&nvcc);
        cmd.args(["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-lineinfo"])
            .args(["-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"])
            .arg("-I")
            .arg(&include);
        if EXACT_UNITS.contains(&name.as_str()) {
            cmd.arg("-fmad=false");
        }
        cmd.arg("-c").arg(src).arg("-o").arg(&obj);
        let status = cmd.status().unwrap_or_else(|e| panic!("cannot run {nvcc}: {e}"));
        assert!(status.success(), "nvcc failed on {}", src.display());
        objects.push(obj);
    }
    let lib = out.join("libferrokmeans.a");
    let _ = fs::remove_file(&lib);
    let status = Command::new("ar").arg("crs").arg(&lib).args(&objects).status().expect("cannot run ar");
    assert!(status.success(), "ar failed");

    println!("cargo:rustc-link-search=native={}", out.display());
    println!("cargo:rustc-link-lib=static=ferrokmeans");
    println!("cargo:rustc-link-search=native={cuda_home}/lib64");
    println!("cargo:rustc-link-lib=static=cudart_static");
    for sys in ["stdc++", "dl", "rt", "pthread"] {
        println!("cargo:rustc-link-lib=dylib={sys}");
    }
}
