//! Builds libbioshell_crmsd.so for sm_103a with nvcc and links it, or links
//! a prebuilt copy when BIOSHELL_CRMSD_LIB_DIR names its directory.
//!
//! The sources are the engine's own (`bioshell_gb300/csrc`, two levels up
//! from this crate), compiled with the flags of `bioshell_gb300/_build.py`:
//! every .cu with nvcc for compute_103a/sm_103a, every .cpp with the host C++
//! compiler without floating-point contraction (the clustering code must round
//! as the reference's f32 arithmetic does), then one shared library.  No
//! CPU fallback exists: the library needs an sm_103 GPU at run time.
use std::env;
use std::path::{Path, PathBuf};
use std::process::Command;
use std::thread;

fn nvcc() -> String {
    if let Ok(p) = env::var("NVCC") {
        return p;
    }
    for c in ["/usr/local/cuda/bin/nvcc", "nvcc"] {
        if c == "nvcc" || Path::new(c).exists() {
            return c.to_string();
        }
    }
    unreachable!()
}

fn link(dir: &Path) {
    println!("cargo:rustc-link-search=native={}", dir.display());
    println!("cargo:rustc-link-lib=dylib=bioshell_crmsd");
    println!("cargo:rustc-link-arg=-Wl,-rpath,{}", dir.display());
}

fn main() {
    println!("cargo:rerun-if-env-changed=BIOSHELL_CRMSD_LIB_DIR");
    println!("cargo:rerun-if-env-changed=NVCC");
    if let Ok(dir) = env::var("BIOSHELL_CRMSD_LIB_DIR") {
        link(Path::new(&dir));
        return;
    }
    let root = PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap()).join("..").join("..");
    let csrc = root.join("bioshell_gb300").join("csrc");
    let include = root.join("include");
    println!("cargo:rerun-if-changed={}", csrc.display());
    println!("cargo:rerun-if-changed={}", include.display());
    let out = PathBuf::from(env::var("OUT_DIR").unwrap());
    let nvcc = nvcc();
    let cxx = env::var("CXX").unwrap_or_else(|_| "g++".to_string());
    let inc = format!("-I{}", include.display());
    let mut jobs = Vec::new();
    let mut objs = Vec::new();
    let mut srcs: Vec<PathBuf> = std::fs::read_dir(&csrc)
        .expect("bioshell_gb300/csrc not found beside this crate")
        .map(|e| e.unwrap().path())
        .filter(|p| matches!(p.extension().and_then(|e| e.to_str()), Some("cu") | Some("cpp")))
        .collect();
    srcs.sort();
    for src in srcs {
        let obj = out.join(format!("{}.o", src.file_stem().unwrap().to_str().unwrap()));
        objs.push(obj.clone());
        let mut cmd = if src.extension().unwrap() == "cpp" {
            let mut c = Command::new(&cxx);
            c.args(["-O3", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off", &inc]);
            c
        } else {
            let mut c = Command::new(&nvcc);
            c.args(["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-lineinfo",
                    "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-fvisibility=hidden", &inc]);
            c
        };
        cmd.arg("-c").arg(&src).arg("-o").arg(&obj);
        jobs.push(thread::spawn(move || {
            let st = cmd.status().expect("nvcc / the C++ compiler could not be run");
            assert!(st.success(), "compiling {} failed", src.display());
        }));
    }
    for j in jobs {
        j.join().unwrap();
    }
    let lib = out.join("libbioshell_crmsd.so");
    let st = Command::new(&nvcc)
        .args(["-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-o"])
        .arg(&lib)
        .args(&objs)
        .status()
        .expect("nvcc could not be run");
    assert!(st.success(), "linking libbioshell_crmsd.so failed");
    link(&out);
}
