//! Raw binding of the GB300 crmsd engine's C ABI (`include/bioshell_crmsd.h`).
//!
//! One `extern "C"` declaration per exported function and one `#[repr(C)]`
//! mirror per struct of the header, in the header's order.  The safe API that
//! `bioshell_pdb::calc` exposes on top of it (`crmsd`, `crmsd_all_vs_all`,
//! `crmsd_batched`, `CrmsdServer`, ...) lives in the `bioshell-pdb`
//! sources of this directory; this crate only links the library (see
//! `build.rs`) and states its interface.  The crmsd function the binding
//! serves has no implementation in bioshell-pdb yet: its home is
//! `bioshell-pdb/src/calc/mod.rs`, beside `SubstructureAxis`
//! (`calc/substructures.rs:17`).
//!
//! Conventions of every call: integer status (0 = `BS_OK`), caller-owned
//! inputs and outputs, `[n][L][3]` f64 coordinates (the memory order of
//! `bioshell_core::Vec3` triples), host or device pointers accepted.
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_void};

// ---------------------------------------------------------------- constants
pub const BS_ABI_VERSION: i32 = 3;
pub const BS_OPTS_VERSION: i32 = 1;

pub type BsStatus = i32;
pub const BS_OK: i32 = 0;
pub const BS_ERR_INVALID_ARG: i32 = 1;
pub const BS_ERR_CUDA: i32 = 2;
pub const BS_ERR_OOM: i32 = 3;
pub const BS_ERR_TIMEOUT: i32 = 4;
pub const BS_ERR_UNSUPPORTED: i32 = 5;
pub const BS_ERR_NONFINITE: i32 = 6;
pub const BS_ERR_BUDGET: i32 = 7;
pub const BS_ERR_NO_DEVICE: i32 = 8;
pub const BS_ERR_INTERNAL: i32 = 9;
pub const BS_ERR_CANCELLED: i32 = 10;

pub const BS_PRECISION_PLAIN64: i32 = 0;
pub const BS_PRECISION_MIXED: i32 = 1;
pub const BS_LAYOUT_TRIANGLE: i32 = 0;
pub const BS_LAYOUT_SQUARE: i32 = 1;
pub const BS_OUT_F64: i32 = 0;
pub const BS_OUT_F32: i32 = 1;
pub const BS_FLAG_NO_GRAPH: i32 = 1;
pub const BS_FLAG_AUTOTUNE: i32 = 2;

pub const BS_LINK_SINGLE: i32 = 0;
pub const BS_LINK_COMPLETE: i32 = 1;
pub const BS_LINK_AVERAGE: i32 = 2;
pub const BS_LINK_MEDIAN: i32 = 3;
pub const BS_LINK_CENTROID: i32 = 4;
pub const BS_LINK_WARD: i32 = 5;

// ------------------------------------------------------------ opaque handles
#[repr(C)]
pub struct BsCtx {
    _p: [u8; 0],
}
#[repr(C)]
pub struct BsServer {
    _p: [u8; 0],
}
#[repr(C)]
pub struct BsModels {
    _p: [u8; 0],
}
#[repr(C)]
pub struct BsTsv {
    _p: [u8; 0],
}

// ------------------------------------------------------------------- structs
/// `bs_opts`: options of the all-vs-all fill (initialise with `bs_opts_init`).
#[repr(C)]
#[derive(Debug, Clone, Copy)]
pub struct BsOpts {
    pub version: u32,
    pub precision: i32,
    pub layout: i32,
    pub out_type: i32,
    pub tolerance: f64,
    pub flags: i32,
    pub flag_queue: i32,
    pub row_begin: i32,
    pub row_end: i32,
    pub reserved: [i32; 4],
}

/// `bs_metrics`: per-call counters of the last compute call on a context.
#[repr(C)]
#[derive(Debug, Default, Clone, Copy)]
pub struct BsMetrics {
    pub pairs: i64,
    pub pairs_refined: i64,
    pub ms_total: f64,
    pub ms_h2d: f64,
    pub ms_prep: f64,
    pub ms_main: f64,
    pub ms_refine: f64,
    pub ms_d2h: f64,
    pub scale_exp: i32,
    pub main_launches: i32,
    pub jobs: i32,
    pub graph: i32,
    pub quant_bound: f64,
    pub bytes_h2d: i64,
    pub bytes_d2h: i64,
    pub narrow_jobs: i32,
    pub tuned_classes: i32,
    pub pairs_plain: i64,
}

/// `bs_set_desc`: one structure set of a batched call.
#[repr(C)]
#[derive(Debug, Clone, Copy)]
pub struct BsSetDesc {
    pub xyz: *const f64,
    pub n: i64,
    pub l: i32,
    pub reserved: i32,
    pub out: *mut c_void,
}

/// `bs_server_config`: the library buckets and limits of a server.
#[repr(C)]
#[derive(Debug, Clone, Copy)]
pub struct BsServerConfig {
    pub nbuckets: i32,
    pub bucket_l: *const i32,
    pub bucket_n: *const i64,
    pub bucket_xyz: *const *const f64,
    pub top_k: i32,
    pub max_inflight: i32,
    pub hbm_budget: usize,
    pub precision: i32,
    pub max_batch_rows: i32,
    pub tolerance: f64,
    pub index_min: i32,
    pub reserved: [i32; 5],
}

/// `bs_server_stats`: latency percentiles and throughput of a server.
#[repr(C)]
#[derive(Debug, Default, Clone, Copy)]
pub struct BsServerStats {
    pub queries_done: i64,
    pub clusters_done: i64,
    pub pairs: i64,
    pub batches: i64,
    pub plain_fallbacks: i64,
    pub pending: i64,
    pub p50_ms: f64,
    pub p99_ms: f64,
    pub max_ms: f64,
    pub mean_ms: f64,
    pub cluster_p50_ms: f64,
    pub cluster_p99_ms: f64,
    pub pairs_per_s: f64,
    pub mean_batch_rows: f64,
    pub seconds: f64,
    pub pairs_screened: i64,
}

extern "C" {
    // ---- version / errors / contexts
    pub fn bs_abi_version() -> i32;
    pub fn bs_status_string(s: BsStatus) -> *const c_char;
    pub fn bs_last_error(ctx: *const BsCtx) -> *const c_char;
    pub fn bs_ctx_create(out: *mut *mut BsCtx, device: i32, hbm_budget_bytes: usize) -> BsStatus;
    pub fn bs_ctx_destroy(ctx: *mut BsCtx);
    pub fn bs_opts_init(opts: *mut BsOpts);
    pub fn bs_get_metrics(ctx: *const BsCtx, out: *mut BsMetrics) -> BsStatus;
    pub fn bs_ctx_trim(ctx: *mut BsCtx) -> BsStatus;
    pub fn bs_ctx_stream(ctx: *const BsCtx) -> *mut c_void;

    // ---- compute
    pub fn bs_crmsd(ctx: *mut BsCtx, a: *const f64, b: *const f64, l: i32, out_rmsd: *mut f64) -> BsStatus;
    pub fn bs_superpose(ctx: *mut BsCtx, a: *const f64, b: *const f64, l: i32, rot: *mut f64, trans: *mut f64,
                        rmsd: *mut f64) -> BsStatus;
    pub fn bs_superpose_pairs(ctx: *mut BsCtx, xyz: *const f64, n: i64, l: i32, ii: *const i64, jj: *const i64,
                              npairs: i64, rot: *mut f64, trans: *mut f64, rmsd: *mut f64) -> BsStatus;
    pub fn bs_all_vs_all(ctx: *mut BsCtx, xyz: *const f64, n: i64, l: i32, opts: *const BsOpts,
                         out: *mut c_void) -> BsStatus;
    pub fn bs_batched(ctx: *mut BsCtx, sets: *const BsSetDesc, nsets: i32, opts: *const BsOpts) -> BsStatus;
    pub fn bs_neighbors(ctx: *mut BsCtx, xyz: *const f64, n: i64, l: i32, eps: f64, opts: *const BsOpts,
                        nnz: *mut i64) -> BsStatus;
    pub fn bs_neighbors_get(ctx: *mut BsCtx, row_ptr: *mut i64, col: *mut i32, dist: *mut f32) -> BsStatus;
    pub fn bs_tune_get(ctx: *mut BsCtx, l: i32, n: i64, narrow: *mut i32) -> BsStatus;
    pub fn bs_tune_set(ctx: *mut BsCtx, l: i32, n: i64, narrow: i32) -> BsStatus;
    pub fn bs_tune_list(ctx: *mut BsCtx, l_class: *mut i32, n_class: *mut i64, narrow: *mut i32, cap: i32,
                        count: *mut i32, num_sms: *mut i32) -> BsStatus;
    pub fn bs_pairs(ctx: *mut BsCtx, xyz: *const f64, n: i64, l: i32, ii: *const i64, jj: *const i64,
                    npairs: i64, opts: *const BsOpts, out: *mut f64) -> BsStatus;
    pub fn bs_all_vs_all_static(xyz: *const f64, n: i64, l: i32, out: *mut f64, stream: *mut c_void) -> BsStatus;
    pub fn bs_partition_rows(n: i64, parts: i32, bounds: *mut i64) -> BsStatus;

    // ---- serving
    pub fn bs_server_create(out: *mut *mut BsServer, device: i32, cfg: *const BsServerConfig) -> BsStatus;
    pub fn bs_server_destroy(s: *mut BsServer);
    pub fn bs_server_last_error(s: *const BsServer) -> *const c_char;
    pub fn bs_server_submit(s: *mut BsServer, xyz: *const f64, q: i32, l: i32, ticket: *mut i64) -> BsStatus;
    pub fn bs_server_submit_cluster(s: *mut BsServer, xyz: *const f64, n: i64, l: i32, eps: f64, min_points: i32,
                                    ticket: *mut i64) -> BsStatus;
    pub fn bs_server_poll(s: *mut BsServer, ticket: i64, done: *mut i32) -> BsStatus;
    pub fn bs_server_wait(s: *mut BsServer, ticket: i64, hit_index: *mut i64, hit_rmsd: *mut f64,
                          timeout_s: f64) -> BsStatus;
    pub fn bs_server_wait_cluster(s: *mut BsServer, ticket: i64, cluster_of: *mut i64, timeout_s: f64) -> BsStatus;
    pub fn bs_server_get_stats(s: *mut BsServer, out: *mut BsServerStats) -> BsStatus;
    pub fn bs_server_cancel(s: *mut BsServer, ticket: i64, cancelled: *mut i32) -> BsStatus;
    pub fn bs_server_reset_stats(s: *mut BsServer) -> BsStatus;

    // ---- clustering of a crmsd matrix
    pub fn bs_hierarchical(tri: *const c_void, n: i64, out_type: i32, rule: i32, merges: *mut i64,
                           merge_dist: *mut f32) -> BsStatus;
    pub fn bs_hierarchical_gpu(ctx: *mut BsCtx, tri: *const c_void, n: i64, out_type: i32, rule: i32,
                               merges: *mut i64, merge_dist: *mut f32) -> BsStatus;
    pub fn bs_cut_tree(merges: *const i64, merge_dist: *const f32, n: i64, cutoff: f32,
                       cluster_of: *mut i64) -> BsStatus;
    pub fn bs_optics(tri: *const c_void, n: i64, out_type: i32, eps: f64, min_points: i32, order: *mut i64,
                     reach: *mut f64, cluster_of: *mut i64) -> BsStatus;
    pub fn bs_optics_neighbors(row_ptr: *const i64, col: *const i32, dist: *const f32, n: i64, eps: f64,
                               min_points: i32, order: *mut i64, reach: *mut f64, cluster_of: *mut i64) -> BsStatus;

    // ---- data formats either side of the path
    pub fn bs_io_last_error() -> *const c_char;
    pub fn bs_models_read(path: *const c_char, format: i32, selection: i32, out: *mut *mut BsModels,
                          n_models: *mut i64, n_atoms: *mut i32) -> BsStatus;
    pub fn bs_models_copy(m: *const BsModels, xyz: *mut f64) -> BsStatus;
    pub fn bs_models_free(m: *mut BsModels);
    pub fn bs_tsv_write(path: *const c_char, tri: *const c_void, n: i64, out_type: i32,
                        labels: *const *const c_char, decimals: i32) -> BsStatus;
    pub fn bs_tsv_read(path: *const c_char, default_value: f64, symmetric: i32, out: *mut *mut BsTsv,
                       n: *mut i64) -> BsStatus;
    pub fn bs_tsv_matrix(t: *const BsTsv, tri: *mut f32) -> BsStatus;
    pub fn bs_tsv_label(t: *const BsTsv, i: i64) -> *const c_char;
    pub fn bs_tsv_free(t: *mut BsTsv);

    // ---- pinned host memory
    pub fn bs_host_alloc(bytes: usize, out: *mut *mut c_void) -> BsStatus;
    pub fn bs_host_free(p: *mut c_void) -> BsStatus;

    // ---- test and diagnostic hooks (no counterpart in the reference)
    pub fn bs_selftest_bands(n: i64, bands: i32, elem_end: *mut i64, cap: i32, count: *mut i32) -> BsStatus;
    pub fn bs_selftest_digits(xyz: *const f64, l: i32, scale_exp: i32, digits: *mut i32, g_exact: *mut i64,
                              qres: *mut f64) -> BsStatus;
    pub fn bs_selftest_epilogue(levels: *const f32, ga: i64, gb: i64, qa: f64, qb: f64, d34: f64, scale_exp: i32,
                                l: i32, tolerance: f64, rmsd: *mut f64, flag: *mut i32) -> BsStatus;
    pub fn bs_selftest_screen(m9: *const f32, gsum: f64, de: f64, dr: f64, scale_exp: i32, l: i32, lo: *mut f32,
                              hi: *mut f32) -> BsStatus;
    pub fn bs_selftest_exact(na: *const i32, nb: *const i32, l: i32, scale_exp: i32, rmsd: *mut f64) -> BsStatus;
    pub fn bs_selftest_superpose(a: *const f64, b: *const f64, l: i32, rot: *mut f64, trans: *mut f64,
                                 rmsd: *mut f64) -> BsStatus;
    pub fn bs_debug_tile_levels(ctx: *mut BsCtx, xyz: *const f64, n: i64, l: i32, levels: *mut f32) -> BsStatus;
    pub fn bs_debug_pair_levels(ctx: *mut BsCtx, xyz: *const f64, n: i64, l: i32, ii: *const i64, jj: *const i64,
                                npairs: i64, levels: *mut f32, rmsd: *mut f64) -> BsStatus;
    pub fn bs_debug_set_wait_limit(ctx: *mut BsCtx, ns: i64) -> BsStatus;
    pub fn bs_debug_fail_alloc(ctx: *mut BsCtx, after: i64) -> BsStatus;
    pub fn bs_diag_fp64_peak(device: i32, flops_per_s: *mut f64) -> BsStatus;
}

#[cfg(test)]
mod tests {
    use super::*;

    /// The library links and answers without a GPU; with one, a pair of
    /// identical structures has crmsd 0.
    #[test]
    fn abi_version_and_identity_pair() {
        unsafe {
            assert_eq!(bs_abi_version(), BS_ABI_VERSION);
            let mut ctx: *mut BsCtx = std::ptr::null_mut();
            let st = bs_ctx_create(&mut ctx, 0, 0);
            if st == BS_ERR_NO_DEVICE {
                return;
            }
            assert_eq!(st, BS_OK);
            let a: Vec<f64> = (0..30).map(|k| (k as f64 * 0.37).sin() * 10.0).collect();
            let mut r = -1.0;
            assert_eq!(bs_crmsd(ctx, a.as_ptr(), a.as_ptr(), 10, &mut r), BS_OK);
            assert!(r.abs() <= 1e-4);
            bs_ctx_destroy(ctx);
        }
    }
}
