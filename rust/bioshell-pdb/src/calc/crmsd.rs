//! crmsd on the GB300 engine: the safe API of `bioshell_pdb::calc`.
//!
//! This file goes to `bioshell-pdb/src/calc/crmsd.rs`; `calc/mod.rs`
//! (bioshell-pdb/src/calc/mod.rs:1-10) adds
//!
//! ```text
//! mod crmsd;
//! pub use crmsd::{crmsd, crmsd_all_vs_all, crmsd_batched, crmsd_neighbors, read_models, superpose,
//!                 CrmsdMatrix, CrmsdNeighborLists, CrmsdOptions, CrmsdServer, Ticket, TopK};
//! ```
//!
//! `bioshell-pdb/Cargo.toml` gains `bioshell-crmsd-sys = { path = "<engine>/rust/bioshell-crmsd-sys" }`,
//! and `PDBError` (bioshell-pdb/src/pdb_parsing_error.rs:7) one variant:
//!
//! ```text
//! #[error("crmsd engine error {status}: {reason}")]
//! /// The GPU crmsd engine returned a non-zero bs_status
//! CrmsdEngine { status: i32, reason: String },
//! ```
//!
//! Every function runs on the GPU through `bioshell-crmsd-sys`; there is no
//! CPU fallback.  Inputs follow the crate's conventions: point sets are
//! `&[T: HasCartesians]` (bioshell-core/src/has_cartesians.rs:6-8), as in
//! `SubstructureAxis::from_3d_points` (calc/substructures.rs:17), equal atom
//! weights, centring on the arithmetic mean, proper rotations only.
use std::os::raw::c_void;
use std::sync::Mutex;

use bioshell_core::{HasCartesians, Matrix3x3, Vec3};
use bioshell_crmsd_sys::*;

use super::Rototranslation;
use crate::{PDBError, Structure};

impl Structure {
    /// Coordinates of the `i`-th model (structure.rs:100 keeps them as
    /// `model_coordinates: Vec<Vec<Vec3>>`), without switching the
    /// structure's atoms to that model as `set_model` does.
    pub fn model_coordinates(&self, i: usize) -> &[Vec3] { &self.model_coordinates[i] }
}

/// Options of the all-vs-all fill (mirrors `bs_opts`).
#[derive(Clone, Debug)]
pub struct CrmsdOptions {
    /// FP64 throughout (the plain method) instead of the mixed-precision path
    pub plain_fp64: bool,
    /// certified per-pair |dRMSD| bound in Angstrom; <= 0 selects 1e-4
    pub tolerance: f64,
    /// time the tile shapes of each new (chain length, size) class once
    pub autotune: bool,
    /// replay a CUDA graph captured for the call's shape
    pub graph: bool,
}

impl Default for CrmsdOptions {
    fn default() -> Self { CrmsdOptions { plain_fp64: false, tolerance: 0.0, autotune: false, graph: true } }
}

impl CrmsdOptions {
    fn to_c(&self) -> BsOpts {
        let mut o = std::mem::MaybeUninit::<BsOpts>::uninit();
        let mut o = unsafe {
            bs_opts_init(o.as_mut_ptr());
            o.assume_init()
        };
        if self.plain_fp64 { o.precision = BS_PRECISION_PLAIN64; }
        o.tolerance = self.tolerance;
        if self.autotune { o.flags |= BS_FLAG_AUTOTUNE; }
        if !self.graph { o.flags |= BS_FLAG_NO_GRAPH; }
        o
    }
}

/// All-vs-all crmsd values of n structures: the packed upper triangle
/// (i < j, row-major), the order in which `HierarchicalClusteringMatrix::new`
/// (bioshell-clustering/src/hierarchical/clustering_matrix.rs:14-19) visits the pairs.
pub struct CrmsdMatrix {
    n: usize,
    tri: Vec<f64>,
}

impl CrmsdMatrix {
    /// Number of structures.
    pub fn n(&self) -> usize { self.n }
    /// crmsd of structures i and j (0 on the diagonal).
    pub fn get(&self, i: usize, j: usize) -> f64 {
        if i == j { return 0.0; }
        let (i, j) = if i < j { (i, j) } else { (j, i) };
        self.tri[i * self.n - i * (i + 1) / 2 + (j - i - 1)]
    }
    /// The packed triangle itself.
    pub fn values(&self) -> &[f64] { &self.tri }
    /// The `Fn(usize, usize) -> f32` closure `hierarchical_clustering` takes.
    pub fn as_f32_closure(&self) -> impl Fn(usize, usize) -> f32 + '_ { move |i, j| self.get(i, j) as f32 }
}

struct Ctx(*mut BsCtx);
unsafe impl Send for Ctx {}
static CTX: Mutex<Option<Ctx>> = Mutex::new(None);

/// Runs `f` on the process's engine context (created on first use, GPU 0).
fn with_ctx<R>(f: impl FnOnce(*mut BsCtx) -> Result<R, PDBError>) -> Result<R, PDBError> {
    let mut g = CTX.lock().unwrap();
    if g.is_none() {
        let mut p = std::ptr::null_mut();
        let st = unsafe { bs_ctx_create(&mut p, 0, 0) };
        if st != BS_OK { return Err(status_error(st)); }
        *g = Some(Ctx(p));
    }
    f(g.as_ref().unwrap().0)
}

fn status_error(status: i32) -> PDBError {
    let reason = unsafe { std::ffi::CStr::from_ptr(bs_status_string(status)) }.to_string_lossy().into_owned();
    PDBError::CrmsdEngine { status, reason }
}

fn engine_error(status: i32, ctx: *const BsCtx) -> PDBError {
    let reason = unsafe { std::ffi::CStr::from_ptr(bs_last_error(ctx)) }.to_string_lossy().into_owned();
    PDBError::CrmsdEngine { status, reason }
}

/// `[n][L][3]` f64: `Vec3` has the default (Rust) representation, so a slice
/// of it is not guaranteed to be a C array of xyz triples; this copy is
/// O(nL), small next to the O(n^2 L) work.
fn pack<T: HasCartesians>(sets: &[&[T]]) -> Vec<f64> {
    let mut v = Vec::with_capacity(sets.len() * sets.first().map_or(0, |s| s.len()) * 3);
    for s in sets {
        for a in s.iter() {
            let p: &Vec3 = a.position();
            v.extend_from_slice(&[p.x, p.y, p.z]);
        }
    }
    v
}

fn check_lengths<T>(models: &[&[T]]) -> Result<(), PDBError> {
    if let Some(first) = models.first() {
        if first.is_empty() || models.iter().any(|m| m.len() != first.len()) {
            return Err(PDBError::CrmsdEngine { status: BS_ERR_INVALID_ARG,
                                               reason: "structures must hold the same, non-zero number of atoms".into() });
        }
    }
    Ok(())
}

/// crmsd of two index-matched point sets (computed on the GPU).
pub fn crmsd<T: HasCartesians>(a: &[T], b: &[T]) -> Result<f64, PDBError> {
    check_lengths(&[a, b])?;
    let xyz = pack(&[a, b]);
    with_ctx(|c| {
        let mut r = 0.0;
        let st = unsafe { bs_crmsd(c, xyz.as_ptr(), xyz.as_ptr().add(3 * a.len()), a.len() as i32, &mut r) };
        if st == BS_OK { Ok(r) } else { Err(engine_error(st, c)) }
    })
}

/// The optimal superposition of `b` onto `a` as the crate's own
/// `Rototranslation` (calc/transformation.rs:22-37): `apply` maps b_k close to
/// a_k.  Also returns the RMSD of that superposition.
pub fn superpose<T: HasCartesians>(a: &[T], b: &[T]) -> Result<(Rototranslation, f64), PDBError> {
    check_lengths(&[a, b])?;
    let xyz = pack(&[a, b]);
    with_ctx(|c| {
        let (mut rot, mut t, mut r) = ([0.0f64; 9], [0.0f64; 3], 0.0f64);
        let st = unsafe {
            bs_superpose(c, xyz.as_ptr(), xyz.as_ptr().add(3 * a.len()), a.len() as i32, rot.as_mut_ptr(),
                         t.as_mut_ptr(), &mut r)
        };
        if st != BS_OK { return Err(engine_error(st, c)); }
        Ok((Rototranslation::new(Matrix3x3::from_array(rot), Vec3::new(t[0], t[1], t[2])), r))
    })
}

/// All-vs-all crmsd of equally long models, e.g. the CA coordinates of the
/// models of a multi-model `Structure` (`model_coordinates(i)`).
pub fn crmsd_all_vs_all<T: HasCartesians>(models: &[&[T]], opts: &CrmsdOptions) -> Result<CrmsdMatrix, PDBError> {
    check_lengths(models)?;
    let n = models.len();
    let xyz = pack(models);
    let mut tri = vec![0.0f64; n * n.saturating_sub(1) / 2];
    let o = opts.to_c();
    let l = models.first().map_or(1, |m| m.len() as i32);
    with_ctx(|c| {
        let st = unsafe { bs_all_vs_all(c, xyz.as_ptr(), n as i64, l, &o, tri.as_mut_ptr() as *mut c_void) };
        if st == BS_OK { Ok(CrmsdMatrix { n, tri }) } else { Err(engine_error(st, c)) }
    })
}

/// All-vs-all crmsd of many decoy sets in one call (one persistent GPU
/// launch); set s may have its own size and chain length.
pub fn crmsd_batched<T: HasCartesians>(sets: &[&[&[T]]], opts: &CrmsdOptions) -> Result<Vec<CrmsdMatrix>, PDBError> {
    for s in sets { check_lengths(s)?; }
    let packed: Vec<Vec<f64>> = sets.iter().map(|m| pack(m)).collect();
    let mut out: Vec<CrmsdMatrix> = sets.iter()
        .map(|m| CrmsdMatrix { n: m.len(), tri: vec![0.0; m.len() * m.len().saturating_sub(1) / 2] })
        .collect();
    let descs: Vec<BsSetDesc> = sets.iter().zip(packed.iter()).zip(out.iter_mut())
        .map(|((m, x), o)| BsSetDesc { xyz: x.as_ptr(), n: m.len() as i64,
                                       l: m.first().map_or(1, |s| s.len() as i32), reserved: 0,
                                       out: o.tri.as_mut_ptr() as *mut c_void })
        .collect();
    let o = opts.to_c();
    with_ctx(|c| {
        let st = unsafe { bs_batched(c, descs.as_ptr(), descs.len() as i32, &o) };
        if st == BS_OK { Ok(()) } else { Err(engine_error(st, c)) }
    })?;
    Ok(out)
}

/// eps-neighbour lists of n models straight from the GPU (no dense matrix):
/// row i holds every j != i with crmsd <= eps, ordered by (distance, j) --
/// `CartesianPoints::neighbors_of` (bioshell-clustering/src/points_set.rs:150-169)
/// without the point itself.  CSR: row i is `col[row_ptr[i]..row_ptr[i+1]]`.
pub struct CrmsdNeighborLists {
    pub n: usize,
    pub eps: f64,
    pub row_ptr: Vec<i64>,
    pub col: Vec<i32>,
    pub dist: Vec<f32>,
}

/// The neighbour lists of `models` within `eps` (mixed precision).
pub fn crmsd_neighbors<T: HasCartesians>(models: &[&[T]], eps: f64) -> Result<CrmsdNeighborLists, PDBError> {
    check_lengths(models)?;
    let n = models.len();
    let xyz = pack(models);
    let o = CrmsdOptions::default().to_c();
    let l = models.first().map_or(1, |m| m.len() as i32);
    with_ctx(|c| {
        let mut nnz = 0i64;
        let st = unsafe { bs_neighbors(c, xyz.as_ptr(), n as i64, l, eps, &o, &mut nnz) };
        if st != BS_OK { return Err(engine_error(st, c)); }
        let mut p = CrmsdNeighborLists { n, eps, row_ptr: vec![0; n + 1], col: vec![0; nnz as usize],
                                         dist: vec![0.0; nnz as usize] };
        let st = unsafe { bs_neighbors_get(c, p.row_ptr.as_mut_ptr(), p.col.as_mut_ptr(), p.dist.as_mut_ptr()) };
        if st == BS_OK { Ok(p) } else { Err(engine_error(st, c)) }
    })
}

/// Every model of a PDB or mmCIF ensemble file as `(n_models, n_atoms,
/// [n][L][3] coordinates)`, CA atoms only when `ca` (the rules of
/// load_pdb.rs:52-115, load_cif.rs:136-168 and IsCA), read in one pass instead
/// of `Structure::from_file` and a `set_model` per model.
pub fn read_models(path: &str, ca: bool) -> Result<(usize, usize, Vec<f64>), PDBError> {
    let c = std::ffi::CString::new(path).map_err(|_| PDBError::CrmsdEngine {
        status: BS_ERR_INVALID_ARG, reason: "path contains a NUL byte".into() })?;
    let (mut h, mut n, mut l) = (std::ptr::null_mut(), 0i64, 0i32);
    let st = unsafe { bs_models_read(c.as_ptr(), 0, ca as i32, &mut h, &mut n, &mut l) };
    if st != BS_OK {
        let reason = unsafe { std::ffi::CStr::from_ptr(bs_io_last_error()) }.to_string_lossy().into_owned();
        return Err(PDBError::CrmsdEngine { status: st, reason });
    }
    let mut xyz = vec![0.0; n as usize * l as usize * 3];
    let st = unsafe {
        let st = bs_models_copy(h, xyz.as_mut_ptr());
        bs_models_free(h);
        st
    };
    if st != BS_OK { return Err(status_error(st)); }
    Ok((n as usize, l as usize, xyz))
}

/// Top-k search over a device-resident structure library, bucketed by chain
/// length, with clustering jobs mixed in (continuous batching on the GPU).
/// `submit` and `wait` may be called from any thread.
pub struct CrmsdServer {
    s: *mut BsServer,
    top_k: usize,
}
unsafe impl Send for CrmsdServer {}
unsafe impl Sync for CrmsdServer {}

/// A queued request; `rows` is the number of query structures (or models).
pub struct Ticket {
    id: i64,
    rows: usize,
}

/// Hits of every query structure: `index[r]` (library index within the
/// bucket, -1 where the bucket is smaller than k) and `rmsd[r]`, ascending.
pub struct TopK {
    pub index: Vec<Vec<i64>>,
    pub rmsd: Vec<Vec<f64>>,
}

impl CrmsdServer {
    /// `library[b]` holds the structures of bucket b, all of one chain length;
    /// the library is copied to the GPU once.
    pub fn new<T: HasCartesians>(library: &[&[&[T]]], top_k: usize, max_inflight: i32) -> Result<Self, PDBError> {
        for b in library { check_lengths(b)?; }
        let packed: Vec<Vec<f64>> = library.iter().map(|b| pack(b)).collect();
        let ls: Vec<i32> = library.iter().map(|b| b.first().map_or(1, |m| m.len() as i32)).collect();
        let ns: Vec<i64> = library.iter().map(|b| b.len() as i64).collect();
        let ptrs: Vec<*const f64> = packed.iter().map(|v| v.as_ptr()).collect();
        let cfg = BsServerConfig { nbuckets: library.len() as i32, bucket_l: ls.as_ptr(), bucket_n: ns.as_ptr(),
                                   bucket_xyz: ptrs.as_ptr(), top_k: top_k as i32, max_inflight, hbm_budget: 0,
                                   precision: BS_PRECISION_MIXED, max_batch_rows: 0, tolerance: 0.0,
                                   index_min: 0, reserved: [0; 5] };
        let mut s = std::ptr::null_mut();
        let st = unsafe { bs_server_create(&mut s, 0, &cfg) };
        if st != BS_OK { return Err(status_error(st)); }
        Ok(CrmsdServer { s, top_k })
    }

    fn error(&self, status: i32) -> PDBError {
        let reason = unsafe { std::ffi::CStr::from_ptr(bs_server_last_error(self.s)) }.to_string_lossy().into_owned();
        PDBError::CrmsdEngine { status, reason }
    }

    /// Queues the query structures (all of one bucket's chain length).
    pub fn submit<T: HasCartesians>(&self, query: &[&[T]]) -> Result<Ticket, PDBError> {
        check_lengths(query)?;
        let x = pack(query);
        let l = query.first().map_or(1, |m| m.len() as i32);
        let mut t = 0i64;
        let st = unsafe { bs_server_submit(self.s, x.as_ptr(), query.len() as i32, l, &mut t) };
        if st == BS_OK { Ok(Ticket { id: t, rows: query.len() }) } else { Err(self.error(st)) }
    }

    /// The top-k hits of every query structure of the request.
    pub fn wait(&self, t: Ticket) -> Result<TopK, PDBError> {
        let k = self.top_k;
        let (mut idx, mut val) = (vec![0i64; t.rows * k], vec![0f64; t.rows * k]);
        let st = unsafe { bs_server_wait(self.s, t.id, idx.as_mut_ptr(), val.as_mut_ptr(), 0.0) };
        if st != BS_OK { return Err(self.error(st)); }
        Ok(TopK { index: idx.chunks(k).map(|c| c.to_vec()).collect(),
                  rmsd: val.chunks(k).map(|c| c.to_vec()).collect() })
    }

    /// Cancels a request still in the queue (true); one already on the GPU
    /// runs to completion (false).  A cancelled request's wait returns
    /// `CrmsdEngine { status: BS_ERR_CANCELLED, .. }`.
    pub fn cancel(&self, t: &Ticket) -> Result<bool, PDBError> {
        let mut c = 0i32;
        let st = unsafe { bs_server_cancel(self.s, t.id, &mut c) };
        if st == BS_OK { Ok(c != 0) } else { Err(self.error(st)) }
    }

    /// An all-vs-all + OPTICS job over `models` (optics.rs:51-148);
    /// `wait_cluster` returns the OPTICS cluster index of every model.
    pub fn submit_cluster<T: HasCartesians>(&self, models: &[&[T]], eps: f64, min_points: i32)
                                            -> Result<Ticket, PDBError> {
        check_lengths(models)?;
        let x = pack(models);
        let l = models.first().map_or(1, |m| m.len() as i32);
        let mut t = 0i64;
        let st = unsafe { bs_server_submit_cluster(self.s, x.as_ptr(), models.len() as i64, l, eps, min_points, &mut t) };
        if st == BS_OK { Ok(Ticket { id: t, rows: models.len() }) } else { Err(self.error(st)) }
    }

    pub fn wait_cluster(&self, t: Ticket) -> Result<Vec<i64>, PDBError> {
        let mut cl = vec![0i64; t.rows];
        let st = unsafe { bs_server_wait_cluster(self.s, t.id, cl.as_mut_ptr(), 0.0) };
        if st == BS_OK { Ok(cl) } else { Err(self.error(st)) }
    }

    /// Latency percentiles (p50/p99) and pairs/s since the last reset.
    pub fn stats(&self) -> BsServerStats {
        let mut st = BsServerStats::default();
        unsafe { bs_server_get_stats(self.s, &mut st) };
        st
    }
}

impl Drop for CrmsdServer {
    fn drop(&mut self) { unsafe { bs_server_destroy(self.s) } }
}
