//! OPTICS and hierarchical clustering over crmsd values from the GB300 engine.
//!
//! This file goes to `bioshell-clustering/src/crmsd_points.rs`, with
//! `pub mod crmsd_points;` in `lib.rs` and `bioshell-pdb = { path = "../bioshell-pdb" }`
//! in `bioshell-clustering/Cargo.toml` (bioshell-datastructures, which
//! bioshell-clustering already depends on, depends on bioshell-pdb itself).
//! The impls live here, beside the traits (points_set.rs:29-62), because the
//! orphan rule forbids them in bioshell-pdb and bioshell-pdb cannot depend
//! on bioshell-clustering.
//!
//! Hierarchical clustering needs no type of its own: the matrix replaces the
//! n(n-1)/2 closure calls of `HierarchicalClusteringMatrix::new`
//! (hierarchical/clustering_matrix.rs:11-22):
//!
//! ```text
//! let m = crmsd_all_vs_all(&models, &CrmsdOptions::default())?;
//! let tree = hierarchical_clustering(m.n(), m.as_f32_closure(), &single_link);
//! ```
use bioshell_pdb::calc::{CrmsdMatrix, CrmsdNeighborLists};

use crate::optics::OpticsPoints;
use crate::{DistanceByIndex, Neighbor, NeighborsOf};

/// OPTICS points backed by a dense crmsd matrix (owned, so that
/// `Box<dyn OpticsPoints>` is 'static).
pub struct CrmsdPoints(pub CrmsdMatrix);

impl DistanceByIndex for CrmsdPoints {
    fn distance(&self, i: usize, j: usize) -> f64 { self.0.get(i, j) }
    fn count_points(&self) -> usize { self.0.n() }
}

impl NeighborsOf for CrmsdPoints {
    /// The semantics of `CartesianPoints::neighbors_of` (points_set.rs:150-169):
    /// the point itself included, every point with d <= cutoff kept, ordered
    /// by a stable sort on the distance of an ascending-index scan.
    fn neighbors_of(&self, idx: usize, cutoff: f64) -> Vec<Neighbor> {
        let mut out: Vec<Neighbor> = (0..self.0.n())
            .map(|j| Neighbor { idx: j, d: self.0.get(idx, j) })
            .filter(|n| n.d <= cutoff)
            .collect();
        out.sort_by(|a, b| a.d.partial_cmp(&b.d).unwrap());
        out
    }
}

impl OpticsPoints for CrmsdPoints {}

/// OPTICS points backed by the GPU's eps-neighbour lists: no dense matrix,
/// so ensembles far beyond what an n x n matrix allows.  Distances beyond the
/// lists' eps are unknown and read as infinite; OPTICS asks for neighbours
/// within its own eps only, which must not exceed the lists' eps.
pub struct CrmsdNeighborPoints(pub CrmsdNeighborLists);

impl DistanceByIndex for CrmsdNeighborPoints {
    fn distance(&self, i: usize, j: usize) -> f64 {
        if i == j { return 0.0; }
        let l = &self.0;
        let (b, e) = (l.row_ptr[i] as usize, l.row_ptr[i + 1] as usize);
        l.col[b..e].iter().position(|&c| c as usize == j).map_or(f64::INFINITY, |k| l.dist[b + k] as f64)
    }
    fn count_points(&self) -> usize { self.0.n }
}

impl NeighborsOf for CrmsdNeighborPoints {
    /// The row as the engine orders it, (d, j), with the point itself put
    /// where the stable sort of an ascending scan places it: at distance 0,
    /// after every j < idx at distance 0.
    fn neighbors_of(&self, idx: usize, cutoff: f64) -> Vec<Neighbor> {
        let l = &self.0;
        let (b, e) = (l.row_ptr[idx] as usize, l.row_ptr[idx + 1] as usize);
        let mut out = Vec::with_capacity(e - b + 1);
        let mut self_done = false;
        for k in b..e {
            let (j, d) = (l.col[k] as usize, l.dist[k] as f64);
            if d > cutoff.min(l.eps) { break; }
            if !self_done && (d > 0.0 || j > idx) {
                out.push(Neighbor { idx, d: 0.0 });
                self_done = true;
            }
            out.push(Neighbor { idx: j, d });
        }
        if !self_done { out.push(Neighbor { idx, d: 0.0 }); }
        out
    }
}

impl OpticsPoints for CrmsdNeighborPoints {}
