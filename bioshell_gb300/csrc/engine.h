// engine.h -- internals shared by the C-ABI layer (api.cu), the serving loop
// (server.cu) and the allocation-free entry point (noalloc.cu): device
// workspaces, the mixed-path launch plan, the graph cache and the call
// sequence.  Not part of the public interface.
#pragma once
#include <cudaTypedefs.h>

#include <map>
#include <string>
#include <vector>

#include "../../include/bioshell_crmsd.h"
#include "kernels.h"

namespace bs {

struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
};

// Device buffers of one mixed-path launch.  The A side holds the jobs' own
// structures; the B side is the same buffers for symmetric jobs, or a
// resident library's for rectangular ones.
struct MixedBuffers {
  long long *ctr = nullptr;  // [structures][3] fixed-point centroids
  SInfo *info_a = nullptr;
  const SInfo *info_b = nullptr;
  float2 *tinfo_a = nullptr;  // screen jobs only
  const float2 *tinfo_b = nullptr;
  __nv_bfloat16 *dig_a[4] = {};
  const __nv_bfloat16 *dig_b[3] = {};
  int64_t pitch_a = 0, pitch_b = 0;  // digit row length (atoms)
  int64_t rows_a = 0, rows_b = 0;    // digit rows allocated
  Job *jobs = nullptr;
  int *jobmap = nullptr;  // job of each 40-structure A block
  Tile *tiles = nullptr;
  unsigned long long *flags = nullptr;
  unsigned long long flag_cap = 0;
  DevScalars *sc = nullptr;
  uint64_t wait_ns = 0;  // bound of the tensor-core kernels' pipeline waits (0: their default)
};

// A symmetric job as the host describes it (device coordinates and output;
// narrow: 40 x 10 tiles, chosen by the autotuner for small sets).
struct JobSpec {
  const double *xyz;
  int64_t n;
  int L;
  OutDesc out;
  int narrow = 0;
  int64_t row_lo = 0, row_hi = -1;  // rows of the pairs to compute (multiples of 40, or n); -1: all
};

struct Plan {
  // overflow scan of the recomputation (non-banded launches): output
  // elements [scan_lo, scan_hi) of job 0, or everything (scan_hi < 0)
  int64_t scan_lo = 0, scan_hi = -1;
  std::vector<Job> jobs;  // host part filled, device part zero
  std::vector<int> jobmap;
  std::vector<Tile> tiles;
  int64_t nblocks = 0;  // 40-structure A blocks
  int pitch = 0;
  bool strips = false;  // screen plan whose `tiles` are strip records (launch_screen_tc)
};

// Builds the jobs, block map and tile table of symmetric jobs.  Tiles of the
// longest chains come first so that the persistent kernel ends with short
// tiles; within a job they run in super-blocks that keep the working set in
// L2.  Returns an empty string on success, else the reason.
std::string make_symmetric_plan(const std::vector<JobSpec> &specs, float tol, bool with_tiles, Plan &plan);

// The seven tensor maps (A digits e0 e1 e2 d2/32, B digits e0 e1 e2).
std::string encode_maps(PFN_cuTensorMapEncodeTiled_v12000 encode, const MixedBuffers &b, CUtensorMap tm[7]);
std::string get_encoder(PFN_cuTensorMapEncodeTiled_v12000 *out);

// Read-back of one symmetric job's packed triangle in row bands, each band
// copied to pinned host memory on a second stream while the next computes.
// Band k is tiles [tile_end[k-1], tile_end[k]) of the plan (whole super-rows
// of A blocks, so its rows are complete when they and their recomputations
// are done) and output elements [elem_end[k-1], elem_end[k]).
struct Readback {
  std::vector<int64_t> tile_end, elem_end;
  const char *dev = nullptr;
  char *host = nullptr;
  size_t esz = 0;
  cudaStream_t copy = nullptr;
  const cudaEvent_t *ev = nullptr;  // tile_end.size() + 1 events
  // many sets (batched): band k ends at tile_end[k] on a set boundary and
  // copies the outputs of its sets (copies[k]); elem_end is unused, and the
  // overflow scan of each band covers every set
  struct Copy {
    const char *dev;
    char *host;
    size_t bytes;
  };
  std::vector<std::vector<Copy>> copies;
  // ... and, when their inputs are in pinned host memory, the uploads of
  // each band's sets (on `upload`, band k signalling up_ev[k]) and the end
  // of each band's structure range: each band is prepared after its upload,
  // so the uploads of later bands overlap the work of earlier ones
  struct Upload {
    char *dev;
    const char *host;
    size_t bytes;
  };
  std::vector<std::vector<Upload>> uploads;
  std::vector<int64_t> struct_end;
  cudaStream_t upload = nullptr;
  const cudaEvent_t *up_ev = nullptr;  // tile_end.size() events
};

// Band boundaries for many symmetric jobs whose tiles lie job by job in the
// plan (make_symmetric_plan): bands end on job boundaries, about `bands`
// bands of equal pair counts with the last ones halved, as make_bands does.
void make_set_bands(const Plan &plan, int bands, Readback &rb);

// Band boundaries for a single symmetric job of n structures: whole
// super-rows, about `bands` bands of equal pair counts, the last two bands'
// worth split in halves down to a sixteenth of a band (the last band's copy
// is the part of the read-back that no computation hides).
void make_bands(const Plan &plan, int64_t n, int bands, Readback &rb);

// Enqueues the mixed-path sequence of a plan whose tables are on the
// device: counters reset, job table upload from `job_stage` (pinned or
// pageable; pinned when captured), preparation, tensor-core tiles, exact
// recomputation.  `ev` (optional, 4 events) marks prep / main / refine
// boundaries; `capturing` records them as graph event nodes.  With `rb`
// (not captured) the tiles run band by band and each band is read back
// as soon as it is final; the stream waits for the last copy.
cudaError_t enqueue_mixed(const Plan &plan, const MixedBuffers &b, const Job *job_stage, const CUtensorMap tm[7],
                          int num_sms, cudaStream_t st, cudaEvent_t *ev, bool capturing, float *dbg = nullptr,
                          const Readback *rb = nullptr);

// Maps the device error bits of a finished launch to a status and message.
bs_status collect_errors(const DevScalars &sc, const Job *jobs, int njobs, std::string &msg);

}  // namespace bs

struct bs_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[6] = {};
  // banded read-back of large results: its copy stream and band events
  cudaStream_t copy_stream = nullptr;
  std::vector<cudaEvent_t> band_ev;
  // banded uploads of many sets' inputs: their stream and band events
  cudaStream_t upload_stream = nullptr;
  std::vector<cudaEvent_t> up_ev;
  size_t budget = 0;
  size_t used = 0;
  uint64_t gen = 0;  // bumped whenever a workspace moves (graphs hold addresses)
  std::string err;
  bs_metrics metrics{};
  // workspaces
  bs::DevBuf xyz, out, ctr, info, dig[4], jobs, jobmap, tiles, flags, scal, y, g, ctrd, pairs_i, pairs_j, pout;
  // eps-neighbour lists: appended pairs, then the CSR of the last bs_neighbors
  bs::DevBuf nbr_sink, nbr_count, nbr_ij, nbr_d, nbr_rows, nbr_key, nbr_tmp, nbr_rowptr, nbr_col, nbr_dist;
  int64_t nbr_n = -1, nbr_nnz = 0;
  // hierarchical clustering on the device: workspace, staged triangle, results
  bs::DevBuf hier_ws, hier_tri, hier_out;
  // superposition results staged for host outputs: rot, trans, rmsd per pair
  bs::DevBuf sp_out;
  unsigned long long nbr_cap_hint = 0;
  void *job_stage = nullptr;  // pinned host copy of the job table
  size_t job_stage_cap = 0;
  void *job_back = nullptr;  // pinned read-back of the job table
  bs::DevScalars *sc_back = nullptr;
  // cached tables of the last plan
  std::vector<int64_t> plan_key;
  // host tile table of the last symmetric plan, reused by a call whose jobs
  // have the same sizes, chain lengths, tile shapes and row ranges; and the
  // row bands of its banded read-back
  std::vector<bs::Tile> tile_cache;
  std::vector<int64_t> tile_key;
  std::vector<int64_t> band_key, band_tile_end, band_elem_end;
  // graph cache
  struct Graph {
    std::vector<int64_t> key;
    cudaGraphExec_t exec = nullptr;
    uint64_t last = 0;
  };
  std::vector<Graph> graphs;
  uint64_t tick = 0;
  PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  // autotuner: shape class (64-atom chain bucket, log2 size) -> narrow tiles
  std::map<int64_t, int> tune;
  // test hooks (bs_debug_set_wait_limit, bs_debug_fail_alloc)
  uint64_t wait_limit_ns = 0;     // 0: the kernels' default bounds
  int64_t fail_alloc_after = -1;  // allocations left before an injected failure (-1: off)
};

namespace bs {
bs_status set_err(bs_ctx *ctx, bs_status s, const char *fmt, ...);
bs_status cuda_err(bs_ctx *ctx, cudaError_t e, const char *what);
bs_status ensure(bs_ctx *ctx, DevBuf &b, size_t bytes, const char *what);
void release(bs_ctx *ctx, DevBuf &b);
bool is_device_ptr(const void *p);
bool is_pinned_host(const void *p);
}  // namespace bs
