// kernels.h -- data layout, device-side job descriptors and launch wrappers
// shared between the kernel translation units and the C-ABI layer.  Internal
// to the library.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace bs {

// ---------------------------------------------------------------- layout
// Digit matrices: one row per (structure, coordinate), `pitch` bf16 columns
// (atoms; a job uses the first lp = L rounded up to 16, zero padded).
// Structures are packed ten to a 32-row group, four groups to a 128-row
// block, so that a tensor-core A tile of 128 rows holds 40 whole structures
// (B tiles: 64 rows, 20 structures) and each structure's three rows sit in
// one warp's TMEM lanes.  Within a group, structures 0-4 take rows 0-14 and
// structures 5-9 rows 16-30 (rows 15 and 31 are zero): each half of a group
// is then one aligned 16-column TMEM load in the epilogue.  Structures are
// numbered globally across the jobs of one launch; every job starts on a
// 40-structure block boundary.
constexpr int kGroupRows = 32;
constexpr int kGroupStructs = 10;
constexpr int kBlockRows = 128;
constexpr int kBlockStructs = 40;
constexpr int kBStructs = 20;
constexpr int kKChunk = 64;  // atoms per 128-byte swizzled TMA box row

// row of coordinate c of structure s (0..9) within its group
__host__ __device__ inline int group_row(int s, int c) { return 3 * s + (s >= 5 ? 1 : 0) + c; }
__host__ __device__ inline int64_t digit_row(int64_t s, int c) {
  return (s / kGroupStructs) * kGroupRows + group_row((int)(s % kGroupStructs), c);
}
inline int64_t blocks_for(int64_t n) { return (n + kBlockStructs - 1) / kBlockStructs; }
inline int lp_for(int L) { return ((L + 15) / 16) * 16; }
inline int pitch_for(int L) { return ((L + kKChunk - 1) / kKChunk) * kKChunk; }

// Fixed-point unit of the preparation pass: coordinates are read as
// integers in units of 2^-32 Angstrom.
constexpr int kFixBits = 32;

// Per-structure data of the mixed path (one 16-byte load per structure).
struct __align__(16) SInfo {
  long long ghat;  // exact sum of squared quantised coordinates (units u)
  float gf;        // ghat as float
  float qres;      // RMS of the quantisation residual y - 2^e n (Angstrom, rounded up)
};

// Output description shared by every kernel that writes pair values.
struct OutDesc {
  void *ptr;     // neighbour layout: a NbrSink in device memory
  int64_t n;     // rows
  int64_t ld;    // row stride of the square / rectangular layouts
  int layout;    // 0 packed triangle, 1 square (both halves), 2 rectangular n x ld, 3 neighbour pairs
  int out_type;  // 0 f64, 1 f32
  float eps;     // neighbour layout: pairs with crmsd <= eps are kept
  int pad;
};
constexpr int kLayoutTriangle = 0;
constexpr int kLayoutSquare = 1;
constexpr int kLayoutRect = 2;
constexpr int kLayoutNeighbors = 3;

// Where the neighbour layout appends: every kept pair i < j of a job as the
// two entries (i, j, d) and (j, i, d), job-local indices; `count` may end
// above `cap` (the entries past cap are dropped and the caller retries).
struct NbrSink {
  unsigned long long *count;
  unsigned long long cap;
  int2 *ij;
  float *d;
};

// One block of pairs of a launch: all pairs i < j of one structure set
// (symmetric), or every pair of a query set against a library range
// (rectangular).  The host fills the first part; the preparation kernels
// fill the second on the device, so the whole call sequence needs no host
// round trip (and can be captured in a CUDA graph).
struct __align__(16) Job {  // 16-byte multiple: the tensor-core kernel bulk-copies it
  // ---- host
  const double *xyz;      // [n][L][3] f64 AoS of the A-side structures (device)
  long long n;            // A-side structures
  long long first_a;      // global index of A structure 0 (multiple of 40)
  long long first_b;      // global index of B structure 0 (multiple of 20)
  long long n_b;          // B-side structures (symmetric: n)
  OutDesc out;
  int L, lp;              // atoms; digit columns used (L rounded up to 16)
  int mode;               // 0 symmetric, 1 rectangular
  int fixed_scale;        // 1: grid exponent given (scale_min), no candidate search
  int scale_min;          // smallest grid exponent allowed
  float tol;              // certified |dRMSD| budget per pair (Angstrom)
  // B-side digit norms for rectangular jobs with a fixed grid (the
  // library's maxima, per digit), used in the exactness bound
  float norm_b[3];
  float qres_b;           // largest B-side quantisation residual RMS
  int screen;             // 1: rectangular screen job (bounds from the leading levels)
  int narrow;             // 1: tiles of 40 x 10 structures (MMA N = 32) instead of 40 x 20
  // ---- device (preparation)
  unsigned long long maxabs;        // max |centred coordinate|, fixed-point units
  unsigned long long norm[4][3];    // per candidate grid: max row sum of squared digits (d0, d1, d2)
  unsigned long long normh[4][3];   // per candidate grid: max over rows and halves of the half-row sums
  unsigned long long normq[4][3];   // the same over quarters (the parts of a long-layout tile)
  unsigned int qres_max_bits;       // largest A-side quantisation residual RMS (float bits)
  int scale_base;                   // grid of candidate 0
  int scale_exp;                    // chosen grid exponent e
  int err;                          // kErr* bits of this job
  float u;                          // Angstrom^2 per unit of quantised products (2^2e)
  float d34;                        // rounding bound of accumulator levels 2-3, as an error of E (units u)
  int layout;                       // accumulator layout of the job's tiles (kAcc*)
  int allow_long;                   // (host) the long layout may be chosen
  int pad2;
};

// Accumulator layouts of a tile.  Normal: the four levels, one 64-column
// accumulator each, in one TMEM buffer.  Long (long chains): eight
// accumulators over both buffers -- level 0 over the whole chain, level 1
// in two and level 2 in four consecutive parts of the chain (16-atom steps
// split evenly), level 3 whole -- so that each part's sum stays below 2^24
// where the whole chain's would not.
constexpr int kAccNormal = 0;
constexpr int kAccLong = 1;
// Screen tiles: only the leading digit products (levels 0 and 1, three per
// 16-atom step, digits 0 and 1 of each side) and an FP32 epilogue writing
// crmsd bounds -- the first stage of top-k queries.
constexpr int kAccScreen = 2;
// Half (chains up to about twice the normal layout's reach): the four levels
// accumulated separately over each half of the chain (16-atom steps split
// evenly), [L0 | L1 | L2 | L3] of the first half in one TMEM buffer and of
// the second half in the other.  Each half's sums stay below 2^24 where the
// whole chain's would not, and each half keeps the normal layout's column
// order, so one MMA still covers several levels.
constexpr int kAccHalf = 3;
__host__ __device__ inline int acc_part(int k16, int nk16, int parts) { return (k16 * parts) / nk16; }
// layouts whose tile takes both TMEM buffers
__host__ __device__ inline bool acc_two_buffers(int layout) { return layout == kAccLong || layout == kAccHalf; }
// accumulator index (0..7) of level `lv` at 16-atom step k16
__host__ __device__ inline int acc_index(int layout, int lv, int k16, int nk16) {
  if (layout == kAccNormal) return lv;
  if (layout == kAccHalf) return 4 * acc_part(k16, nk16, 2) + lv;
  if (lv == 0) return 0;
  if (lv == 1) return 1 + acc_part(k16, nk16, 2);
  if (lv == 2) return 3 + acc_part(k16, nk16, 4);
  return 7;
}

// Counters shared by the kernels of one launch.
struct DevScalars {
  unsigned long long flag_count;  // pairs queued for exact recomputation
  int err;                        // kErr* bits not tied to one job
  int pad;
  unsigned long long flag_done;   // queue entries already recomputed (banded launches)
  unsigned long long tile_next;   // next tile of the running k_mixed_tc launch (zero before each)
};
constexpr int kErrTimeout = 1;
constexpr int kErrNonFinite = 2;
constexpr int kErrBounds = 4;
constexpr int kErrInternal = 8;
constexpr int kErrUnsupported = 16;  // no grid meets the exactness bound / coordinates out of range

// Flag entries: job (16 bits) | global i (24 bits) | global j (24 bits).
constexpr int64_t kMaxGlobalStructs = 1ll << 24;
__host__ __device__ inline unsigned long long flag_pack(int job, int64_t i, int64_t j) {
  return ((unsigned long long)job << 48) | ((unsigned long long)i << 24) | (unsigned long long)j;
}

// Tensor-core tile: A block (40 structures), B block (20 structures; 10 for
// a narrow job's tiles), job, and the job's shape (16-atom steps | layout <<
// 16 | narrow << 24), written on the device once the preparation has chosen
// the layout, so that the TMA and MMA threads read one record per tile.
struct __align__(16) Tile {
  int a_blk, b_blk, job, shape;
};
__host__ __device__ inline int tile_nk16(const Tile &t) { return t.shape & 0xffff; }
__host__ __device__ inline int tile_layout(const Tile &t) { return (t.shape >> 16) & 0xff; }
__host__ __device__ inline bool tile_narrow(const Tile &t) { return (t.shape >> 24) & 1; }
constexpr int kNarrowStructs = 10;  // B structures of a narrow tile (one 32-row group)

// ------------------------------------------------------------- launches
// prep.cu -- mixed path, all jobs of a launch at once
struct PrepArgs {
  Job *jobs;
  int njobs;
  const int *job_of_struct_block;  // job of each 40-structure block (A side)
  int64_t nblocks;                 // 40-structure blocks
  long long *ctr;                  // fixed-point centroid per global structure [3]
  __nv_bfloat16 *dig[4];           // e0, e1, e2 = 16 d2, d2 / 32
  int64_t pitch;
  SInfo *info;
  // optional (screen jobs): per structure {G of the coordinates without
  // digit 2, RMS of digit 2 in Angstrom} -- the truncated structure the
  // screen's levels 0 and 1 describe, and its distance from the full one
  float2 *tinfo;
  DevScalars *sc;
  // structures [s_lo, s_hi) only (s_hi < 0: all), and of the per-job
  // kernels only the jobs whose first structure lies there: the preparation
  // of one band of a banded call
  int64_t s_lo = 0, s_hi = -1;
};
cudaError_t launch_prep_mixed(const PrepArgs &p, cudaStream_t st);
int prep_max_pitch();
cudaError_t prep_prepare();

// plain path (single set, FP64 throughout)
cudaError_t launch_prep_plain(const double *xyz, int64_t n, int L, int lp, double *ctr, double *y, double *g,
                              int *err, cudaStream_t st);

// plain64.cu
cudaError_t launch_plain64_all(const double *y, const double *g, int64_t n, int L, int lp, OutDesc out,
                               cudaStream_t st);
cudaError_t launch_plain64_pairs(const double *y, const double *g, int64_t n, int L, int lp, const int64_t *ii,
                                 const int64_t *jj, int64_t np, double *out, cudaStream_t st);
cudaError_t launch_plain64_rect(const double *ya, const double *ga, int64_t na, const double *yb, const double *gb,
                                int64_t nb, int L, int lp, OutDesc out, cudaStream_t st);

// mixed_tc.cu
struct TcArgs {
  const Tile *tiles;
  int64_t ntiles;
  const Job *jobs;
  const SInfo *info_a;
  const SInfo *info_b;
  const float2 *tinfo_a;  // screen jobs: truncated-structure data (PrepArgs::tinfo)
  const float2 *tinfo_b;
  DevScalars *sc;
  unsigned long long *flags;
  unsigned long long flag_cap;
  float *dbg;  // optional dump of the raw level sums of tiles (0,0) and (0,1)
  int num_sms;
  uint64_t wait_ns;  // bound of each pipeline wait (0: the kernel's default); a test hook
};
cudaError_t launch_mixed_tc(const CUtensorMap *tm /* [7]: A digits e0 e1 e2 d2/32, B digits e0 e1 e2 */,
                            const TcArgs &a, cudaStream_t st);
// writes every tile's shape from its job (after the preparation)
cudaError_t launch_tile_shapes(Tile *tiles, int64_t ntiles, const Job *jobs, int num_sms, cudaStream_t st);
size_t mixed_tc_smem_bytes();
cudaError_t mixed_tc_prepare();
// screen_tc.cu -- the same for launches whose tiles are all screen tiles
// (tensor maps 0, 1, 4, 5 of the seven).  strips: a.tiles holds strip
// records {query block, first library block, job, nk16 | count << 16} (chains
// of at most screen_strip_max_nk16() 16-atom steps); else screen tiles.
cudaError_t launch_screen_tc(const CUtensorMap *tm, const TcArgs &a, bool strips, cudaStream_t st);
// superpose.cu -- for each pair (pi[p], pj[p]) of xyz[n][L][3]: rot[p] (3x3
// row-major), trans[p] with rot x_j + trans ~ x_i, and the RMSD of that
// superposition (rmsd may be null); bad indices set kErrBounds, non-finite
// input kErrNonFinite in *err.
cudaError_t launch_superpose(const double *xyz, int64_t n, int L, const int64_t *pi, const int64_t *pj, int64_t np,
                             double *rot, double *trans, double *rmsd, int *err, int num_sms, cudaStream_t st);
cudaError_t screen_tc_prepare();
int screen_strip_max_nk16();

// refine.cu
struct DigitsView {
  const __nv_bfloat16 *d0, *d1, *d2;
  int64_t pitch;
};
struct RefineArgs {
  DigitsView da, db;
  const SInfo *info_a, *info_b;
  const Job *jobs;
  int njobs;
  DevScalars *sc;
  const unsigned long long *flags;
  unsigned long long cap;
  int num_sms;
  // banded launches: queue entries from sc->flag_done on are new; `mark`
  // advances flag_done afterwards, and the overflow scan covers only the
  // output elements [scan_lo, scan_hi) of job 0 (scan_hi < 0: everything)
  bool mark = false;
  int64_t scan_lo = 0, scan_hi = -1;
};
// exact recomputation of the queued pairs; then, only when the queue
// overflowed (checked on the device), of every sentinel left in the outputs
cudaError_t launch_refine(const RefineArgs &r, cudaStream_t st);
// Certified crmsd of the screen candidates of rectangular jobs: row r is
// global A structure row_ig[r] of job row_job[r]; candidate c of the row is
// B structure cand_j[r * cap + c] (c < min(cand_n[r], cap)); values go to
// cand_v[r * cap + c].
cudaError_t launch_exact_candidates(const DigitsView &da, const DigitsView &db, const SInfo *info_a,
                                    const SInfo *info_b, const Job *jobs, const int *row_job, const int64_t *row_ig,
                                    int64_t rows, const int *cand_j, const int *cand_n, int cap, float *cand_v,
                                    cudaStream_t st);
// CUDA-core level sums + the same epilogue for an explicit pair list of job 0
// (used for sparse pair lists and as the tensor-core path's independent check)
cudaError_t launch_mixed_pairs(const DigitsView &dg, const SInfo *info, const Job *job, DevScalars *sc,
                               const int64_t *ii, const int64_t *jj, int64_t np, double *out, float *levels_out,
                               cudaStream_t st);

// topk.cu -- per row of a dense [rows][ld] f32 block: the k <= kTopkMax
// smallest of the first n values, ascending by (value, library index), the
// library index of column c being perm[c] (perm may be null: c); results
// report library indices, and entries that do not exist come back as -1.
constexpr int kTopkMax = 64;
cudaError_t launch_topk(const float *vals, int64_t rows, int64_t n, int64_t ld, int k, const int *perm,
                        int64_t *out_idx, float *out_val, cudaStream_t st);
// The same with a per-row count of valid values (row_n[r] <= n) and a map
// from position to column (col_map[r * ld + c]; may be null).
cudaError_t launch_topk_rows(const float *vals, int64_t rows, const int *row_n, int64_t ld, int k,
                             const int *col_map, const int *perm, int64_t *out_idx, float *out_val, cudaStream_t st);
// Screen candidates from the packed brackets of a screen job (one word per
// pair: hi rounded up to half precision in the top 16 bits, lo rounded down
// in the bottom 16).  Per row r: T[r] = an upper bound of the row's k-th
// smallest hi -- the top edge of the bin of the 4096-bin histogram of hi
// (bins of 1/64 of an octave) that holds it -- then every column c with
// lo[r][c] <= T[r], up to cap per row (cand_n[r] counts all, so
// cand_n[r] > cap marks an overflowing row).  hist ([rows][4096] u32),
// thresholds ([rows] u32) and cand_n are scratch the call clears itself.
constexpr int kScreenBins = 4096;

// hier.cu -- hierarchical clustering of a packed triangle on the device (one
// cooperative launch; merges[n-1][4] and merge_dist[n-1] device buffers)
size_t hier_workspace_bytes(int64_t n, int grid);
int hier_grid(int num_sms);
// *err_out: a device int, 0 after a complete run, else 1 + the phase whose
// grid barrier timed out (100: an inconsistent merge pair)
cudaError_t launch_hierarchical(const void *tri, int out_type, int64_t n, int rule, void *ws, int grid,
                                int64_t *merges, float *merge_dist, int **err_out, uint64_t wait_ns, cudaStream_t st);

// neighbors.cu -- CSR rows (ordered by (d, j), without i itself) from the
// cnt entries a neighbour-layout launch appended.  scratch_rows: 2n words;
// key, tmp: cnt words each.
cudaError_t launch_neighbors_csr(const int2 *ij, const float *d, int64_t cnt, int64_t n, int num_sms,
                                 int64_t *row_ptr, int32_t *col, float *dist, unsigned long long *scratch_rows,
                                 unsigned long long *key, unsigned long long *tmp, cudaStream_t st);
// A row-block segment of a pruned screen's brackets: rows r0 .. r0 + nr - 1,
// columns [c0, c1) (at most screen_select_chunk(), c0 a multiple of 4).
struct SelSeg {
  int64_t r0;
  int nr, pad;
  int64_t c0, c1;
};
int screen_select_chunk();
// launch_screen_select over the listed segments only (the rest of each row
// is never read); max_rows bounds nr.
cudaError_t launch_screen_select_seg(const uint32_t *packed, int64_t rows, int64_t ld, int k, int cap,
                                     const SelSeg *segs, int64_t nsegs, int max_rows, uint32_t *hist,
                                     uint32_t *thresholds, int *cand_j, int *cand_n, cudaStream_t st);
cudaError_t launch_screen_select(const uint32_t *packed, int64_t rows, int64_t n, int64_t ld, int k, int cap,
                                 uint32_t *hist, uint32_t *thresholds, int *cand_j, int *cand_n, cudaStream_t st);

}  // namespace bs
