// kernels.h -- launch wrappers shared between the kernel translation units
// and the C-ABI layer.  Internal to the library.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace bs {

// ---------------------------------------------------------------- layout
// Digit matrices: one row per (structure, coordinate), `lp` bf16 columns
// (atoms, zero padded to a multiple of 16).  Structures are packed ten to a
// 32-row group (rows 30 and 31 of each group are zero), four groups to a
// 128-row block, so that a tensor-core A tile of 128 rows holds 40 whole
// structures (B tiles: 64 rows, 20 structures) and each structure's three
// rows sit in one warp's TMEM lanes.
constexpr int kGroupRows = 32;
constexpr int kGroupStructs = 10;
constexpr int kBlockRows = 128;
constexpr int kBlockStructs = 40;

__host__ __device__ inline int64_t digit_row(int64_t s, int c) {
  return (s / kGroupStructs) * kGroupRows + (s % kGroupStructs) * 3 + c;
}
inline int64_t blocks_for(int64_t n) { return (n + kBlockStructs - 1) / kBlockStructs; }
inline int lp_for(int L) { return ((L + 15) / 16) * 16; }

// Per-structure data of the mixed path (one 16-byte load per structure).
struct __align__(16) SInfo {
  long long ghat;  // exact sum of squared quantised coordinates (units u)
  float gf;        // ghat as float
  float qres;      // RMS of the quantisation residual y - 2^e n (Angstrom, rounded up)
};

// Scalars the kernels exchange through device memory.
struct DevScalars {
  unsigned long long maxabs_bits;   // max |centred coordinate| (double bits)
  unsigned long long norm_max[3];   // max over (structure, coord) of sum d_i^2
  unsigned long long flag_count;    // pairs queued for exact recomputation
  unsigned long long qres_max_bits; // max per-structure quantisation residual RMS (float bits)
  int scale_exp;                    // grid exponent e (coordinates in units 2^e A)
  int err;                          // error bits (kErr*)
  int scale_min;                    // lower bound on e requested by the host
  int pad;
};
constexpr int kErrTimeout = 1;
constexpr int kErrNonFinite = 2;
constexpr int kErrBounds = 4;
constexpr int kErrInternal = 8;

// Output description shared by every kernel that writes pair values.
struct OutDesc {
  void *ptr;
  int64_t n;
  int layout;    // 0 triangle, 1 square
  int out_type;  // 0 f64, 1 f32
};

// ------------------------------------------------------------- launches
// prep.cu
cudaError_t launch_prep_stats(const double *xyz, int64_t n, int L, double *ctr, DevScalars *sc,
                              cudaStream_t st);
cudaError_t launch_prep_scale(DevScalars *sc, cudaStream_t st);
// dig[0..3]: e0, e1, e2 = 16 d2, and d2 / 32 (the level-4 operand)
cudaError_t launch_prep_digits(const double *xyz, const double *ctr, int64_t n, int L, int lp,
                               __nv_bfloat16 *const *dig, SInfo *info, DevScalars *sc, cudaStream_t st);
cudaError_t launch_prep_plain(const double *xyz, const double *ctr, int64_t n, int L, int lp, double *y,
                              double *g, cudaStream_t st);

// plain64.cu
cudaError_t launch_plain64_all(const double *y, const double *g, int64_t n, int L, int lp, OutDesc out,
                               cudaStream_t st);
cudaError_t launch_plain64_pairs(const double *y, const double *g, int64_t n, int L, int lp, const int64_t *ii,
                                 const int64_t *jj, int64_t np, double *out, cudaStream_t st);

// mixed_tc.cu
struct TcArgs {
  const int2 *tiles;
  int64_t ntiles;
  int64_t n;
  int L, lp;
  const SInfo *info;
  DevScalars *sc;
  float tol;  // certified |dRMSD| budget per pair (Angstrom)
  float u;    // Angstrom^2 per unit of the quantised products
  float d34;  // level-3 accumulator rounding bound, as an error of E (units u)
  OutDesc out;
  unsigned long long *flags;
  unsigned long long flag_cap;
  float *dbg;  // optional dump of the first tile's raw level sums
  int num_sms;
};
cudaError_t launch_mixed_tc(const CUtensorMap *tm /* [7]: A digits e0 e1 e2 d2/32, B digits e0 e1 e2 */,
                            const TcArgs &a, cudaStream_t st);
size_t mixed_tc_smem_bytes();

// refine.cu
cudaError_t launch_refine_list(__nv_bfloat16 *const *dig, int lp, int L, const SInfo *info, DevScalars *sc,
                               const unsigned long long *flags, unsigned long long cap, OutDesc out, int num_sms,
                               cudaStream_t st);
cudaError_t launch_refine_scan(__nv_bfloat16 *const *dig, int lp, int L, const SInfo *info, DevScalars *sc,
                               OutDesc out, int num_sms, cudaStream_t st);
// CUDA-core level sums + the same epilogue for an explicit pair list (used
// for sparse pair lists and as the tensor-core path's independent check).
cudaError_t launch_mixed_pairs(__nv_bfloat16 *const *dig, int lp, int L, const SInfo *info, DevScalars *sc,
                               float tol, float u, float d34, const int64_t *ii, const int64_t *jj, int64_t np,
                               double *out, float *levels_out, cudaStream_t st);

}  // namespace bs
