// api.cu -- the C ABI (include/bioshell_crmsd.h): contexts, device
// workspaces, host<->device staging, the call sequences of the plain and
// mixed paths, metrics, and the host-side self-test hooks.
#include <cudaTypedefs.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <string>
#include <vector>

#include "../../include/bioshell_crmsd.h"
#include "crmsd_math.cuh"
#include "kernels.h"

using namespace bs;

namespace {

constexpr double kDefaultTol = 1e-4;  // Angstrom, certified total |dRMSD| per pair
constexpr unsigned long long kFlagCap = 1ull << 24;  // queued exact recomputations

struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
};

}  // namespace

struct bs_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[6] = {};
  size_t budget = 0;
  size_t used = 0;
  std::string err;
  bs_metrics metrics{};
  // workspaces
  DevBuf xyz, ctr, info, dig[4], y, g, out, tiles, flags, scal, pairs_i, pairs_j, pout;
  double d34 = 0.0;  // level-3 rounding bound of the last preparation (units u)
  int64_t tiles_nb = -1;
  int64_t tiles_count = 0;
  PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
};

namespace {

bs_status set_err(bs_ctx *ctx, bs_status s, const char *fmt, ...) {
  if (ctx) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    ctx->err = buf;
  }
  return s;
}

bs_status cuda_err(bs_ctx *ctx, cudaError_t e, const char *what) {
  const bs_status s = (e == cudaErrorMemoryAllocation) ? BS_ERR_OOM : BS_ERR_CUDA;
  return set_err(ctx, s, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(call, what)                                  \
  do {                                                  \
    cudaError_t _e = (call);                            \
    if (_e != cudaSuccess) return cuda_err(ctx, _e, what); \
  } while (0)

bs_status ensure(bs_ctx *ctx, DevBuf &b, size_t bytes, const char *what) {
  if (bytes == 0) bytes = 16;
  if (b.cap >= bytes) return BS_OK;
  if (b.p) {
    cudaFree(b.p);
    ctx->used -= b.cap;
    b.p = nullptr;
    b.cap = 0;
  }
  if (ctx->used + bytes > ctx->budget)
    return set_err(ctx, BS_ERR_BUDGET, "%s: %zu bytes would exceed the context budget (%zu of %zu in use)", what,
                   bytes, ctx->used, ctx->budget);
  cudaError_t e = cudaMalloc(&b.p, bytes);
  if (e != cudaSuccess) {
    b.p = nullptr;
    return cuda_err(ctx, e, what);
  }
  ctx->used += bytes;
  b.cap = bytes;
  return BS_OK;
}

void release(bs_ctx *ctx, DevBuf &b) {
  if (b.p) {
    cudaFree(b.p);
    ctx->used -= b.cap;
  }
  b.p = nullptr;
  b.cap = 0;
}

bool is_device_ptr(const void *p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

bs_status check_opts(bs_ctx *ctx, const bs_opts *o) {
  if (o->version != BS_OPTS_VERSION) return set_err(ctx, BS_ERR_INVALID_ARG, "bs_opts.version %u != %d", o->version, BS_OPTS_VERSION);
  if (o->precision != BS_PRECISION_PLAIN64 && o->precision != BS_PRECISION_MIXED)
    return set_err(ctx, BS_ERR_INVALID_ARG, "bs_opts.precision %d unknown", o->precision);
  if (o->layout != BS_LAYOUT_TRIANGLE && o->layout != BS_LAYOUT_SQUARE)
    return set_err(ctx, BS_ERR_INVALID_ARG, "bs_opts.layout %d unknown", o->layout);
  if (o->out_type != BS_OUT_F64 && o->out_type != BS_OUT_F32)
    return set_err(ctx, BS_ERR_INVALID_ARG, "bs_opts.out_type %d unknown", o->out_type);
  return BS_OK;
}

// Coordinates on the device (copied from the host when needed).
bs_status stage_coords(bs_ctx *ctx, const double *xyz, int64_t n, int L, const double **dev) {
  const size_t bytes = (size_t)n * (size_t)L * 3 * sizeof(double);
  if (is_device_ptr(xyz)) {
    *dev = xyz;
    return BS_OK;
  }
  bs_status s = ensure(ctx, ctx->xyz, bytes, "coordinates");
  if (s) return s;
  CK(cudaMemcpyAsync(ctx->xyz.p, xyz, bytes, cudaMemcpyHostToDevice, ctx->stream), "copy coordinates to device");
  ctx->metrics.bytes_h2d += (int64_t)bytes;
  *dev = static_cast<const double *>(ctx->xyz.p);
  return BS_OK;
}

bs_status read_scalars(bs_ctx *ctx, DevScalars *host) {
  CK(cudaMemcpyAsync(host, ctx->scal.p, sizeof(DevScalars), cudaMemcpyDeviceToHost, ctx->stream), "read scalars");
  CK(cudaStreamSynchronize(ctx->stream), "synchronize");
  return BS_OK;
}

// Mixed path preparation: centring, grid choice, digits, and the exactness
// bound: levels 0-2 must stay below 2^24 in magnitude.  With n_i = max over
// (structure, coordinate) of sqrt(sum e_i^2), Cauchy-Schwarz bounds |S_l| by
// sum_{i+j=l} n_i n_j; when that reaches 2^24 the grid is coarsened by one bit
// and the digits are recomputed.  Level 3 (S3 + S4/512) is exact below 2^23;
// above, its FP32 rounding is bounded here and charged to the error budget.
bs_status prep_mixed(bs_ctx *ctx, const double *dxyz, int64_t n, int L, int lp, DevScalars *hs) {
  const int64_t rows = blocks_for(n) * kBlockRows;
  const size_t dbytes = (size_t)rows * lp * sizeof(__nv_bfloat16);
  bs_status s;
  if ((s = ensure(ctx, ctx->ctr, (size_t)n * 3 * sizeof(double), "centroids"))) return s;
  if ((s = ensure(ctx, ctx->info, (size_t)n * sizeof(SInfo), "structure data"))) return s;
  for (int d = 0; d < 4; ++d)
    if ((s = ensure(ctx, ctx->dig[d], dbytes, "digit matrices"))) return s;
  __nv_bfloat16 *digs[4];
  for (int d = 0; d < 4; ++d) digs[d] = static_cast<__nv_bfloat16 *>(ctx->dig[d].p);
  DevScalars *sc = static_cast<DevScalars *>(ctx->scal.p);
  int scale_min = -1000;
  for (int attempt = 0; attempt < 8; ++attempt) {
    DevScalars init{};
    init.scale_min = scale_min;
    CK(cudaMemcpyAsync(sc, &init, sizeof(init), cudaMemcpyHostToDevice, ctx->stream), "init scalars");
    for (int d = 0; d < 4; ++d) CK(cudaMemsetAsync(digs[d], 0, dbytes, ctx->stream), "clear digits");
    CK(launch_prep_stats(dxyz, n, L, static_cast<double *>(ctx->ctr.p), sc, ctx->stream), "prep stats");
    CK(launch_prep_scale(sc, ctx->stream), "prep scale");
    CK(launch_prep_digits(dxyz, static_cast<const double *>(ctx->ctr.p), n, L, lp, digs,
                          static_cast<SInfo *>(ctx->info.p), sc, ctx->stream),
       "prep digits");
    if ((s = read_scalars(ctx, hs))) return s;
    if (hs->err & kErrNonFinite) return set_err(ctx, BS_ERR_NONFINITE, "input coordinates contain NaN or Inf");
    const double n0 = sqrt((double)hs->norm_max[0]), n1 = sqrt((double)hs->norm_max[1]),
                 n2 = sqrt((double)hs->norm_max[2]);
    const double b0 = n0 * n0, b1 = 2 * n0 * n1, b2 = 2 * n0 * n2 + n1 * n1;
    const double lim = 16777216.0;  // 2^24
    if (b0 < lim && b1 < lim && b2 < lim) {
      const double b34 = 2 * n1 * n2 + n2 * n2 / 512.0;
      double err3 = 0.0;  // level-3 units
      if (b34 >= 8388608.0) {  // 2^23: half-integers no longer exact
        const int k = (int)floor(log2(b34));
        err3 = 3.0 * (double)L * ldexp(1.0, k - 24);
      }
      // Mhat carries 2 S3' -> |dM| <= 2 err3 u per entry; |dE| <= 2 sqrt(3) ||dM||_F
      ctx->d34 = 12.0 * sqrt(3.0) * err3;
      return BS_OK;
    }
    scale_min = hs->scale_exp + 1;
  }
  return set_err(ctx, BS_ERR_UNSUPPORTED,
                 "chain length %d too long for exact 3-digit level sums (bound not met after 8 coarsenings)", L);
}

// Tensor-core tiles: row blocks I of 40 structures against column blocks J
// of 20 structures, kept when some pair i < j falls in the tile (J >= 2I),
// in super-block order so that the tiles in flight at any time touch a
// working set that stays in L2.
void build_tiles(int64_t n, std::vector<int2> &t) {
  const int64_t nba = blocks_for(n), nbb = (n + 19) / 20;
  const int64_t SA = 32, SBB = 64;
  t.clear();
  for (int64_t sa = 0; sa < nba; sa += SA)
    for (int64_t sb = 2 * sa; sb < nbb; sb += SBB)
      for (int64_t I = sa; I < std::min(sa + SA, nba); ++I)
        for (int64_t J = std::max(sb, 2 * I); J < std::min(sb + SBB, nbb); ++J)
          t.push_back(make_int2((int)I, (int)J));
}

bs_status encode_maps(bs_ctx *ctx, int64_t rows, int lp, CUtensorMap *tm) {
  if (!ctx->encode) {
    cudaDriverEntryPointQueryResult q;
    void *fn = nullptr;
    CK(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q),
       "driver entry point cuTensorMapEncodeTiled");
    if (q != cudaDriverEntryPointSuccess || !fn)
      return set_err(ctx, BS_ERR_CUDA, "cuTensorMapEncodeTiled unavailable in the driver");
    ctx->encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  // maps 0-3: A operand boxes (64 atoms x 128 rows) of e0, e1, e2, d2/32;
  // maps 4-6: B boxes (64 x 64) of e0, e1, e2
  for (int m = 0; m < 7; ++m) {
    const int d = m < 4 ? m : m - 4;
    cuuint64_t gdim[2] = {(cuuint64_t)lp, (cuuint64_t)rows};
    cuuint64_t gstride[1] = {(cuuint64_t)lp * 2};
    cuuint32_t box[2] = {64, m < 4 ? 128u : 64u};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = ctx->encode(&tm[m], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, ctx->dig[d].p, gdim, gstride, box, estr,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_err(ctx, BS_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  }
  return BS_OK;
}

size_t out_elems(int64_t n, int layout) {
  return layout == BS_LAYOUT_TRIANGLE ? (size_t)(n * (n - 1) / 2) : (size_t)n * (size_t)n;
}

// Certified per-pair |dRMSD| budget: the kernels charge each pair its two
// structures' quantisation residuals (Minkowski) and give the fast path the
// rest (at least 1e-5 A).
float total_tolerance(const bs_opts &o) { return (float)(o.tolerance > 0 ? o.tolerance : kDefaultTol); }
float qres_max(const DevScalars &hs) {
  float f;
  const unsigned b = (unsigned)hs.qres_max_bits;
  memcpy(&f, &b, 4);
  return f;
}

bs_status check_device_errors(bs_ctx *ctx, DevScalars *hs) {
  bs_status s = read_scalars(ctx, hs);
  if (s) return s;
  if (hs->err & kErrTimeout) return set_err(ctx, BS_ERR_TIMEOUT, "a device-side wait timed out");
  if (hs->err & kErrNonFinite) return set_err(ctx, BS_ERR_NONFINITE, "input coordinates contain NaN or Inf");
  if (hs->err & kErrInternal) return set_err(ctx, BS_ERR_INTERNAL, "device-side invariant violated");
  return BS_OK;
}

float elapsed(bs_ctx *ctx, int a, int b) {
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev[a], ctx->ev[b]);
  return ms;
}

bs_status all_vs_all_impl(bs_ctx *ctx, const double *xyz, int64_t n, int L, const bs_opts &o, void *out) {
  ctx->metrics = bs_metrics{};
  const size_t esz = o.out_type == BS_OUT_F64 ? 8 : 4;
  const size_t nout = out_elems(n, o.layout);
  const bool out_dev = is_device_ptr(out);
  const int lp = lp_for(L);
  bs_status s;
  CK(cudaEventRecord(ctx->ev[0], ctx->stream), "event");
  const double *dxyz = nullptr;
  if ((s = stage_coords(ctx, xyz, n, L, &dxyz))) return s;
  CK(cudaEventRecord(ctx->ev[1], ctx->stream), "event");
  void *dout = out;
  if (!out_dev) {
    if ((s = ensure(ctx, ctx->out, nout * esz, "result buffer"))) return s;
    dout = ctx->out.p;
  }
  if (o.layout == BS_LAYOUT_SQUARE)
    CK(cudaMemset2DAsync(dout, (size_t)(n + 1) * esz, 0, esz, (size_t)n, ctx->stream), "zero diagonal");
  OutDesc od{dout, n, o.layout, o.out_type};
  DevScalars hs{};
  if (o.precision == BS_PRECISION_PLAIN64) {
    if ((s = ensure(ctx, ctx->ctr, (size_t)n * 3 * sizeof(double), "centroids"))) return s;
    if ((s = ensure(ctx, ctx->y, (size_t)n * 3 * lp * sizeof(double), "centred coordinates"))) return s;
    if ((s = ensure(ctx, ctx->g, (size_t)n * sizeof(double), "norms"))) return s;
    DevScalars init{};
    CK(cudaMemcpyAsync(ctx->scal.p, &init, sizeof(init), cudaMemcpyHostToDevice, ctx->stream), "init scalars");
    DevScalars *sc = static_cast<DevScalars *>(ctx->scal.p);
    CK(launch_prep_stats(dxyz, n, L, static_cast<double *>(ctx->ctr.p), sc, ctx->stream), "prep stats");
    CK(launch_prep_plain(dxyz, static_cast<const double *>(ctx->ctr.p), n, L, lp, static_cast<double *>(ctx->y.p),
                         static_cast<double *>(ctx->g.p), ctx->stream),
       "prep plain");
    CK(cudaEventRecord(ctx->ev[2], ctx->stream), "event");
    CK(launch_plain64_all(static_cast<const double *>(ctx->y.p), static_cast<const double *>(ctx->g.p), n, L, lp, od,
                          ctx->stream),
       "plain64 all-vs-all");
    CK(cudaEventRecord(ctx->ev[3], ctx->stream), "event");
    CK(cudaEventRecord(ctx->ev[4], ctx->stream), "event");
    ctx->metrics.main_launches = 3;
  } else {
    if ((s = prep_mixed(ctx, dxyz, n, L, lp, &hs))) return s;
    CK(cudaEventRecord(ctx->ev[2], ctx->stream), "event");
    const int64_t nb = blocks_for(n);
    if (ctx->tiles_nb != n) {
      std::vector<int2> t;
      build_tiles(n, t);
      if ((s = ensure(ctx, ctx->tiles, t.size() * sizeof(int2), "tile table"))) return s;
      CK(cudaMemcpy(ctx->tiles.p, t.data(), t.size() * sizeof(int2), cudaMemcpyHostToDevice), "upload tile table");
      ctx->tiles_nb = n;
      ctx->tiles_count = (int64_t)t.size();
    }
    if ((s = ensure(ctx, ctx->flags, kFlagCap * sizeof(unsigned long long), "flag list"))) return s;
    CUtensorMap tm[7];
    if ((s = encode_maps(ctx, nb * kBlockRows, lp, tm))) return s;
    TcArgs a{};
    a.tiles = static_cast<const int2 *>(ctx->tiles.p);
    a.ntiles = ctx->tiles_count;
    a.n = n;
    a.L = L;
    a.lp = lp;
    a.info = static_cast<const SInfo *>(ctx->info.p);
    a.sc = static_cast<DevScalars *>(ctx->scal.p);
    a.tol = total_tolerance(o);
    a.u = ldexpf(1.0f, 2 * hs.scale_exp);
    a.d34 = (float)ctx->d34;
    a.out = od;
    a.flags = static_cast<unsigned long long *>(ctx->flags.p);
    a.flag_cap = kFlagCap;
    a.dbg = nullptr;
    a.num_sms = ctx->num_sms;
    CK(launch_mixed_tc(tm, a, ctx->stream), "tensor-core all-vs-all");
    CK(cudaEventRecord(ctx->ev[3], ctx->stream), "event");
    __nv_bfloat16 *digs[4];
    for (int d = 0; d < 4; ++d) digs[d] = static_cast<__nv_bfloat16 *>(ctx->dig[d].p);
    CK(launch_refine_list(digs, lp, L, a.info, a.sc, a.flags, kFlagCap, od, ctx->num_sms, ctx->stream),
       "exact recomputation");
    if ((s = check_device_errors(ctx, &hs))) return s;
    if (hs.flag_count > kFlagCap) {
      CK(launch_refine_scan(digs, lp, L, a.info, a.sc, od, ctx->num_sms, ctx->stream), "exact recomputation (scan)");
    }
    CK(cudaEventRecord(ctx->ev[4], ctx->stream), "event");
    ctx->metrics.pairs_refined = (int64_t)hs.flag_count;
    ctx->metrics.scale_exp = hs.scale_exp;
    ctx->metrics.quant_bound = 2.0 * qres_max(hs);  // worst pair's |dRMSD| from the grid
    ctx->metrics.main_launches = 5 + (hs.flag_count > kFlagCap ? 1 : 0);
  }
  if (!out_dev) {
    CK(cudaMemcpyAsync(out, dout, nout * esz, cudaMemcpyDeviceToHost, ctx->stream), "copy result to host");
    ctx->metrics.bytes_d2h += (int64_t)(nout * esz);
  }
  CK(cudaEventRecord(ctx->ev[5], ctx->stream), "event");
  if ((s = check_device_errors(ctx, &hs))) return s;
  ctx->metrics.pairs = n * (n - 1) / 2;
  ctx->metrics.ms_h2d = elapsed(ctx, 0, 1);
  ctx->metrics.ms_prep = elapsed(ctx, 1, 2);
  ctx->metrics.ms_main = elapsed(ctx, 2, 3);
  ctx->metrics.ms_refine = elapsed(ctx, 3, 4);
  ctx->metrics.ms_d2h = elapsed(ctx, 4, 5);
  ctx->metrics.ms_total = elapsed(ctx, 0, 5);
  return BS_OK;
}

bs_status pairs_impl(bs_ctx *ctx, const double *xyz, int64_t n, int L, const int64_t *ii, const int64_t *jj,
                     int64_t np, const bs_opts &o, double *out, float *levels_dbg) {
  ctx->metrics = bs_metrics{};
  const int lp = lp_for(L);
  bs_status s;
  CK(cudaEventRecord(ctx->ev[0], ctx->stream), "event");
  const double *dxyz = nullptr;
  if ((s = stage_coords(ctx, xyz, n, L, &dxyz))) return s;
  const int64_t *dii = ii, *djj = jj;
  if (!is_device_ptr(ii)) {
    if ((s = ensure(ctx, ctx->pairs_i, (size_t)np * 8, "pair list"))) return s;
    CK(cudaMemcpyAsync(ctx->pairs_i.p, ii, (size_t)np * 8, cudaMemcpyHostToDevice, ctx->stream), "copy pair list");
    dii = static_cast<const int64_t *>(ctx->pairs_i.p);
  }
  if (!is_device_ptr(jj)) {
    if ((s = ensure(ctx, ctx->pairs_j, (size_t)np * 8, "pair list"))) return s;
    CK(cudaMemcpyAsync(ctx->pairs_j.p, jj, (size_t)np * 8, cudaMemcpyHostToDevice, ctx->stream), "copy pair list");
    djj = static_cast<const int64_t *>(ctx->pairs_j.p);
  }
  const bool out_dev = is_device_ptr(out);
  double *dout = out;
  if (!out_dev) {
    if ((s = ensure(ctx, ctx->pout, (size_t)np * 8, "pair results"))) return s;
    dout = static_cast<double *>(ctx->pout.p);
  }
  CK(cudaEventRecord(ctx->ev[1], ctx->stream), "event");
  DevScalars hs{};
  if (o.precision == BS_PRECISION_PLAIN64) {
    if ((s = ensure(ctx, ctx->ctr, (size_t)n * 3 * sizeof(double), "centroids"))) return s;
    if ((s = ensure(ctx, ctx->y, (size_t)n * 3 * lp * sizeof(double), "centred coordinates"))) return s;
    if ((s = ensure(ctx, ctx->g, (size_t)n * sizeof(double), "norms"))) return s;
    DevScalars init{};
    CK(cudaMemcpyAsync(ctx->scal.p, &init, sizeof(init), cudaMemcpyHostToDevice, ctx->stream), "init scalars");
    DevScalars *sc = static_cast<DevScalars *>(ctx->scal.p);
    CK(launch_prep_stats(dxyz, n, L, static_cast<double *>(ctx->ctr.p), sc, ctx->stream), "prep stats");
    CK(launch_prep_plain(dxyz, static_cast<const double *>(ctx->ctr.p), n, L, lp, static_cast<double *>(ctx->y.p),
                         static_cast<double *>(ctx->g.p), ctx->stream),
       "prep plain");
    CK(cudaEventRecord(ctx->ev[2], ctx->stream), "event");
    CK(launch_plain64_pairs(static_cast<const double *>(ctx->y.p), static_cast<const double *>(ctx->g.p), n, L, lp,
                            dii, djj, np, dout, ctx->stream),
       "plain64 pairs");
  } else {
    if ((s = prep_mixed(ctx, dxyz, n, L, lp, &hs))) return s;
    CK(cudaEventRecord(ctx->ev[2], ctx->stream), "event");
    __nv_bfloat16 *digs[4];
    for (int d = 0; d < 4; ++d) digs[d] = static_cast<__nv_bfloat16 *>(ctx->dig[d].p);
    CK(launch_mixed_pairs(digs, lp, L, static_cast<const SInfo *>(ctx->info.p), static_cast<DevScalars *>(ctx->scal.p),
                          total_tolerance(o), ldexpf(1.0f, 2 * hs.scale_exp), (float)ctx->d34, dii, djj, np, dout,
                          levels_dbg, ctx->stream),
       "mixed pairs");
  }
  CK(cudaEventRecord(ctx->ev[3], ctx->stream), "event");
  CK(cudaEventRecord(ctx->ev[4], ctx->stream), "event");
  if (!out_dev) {
    CK(cudaMemcpyAsync(out, dout, (size_t)np * 8, cudaMemcpyDeviceToHost, ctx->stream), "copy pair results");
    ctx->metrics.bytes_d2h += np * 8;
  }
  CK(cudaEventRecord(ctx->ev[5], ctx->stream), "event");
  if ((s = check_device_errors(ctx, &hs))) return s;
  ctx->metrics.pairs = np;
  ctx->metrics.scale_exp = hs.scale_exp;
  if (o.precision == BS_PRECISION_MIXED) ctx->metrics.quant_bound = 2.0 * qres_max(hs);
  ctx->metrics.ms_h2d = elapsed(ctx, 0, 1);
  ctx->metrics.ms_prep = elapsed(ctx, 1, 2);
  ctx->metrics.ms_main = elapsed(ctx, 2, 3);
  ctx->metrics.ms_d2h = elapsed(ctx, 4, 5);
  ctx->metrics.ms_total = elapsed(ctx, 0, 5);
  return BS_OK;
}

}  // namespace

// ======================================================================
// C ABI
// ======================================================================
extern "C" {

BS_API int32_t bs_abi_version(void) { return BS_ABI_VERSION; }

BS_API const char *bs_status_string(bs_status s) {
  switch (s) {
    case BS_OK: return "ok";
    case BS_ERR_INVALID_ARG: return "invalid argument";
    case BS_ERR_CUDA: return "CUDA error";
    case BS_ERR_OOM: return "out of memory";
    case BS_ERR_TIMEOUT: return "device-side wait timed out";
    case BS_ERR_UNSUPPORTED: return "unsupported shape";
    case BS_ERR_NONFINITE: return "non-finite input";
    case BS_ERR_BUDGET: return "HBM budget exceeded";
    case BS_ERR_NO_DEVICE: return "no usable sm_103 GPU";
    case BS_ERR_INTERNAL: return "internal error";
    default: return "unknown status";
  }
}

BS_API const char *bs_last_error(const bs_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

BS_API void bs_opts_init(bs_opts *o) {
  if (!o) return;
  memset(o, 0, sizeof(*o));
  o->version = BS_OPTS_VERSION;
  o->precision = BS_PRECISION_MIXED;
  o->layout = BS_LAYOUT_TRIANGLE;
  o->out_type = BS_OUT_F64;
  o->tolerance = 0.0;
}

BS_API bs_status bs_ctx_create(bs_ctx **out, int32_t device, size_t hbm_budget_bytes) {
  if (!out) return BS_ERR_INVALID_ARG;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
    cudaGetLastError();
    return BS_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= count) return BS_ERR_INVALID_ARG;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return BS_ERR_NO_DEVICE;
  if (!(prop.major == 10 && prop.minor == 3)) return BS_ERR_NO_DEVICE;  // built for sm_103a only
  bs_ctx *ctx = new (std::nothrow) bs_ctx();
  if (!ctx) return BS_ERR_OOM;
  ctx->device = device;
  ctx->num_sms = prop.multiProcessorCount;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return BS_ERR_CUDA;
  }
  for (auto &e : ctx->ev) cudaEventCreate(&e);
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  ctx->budget = hbm_budget_bytes ? hbm_budget_bytes : (size_t)(0.9 * (double)free_b);
  if (ensure(ctx, ctx->scal, sizeof(DevScalars), "scalars") != BS_OK) {
    bs_ctx_destroy(ctx);
    return BS_ERR_OOM;
  }
  *out = ctx;
  return BS_OK;
}

BS_API void bs_ctx_destroy(bs_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  DevBuf *bufs[] = {&ctx->xyz, &ctx->ctr, &ctx->info, &ctx->dig[0], &ctx->dig[1], &ctx->dig[2], &ctx->dig[3],
                    &ctx->y, &ctx->g, &ctx->out, &ctx->tiles, &ctx->flags, &ctx->scal, &ctx->pairs_i,
                    &ctx->pairs_j, &ctx->pout};
  for (DevBuf *b : bufs) release(ctx, *b);
  for (auto &e : ctx->ev)
    if (e) cudaEventDestroy(e);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

BS_API bs_status bs_ctx_trim(bs_ctx *ctx) {
  if (!ctx) return BS_ERR_INVALID_ARG;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  DevBuf *bufs[] = {&ctx->xyz, &ctx->ctr, &ctx->info, &ctx->dig[0], &ctx->dig[1], &ctx->dig[2], &ctx->dig[3],
                    &ctx->y, &ctx->g, &ctx->out, &ctx->tiles, &ctx->flags, &ctx->pairs_i, &ctx->pairs_j, &ctx->pout};
  for (DevBuf *b : bufs) release(ctx, *b);
  ctx->tiles_nb = -1;
  return BS_OK;
}

BS_API void *bs_ctx_stream(const bs_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

BS_API bs_status bs_get_metrics(const bs_ctx *ctx, bs_metrics *out) {
  if (!ctx || !out) return BS_ERR_INVALID_ARG;
  *out = ctx->metrics;
  return BS_OK;
}

BS_API bs_status bs_all_vs_all(bs_ctx *ctx, const double *xyz, int64_t n, int32_t L, const bs_opts *opts, void *out) {
  if (!ctx) return BS_ERR_INVALID_ARG;
  bs_opts o;
  bs_opts_init(&o);
  if (opts) o = *opts;
  bs_status s = check_opts(ctx, &o);
  if (s) return s;
  if (n < 0 || L < 1) return set_err(ctx, BS_ERR_INVALID_ARG, "n must be >= 0 and L >= 1 (n=%lld, L=%d)", (long long)n, L);
  if (n > 0 && (!xyz || !out)) return set_err(ctx, BS_ERR_INVALID_ARG, "null coordinate or result pointer");
  if (n > (1LL << 31) - 1) return set_err(ctx, BS_ERR_UNSUPPORTED, "n above 2^31-1");
  if (n < 2) {
    ctx->metrics = bs_metrics{};
    if (n == 1 && o.layout == BS_LAYOUT_SQUARE) {
      const size_t esz = o.out_type == BS_OUT_F64 ? 8 : 4;
      double z = 0.0;
      if (cudaMemcpy(out, &z, esz, cudaMemcpyDefault) != cudaSuccess) return cuda_err(ctx, cudaGetLastError(), "write result");
    }
    return BS_OK;
  }
  if (cudaSetDevice(ctx->device) != cudaSuccess) return set_err(ctx, BS_ERR_CUDA, "cudaSetDevice failed");
  return all_vs_all_impl(ctx, xyz, n, L, o, out);
}

BS_API bs_status bs_pairs(bs_ctx *ctx, const double *xyz, int64_t n, int32_t L, const int64_t *ii, const int64_t *jj,
                          int64_t npairs, const bs_opts *opts, double *out) {
  if (!ctx) return BS_ERR_INVALID_ARG;
  bs_opts o;
  bs_opts_init(&o);
  if (opts) o = *opts;
  bs_status s = check_opts(ctx, &o);
  if (s) return s;
  if (n < 1 || L < 1 || npairs < 0) return set_err(ctx, BS_ERR_INVALID_ARG, "n >= 1, L >= 1, npairs >= 0 required");
  if (npairs == 0) return BS_OK;
  if (!xyz || !ii || !jj || !out) return set_err(ctx, BS_ERR_INVALID_ARG, "null pointer argument");
  if (!is_device_ptr(ii) && !is_device_ptr(jj)) {
    for (int64_t t = 0; t < npairs; ++t)
      if (ii[t] < 0 || ii[t] >= n || jj[t] < 0 || jj[t] >= n)
        return set_err(ctx, BS_ERR_INVALID_ARG, "pair %lld = (%lld, %lld) out of range [0, %lld)", (long long)t,
                       (long long)ii[t], (long long)jj[t], (long long)n);
  }
  if (cudaSetDevice(ctx->device) != cudaSuccess) return set_err(ctx, BS_ERR_CUDA, "cudaSetDevice failed");
  return pairs_impl(ctx, xyz, n, L, ii, jj, npairs, o, out, nullptr);
}

BS_API bs_status bs_crmsd(bs_ctx *ctx, const double *a, const double *b, int32_t L, double *out_rmsd) {
  if (!ctx) return BS_ERR_INVALID_ARG;
  if (!a || !b || !out_rmsd || L < 1) return set_err(ctx, BS_ERR_INVALID_ARG, "null pointer or L < 1");
  if (cudaSetDevice(ctx->device) != cudaSuccess) return set_err(ctx, BS_ERR_CUDA, "cudaSetDevice failed");
  const size_t one = (size_t)L * 3 * sizeof(double);
  bs_status s = ensure(ctx, ctx->xyz, 2 * one, "coordinates");
  if (s) return s;
  double *d = static_cast<double *>(ctx->xyz.p);
  CK(cudaMemcpyAsync(d, a, one, cudaMemcpyDefault, ctx->stream), "copy a");
  CK(cudaMemcpyAsync(d + (size_t)L * 3, b, one, cudaMemcpyDefault, ctx->stream), "copy b");
  const int64_t ii = 0, jj = 1;
  bs_opts o;
  bs_opts_init(&o);
  double r = 0.0;
  s = pairs_impl(ctx, d, 2, L, &ii, &jj, 1, o, &r, nullptr);
  if (s) return s;
  *out_rmsd = r;
  return BS_OK;
}

BS_API bs_status bs_host_alloc(size_t bytes, void **out) {
  if (!out) return BS_ERR_INVALID_ARG;
  *out = nullptr;
  if (bytes == 0) return BS_OK;
  cudaError_t e = cudaHostAlloc(out, bytes, cudaHostAllocDefault);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *out = nullptr;
    return e == cudaErrorMemoryAllocation ? BS_ERR_OOM : BS_ERR_CUDA;
  }
  return BS_OK;
}

BS_API bs_status bs_host_free(void *p) {
  if (!p) return BS_OK;
  return cudaFreeHost(p) == cudaSuccess ? BS_OK : BS_ERR_CUDA;
}

BS_API bs_status bs_debug_tile_levels(bs_ctx *ctx, const double *xyz, int64_t n, int32_t L, float *levels) {
  if (!ctx || !xyz || !levels || n < 1 || L < 1) return BS_ERR_INVALID_ARG;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return set_err(ctx, BS_ERR_CUDA, "cudaSetDevice failed");
  const int lp = lp_for(L);
  const double *dxyz = nullptr;
  bs_status s;
  if ((s = stage_coords(ctx, xyz, n, L, &dxyz))) return s;
  DevScalars hs{};
  if ((s = prep_mixed(ctx, dxyz, n, L, lp, &hs))) return s;
  const int64_t nb = blocks_for(n);
  const int2 first[2] = {make_int2(0, 0), make_int2(0, 1)};
  if ((s = ensure(ctx, ctx->tiles, sizeof(first), "tile table"))) return s;
  CK(cudaMemcpy(ctx->tiles.p, first, sizeof(first), cudaMemcpyHostToDevice), "upload tiles");
  ctx->tiles_nb = -1;  // the cached table was replaced
  const size_t nout = (size_t)n * (size_t)(n > 1 ? n - 1 : 1) / 2 + 1;
  if ((s = ensure(ctx, ctx->out, nout * 8, "result buffer"))) return s;
  if ((s = ensure(ctx, ctx->flags, kFlagCap * sizeof(unsigned long long), "flag list"))) return s;
  if ((s = ensure(ctx, ctx->pout, (size_t)4 * 128 * 128 * sizeof(float), "level dump"))) return s;
  CK(cudaMemsetAsync(ctx->pout.p, 0, (size_t)4 * 128 * 128 * sizeof(float), ctx->stream), "clear level dump");
  CUtensorMap tm[7];
  if ((s = encode_maps(ctx, nb * kBlockRows, lp, tm))) return s;
  TcArgs a{};
  a.tiles = static_cast<const int2 *>(ctx->tiles.p);
  a.ntiles = (n > 20) ? 2 : 1;
  a.n = n;
  a.L = L;
  a.lp = lp;
  a.info = static_cast<const SInfo *>(ctx->info.p);
  a.sc = static_cast<DevScalars *>(ctx->scal.p);
  a.tol = (float)kDefaultTol;
  a.u = ldexpf(1.0f, 2 * hs.scale_exp);
  a.d34 = (float)ctx->d34;
  a.out = OutDesc{ctx->out.p, n, BS_LAYOUT_TRIANGLE, BS_OUT_F64};
  a.flags = static_cast<unsigned long long *>(ctx->flags.p);
  a.flag_cap = kFlagCap;
  a.dbg = static_cast<float *>(ctx->pout.p);
  a.num_sms = ctx->num_sms;
  CK(launch_mixed_tc(tm, a, ctx->stream), "tensor-core tile");
  CK(cudaMemcpyAsync(levels, a.dbg, (size_t)4 * 128 * 128 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream),
     "copy level dump");
  return check_device_errors(ctx, &hs);
}

BS_API bs_status bs_debug_pair_levels(bs_ctx *ctx, const double *xyz, int64_t n, int32_t L, const int64_t *ii,
                                      const int64_t *jj, int64_t npairs, float *levels, double *rmsd) {
  if (!ctx || !xyz || !ii || !jj || !levels || !rmsd || n < 1 || L < 1 || npairs < 1) return BS_ERR_INVALID_ARG;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return set_err(ctx, BS_ERR_CUDA, "cudaSetDevice failed");
  for (int64_t t = 0; t < npairs; ++t)
    if (ii[t] < 0 || ii[t] >= n || jj[t] < 0 || jj[t] >= n) return set_err(ctx, BS_ERR_INVALID_ARG, "pair out of range");
  DevBuf lv;
  bs_status s = ensure(ctx, lv, (size_t)npairs * 36 * sizeof(float), "level dump");
  if (s) return s;
  bs_opts o;
  bs_opts_init(&o);
  s = pairs_impl(ctx, xyz, n, L, ii, jj, npairs, o, rmsd, static_cast<float *>(lv.p));
  if (s == BS_OK) {
    cudaError_t e = cudaMemcpy(levels, lv.p, (size_t)npairs * 36 * sizeof(float), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) s = cuda_err(ctx, e, "copy level dump");
  }
  release(ctx, lv);
  return s;
}

// ------------------------------------------------------------ test hooks
BS_API bs_status bs_selftest_digits(const double *xyz, int32_t L, int32_t scale_exp, int32_t *digits,
                                    int64_t *g_exact, double *qres) {
  if (!xyz || !digits || !g_exact || !qres || L < 1) return BS_ERR_INVALID_ARG;
  double c[3] = {0, 0, 0};
  for (int k = 0; k < L; ++k)
    for (int d = 0; d < 3; ++d) c[d] += xyz[3 * k + d];
  for (int d = 0; d < 3; ++d) c[d] /= (double)L;
  long long g = 0;
  double res = 0.0;
  for (int k = 0; k < L; ++k)
    for (int d = 0; d < 3; ++d) {
      const double y = xyz[3 * k + d] - c[d];
      const double r = nearbyint(ldexp(y, -scale_exp));
      if (!(fabs(r) < 4194304.0)) return BS_ERR_UNSUPPORTED;
      const int q = (int)r;
      res += (y - ldexp(r, scale_exp)) * (y - ldexp(r, scale_exp));
      int a, b, e;
      bsm::split_digits(q, a, b, e);
      digits[(0 * 3 + d) * L + k] = a;
      digits[(1 * 3 + d) * L + k] = b;
      digits[(2 * 3 + d) * L + k] = e;
      g += (long long)q * q;
    }
  *g_exact = g;
  *qres = sqrt(res / (double)L);
  return BS_OK;
}

BS_API bs_status bs_selftest_epilogue(const float *levels, int64_t ga, int64_t gb, double qa, double qb, double d34,
                                      int32_t scale_exp, int32_t L, double tolerance, double *rmsd, int32_t *flag) {
  if (!levels || !rmsd || !flag || L < 1) return BS_ERR_INVALID_ARG;
  bsm::EpilogueIn in;
  for (int e = 0; e < 9; ++e) {
    in.s0[e] = levels[e];
    in.s1[e] = levels[9 + e];
    in.s2[e] = levels[18 + e];
    in.s3[e] = levels[27 + e];
  }
  in.ga = ga;
  in.gb = gb;
  in.gfa = (float)ga;
  in.gfb = (float)gb;
  in.qa = (float)qa;
  in.qb = (float)qb;
  int f = 0;
  const float r = bsm::pair_rmsd_fast(in, ldexpf(1.0f, 2 * scale_exp), (float)d34, L,
                                      (float)(tolerance > 0 ? tolerance : kDefaultTol), f);
  *rmsd = (double)r;
  *flag = f;
  return BS_OK;
}

BS_API bs_status bs_selftest_exact(const int32_t *na, const int32_t *nb, int32_t L, int32_t scale_exp, double *rmsd) {
  if (!na || !nb || !rmsd || L < 1) return BS_ERR_INVALID_ARG;
  long long mh[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  long long ga = 0, gb = 0;
  for (int k = 0; k < L; ++k)
    for (int x = 0; x < 3; ++x) {
      const long long ax = na[x * L + k];
      ga += ax * ax;
      const long long bx = nb[x * L + k];
      gb += bx * bx;
      for (int y = 0; y < 3; ++y) mh[3 * x + y] += ax * (long long)nb[y * L + k];
    }
  *rmsd = bsm::pair_rmsd_exact(mh, ga, gb, scale_exp, L);
  return BS_OK;
}

}  // extern "C"
