// noalloc.cu -- bs_all_vs_all_static: the mixed-precision all-vs-all for
// callers that cannot allocate device memory.
//
// Some hosts embed the engine where device allocation is not theirs to do:
// a caller running inside another framework's memory pool, a plugin that may
// only use the buffers it is handed, or code that must not call cudaMalloc /
// cudaFree at all (for example to keep a process's device footprint fixed, or
// because the allocator is owned by someone else).  For them this entry point
// takes device pointers for the coordinates and the result and keeps every
// piece of scratch (digit matrices, per-structure data, tile table, queue of
// pairs to recompute, scalars) in file-scope static device arrays sized for at
// most kMaxN structures of at most kMaxL atoms.  Every GPU that loads this
// library holds those arrays (about 7.4 MB) until the process exits.
//
// The arrays are shared by all calls: each call clears what must start at
// zero, and calls whose work overlaps on the GPU (for example on two streams
// at once) race on the same scratch and must not be issued.
#include <math.h>
#include <string.h>

#include <cudaTypedefs.h>

#include "../../include/bioshell_crmsd.h"
#include "kernels.h"

namespace bs {
namespace {

constexpr int64_t kMaxN = 512;                                   // structures per call
constexpr int kMaxL = 512;                                       // atoms per structure
constexpr int64_t kMaxBlocks = (kMaxN + kBlockStructs - 1) / kBlockStructs;  // 13
constexpr int64_t kMaxRows = kMaxBlocks * kBlockRows;            // 1664 digit rows
constexpr int64_t kDigitElems = kMaxRows * kMaxL;                // per digit matrix
constexpr int64_t kMaxTiles = kMaxBlocks * ((kMaxN + 19) / 20);  // upper bound of 40x20 tiles
constexpr unsigned long long kStaticFlagCap = 1ull << 16;

// file-scope scratch; its address is taken once per device below
static __device__ __align__(256) __nv_bfloat16 g_digits[4][kDigitElems];
static __device__ __align__(256) SInfo g_info[kMaxN];
static __device__ __align__(256) double g_ctr[kMaxN * 3];
static __device__ __align__(256) int2 g_tiles[kMaxTiles];
static __device__ __align__(256) unsigned long long g_flags[kStaticFlagCap];
static __device__ __align__(256) DevScalars g_scal;

constexpr int kMaxDevices = 64;
struct Scratch {
  bool ready = false;
  __nv_bfloat16 *dig[4] = {};
  SInfo *info = nullptr;
  double *ctr = nullptr;
  int2 *tiles = nullptr;
  unsigned long long *flags = nullptr;
  DevScalars *scal = nullptr;
  int num_sms = 0;
};
Scratch g_scratch[kMaxDevices];
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

// Device addresses of the static arrays on the current device (host code may
// not use the array names as addresses).
bs_status setup(int dev, Scratch **out) {
  if (dev < 0 || dev >= kMaxDevices) return BS_ERR_UNSUPPORTED;
  Scratch &s = g_scratch[dev];
  if (!s.ready) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_digits) != cudaSuccess) return BS_ERR_CUDA;
    for (int d = 0; d < 4; ++d) s.dig[d] = static_cast<__nv_bfloat16 *>(p) + (size_t)d * kDigitElems;
    if (cudaGetSymbolAddress(&p, g_info) != cudaSuccess) return BS_ERR_CUDA;
    s.info = static_cast<SInfo *>(p);
    if (cudaGetSymbolAddress(&p, g_ctr) != cudaSuccess) return BS_ERR_CUDA;
    s.ctr = static_cast<double *>(p);
    if (cudaGetSymbolAddress(&p, g_tiles) != cudaSuccess) return BS_ERR_CUDA;
    s.tiles = static_cast<int2 *>(p);
    if (cudaGetSymbolAddress(&p, g_flags) != cudaSuccess) return BS_ERR_CUDA;
    s.flags = static_cast<unsigned long long *>(p);
    if (cudaGetSymbolAddress(&p, g_scal) != cudaSuccess) return BS_ERR_CUDA;
    s.scal = static_cast<DevScalars *>(p);
    if (cudaDeviceGetAttribute(&s.num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return BS_ERR_CUDA;
    if (!g_encode) {
      cudaDriverEntryPointQueryResult q;
      void *fn = nullptr;
      if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
              cudaSuccess ||
          q != cudaDriverEntryPointSuccess || !fn)
        return BS_ERR_CUDA;
      g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    s.ready = true;
  }
  *out = &s;
  return BS_OK;
}

bool on_device(const void *p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

}  // namespace
}  // namespace bs

using namespace bs;

extern "C" BS_API bs_status bs_all_vs_all_static(const double *xyz, int64_t n, int32_t L, double *out, void *stream) {
  if (n < 0 || L < 1) return BS_ERR_INVALID_ARG;
  if (n > kMaxN || L > kMaxL) return BS_ERR_UNSUPPORTED;  // beyond the static scratch
  if (n < 2) return BS_OK;
  if (!xyz || !out || !on_device(xyz) || !on_device(out)) return BS_ERR_INVALID_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return BS_ERR_NO_DEVICE;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess || !(prop.major == 10 && prop.minor == 3))
    return BS_ERR_NO_DEVICE;
  Scratch *sc = nullptr;
  bs_status s = setup(dev, &sc);
  if (s) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int lp = lp_for(L);
  const int64_t nb = blocks_for(n), rows = nb * kBlockRows;
  const size_t dbytes = (size_t)rows * lp * sizeof(__nv_bfloat16);

  // preparation with the same exactness check as bs_all_vs_all (levels 0-2
  // below 2^24, coarsening the grid when a bound is not met)
  DevScalars hs{};
  double d34 = 0.0;
  bool ok = false;
  int scale_min = -1000;
  for (int attempt = 0; attempt < 8 && !ok; ++attempt) {
    DevScalars init{};
    init.scale_min = scale_min;
    if (cudaMemcpyAsync(sc->scal, &init, sizeof(init), cudaMemcpyHostToDevice, st) != cudaSuccess) return BS_ERR_CUDA;
    for (int d = 0; d < 4; ++d)
      if (cudaMemsetAsync(sc->dig[d], 0, dbytes, st) != cudaSuccess) return BS_ERR_CUDA;
    if (launch_prep_stats(xyz, n, L, sc->ctr, sc->scal, st) != cudaSuccess) return BS_ERR_CUDA;
    if (launch_prep_scale(sc->scal, st) != cudaSuccess) return BS_ERR_CUDA;
    if (launch_prep_digits(xyz, sc->ctr, n, L, lp, sc->dig, sc->info, sc->scal, st) != cudaSuccess)
      return BS_ERR_CUDA;
    if (cudaMemcpyAsync(&hs, sc->scal, sizeof(hs), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return BS_ERR_CUDA;
    if (hs.err & kErrNonFinite) return BS_ERR_NONFINITE;
    const double n0 = sqrt((double)hs.norm_max[0]), n1 = sqrt((double)hs.norm_max[1]),
                 n2 = sqrt((double)hs.norm_max[2]);
    const double lim = 16777216.0;
    if (n0 * n0 < lim && 2 * n0 * n1 < lim && 2 * n0 * n2 + n1 * n1 < lim) {
      const double b34 = 2 * n1 * n2 + n2 * n2 / 512.0;
      const double err3 = b34 >= 8388608.0 ? 3.0 * (double)L * ldexp(1.0, (int)floor(log2(b34)) - 24) : 0.0;
      d34 = 12.0 * sqrt(3.0) * err3;
      ok = true;
    } else {
      scale_min = hs.scale_exp + 1;
    }
  }
  if (!ok) return BS_ERR_UNSUPPORTED;

  // tile table (40 x 20 structure tiles with a pair i < j), on the stack
  int2 tiles[kMaxTiles];
  int64_t nt = 0;
  const int64_t nbb = (n + 19) / 20;
  for (int64_t I = 0; I < nb; ++I)
    for (int64_t J = 2 * I; J < nbb; ++J) tiles[nt++] = make_int2((int)I, (int)J);
  if (cudaMemcpyAsync(sc->tiles, tiles, (size_t)nt * sizeof(int2), cudaMemcpyHostToDevice, st) != cudaSuccess)
    return BS_ERR_CUDA;

  CUtensorMap tm[7];
  for (int m = 0; m < 7; ++m) {
    const int d = m < 4 ? m : m - 4;
    cuuint64_t gdim[2] = {(cuuint64_t)lp, (cuuint64_t)rows};
    cuuint64_t gstride[1] = {(cuuint64_t)lp * 2};
    cuuint32_t box[2] = {64, m < 4 ? 128u : 64u};
    cuuint32_t estr[2] = {1, 1};
    if (g_encode(&tm[m], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, sc->dig[d], gdim, gstride, box, estr,
                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return BS_ERR_CUDA;
  }
  TcArgs a{};
  a.tiles = sc->tiles;
  a.ntiles = nt;
  a.n = n;
  a.L = L;
  a.lp = lp;
  a.info = sc->info;
  a.sc = sc->scal;
  a.tol = 1e-4f;
  a.u = ldexpf(1.0f, 2 * hs.scale_exp);
  a.d34 = (float)d34;
  a.out = OutDesc{out, n, BS_LAYOUT_TRIANGLE, BS_OUT_F64};
  a.flags = sc->flags;
  a.flag_cap = kStaticFlagCap;
  a.dbg = nullptr;
  a.num_sms = sc->num_sms;
  if (launch_mixed_tc(tm, a, st) != cudaSuccess) return BS_ERR_CUDA;
  if (launch_refine_list(sc->dig, lp, L, sc->info, sc->scal, sc->flags, kStaticFlagCap, a.out, sc->num_sms, st) !=
      cudaSuccess)
    return BS_ERR_CUDA;
  if (cudaMemcpyAsync(&hs, sc->scal, sizeof(hs), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return BS_ERR_CUDA;
  if (hs.flag_count > kStaticFlagCap) {
    if (launch_refine_scan(sc->dig, lp, L, sc->info, sc->scal, a.out, sc->num_sms, st) != cudaSuccess)
      return BS_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return BS_ERR_CUDA;
  }
  if (hs.err & kErrTimeout) return BS_ERR_TIMEOUT;
  return BS_OK;
}
