// noalloc.cu -- bs_all_vs_all_static: the mixed-precision all-vs-all for
// callers that cannot allocate device memory.
//
// Some hosts embed the engine where device allocation is not theirs to do:
// a caller running inside another framework's memory pool, a plugin that may
// only use the buffers it is handed, or code that must not call cudaMalloc /
// cudaFree at all (for example to keep a process's device footprint fixed, or
// because the allocator is owned by someone else).  For them this entry point
// takes device pointers for the coordinates and the result and keeps every
// piece of scratch (digit matrices, per-structure data, job and tile tables,
// queue of pairs to recompute, counters) in file-scope static device arrays
// sized for at most kMaxN structures of at most kMaxL atoms.  Every GPU that
// loads this library holds those arrays (about 7.4 MB) until the process
// exits.
//
// The arrays are shared by all calls: each call clears what must start at
// zero, and calls whose work overlaps on the GPU (for example on two streams
// at once) race on the same scratch and must not be issued.
#include <string.h>

#include <mutex>

#include "engine.h"

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
static __device__ __align__(256) SInfo g_info[kMaxBlocks * kBlockStructs];
static __device__ __align__(256) long long g_ctr[kMaxBlocks * kBlockStructs * 3];
static __device__ __align__(256) Job g_job[1];
static __device__ __align__(256) int g_jobmap[kMaxBlocks];
static __device__ __align__(256) Tile g_tiles[kMaxTiles];
static __device__ __align__(256) unsigned long long g_flags[kStaticFlagCap];
static __device__ __align__(256) DevScalars g_scal;

constexpr int kMaxDevices = 64;
struct Scratch {
  bool ready = false;
  bool sm103 = false;  // the device is an sm_103 GPU (checked once, at set-up)
  __nv_bfloat16 *dig[4] = {};
  SInfo *info = nullptr;
  long long *ctr = nullptr;
  Job *job = nullptr;
  int *jobmap = nullptr;
  Tile *tiles = nullptr;
  unsigned long long *flags = nullptr;
  DevScalars *scal = nullptr;
  int num_sms = 0;
};
Scratch g_scratch[kMaxDevices];
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::mutex g_setup_mu;  // first calls on different devices may come from different threads

template <typename T>
bool symbol(T &sym, void **p) {
  return cudaGetSymbolAddress(p, sym) == cudaSuccess;
}

// Device addresses of the static arrays on the current device (host code may
// not use the array names as addresses), and the device's compute capability,
// looked up once per device.
bs_status setup(int dev, Scratch **out) {
  if (dev < 0 || dev >= kMaxDevices) return BS_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_setup_mu);
  Scratch &s = g_scratch[dev];
  if (!s.ready) {
    int major = 0, minor = 0;
    if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess)
      return BS_ERR_NO_DEVICE;
    s.sm103 = major == 10 && minor == 3;
    if (!s.sm103) {
      s.ready = true;
      return BS_ERR_NO_DEVICE;
    }
    void *p = nullptr;
    if (!symbol(g_digits, &p)) return BS_ERR_CUDA;
    for (int d = 0; d < 4; ++d) s.dig[d] = static_cast<__nv_bfloat16 *>(p) + (size_t)d * kDigitElems;
    if (!symbol(g_info, &p)) return BS_ERR_CUDA;
    s.info = static_cast<SInfo *>(p);
    if (!symbol(g_ctr, &p)) return BS_ERR_CUDA;
    s.ctr = static_cast<long long *>(p);
    if (!symbol(g_job, &p)) return BS_ERR_CUDA;
    s.job = static_cast<Job *>(p);
    if (!symbol(g_jobmap, &p)) return BS_ERR_CUDA;
    s.jobmap = static_cast<int *>(p);
    if (!symbol(g_tiles, &p)) return BS_ERR_CUDA;
    s.tiles = static_cast<Tile *>(p);
    if (!symbol(g_flags, &p)) return BS_ERR_CUDA;
    s.flags = static_cast<unsigned long long *>(p);
    if (!symbol(g_scal, &p)) return BS_ERR_CUDA;
    s.scal = static_cast<DevScalars *>(p);
    if (cudaDeviceGetAttribute(&s.num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return BS_ERR_CUDA;
    if (mixed_tc_prepare() != cudaSuccess || prep_prepare() != cudaSuccess) return BS_ERR_CUDA;
    if (!get_encoder(&g_encode).empty()) return BS_ERR_CUDA;
    s.ready = true;
  }
  if (!s.sm103) return BS_ERR_NO_DEVICE;
  *out = &s;
  return BS_OK;
}

}  // namespace
}  // namespace bs

using namespace bs;

extern "C" BS_API bs_status bs_all_vs_all_static(const double *xyz, int64_t n, int32_t L, double *out, void *stream) {
  if (n < 0 || L < 1) return BS_ERR_INVALID_ARG;
  if (n > kMaxN || L > kMaxL) return BS_ERR_UNSUPPORTED;  // beyond the static scratch
  if (n < 2) return BS_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the call copies tables from host memory, reads its counters back and
  // synchronises, none of which a stream capture allows: refuse before any
  // other CUDA call, so the caller's capture stays valid
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) return BS_ERR_CUDA;
  if (cap != cudaStreamCaptureStatusNone) return BS_ERR_UNSUPPORTED;
  if (!xyz || !out || !is_device_ptr(xyz) || !is_device_ptr(out)) return BS_ERR_INVALID_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return BS_ERR_NO_DEVICE;
  Scratch *sc = nullptr;
  bs_status s = setup(dev, &sc);
  if (s) return s;

  std::vector<JobSpec> specs{JobSpec{xyz, n, L, OutDesc{out, n, n, kLayoutTriangle, 0}}};
  Plan plan;
  if (!make_symmetric_plan(specs, 1e-4f, true, plan).empty()) return BS_ERR_UNSUPPORTED;
  MixedBuffers b{};
  b.ctr = sc->ctr;
  b.info_a = sc->info;
  b.info_b = sc->info;
  for (int d = 0; d < 4; ++d) b.dig_a[d] = sc->dig[d];
  for (int d = 0; d < 3; ++d) b.dig_b[d] = sc->dig[d];
  b.pitch_a = b.pitch_b = plan.pitch;
  b.rows_a = b.rows_b = plan.nblocks * kBlockRows;
  b.jobs = sc->job;
  b.jobmap = sc->jobmap;
  b.tiles = sc->tiles;
  b.flags = sc->flags;
  b.flag_cap = kStaticFlagCap;
  b.sc = sc->scal;
  if (cudaMemcpyAsync(b.jobmap, plan.jobmap.data(), plan.jobmap.size() * sizeof(int), cudaMemcpyHostToDevice, st) !=
          cudaSuccess ||
      cudaMemcpyAsync(b.tiles, plan.tiles.data(), plan.tiles.size() * sizeof(Tile), cudaMemcpyHostToDevice, st) !=
          cudaSuccess)
    return BS_ERR_CUDA;
  CUtensorMap tm[7];
  if (!encode_maps(g_encode, b, tm).empty()) return BS_ERR_CUDA;
  Job job = plan.jobs[0];
  if (enqueue_mixed(plan, b, &job, tm, sc->num_sms, st, nullptr, false) != cudaSuccess) return BS_ERR_CUDA;
  DevScalars hs{};
  Job back{};
  if (cudaMemcpyAsync(&back, b.jobs, sizeof(Job), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(&hs, b.sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return BS_ERR_CUDA;
  std::string msg;
  return collect_errors(hs, &back, 1, msg);
}
