// mixed_tc.cu -- all-vs-all crmsd on tcgen05 tensor cores (sm_103a).
//
// The per-pair 3x3 covariances of a 40 x 20 block of structures are the
// 3x3 blocks of one 128 x 64 tile of X X^T, where X holds a row per
// (structure, coordinate) and a column per atom (layout in kernels.h).  X is
// split into exact bf16 digit matrices D0, D1, D2 (prep.cu) and D2s = D2/512;
// per 16-atom step the kernel issues the nine digit products
//     L0 += D0 D0'   L1 += D0 D1' + D1 D0'
//     L2 += D0 D2' + D1 D1' + D2 D0'   L3 += D1 D2' + D2 D1' + D2s D2'
// into four FP32 accumulators of 128 lanes x 64 columns in TMEM.  Levels 0-2
// are integers below 2^24, so their accumulation is exact; L3 carries the
// level-4 products at 1/512 scale with a bounded rounding error.  TMEM
// holds two such accumulator sets, so the epilogue of one tile overlaps the
// MMAs of the next.
//
// Roles (one persistent CTA per SM, 384 threads):
//   warp 0  TMA producer: 4 A digit boxes (128 rows x 64 atoms) and 3 B
//           digit boxes (64 rows x 64 atoms), 128-byte swizzle, 2 stages;
//   warp 1  MMA issuer (one thread), tcgen05.mma kind::f16, M = 128, N = 64;
//   warp 2  TMEM allocation (512 columns);
//   warps 4-11  epilogue: warp w owns TMEM lanes 32 (w % 4) .. +31 (10 row
//           structures) and column group (w - 4) / 4 (10 column structures);
//           it stages one level at a time in shared memory, the thread of
//           coordinate x of structure i finishes pairs (i, j) with
//           j = x mod 3 through the three phases of crmsd_math.cuh, and
//           writes the result.
// Every mbarrier wait is bounded; a timeout sets an error bit and all roles
// leave their loops so the block always reaches TMEM deallocation.
#include "crmsd_math.cuh"
#include "kernels.h"
#include "ptx.cuh"

namespace bs {
namespace {

constexpr int kStages = 2;
constexpr int kKChunk = 64;                              // atoms per 128-byte swizzle row
constexpr int kBRows = 64;                               // B tile rows = 20 structures
constexpr int kAOpBytes = kBlockRows * kKChunk * 2;      // 16 KB
constexpr int kBOpBytes = kBRows * kKChunk * 2;          // 8 KB
constexpr int kStageBytes = 4 * kAOpBytes + 3 * kBOpBytes;
constexpr int kThreads = 384;
constexpr int kEpiWarp0 = 4;
constexpr int kEpiWarps = 8;
constexpr int kTmemCols = 512;                           // 2 buffers x 4 levels x 64 columns
constexpr int kPitch = 33;                               // staging pitch in floats
constexpr int kEpiStageBytes = kEpiWarps * 32 * kPitch * 4;
constexpr int kBarBytes = 256;
constexpr size_t kSmemBytes = 1024 + (size_t)kStages * kStageBytes + kEpiStageBytes + kBarBytes;
constexpr uint64_t kTimeoutNs = 4000000000ull;
constexpr uint32_t kIdesc = ptx::idesc_bf16_f32(128, kBRows);

struct Shared {
  uint64_t full[kStages];
  uint64_t empty[kStages];
  uint64_t tfull[2];
  uint64_t tempty[2];
  uint64_t drain;
  uint32_t tmem_base;
  int abort;
};

__device__ __forceinline__ int64_t tri_index(int64_t n, int64_t i, int64_t j) {
  return i * n - i * (i + 1) / 2 + (j - i - 1);
}

// f64 results are written as bit patterns built with integer operations
// (a float -> double conversion would run on the slow FP64 pipe).
__device__ __forceinline__ void store_pair(const OutDesc &o, int64_t i, int64_t j, float v) {
  if (o.layout == 0) {
    const int64_t idx = tri_index(o.n, i, j);
    if (o.out_type == 0) static_cast<unsigned long long *>(o.ptr)[idx] = bsm::f32_to_f64_bits(v);
    else static_cast<float *>(o.ptr)[idx] = v;
  } else {
    if (o.out_type == 0) {
      const unsigned long long b = bsm::f32_to_f64_bits(v);
      static_cast<unsigned long long *>(o.ptr)[i * o.n + j] = b;
      static_cast<unsigned long long *>(o.ptr)[j * o.n + i] = b;
    } else {
      static_cast<float *>(o.ptr)[i * o.n + j] = v;
      static_cast<float *>(o.ptr)[j * o.n + i] = v;
    }
  }
}

__device__ __forceinline__ void fail(Shared *sh, DevScalars *sc) {
  sh->abort = 1;
  atomicOr(&sc->err, kErrTimeout);
}

__global__ void __launch_bounds__(kThreads, 1)
    k_mixed_tc(const __grid_constant__ CUtensorMap ta0, const __grid_constant__ CUtensorMap ta1,
               const __grid_constant__ CUtensorMap ta2, const __grid_constant__ CUtensorMap ta3,
               const __grid_constant__ CUtensorMap tb0, const __grid_constant__ CUtensorMap tb1,
               const __grid_constant__ CUtensorMap tb2, TcArgs a) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  float *stage_epi = reinterpret_cast<float *>(smem + (size_t)kStages * kStageBytes);
  Shared *sh = reinterpret_cast<Shared *>(smem + (size_t)kStages * kStageBytes + kEpiStageBytes);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nk16 = a.lp / 16;
  const int nchunks = (a.lp + kKChunk - 1) / kKChunk;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      ptx::mbar_init(&sh->full[s], 1);
      ptx::mbar_init(&sh->empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      ptx::mbar_init(&sh->tfull[b], 1);
      ptx::mbar_init(&sh->tempty[b], kEpiWarps * 32);
    }
    ptx::mbar_init(&sh->drain, 1);
    sh->abort = 0;
    ptx::fence_mbar_init();
    ptx::prefetch_tmap(&ta0);
    ptx::prefetch_tmap(&ta1);
    ptx::prefetch_tmap(&ta2);
    ptx::prefetch_tmap(&ta3);
    ptx::prefetch_tmap(&tb0);
    ptx::prefetch_tmap(&tb1);
    ptx::prefetch_tmap(&tb2);
  }
  if (warp == 2) {
    ptx::tmem_alloc(&sh->tmem_base, kTmemCols);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = sh->tmem_base;
  volatile int *abort = &sh->abort;

  if (warp == 0) {
    if (lane == 0) {
      // ------------------------------------------------------ TMA producer
      uint32_t it = 0;
      for (int64_t t = blockIdx.x; t < a.ntiles && !*abort; t += gridDim.x) {
        const int2 tile = a.tiles[t];
        const int rowA = tile.x * kBlockRows, rowB = tile.y * kBRows;
        for (int kc = 0; kc < nchunks; ++kc, ++it) {
          const int s = it % kStages;
          const uint32_t ph = (it / kStages) & 1u;
          if (!ptx::mbar_wait(&sh->empty[s], ph ^ 1u, abort, kTimeoutNs)) {
            fail(sh, a.sc);
            break;
          }
          ptx::mbar_arrive_expect_tx(&sh->full[s], kStageBytes);
          uint8_t *st = smem + (size_t)s * kStageBytes;
          const int k0 = kc * kKChunk;
          ptx::tma_load_2d(st + 0 * kAOpBytes, &ta0, k0, rowA, &sh->full[s]);
          ptx::tma_load_2d(st + 1 * kAOpBytes, &ta1, k0, rowA, &sh->full[s]);
          ptx::tma_load_2d(st + 2 * kAOpBytes, &ta2, k0, rowA, &sh->full[s]);
          ptx::tma_load_2d(st + 3 * kAOpBytes, &ta3, k0, rowA, &sh->full[s]);
          ptx::tma_load_2d(st + 4 * kAOpBytes + 0 * kBOpBytes, &tb0, k0, rowB, &sh->full[s]);
          ptx::tma_load_2d(st + 4 * kAOpBytes + 1 * kBOpBytes, &tb1, k0, rowB, &sh->full[s]);
          ptx::tma_load_2d(st + 4 * kAOpBytes + 2 * kBOpBytes, &tb2, k0, rowB, &sh->full[s]);
        }
      }
      // let the stages still in flight land before the block can retire
      for (uint32_t d = (it > kStages ? it - kStages : 0); d < it; ++d) {
        volatile int no_abort = 0;
        ptx::mbar_wait(&sh->full[d % kStages], (d / kStages) & 1u, &no_abort, 100000000ull);
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {
      // ------------------------------------------------------- MMA issuer
      uint32_t it = 0, tt = 0;
      for (int64_t t = blockIdx.x; t < a.ntiles && !*abort; t += gridDim.x, ++tt) {
        const uint32_t buf = tt & 1u, use = tt >> 1;
        if (!ptx::mbar_wait(&sh->tempty[buf], (use & 1u) ^ 1u, abort, kTimeoutNs)) {
          fail(sh, a.sc);
          break;
        }
        ptx::tc_fence_after();
        const uint32_t acc0 = tmem + buf * 256u;
        bool ok = true;
        for (int kc = 0; kc < nchunks; ++kc, ++it) {
          const int s = it % kStages;
          const uint32_t ph = (it / kStages) & 1u;
          if (!ptx::mbar_wait(&sh->full[s], ph, abort, kTimeoutNs)) {
            fail(sh, a.sc);
            ok = false;
            break;
          }
          ptx::tc_fence_after();
          const uint32_t base = ptx::smem_u32(smem + (size_t)s * kStageBytes);
          const uint32_t bbase = base + 4 * kAOpBytes;
          const int ksteps = min(4, nk16 - kc * 4);
          for (int kk = 0; kk < ksteps; ++kk) {
            const uint32_t off = (uint32_t)kk * 32u;
            const uint64_t da0 = ptx::smem_desc_sw128(base + 0 * kAOpBytes + off);
            const uint64_t da1 = ptx::smem_desc_sw128(base + 1 * kAOpBytes + off);
            const uint64_t da2 = ptx::smem_desc_sw128(base + 2 * kAOpBytes + off);
            const uint64_t da3 = ptx::smem_desc_sw128(base + 3 * kAOpBytes + off);
            const uint64_t db0 = ptx::smem_desc_sw128(bbase + 0 * kBOpBytes + off);
            const uint64_t db1 = ptx::smem_desc_sw128(bbase + 1 * kBOpBytes + off);
            const uint64_t db2 = ptx::smem_desc_sw128(bbase + 2 * kBOpBytes + off);
            const uint32_t acc = (kc | kk) ? 1u : 0u;
            ptx::tc_mma_f16(acc0 + 0 * 64, da0, db0, kIdesc, acc);
            ptx::tc_mma_f16(acc0 + 1 * 64, da0, db1, kIdesc, acc);
            ptx::tc_mma_f16(acc0 + 1 * 64, da1, db0, kIdesc, 1u);
            ptx::tc_mma_f16(acc0 + 2 * 64, da0, db2, kIdesc, acc);
            ptx::tc_mma_f16(acc0 + 2 * 64, da1, db1, kIdesc, 1u);
            ptx::tc_mma_f16(acc0 + 2 * 64, da2, db0, kIdesc, 1u);
            ptx::tc_mma_f16(acc0 + 3 * 64, da1, db2, kIdesc, acc);
            ptx::tc_mma_f16(acc0 + 3 * 64, da2, db1, kIdesc, 1u);
            ptx::tc_mma_f16(acc0 + 3 * 64, da3, db2, kIdesc, 1u);
          }
          ptx::tc_commit(&sh->empty[s]);
        }
        if (!ok) break;
        ptx::tc_commit(&sh->tfull[buf]);
      }
      // all MMAs of this thread complete before teardown
      ptx::tc_commit(&sh->drain);
      volatile int no_abort = 0;
      ptx::mbar_wait(&sh->drain, 0, &no_abort, 1000000000ull);
    }
    __syncwarp();
  } else if (warp >= kEpiWarp0) {
    // ---------------------------------------------------------- epilogue
    const int qd = warp & 3;                // TMEM lane quarter of this warp
    const int g = (warp - kEpiWarp0) >> 2;  // column group (10 structures)
    float *stg = stage_epi + (warp - kEpiWarp0) * 32 * kPitch;
    const int il = lane / 3, x = lane - 3 * (lane / 3);
    const int ilr = il < kGroupStructs ? il : kGroupStructs - 1;  // pad lanes read a valid row
    const uint32_t lane_base = tmem + ((uint32_t)(qd * 32) << 16) + 32u * g;
    uint32_t tt = 0;
    for (int64_t t = blockIdx.x; t < a.ntiles; t += gridDim.x, ++tt) {
      const uint32_t buf = tt & 1u, use = tt >> 1;
      if (!ptx::mbar_wait(&sh->tfull[buf], use & 1u, abort, kTimeoutNs)) {
        fail(sh, a.sc);
        break;
      }
      ptx::tc_fence_after();
      const int2 tile = a.tiles[t];
      const uint32_t col0 = lane_base + buf * 256u;
      const int64_t i = (int64_t)tile.x * kBlockStructs + qd * kGroupStructs + il;
      const bool row_ok = (lane < 30) && (i < a.n);
      SInfo ia{};
      if (row_ok) ia = a.info[i];
      const bool dump = (a.dbg != nullptr) && (tile.x == 0) && (tile.y < 2);
      // The group's 10 column structures are finished in two halves of five
      // (columns 15h .. 15h+14), so a lane carries at most two pairs at once.
#pragma unroll 1
      for (int h = 0; h < 2; ++h) {
        const int c0 = 15 * h;  // first TMEM column of this half within the group
        // ---- pass A: FP32 covariance rows of this half, staged per lane
        {
          float m[32], v[32];
          ptx::tmem_ld_32x32b_x32(col0 + 0 * 64, m);
          ptx::tmem_ld_32x32b_x32(col0 + 1 * 64, v);
#pragma unroll
          for (int c = 0; c < 32; ++c) m[c] = fmaf(v[c], 0.001953125f, m[c]);  // 2^-9
          ptx::tmem_ld_32x32b_x32(col0 + 2 * 64, v);
#pragma unroll
          for (int c = 0; c < 32; ++c) m[c] = fmaf(v[c], 3.814697265625e-6f, m[c]);  // 2^-18
          ptx::tmem_ld_32x32b_x32(col0 + 3 * 64, v);
#pragma unroll
          for (int c = 0; c < 32; ++c) m[c] = fmaf(v[c], 7.450580596923828125e-9f, m[c]);  // 2^-27
#pragma unroll
          for (int c = 0; c < 16; ++c) stg[lane * kPitch + c] = h ? m[15 + c] : m[c];
        }
        __syncwarp();
        bsm::FastState st[2];
        int64_t jj[2];
        bool valid[2];
        SInfo ib[2];
#pragma unroll
        for (int sl = 0; sl < 2; ++sl) {
          const int jh = 3 * sl + x;  // owned structure within the half (0..5, valid < 5)
          const int jc = jh < 5 ? jh : 4;
          jj[sl] = (int64_t)tile.y * 20 + g * kGroupStructs + 5 * h + jh;
          valid[sl] = row_ok && (jh < 5) && (jj[sl] < a.n) && (jj[sl] > i);
          ib[sl] = SInfo{};
          if (valid[sl]) ib[sl] = a.info[jj[sl]];
          float m9[9];
#pragma unroll
          for (int xr = 0; xr < 3; ++xr)
#pragma unroll
            for (int y = 0; y < 3; ++y) m9[3 * xr + y] = stg[(3 * ilr + xr) * kPitch + 3 * jc + y];
          bsm::fast_begin(m9, valid[sl] ? ia.gf + ib[sl].gf : 0.f, st[sl]);
        }
        __syncwarp();
        // ---- pass B: exact level sums, one level at a time
#pragma unroll
        for (int lv = 0; lv < 4; ++lv) {
          float v[32];
          ptx::tmem_ld_32x32b_x32(col0 + lv * 64, v);
          if (dump && h == 0) {
            float *drow = a.dbg + ((size_t)(lv * 128 + qd * 32 + lane)) * 128 + 64 * tile.y + 32 * g;
#pragma unroll
            for (int c = 0; c < 32; ++c) drow[c] = v[c];
          }
#pragma unroll
          for (int c = 0; c < 16; ++c) stg[lane * kPitch + c] = h ? v[15 + c] : v[c];
          __syncwarp();
#pragma unroll
          for (int sl = 0; sl < 2; ++sl) {
            const int jh = 3 * sl + x;
            const int jc = jh < 5 ? jh : 4;
            float s9[9];
#pragma unroll
            for (int xr = 0; xr < 3; ++xr)
#pragma unroll
              for (int y = 0; y < 3; ++y) s9[3 * xr + y] = stg[(3 * ilr + xr) * kPitch + 3 * jc + y];
            bsm::fast_level(st[sl], lv, s9);
          }
          __syncwarp();
        }
        if (h == 1) {
          // all TMEM reads of this buffer are done: hand it back to the MMA warp
          ptx::tc_fence_before();
          ptx::mbar_arrive(&sh->tempty[buf]);
        }
        // ---- finish and store
#pragma unroll
        for (int sl = 0; sl < 2; ++sl) {
          if (!valid[sl]) continue;
          const int64_t j = jj[sl];
          int flag = 0;
          const float r = bsm::fast_finish(st[sl], ia.ghat + ib[sl].ghat, ia.gf + ib[sl].gf, ia.qres + ib[sl].qres,
                                           a.d34, a.u, a.L, a.tol, flag);
          if (flag) {
            store_pair(a.out, i, j, -1.0f);
            const unsigned long long slot = atomicAdd(&a.sc->flag_count, 1ull);
            if (slot < a.flag_cap) a.flags[slot] = ((unsigned long long)i << 32) | (unsigned long long)j;
          } else {
            store_pair(a.out, i, j, r);
          }
        }
      }
    }
  }
  __syncthreads();
  if (warp == 2) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, kTmemCols);
  }
}

}  // namespace

size_t mixed_tc_smem_bytes() { return kSmemBytes; }

cudaError_t launch_mixed_tc(const CUtensorMap *tm, const TcArgs &a, cudaStream_t st) {
  if (a.ntiles <= 0) return cudaSuccess;
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(k_mixed_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  const int64_t grid = a.ntiles < a.num_sms ? a.ntiles : a.num_sms;
  k_mixed_tc<<<(unsigned)grid, kThreads, kSmemBytes, st>>>(tm[0], tm[1], tm[2], tm[3], tm[4], tm[5], tm[6], a);
  return cudaGetLastError();
}

}  // namespace bs
