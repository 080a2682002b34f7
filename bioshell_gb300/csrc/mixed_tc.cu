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
// level-4 products at 1/512 scale with a bounded rounding error.  TMEM holds
// two such accumulator sets, so the epilogue of one tile overlaps the MMAs
// of the next.  Tiles of long chains use both sets at once (the long
// layout, kernels.h): level 1 accumulated in two and level 2 in four parts
// of the chain, so each part stays exact where the whole chain's sum would
// not; the epilogue adds the parts as integers.  (When even that does not
// bound level 2 below 2^24, it accumulates up to 2^26 with its rounding
// charged to the job's error budget.)
//
// Roles (one persistent CTA per SM, 384 threads):
//   warp 0  TMA producer: 4 A digit boxes (128 rows x 64 atoms) and 3 B
//           digit boxes (64 rows x 64 atoms), 128-byte swizzle, 2 stages;
//           and per tile a bulk copy of its job and per-structure data
//           (kMetaSlots tiles ahead);
//   warp 1  MMA issuer: the whole warp runs the loop (its values stay
//           warp-uniform) and one elected lane issues tcgen05.mma kind::f16,
//           M = 128, N = 64 to 192: one instruction per A digit covers the
//           adjacent level accumulators its products go to (4 instructions
//           per 16-atom step instead of 9);
//   warp 2  TMEM allocation (512 columns);
//   warp 3  idle (keeps the epilogue warps on TMEM lane quarters w % 4);
//   warps 4-11  epilogue: warp w owns TMEM lanes 32 (w % 4) .. +31 (10 row
//           structures) and column group (w - 4) / 4 (10 column structures);
//           it stages one level at a time in shared memory, the thread of
//           coordinate x of structure i finishes pairs (i, j) with
//           j = x mod 3 through the three phases of crmsd_math.cuh, and
//           writes the result.
// Tiles come from a table of (A block, B block, job), handed out one at a
// time by a counter (DevScalars::tile_next, zero at launch): the TMA thread
// takes the next tile and passes its record to the MMA thread and the
// epilogue through the metadata slot, so all SMs work on a narrow window of
// the table and its operands stay in L2.  One launch serves any number of
// jobs -- the symmetric all-vs-all of one or many structure sets
// (pairs i < j), and query-vs-library blocks (every pair) -- each with its
// own chain length, grid and output.
// Every mbarrier wait is bounded; a timeout sets an error bit and all roles
// leave their loops so the block always reaches TMEM deallocation.
#include <cuda_fp16.h>

#include <type_traits>

#include "crmsd_math.cuh"
#include "kernels.h"
#include "ptx.cuh"

namespace bs {
namespace {

constexpr int kStages = 2;
constexpr int kBRows = 64;                               // B tile rows = 20 structures
constexpr int kAOpBytes = kBlockRows * kKChunk * 2;      // 16 KB
constexpr int kBOpBytes = kBRows * kKChunk * 2;          // 8 KB
constexpr int kStageBytes = 4 * kAOpBytes + 3 * kBOpBytes;
constexpr int kScreenStageBytes = 2 * kAOpBytes + 2 * kBOpBytes;  // digits 0 and 1 only
constexpr int kThreads = 384;
constexpr int kEpiWarp0 = 4;
constexpr int kEpiWarps = 8;
constexpr int kTmemCols = 512;                           // 2 buffers x 4 levels x 64 columns
// Epilogue staging per warp: two buffers of 32 rows x 16 columns, or for
// screen tiles one area of 32 rows x 32 columns (pitch 33).  Pitch 19: a
// lane's pair reads rows 3 il + [il >= 5] + xr at columns 3 x + c, and with
// 19 floats per row the 30 (il, x) of a warp fall in 30 different banks (17
// made 3-way conflicts); the per-lane row writes stay conflict-free (odd).
constexpr int kPitch = 19;
constexpr int kPitchWide = 33;
constexpr int kEpiStageFloats = 2 * 32 * kPitch;
static_assert(32 * kPitchWide <= kEpiStageFloats, "screen staging exceeds the warp's area");
constexpr int kEpiStageBytes = kEpiWarps * kEpiStageFloats * 4;
constexpr int kBarBytes = 256;

// What the epilogue needs of one tile: its record, its job and the
// per-structure data of its A and B blocks, bulk-copied into shared memory by
// the TMA thread together with the tile's operands, kMetaSlots tiles deep.
constexpr int kMetaSlots = 4;
struct __align__(16) TileMeta {
  SInfo ia[kBlockStructs];   // A-block structures (normal and long tiles)
  SInfo ib[kBStructs];       // B-block structures
  float2 ta[kBlockStructs];  // screen tiles: {G, RMS of digit 2} of the truncated structures
  float2 tb[kBStructs];
  Job job;
  Tile tile;
};
constexpr int kMetaBytes = kMetaSlots * (int)sizeof(TileMeta);
constexpr size_t kSmemBytes = 1024 + (size_t)kStages * kStageBytes + kEpiStageBytes + kMetaBytes + kBarBytes;
static_assert(kSmemBytes <= 232448, "dynamic shared memory above the 227 KB a block may use");
constexpr uint64_t kTimeoutNs = 4000000000ull;
constexpr uint32_t kIdesc = ptx::idesc_bf16_f32(128, kBRows);
constexpr uint32_t kIdescNarrow = ptx::idesc_bf16_f32(128, 32);  // narrow tiles: first 32 B rows
// One instruction per A digit against several B digits at once: the B digit
// boxes of a stage lie back to back (64 rows each), so an N = 128 or 192
// operand starting at digit d spans digits d, d+1 (, d+2), and the product
// lands in as many adjacent 64-column accumulators -- which is where the
// levels sit (level l at column 64 l).  An M = 128 instruction costs about
// the same up to N = 128, so this halves the instruction count.
constexpr uint32_t kIdesc128 = ptx::idesc_bf16_f32(128, 128);
constexpr uint32_t kIdesc192 = ptx::idesc_bf16_f32(128, 192);

struct Shared {
  uint64_t full[kStages];
  uint64_t empty[kStages];
  uint64_t tfull[2];
  uint64_t tempty[2];
  uint64_t mfull[kMetaSlots];   // tile metadata slot landed (bulk copies)
  uint64_t mempty[kMetaSlots];  // tile metadata slot released (epilogue)
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
  if (o.layout == kLayoutTriangle) {
    const int64_t idx = tri_index(o.n, i, j);
    if (o.out_type == 0) static_cast<unsigned long long *>(o.ptr)[idx] = bsm::f32_to_f64_bits(v);
    else static_cast<float *>(o.ptr)[idx] = v;
  } else if (o.layout == kLayoutRect) {
    const int64_t idx = i * o.ld + j;
    if (o.out_type == 0) static_cast<unsigned long long *>(o.ptr)[idx] = bsm::f32_to_f64_bits(v);
    else static_cast<float *>(o.ptr)[idx] = v;
  } else {
    if (o.out_type == 0) {
      const unsigned long long b = bsm::f32_to_f64_bits(v);
      static_cast<unsigned long long *>(o.ptr)[i * o.ld + j] = b;
      static_cast<unsigned long long *>(o.ptr)[j * o.ld + i] = b;
    } else {
      static_cast<float *>(o.ptr)[i * o.ld + j] = v;
      static_cast<float *>(o.ptr)[j * o.ld + i] = v;
    }
  }
}

// Neighbour layout: the warp's kept pairs appended with one atomic per warp
// (every lane of the warp calls this).
__device__ __forceinline__ void nbr_append(const OutDesc &o, bool hit, int64_t i, int64_t j, float v, int lane) {
  const unsigned m = __ballot_sync(0xffffffffu, hit);
  if (!m) return;
  const NbrSink *sk = static_cast<const NbrSink *>(o.ptr);
  const int lead = __ffs(m) - 1;
  unsigned long long base = 0;
  if (lane == lead) base = atomicAdd(sk->count, 2ull * (unsigned long long)__popc(m));
  base = __shfl_sync(0xffffffffu, base, lead);
  if (hit) {
    const unsigned long long s = base + 2ull * (unsigned long long)__popc(m & ((1u << lane) - 1u));
    if (s + 1 < sk->cap) {
      sk->ij[s] = make_int2((int)i, (int)j);
      sk->d[s] = v;
      sk->ij[s + 1] = make_int2((int)j, (int)i);
      sk->d[s + 1] = v;
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
  // 1024-byte aligned (128-byte swizzle atoms); offset arithmetic on the
  // shared array keeps every access below in the shared address space
  uint8_t *smem = smem_raw + ((1024u - (ptx::smem_u32(smem_raw) & 1023u)) & 1023u);
  float *stage_epi = reinterpret_cast<float *>(smem + (size_t)kStages * kStageBytes);
  TileMeta *meta = reinterpret_cast<TileMeta *>(smem + (size_t)kStages * kStageBytes + kEpiStageBytes);
  Shared *sh = reinterpret_cast<Shared *>(smem + (size_t)kStages * kStageBytes + kEpiStageBytes + kMetaBytes);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      ptx::mbar_init(&sh->full[s], 1);
      ptx::mbar_init(&sh->empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      ptx::mbar_init(&sh->tfull[b], 1);
      ptx::mbar_init(&sh->tempty[b], kEpiWarps * 32);
    }
    for (int b = 0; b < kMetaSlots; ++b) {
      ptx::mbar_init(&sh->mfull[b], 1);
      ptx::mbar_init(&sh->mempty[b], kEpiWarps * 32);
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
  // bound of the producer's and the MMA issuer's pipeline waits; the
  // epilogue keeps the default and leaves when they give up (abort)
  const uint64_t tmo = a.wait_ns ? a.wait_ns : kTimeoutNs;

  if (warp == 0) {
    if (lane == 0) {
      // ------------------------------------------------------ TMA producer
      uint32_t it = 0, tt = 0;
      unsigned long long *ctr = &a.sc->tile_next;
      int64_t t = (int64_t)atomicAdd(ctr, 1ull);
      Tile next = t < a.ntiles ? a.tiles[t] : Tile{};
      unsigned long long tn = 0;
      for (; !*abort; ++tt) {
        const Tile tile = next;
        {
          // the tile's metadata: record, job, per-structure data
          const uint32_t ms = tt % kMetaSlots;
          if (!ptx::mbar_wait(&sh->mempty[ms], ((tt / kMetaSlots) & 1u) ^ 1u, abort, tmo)) {
            fail(sh, a.sc);
            break;
          }
          TileMeta &mt = meta[ms];
          if (t >= a.ntiles) {
            // end of the table: a record with job -1 tells the MMA thread and
            // the epilogue to stop
            mt.tile = Tile{0, 0, -1, 0};
            ptx::mbar_arrive(&sh->mfull[ms]);
            ++tt;
            break;
          }
          mt.tile = tile;
          tn = atomicAdd(ctr, 1ull);  // used after this tile's loads are issued
          const bool nar = tile_narrow(tile), scr = tile_layout(tile) == kAccScreen;
          const int nbs = nar ? kNarrowStructs : kBStructs;
          const int64_t a0 = (int64_t)tile.a_blk * kBlockStructs, b0 = (int64_t)tile.b_blk * nbs;
          const uint32_t per = scr ? 8u : 16u;
          ptx::mbar_arrive_expect_tx(&sh->mfull[ms], (uint32_t)sizeof(Job) + per * (kBlockStructs + nbs));
          ptx::bulk_load(&mt.job, a.jobs + tile.job, (uint32_t)sizeof(Job), &sh->mfull[ms]);
          if (scr) {
            ptx::bulk_load(mt.ta, a.tinfo_a + a0, 8u * kBlockStructs, &sh->mfull[ms]);
            ptx::bulk_load(mt.tb, a.tinfo_b + b0, 8u * nbs, &sh->mfull[ms]);
          } else {
            ptx::bulk_load(mt.ia, a.info_a + a0, 16u * kBlockStructs, &sh->mfull[ms]);
            ptx::bulk_load(mt.ib, a.info_b + b0, 16u * nbs, &sh->mfull[ms]);
          }
        }
        const int rowA = tile.a_blk * kBlockRows;
        const int rowB = tile_narrow(tile) ? tile.b_blk * kGroupRows : tile.b_blk * kBRows;
        const int nchunks = (tile_nk16(tile) * 16 + kKChunk - 1) / kKChunk;
        const bool scr = tile_layout(tile) == kAccScreen;
        for (int kc = 0; kc < nchunks; ++kc, ++it) {
          const int s = it % kStages;
          const uint32_t ph = (it / kStages) & 1u;
          if (!ptx::mbar_wait(&sh->empty[s], ph ^ 1u, abort, tmo)) {
            fail(sh, a.sc);
            break;
          }
          ptx::mbar_arrive_expect_tx(&sh->full[s], scr ? kScreenStageBytes : kStageBytes);
          uint8_t *st = smem + (size_t)s * kStageBytes;
          const int k0 = kc * kKChunk;
          ptx::tma_load_2d(st + 0 * kAOpBytes, &ta0, k0, rowA, &sh->full[s]);
          ptx::tma_load_2d(st + 1 * kAOpBytes, &ta1, k0, rowA, &sh->full[s]);
          if (!scr) {
            ptx::tma_load_2d(st + 2 * kAOpBytes, &ta2, k0, rowA, &sh->full[s]);
            ptx::tma_load_2d(st + 3 * kAOpBytes, &ta3, k0, rowA, &sh->full[s]);
          }
          ptx::tma_load_2d(st + 4 * kAOpBytes + 0 * kBOpBytes, &tb0, k0, rowB, &sh->full[s]);
          ptx::tma_load_2d(st + 4 * kAOpBytes + 1 * kBOpBytes, &tb1, k0, rowB, &sh->full[s]);
          if (!scr) ptx::tma_load_2d(st + 4 * kAOpBytes + 2 * kBOpBytes, &tb2, k0, rowB, &sh->full[s]);
        }
        // the next tile: its record loads while this block waits for slots
        t = (int64_t)tn;
        if (t < a.ntiles) next = a.tiles[t];
      }
      // let the copies still in flight land before the block can retire
      for (uint32_t d = (it > kStages ? it - kStages : 0); d < it; ++d) {
        volatile int no_abort = 0;
        ptx::mbar_wait(&sh->full[d % kStages], (d / kStages) & 1u, &no_abort, 100000000ull);
      }
      for (uint32_t d = (tt > kMetaSlots ? tt - kMetaSlots : 0); d < tt; ++d) {
        volatile int no_abort = 0;
        ptx::mbar_wait(&sh->mfull[d % kMetaSlots], (d / kMetaSlots) & 1u, &no_abort, 100000000ull);
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    {
      // ------------------------------------------------------- MMA issuer
      // The whole warp runs the loop, so its values stay warp-uniform; one
      // elected lane issues the tensor-core instructions and their commits
      // (a commit tracks the MMAs of the thread that issues it).
      const bool leader = ptx::elect_one();
      // TMEM buffer slots are used in order: slot p is buffer p & 1 for the
      // (p >> 1)-th time.  A long- or half-layout tile takes two consecutive
      // slots (eight accumulators: accumulator a lives in slot p + a / 4).
      uint32_t it = 0, p = 0;
      for (uint32_t tt = 0; !*abort; ++tt) {
        // the tile's record, as the TMA thread took it from the table
        const uint32_t ms = tt % kMetaSlots;
        if (!__all_sync(0xffffffffu, ptx::mbar_wait(&sh->mfull[ms], (tt / kMetaSlots) & 1u, abort, tmo))) {
          fail(sh, a.sc);
          break;
        }
        const Tile tile = meta[ms].tile;
        if (tile.job < 0) break;
        const int nk16 = tile_nk16(tile);
        const int nchunks = (nk16 * 16 + kKChunk - 1) / kKChunk;
        const int lay = tile_layout(tile);
        const uint32_t idesc = tile_narrow(tile) ? kIdescNarrow : kIdesc;
        const uint32_t need = acc_two_buffers(lay) ? 2u : 1u;
        // half layout: the first 16-atom step of the second half
        // (acc_part(k, nk16, 2) == 1 from there on); never reached otherwise
        const int khalf = lay == kAccHalf ? (nk16 + 1) / 2 : 1 << 30;
        bool ok = true;
        for (uint32_t u = 0; u < need && ok; ++u) {
          const uint32_t q = p + u;
          if (!__all_sync(0xffffffffu, ptx::mbar_wait(&sh->tempty[q & 1u], ((q >> 1) & 1u) ^ 1u, abort, tmo))) {
            fail(sh, a.sc);
            ok = false;
          }
        }
        if (!ok) break;
        ptx::tc_fence_after();
        auto acc_col = [&](int ai) -> uint32_t { return tmem + ((p + (uint32_t)(ai >> 2)) & 1u) * 256u + (ai & 3) * 64u; };
        // the common tiles (normal or half layout, 20 B structures): four
        // side-by-side MMAs per step into [L0 | L1 | L2 | L3] at c_lo (the
        // half layout's second half at c_hi), the tile's columns fixed here
        const bool wide4 = (lay == kAccNormal || lay == kAccHalf) && !tile_narrow(tile);
        const uint32_t c_lo = acc_col(0), c_hi = acc_col(4);
        for (int kc = 0; kc < nchunks; ++kc, ++it) {
          const int s = it % kStages;
          const uint32_t ph = (it / kStages) & 1u;
          if (!__all_sync(0xffffffffu, ptx::mbar_wait(&sh->full[s], ph, abort, tmo))) {
            fail(sh, a.sc);
            ok = false;
            break;
          }
          ptx::tc_fence_after();
          const uint32_t base = ptx::smem_u32(smem + (size_t)s * kStageBytes);
          const uint32_t bbase = base + 4 * kAOpBytes;
          const int ksteps = min(4, nk16 - kc * 4);
          if (wide4) {
            // descriptors of the stage's boxes at step 0; a step, a digit
            // box or the B boxes are whole multiples of 16 bytes further on,
            // and the 14-bit address field cannot carry (shared addresses
            // stay below 2^18), so each descriptor is one addition away
            const uint64_t dA = ptx::smem_desc_sw128(base), dB = ptx::smem_desc_sw128(bbase);
            constexpr uint64_t kA16 = kAOpBytes >> 4, kB16 = kBOpBytes >> 4;
            for (int kk = 0; kk < ksteps; ++kk) {
              const int k = kc * 4 + kk;
              const uint64_t o = (uint64_t)kk * 2u;  // 32 bytes per 16-atom step
              const uint64_t da0 = dA + o, da1 = dA + kA16 + o, da2 = dA + 2 * kA16 + o, da3 = dA + 3 * kA16 + o;
              const uint64_t db0 = dB + o, db1 = dB + kB16 + o, db2 = dB + 2 * kB16 + o;
              const uint32_t c0 = k >= khalf ? c_hi : c_lo;
              if (k == 0 || k == khalf) {  // each accumulator's first write overwrites
                if (leader) ptx::tc_mma_f16(c0, da0, db0, kIdesc, 0u);           // L0 = e0e0
                if (leader) ptx::tc_mma_f16(c0 + 64, da1, db0, kIdesc192, 0u);   // L1 = e1e0, L2 = e1e1, L3 = e1e2
                if (leader) ptx::tc_mma_f16(c0 + 64, da0, db1, kIdesc128, 1u);   // L1 += e0e1, L2 += e0e2
              } else {
                if (leader) ptx::tc_mma_f16(c0, da0, db0, kIdesc192, 1u);        // L0 += e0e0, L1 += e0e1, L2 += e0e2
                if (leader) ptx::tc_mma_f16(c0 + 64, da1, db0, kIdesc192, 1u);   // L1 += e1e0, L2 += e1e1, L3 += e1e2
              }
              if (leader) ptx::tc_mma_f16(c0 + 128, da2, db0, kIdesc128, 1u);    // L2 += e2e0, L3 += e2e1
              if (leader) ptx::tc_mma_f16(c0 + 192, da3, db2, kIdesc, 1u);       // L3 += (e2/512) e2
            }
            if (leader) ptx::tc_commit(&sh->empty[s]);
            continue;
          }
          for (int kk = 0; kk < ksteps; ++kk) {
            const int k = kc * 4 + kk;
            const uint32_t off = (uint32_t)kk * 32u;
            const uint64_t da0 = ptx::smem_desc_sw128(base + 0 * kAOpBytes + off);
            const uint64_t da1 = ptx::smem_desc_sw128(base + 1 * kAOpBytes + off);
            const uint64_t da2 = ptx::smem_desc_sw128(base + 2 * kAOpBytes + off);
            const uint64_t da3 = ptx::smem_desc_sw128(base + 3 * kAOpBytes + off);
            const uint64_t db0 = ptx::smem_desc_sw128(bbase + 0 * kBOpBytes + off);
            const uint64_t db1 = ptx::smem_desc_sw128(bbase + 1 * kBOpBytes + off);
            const uint64_t db2 = ptx::smem_desc_sw128(bbase + 2 * kBOpBytes + off);
            if (lay == kAccScreen) {
              // digits 0 and 1 only: [L0 | L1 | L11] = [e0e0 | e0e1 + e1e0 |
              // e1e1], the exact covariance of the structures without digit 2
              const uint32_t c0 = acc_col(0);
              if (k == 0) {  // each accumulator's first write overwrites
                if (leader) ptx::tc_mma_f16(c0, da0, db0, kIdesc, 0u);           // L0 = e0e0
                if (leader) ptx::tc_mma_f16(c0 + 64, da1, db0, kIdesc128, 0u);   // L1 = e1e0, L11 = e1e1
                if (leader) ptx::tc_mma_f16(c0 + 64, da0, db1, kIdesc, 1u);      // L1 += e0e1
              } else {
                if (leader) ptx::tc_mma_f16(c0, da0, db0, kIdesc128, 1u);        // L0 += e0e0, L1 += e0e1
                if (leader) ptx::tc_mma_f16(c0 + 64, da1, db0, kIdesc128, 1u);   // L1 += e1e0, L11 += e1e1
              }
              continue;
            }
            uint32_t col[4], acc[4];  // per level: accumulator column, accumulate (vs overwrite)
            if (lay == kAccNormal) {
              // one buffer, level lv at column 64 lv; every level starts at step 0
              const uint32_t c0 = acc_col(0);
              const uint32_t first = k > 0 ? 1u : 0u;
#pragma unroll
              for (int lv = 0; lv < 4; ++lv) {
                col[lv] = c0 + lv * 64u;
                acc[lv] = first;
              }
            } else {
#pragma unroll
              for (int lv = 0; lv < 4; ++lv) {
                const int ai = acc_index(lay, lv, k, nk16);
                col[lv] = acc_col(ai);
                acc[lv] = (k > 0 && acc_index(lay, lv, k - 1, nk16) == ai) ? 1u : 0u;
              }
            }
            if (leader) ptx::tc_mma_f16(col[0], da0, db0, idesc, acc[0]);
            if (leader) ptx::tc_mma_f16(col[1], da0, db1, idesc, acc[1]);
            if (leader) ptx::tc_mma_f16(col[1], da1, db0, idesc, 1u);
            if (leader) ptx::tc_mma_f16(col[2], da0, db2, idesc, acc[2]);
            if (leader) ptx::tc_mma_f16(col[2], da1, db1, idesc, 1u);
            if (leader) ptx::tc_mma_f16(col[2], da2, db0, idesc, 1u);
            if (leader) ptx::tc_mma_f16(col[3], da1, db2, idesc, acc[3]);
            if (leader) ptx::tc_mma_f16(col[3], da2, db1, idesc, 1u);
            if (leader) ptx::tc_mma_f16(col[3], da3, db2, idesc, 1u);
          }
          if (leader) ptx::tc_commit(&sh->empty[s]);
        }
        if (!ok) break;
        for (uint32_t u = 0; u < need; ++u) if (leader) ptx::tc_commit(&sh->tfull[(p + u) & 1u]);
        p += need;
      }
      // all MMAs of this thread complete before teardown
      if (leader) ptx::tc_commit(&sh->drain);
      volatile int no_abort = 0;
      ptx::mbar_wait(&sh->drain, 0, &no_abort, 1000000000ull);
    }
    __syncwarp();
  } else if (warp >= kEpiWarp0) {
    // ---------------------------------------------------------- epilogue
    const int qd = warp & 3;                // TMEM lane quarter of this warp
    const int g = (warp - kEpiWarp0) >> 2;  // column group (10 structures)
    float *stg = stage_epi + (warp - kEpiWarp0) * kEpiStageFloats;
    // lane -> (row structure il, coordinate x) of the group layout: lanes
    // 0-14 hold structures 0-4, lanes 16-30 structures 5-9
    const int lt = lane - (lane >= 16 ? 1 : 0);
    const int il = lt / 3, x = lt - 3 * (lt / 3);
    const bool lane_real = lane != 15 && lane < 31;
    const int ilr = il < kGroupStructs ? il : kGroupStructs - 1;  // pad lanes read a valid row
    const uint32_t lane_base = tmem + ((uint32_t)(qd * 32) << 16) + 32u * g;
    uint32_t p = 0;   // TMEM buffer slot, as the MMA issuer counts them
    for (uint32_t tt = 0;; ++tt) {  // tile sequence number (metadata slot)
      const uint32_t slot = tt % kMetaSlots;
      // every lane waits (and so acquires what the phase publishes), and the
      // warp takes one decision: lanes must not part at a timeout, since
      // the tile's work below is warp-collective
      if (!__all_sync(0xffffffffu, ptx::mbar_wait(&sh->mfull[slot], (tt / kMetaSlots) & 1u, abort, kTimeoutNs))) {
        fail(sh, a.sc);
        break;
      }
      const TileMeta &mt = meta[slot];
      if (mt.tile.job < 0) break;  // end of the table
      const Job &mj = mt.job;
      const bool lng = mj.layout == kAccLong;
      const bool hlf = mj.layout == kAccHalf;
      const bool two = lng || hlf;  // the tile holds both TMEM buffers
      bool ok = true;
      for (uint32_t u = 0; u < (two ? 2u : 1u) && ok; ++u) {
        const uint32_t q = p + u;
        if (!__all_sync(0xffffffffu, ptx::mbar_wait(&sh->tfull[q & 1u], (q >> 1) & 1u, abort, kTimeoutNs))) {
          fail(sh, a.sc);
          ok = false;
        }
      }
      if (!ok) break;
      ptx::tc_fence_after();
      // the tile's scalars in registers (shared memory would be re-read
      // after every warp synchronisation)
      const int64_t jn = mj.n, jnb = mj.n_b, fa = mj.first_a, fb = mj.first_b;
      const bool sym = mj.mode == 0;
      const bool job_ok = mj.err == 0;
      const OutDesc out = mj.out;
      const float t_d34 = mj.d34, t_u = mj.u, t_tol = mj.tol;
      const int t_L = mj.L, t_job = mt.tile.job;
      const int t_ablk = mt.tile.a_blk, t_bblk = mt.tile.b_blk;
      // first B structure of this warp's column group (narrow tiles: group 1 has none)
      const int64_t jg0 = (int64_t)t_bblk * (mj.narrow ? kNarrowStructs : kBStructs) + g * kGroupStructs;
      const bool cols_ok = !(mj.narrow && g == 1);
      if (mj.layout == kAccScreen) {
        // ---- screen tile: a crmsd bracket per pair from levels 0 and 1 (the
        // truncated structures), stored as one word: hi (rounded up) and lo
        // (rounded down) halves
        uint32_t *sout = static_cast<uint32_t *>(out.ptr);
        __syncwarp();  // the previous tile's reads of the staging area are done
        {
          // m = L0 + 2^-9 L1 + 2^-18 L11: the covariance of the truncated
          // structures in units of 2^28 grid products
          const uint32_t c0 = lane_base + (p & 1u) * 256u;
          float m[32], v[32];
          ptx::tmem_ld2_32x32b_x32(c0 + 64, c0 + 128, m, v);
#pragma unroll
          for (int c = 0; c < 32; ++c) m[c] = fmaf(v[c], 0.001953125f, m[c]);
          ptx::tmem_ld_32x32b_x32(c0, v);
          ptx::tc_fence_before();
          ptx::mbar_arrive(&sh->tempty[p & 1u]);
#pragma unroll
          for (int c = 0; c < 32; ++c) stg[lane * kPitchWide + c] = fmaf(m[c], 0.001953125f, v[c]);
        }
        __syncwarp();
        // the warp's 10 x 10 pairs over its 32 lanes in four rounds, two
        // rounds at a time (two independent dependency chains per lane)
        const int64_t i0 = (int64_t)t_ablk * kBlockStructs + qd * kGroupStructs - fa;
        const int64_t j0 = jg0 - fb;
#pragma unroll 1
        for (int rd = 0; rd < 4; rd += 2) {
          float lo[2], hi[2];
          bool ok[2];
          int64_t oi[2];
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            const int pp = (rd + u) * 32 + lane;
            const int pc = pp < kGroupStructs * kGroupStructs ? pp : 0;  // pad slots read a valid pair
            const int ir = pc / kGroupStructs, jc = pc - kGroupStructs * (pc / kGroupStructs);
            const int64_t i = i0 + ir, j = j0 + jc;
            ok[u] = job_ok && cols_ok && pp < kGroupStructs * kGroupStructs && i < jn && j < jnb;
            oi[u] = i * out.ld + j;
            float m9[9];
#pragma unroll
            for (int xr = 0; xr < 3; ++xr)
#pragma unroll
              for (int y = 0; y < 3; ++y) m9[3 * xr + y] = stg[group_row(ir, xr) * kPitchWide + group_row(jc, y)];
            const float2 ta = mt.ta[qd * kGroupStructs + ir], tb = mt.tb[g * kGroupStructs + jc];
            bsm::screen_bracket(m9, ta.x + tb.x, t_d34, ta.y + tb.y, t_u, t_L, lo[u], hi[u]);
          }
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            if (!ok[u]) continue;
            const uint32_t wlo = __half_as_ushort(__float2half_rd(lo[u]));
            const uint32_t whi = __half_as_ushort(__float2half_ru(hi[u]));
            sout[oi[u]] = (whi << 16) | wlo;
          }
        }
        ptx::mbar_arrive(&sh->mempty[slot]);
        p += 1u;
        continue;
      }
      // accumulators of level lv: normal layout {lv}; long layout L0 {0},
      // L1 {1, 2}, L2 {3..6}, L3 {7}; half layout {lv, lv + 4};
      // accumulator ai sits in slot p + ai / 4
      auto acc_col = [&](int ai) -> uint32_t { return lane_base + ((p + (uint32_t)(ai >> 2)) & 1u) * 256u + (ai & 3) * 64u; };
      const int64_t ig = (int64_t)t_ablk * kBlockStructs + qd * kGroupStructs + il;
      const int64_t i = ig - fa;
      const bool row_ok = job_ok && cols_ok && lane_real && (il < kGroupStructs) && (i < jn);
      const SInfo ia = mt.ia[qd * kGroupStructs + ilr];
      const bool dump = (a.dbg != nullptr) && (t_ablk == 0) && (t_bblk < 2) && !two;
      // row of coordinate xr of this lane's row structure in the staging buffers
      int srow[3];
#pragma unroll
      for (int xr = 0; xr < 3; ++xr) srow[xr] = group_row(ilr, xr) * kPitch;
      // The group's 10 column structures are finished in two halves of five:
      // half h is TMEM columns 16h .. 16h+14 of the group (one 16-column
      // load per accumulator), and a lane carries at most two pairs at once.
      // The halves' work, compiled once per accumulator layout (the layout
      // is uniform over the tile): runtime layout branches inside it cost
      // the normal layout 10% in an A/B run.
      auto finish_halves = [&](auto layout_tag) {
        constexpr int kLay = decltype(layout_tag)::value;
        constexpr bool lng = kLay == kAccLong;
        constexpr bool hlf = kLay == kAccHalf;
        constexpr bool two = lng || hlf;
  #pragma unroll 1
        for (int h = 0; h < 2; ++h) {
          const uint32_t hc = 16u * (uint32_t)h;
          float *bufm = stg + kPitch * 32;  // FP32 covariance rows (buffer 1)
          // ---- pass A: FP32 covariance rows of this half, staged per lane
          {
            float m[16], v[16];
            ptx::tmem_ld2_32x32b_x16(acc_col(0) + hc, acc_col(1) + hc, m, v);
            if (hlf) {  // level 0 of the second half
              float w[16];
              ptx::tmem_ld_32x32b_x16(acc_col(4) + hc, w);
  #pragma unroll
              for (int c = 0; c < 16; ++c) m[c] += w[c];
            }
  #pragma unroll
            for (int c = 0; c < 16; ++c) m[c] = fmaf(v[c], 0.001953125f, m[c]);
  #pragma unroll
            for (int lv = 1; lv < 4; ++lv) {
              const float wl = lv == 1 ? 0.001953125f : (lv == 2 ? 3.814697265625e-6f : 7.450580596923828125e-9f);
  #pragma unroll
              for (int part = 0; part < 4; ++part) {
                // normal layout: accumulator lv; long: L1 {1, 2}, L2 {3..6},
                // L3 {7}; half: {lv, lv + 4}
                const int ai = lng ? (lv == 1 ? 1 + part : (lv == 2 ? 3 + part : 7)) : lv + 4 * part;
                const bool use = (lv == 1 && two && part == 1) ||
                                 (lv > 1 && (part == 0 || (lng && lv == 2) || (hlf && part == 1)));
                if (use) {
                  ptx::tmem_ld_32x32b_x16(acc_col(ai) + hc, v);
  #pragma unroll
                  for (int c = 0; c < 16; ++c) m[c] = fmaf(v[c], wl, m[c]);
                }
              }
            }
            __syncwarp();  // every lane is done with the previous half's last level (buffer 1)
  #pragma unroll
            for (int c = 0; c < 16; ++c) bufm[lane * kPitch + c] = m[c];
          }
          __syncwarp();
          bsm::FastState st[2];
          int64_t jj[2];
          bool valid[2];
          SInfo ib[2];
          int scol[2];
          {
            // the lane's two pairs through one packed FP32x2 QCP
            float m9[2][9], gs[2];
  #pragma unroll
            for (int sl = 0; sl < 2; ++sl) {
              const int jh = 3 * sl + x;  // owned structure within the half (0..5, valid < 5)
              const int jc = jh < 5 ? jh : 4;
              scol[sl] = 3 * jc;
              const int64_t jg = jg0 + 5 * h + jh;
              jj[sl] = jg - fb;
              valid[sl] = row_ok && (jh < 5) && (jj[sl] < jnb) && (!sym || jj[sl] > i);
              ib[sl] = mt.ib[g * kGroupStructs + 5 * h + jc];
  #pragma unroll
              for (int xr = 0; xr < 3; ++xr)
  #pragma unroll
                for (int y = 0; y < 3; ++y) m9[sl][3 * xr + y] = bufm[srow[xr] + scol[sl] + y];
              gs[sl] = valid[sl] ? ia.gf + ib[sl].gf : 0.f;
            }
            bsm::F2 mm[9];
  #pragma unroll
            for (int e = 0; e < 9; ++e) mm[e] = bsm::f2(m9[0][e], m9[1][e]);
            bsm::fast_begin2(mm, bsm::f2(gs[0], gs[1]), st[0], st[1]);
          }
          // ---- pass B: exact level sums, one level at a time (levels 0-2 as
          // integers: the parts of a long-layout level add exactly); level lv
          // is staged in buffer lv & 1, so one warp synchronisation per level
          // separates each buffer's writes from the previous reads
  #pragma unroll
          for (int lv = 0; lv < 4; ++lv) {
            float *buf = stg + (lv & 1) * kPitch * 32;
            const int a0 = lng ? (lv == 0 ? 0 : lv == 1 ? 1 : lv == 2 ? 3 : 7) : lv;
            float v[16];
            if (hlf) {
              // the level over both halves of the chain: levels 0-2 added as
              // integers (exact; v then holds their bit patterns), level 3 in FP32
              float w[16];
              ptx::tmem_ld2_32x32b_x16(acc_col(a0) + hc, acc_col(a0 + 4) + hc, v, w);
  #pragma unroll
              for (int c = 0; c < 16; ++c)
                v[c] = lv < 3 ? __int_as_float(__float2int_rn(v[c]) + __float2int_rn(w[c])) : v[c] + w[c];
            } else {
              ptx::tmem_ld_32x32b_x16(acc_col(a0) + hc, v);
            }
            if (dump) {
              float *drow = a.dbg + ((size_t)(lv * 128 + qd * 32 + lane)) * 128 + 64 * t_bblk + 32 * g + hc;
  #pragma unroll
              for (int c = 0; c < 16; ++c) drow[c] = v[c];
            }
            if (h == 1 && lv == 3) {
              // all TMEM reads of this tile are done: hand its buffers back to the MMA warp
              ptx::tc_fence_before();
              ptx::mbar_arrive(&sh->tempty[p & 1u]);
              if (two) ptx::mbar_arrive(&sh->tempty[(p + 1u) & 1u]);
            }
  #pragma unroll
            for (int c = 0; c < 16; ++c)
              buf[lane * kPitch + c] = (lv < 3 && !hlf) ? __int_as_float(__float2int_rn(v[c])) : v[c];
            if (lng && (lv == 1 || lv == 2)) {
              // further parts of the level, added into the staged row (integers stay exact)
  #pragma unroll
              for (int part = 1; part < 4; ++part) {
                if (lv == 1 && part > 1) break;
                ptx::tmem_ld_32x32b_x16(acc_col(a0 + part) + hc, v);
  #pragma unroll
                for (int c = 0; c < 16; ++c) {
                  float &d = buf[lane * kPitch + c];
                  d = __int_as_float(__float_as_int(d) + __float2int_rn(v[c]));
                }
              }
            }
            __syncwarp();
  #pragma unroll
            for (int sl = 0; sl < 2; ++sl) {
              float s9[9];
  #pragma unroll
              for (int xr = 0; xr < 3; ++xr)
  #pragma unroll
                for (int y = 0; y < 3; ++y) s9[3 * xr + y] = buf[srow[xr] + scol[sl] + y];
              bsm::fast_level_staged(st[sl], lv, s9);
            }
          }
          // ---- finish and store (neighbour layout: flagged pairs are kept or
          // dropped by the exact recomputation)
          const bool nbr = out.layout == kLayoutNeighbors;  // the same for the whole warp
  #pragma unroll
          for (int sl = 0; sl < 2; ++sl) {
            const int64_t j = jj[sl];
            int flag = 0;
            float r = 0.f;
            if (valid[sl]) {
              r = bsm::fast_finish(st[sl], ia.ghat + ib[sl].ghat, ia.gf + ib[sl].gf, ia.qres + ib[sl].qres, t_d34,
                                   t_u, t_L, t_tol, flag);
              if (flag) {
                if (!nbr) store_pair(out, i, j, -1.0f);
                const unsigned long long q = atomicAdd(&a.sc->flag_count, 1ull);
                if (q < a.flag_cap) a.flags[q] = flag_pack(t_job, ig, j + fb);
              } else if (!nbr) {
                store_pair(out, i, j, r);
              }
            }
            if (nbr) nbr_append(out, valid[sl] && !flag && r <= out.eps, i, j, r, lane);
          }
        }
      };
      if (hlf) finish_halves(std::integral_constant<int, kAccHalf>{});
      else if (lng) finish_halves(std::integral_constant<int, kAccLong>{});
      else finish_halves(std::integral_constant<int, kAccNormal>{});
      // the tile's metadata is no longer read: release its slot
      ptx::mbar_arrive(&sh->mempty[slot]);
      p += two ? 2u : 1u;
    }
  }
  __syncthreads();
  if (warp == 2) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, kTmemCols);
  }
}

__global__ void k_tile_shapes(Tile *tiles, int64_t ntiles, const Job *jobs) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ntiles; t += (int64_t)gridDim.x * blockDim.x) {
    const Job &jb = jobs[tiles[t].job];
    tiles[t].shape = (jb.lp / 16) | (jb.layout << 16) | (jb.narrow << 24);
  }
}

}  // namespace

cudaError_t launch_tile_shapes(Tile *tiles, int64_t ntiles, const Job *jobs, int num_sms, cudaStream_t st) {
  if (ntiles <= 0) return cudaSuccess;
  k_tile_shapes<<<num_sms * 8, 256, 0, st>>>(tiles, ntiles, jobs);
  return cudaGetLastError();
}

size_t mixed_tc_smem_bytes() { return kSmemBytes; }

// Kernel attributes, set once per device before any launch or capture.
cudaError_t mixed_tc_prepare() {
  return cudaFuncSetAttribute(k_mixed_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes);
}

cudaError_t launch_mixed_tc(const CUtensorMap *tm, const TcArgs &a, cudaStream_t st) {
  if (a.ntiles <= 0) return cudaSuccess;
  const int64_t grid = a.ntiles < a.num_sms ? a.ntiles : a.num_sms;
  k_mixed_tc<<<(unsigned)grid, kThreads, kSmemBytes, st>>>(tm[0], tm[1], tm[2], tm[3], tm[4], tm[5], tm[6], a);
  return cudaGetLastError();
}

}  // namespace bs
