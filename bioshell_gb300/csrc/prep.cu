// prep.cu -- streaming preparation passes over the input coordinates.
//
// Mixed path (all jobs of a launch at once, no host round trip):
//   center  per structure: coordinates read as fixed-point integers (units
//           2^-32 A, exact for the 3-decimal coordinates of PDB/mmCIF
//           files), centroid (arithmetic mean, as bioshell-pdb's
//           SubstructureAxis centres, calc/substructures.rs:26-31), largest
//           centred coordinate of the job;
//   scale   per job: the finest grid 2^e with every centred coordinate below
//           (2^22 - 1) 2^e;
//   norms   per structure: for grids e .. e+3, the row norms of the three
//           balanced digits (9, 9 and 5 bits) of the quantised coordinates;
//   choose  per job, from Cauchy-Schwarz bounds on the row norms: the
//           finest grid whose tensor-core level sums 0-2 all stay below 2^24
//           (exact) while its quantisation fits the error budget; for long
//           chains, where no such grid exists, the finest grid with levels 0
//           and 1 exact and level 2 below 2^26, its rounding (and level 3's)
//           charged to the error budget;
//   digits  per structure: digit rows (bf16), exact squared norm, RMS
//           quantisation residual.
// All of it is integer arithmetic: the FP64 pipe is not used.
//
// Plain path: FP64 centring into K-major [n][3][lp] and G.
#include <limits.h>
#include <math.h>

#include "crmsd_math.cuh"
#include "kernels.h"

namespace bs {
namespace {

constexpr int kWarpsPerBlock = 4;

__device__ __forceinline__ long long warp_sum64(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ unsigned warp_sum32(unsigned v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ unsigned long long warp_max64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}

// round(x * 2^32) from the bits of x, with integer operations only.
// Returns 0, or kErrNonFinite for NaN/Inf, or kErrUnsupported for
// |x| >= 2^15 A (outside the fixed-point range).
__device__ __forceinline__ int to_fix(double x, long long &out) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7ff);
  // |x| = mant 2^(ex - 1075) = mant 2^(sh) fixed-point units, mant in [2^52, 2^53)
  const int sh = ex - 1043;
  out = 0;
  if (ex == 0x7ff) return kErrNonFinite;
  if (sh > -6) return kErrUnsupported;  // |x| >= 2^15
  const unsigned long long mant = (b & 0xfffffffffffffull) | 0x10000000000000ull;
  long long v = 0;
  if (ex != 0 && sh > -63) v = (long long)((mant + (1ull << (-sh - 1))) >> (-sh));  // round half up
  out = (b >> 63) ? -v : v;
  return 0;
}

struct Where {
  int job;
  int64_t local;  // structure index within the job (< n when valid)
  bool valid;
};

__device__ __forceinline__ Where locate(const PrepArgs &p, int64_t g) {
  Where w;
  w.job = p.job_of_struct_block[g / kBlockStructs];
  w.local = 0;
  w.valid = false;
  if (w.job < 0) return w;
  const Job &jb = p.jobs[w.job];
  w.local = g - jb.first_a;
  w.valid = w.local >= 0 && w.local < jb.n;
  return w;
}

// Each warp takes a run of consecutive structures (usually all of one job)
// and keeps the job-wide maxima of the run in registers: one atomic per job
// change instead of one per structure (same-address atomics serialise).
// Runs are at most 8 structures, so the block scheduler balances sets of
// different chain lengths, and shorter where that leaves fewer than about
// 32 warps per SM.
struct Run {
  int64_t g0, g1;
};
__device__ __forceinline__ Run warp_run(int64_t s0, int64_t nstructs, int run) {
  const int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  Run r;
  r.g0 = s0 + w * run;
  r.g1 = r.g0 + run < nstructs ? r.g0 + run : nstructs;
  return r;
}

__device__ __forceinline__ long long warp_min64s(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w < v ? w : v;
  }
  return v;
}
__device__ __forceinline__ long long warp_max64s(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}

// ------------------------------------------------------------------ center
// One read of the coordinates: per component the sum (centroid) and the
// extremes; the largest centred coordinate max|v - C| is max(vmax - C,
// C - vmin), the same value a second pass over |v - C| would find.
__global__ void __launch_bounds__(kWarpsPerBlock * 32) k_mx_center(PrepArgs p, int64_t nstructs, int run_len) {
  const int lane = threadIdx.x & 31;
  const Run run = warp_run(p.s_lo, nstructs, run_len);
  int cur = -1;                // job whose maximum is being gathered
  unsigned long long mrun = 0;  // its largest centred coordinate so far
  for (int64_t g = run.g0; g < run.g1; ++g) {
    const Where w = locate(p, g);
    if (!w.valid) continue;
    if (w.job != cur) {
      if (cur >= 0 && lane == 0) atomicMax(&p.jobs[cur].maxabs, mrun);
      cur = w.job;
      mrun = 0;
    }
    Job &jb = p.jobs[w.job];
    const int L = jb.L;
    const double *x = jb.xyz + w.local * 3 * (int64_t)L;
    long long s[3] = {0, 0, 0};
    long long lo[3] = {LLONG_MAX, LLONG_MAX, LLONG_MAX}, hi[3] = {LLONG_MIN, LLONG_MIN, LLONG_MIN};
    int bad = 0;
    int c = lane % 3;
    // four coalesced loads in flight per lane, then their updates in order
    for (int i0 = lane; i0 < 3 * L; i0 += 128) {
      double xv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) xv[u] = i0 + 32 * u < 3 * L ? x[i0 + 32 * u] : 0.0;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (i0 + 32 * u < 3 * L) {
          long long v;
          bad |= to_fix(xv[u], v);
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            if (c == k) {
              s[k] += v;
              lo[k] = v < lo[k] ? v : lo[k];
              hi[k] = v > hi[k] ? v : hi[k];
            }
          }
        }
        c = (c + 2) % 3;  // (i + 32) mod 3
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    if (bad) {
      if (lane == 0) atomicOr(&jb.err, bad);
      continue;
    }
    long long C[3];
    unsigned long long m = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const long long t = warp_sum64(s[k]);
      const long long h = L / 2;
      C[k] = t >= 0 ? (t + h) / L : -((-t + h) / L);
      const long long vlo = warp_min64s(lo[k]), vhi = warp_max64s(hi[k]);
      const unsigned long long a0 = (unsigned long long)(vhi - C[k]), a1 = (unsigned long long)(C[k] - vlo);
      m = a0 > m ? a0 : m;
      m = a1 > m ? a1 : m;
    }
    mrun = m > mrun ? m : mrun;
    if (lane == 0) {
      p.ctr[3 * g + 0] = C[0];
      p.ctr[3 * g + 1] = C[1];
      p.ctr[3 * g + 2] = C[2];
    }
  }
  if (cur >= 0 && lane == 0) atomicMax(&p.jobs[cur].maxabs, mrun);
}

// ------------------------------------------------------------------- scale
// a banded launch prepares only the jobs whose structures lie in its range
__device__ __forceinline__ bool job_in_range(const PrepArgs &p, const Job &jb) {
  return jb.first_a >= p.s_lo && (p.s_hi < 0 || jb.first_a < p.s_hi);
}

__global__ void k_mx_scale(PrepArgs p) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= p.njobs) return;
  Job &jb = p.jobs[j];
  if (!job_in_range(p, jb)) return;
  // smallest e with every centred coordinate <= (2^22 - 1) 2^e (the range of
  // the three balanced digits); one thread per job, so plain FP64 is fine
  const double m = (double)jb.maxabs * 2.3283064365386963e-10;  // Angstrom
  const double lim = 4194303.0;
  int e = -40;
  if (m > 0.0) {
    e = (int)ceil(log2(m / lim));
    while (ldexp(lim, e) < m) ++e;
    while (ldexp(lim, e - 1) >= m) --e;
  }
  if (jb.fixed_scale) {
    if (e > jb.scale_min) atomicOr(&jb.err, kErrUnsupported);  // beyond the given grid's range
    e = jb.scale_min;
  } else if (e < jb.scale_min) {
    e = jb.scale_min;
  }
  if (e < 1 - kFixBits) e = 1 - kFixBits;  // the grid is never finer than 2 fixed-point units
  jb.scale_base = e;
}

// ---------------------------------------------------------------- norms
// Row norms of the digits per candidate grid, over the whole chain, its two
// halves and its four quarters (the accumulator parts of a long-layout
// tile).  Lane group qq (8 lanes) takes quarter qq of the chain, an atom
// (all three coordinate rows) per lane-step; the 36 (row, grid, digit)
// sums are reduced within each group, then combined across the groups into
// half and full sums.  Unsigned sums wrap identically in any order.
__global__ void __launch_bounds__(kWarpsPerBlock * 32, 6) k_mx_norms(PrepArgs p, int64_t nstructs, int run_len) {
  const int lane = threadIdx.x & 31;
  const int qq = lane >> 3, u = lane & 7;
  const Run run = warp_run(p.s_lo, nstructs, run_len);
  int cur = -1;
  // the current job's maxima over the run so far, lane 3a + d holding those
  // of grid a, digit d (every lane sees every sum after the reductions)
  unsigned rf = 0, rh = 0, rq = 0;
  auto flush = [&]() {
    if (cur < 0 || lane >= 12) return;
    Job &jc = p.jobs[cur];
    const int a = lane / 3, d = lane - 3 * (lane / 3);
    if (a >= (jc.fixed_scale ? 1 : 4)) return;
    atomicMax(&jc.norm[a][d], (unsigned long long)rf);
    atomicMax(&jc.normh[a][d], (unsigned long long)rh);
    atomicMax(&jc.normq[a][d], (unsigned long long)rq);
  };
  for (int64_t g = run.g0; g < run.g1; ++g) {
    const Where w = locate(p, g);
    if (!w.valid) continue;
    Job &jb = p.jobs[w.job];
    if (jb.err) continue;
    if (w.job != cur) {
      flush();
      cur = w.job;
      rf = rh = rq = 0;
    }
    const int L = jb.L;
    const int nk16 = jb.lp / 16;
    const double *x = jb.xyz + w.local * 3 * (int64_t)L;
    const int ncand = jb.fixed_scale ? 1 : 4;
    const int t0 = jb.scale_base + kFixBits;
    const long long C[3] = {p.ctr[3 * g], p.ctr[3 * g + 1], p.ctr[3 * g + 2]};
    // quarter qq holds the 16-atom steps k16 with acc_part(k16, nk16, 4) ==
    // qq, i.e. 4 k16 in [qq nk16, (qq + 1) nk16)
    const int k_lo = 16 * ((qq * nk16 + 3) / 4), k_hi = min(L, 16 * (((qq + 1) * nk16 + 3) / 4));
    unsigned acc[3][4][3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int d = 0; d < 3; ++d) acc[r][a][d] = 0;
    for (int k = k_lo + u; k < k_hi; k += 8) {
      const double xr[3] = {x[3 * k], x[3 * k + 1], x[3 * k + 2]};
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        long long v;
        to_fix(xr[r], v);
        const long long y = v - C[r];
        // round-half-up of y / 2^(t0 + a) is ((w >> a) + 1) >> 1 with
        // w = floor(y / 2^(t0 - 1)); |w| <= 2^23 (the grid bounds every
        // centred coordinate by 2^22 2^t0), so the candidates are 32-bit
        const int wv = (int)(y >> (t0 - 1));
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          if (a < ncand) {
            const int q = ((wv >> a) + 1) >> 1;
            int e0, e1, e2;
            bsm::split_digits(q, e0, e1, e2);
            acc[r][a][0] += (unsigned)(e0 * e0);
            acc[r][a][1] += (unsigned)(e1 * e1);
            acc[r][a][2] += (unsigned)(e2 * e2);
          }
        }
      }
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      if (a >= ncand) break;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        unsigned f = 0, h = 0, q4 = 0;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          unsigned v = acc[r][a][d];
          v += __shfl_xor_sync(0xffffffffu, v, 4);
          v += __shfl_xor_sync(0xffffffffu, v, 2);
          v += __shfl_xor_sync(0xffffffffu, v, 1);  // quarter qq's sum
          const unsigned vq = max(v, __shfl_xor_sync(0xffffffffu, v, 8));
          const unsigned hs = v + __shfl_xor_sync(0xffffffffu, v, 8);  // half sum (quarters 0+1 or 2+3)
          const unsigned hx = __shfl_xor_sync(0xffffffffu, hs, 16);
          const unsigned fs = hs + hx;  // the whole chain
          q4 = max(q4, max(vq, __shfl_xor_sync(0xffffffffu, vq, 16)));
          h = max(h, max(hs, hx));
          f = max(f, fs);
        }
        if (lane == 3 * a + d) {
          rf = max(rf, f);
          rh = max(rh, h);
          rq = max(rq, q4);
        }
      }
    }
  }
  flush();
}

// ---------------------------------------------------------------- choose
__global__ void k_mx_choose(PrepArgs p) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= p.njobs) return;
  Job &jb = p.jobs[j];
  if (!job_in_range(p, jb)) return;
  if (jb.err) return;
  // Preference, from Cauchy-Schwarz bounds on the row norms: (1) the finest
  // grid whose level sums 0-2 are all exact (below 2^24) while its
  // quantisation (about 2^e per pair) leaves a quarter of the budget to the
  // arithmetic; (2) the same with the half layout (every level in halves of
  // the chain); (3) the same with the long layout (level 1 in halves, level
  // 2 in quarters; longer chains); (4) the finest grid with levels 0-1 exact
  // and level 2 below 2^26, its rounding charged to the budget.
  const int ncand = jb.fixed_scale ? 1 : 4;
  const bool can_long = jb.mode == 0 && jb.allow_long && jb.lp / 16 >= 4;
  int pick = -1, relaxed = -1, pick_long = -1, pick_half = -1;
  double bb2[4], bb34[4];
  for (int a = 0; a < ncand; ++a) {
    double f[3], hh[3], qq[3], nb[3];
    for (int d = 0; d < 3; ++d) {
      f[d] = sqrt((double)jb.norm[a][d]);
      hh[d] = sqrt((double)jb.normh[a][d]);
      qq[d] = sqrt((double)jb.normq[a][d]);
      nb[d] = jb.mode == 1 ? (double)jb.norm_b[d] : f[d];
    }
    const double b0 = f[0] * nb[0], b1 = f[0] * nb[1] + f[1] * nb[0];
    const double b2 = f[0] * nb[2] + f[1] * nb[1] + f[2] * nb[0];
    bb2[a] = b2;
    bb34[a] = f[1] * nb[2] + f[2] * nb[1] + f[2] * nb[2] / 512.0;
    const bool grid_ok = jb.fixed_scale || ldexp(1.0, jb.scale_base + a) <= 0.75 * (double)jb.tol;
    if (grid_ok && b0 < 16777216.0 && b1 < 16777216.0 && b2 < 16777216.0) {
      pick = a;
      break;
    }
    if (grid_ok && can_long && pick_half < 0 && hh[0] * hh[0] < 16777216.0 && 2.0 * hh[0] * hh[1] < 16777216.0 &&
        2.0 * hh[0] * hh[2] + hh[1] * hh[1] < 16777216.0)
      pick_half = a;
    if (grid_ok && can_long && pick_long < 0 && b0 < 16777216.0 && 2.0 * hh[0] * hh[1] < 16777216.0 &&
        2.0 * qq[0] * qq[2] + qq[1] * qq[1] < 16777216.0)
      pick_long = a;
    if (b0 < 16777216.0 && b1 < 16777216.0 && b2 < 67108864.0 && relaxed < 0) relaxed = a;
  }
  jb.layout = kAccNormal;
  if (pick < 0 && pick_half >= 0) {
    pick = pick_half;
    bb2[pick] = 0.0;  // both halves of level 2 are exact
    jb.layout = kAccHalf;
  } else if (pick < 0 && pick_long >= 0) {
    pick = pick_long;
    bb2[pick] = 0.0;  // every part of level 2 is exact
    jb.layout = kAccLong;
  }
  if (pick < 0) pick = relaxed;
  if (pick < 0) {
    atomicOr(&jb.err, kErrUnsupported);
    return;
  }
  // half-ulp rounding per accumulation step, 3 L steps per entry
  double err2 = 0.0, err3 = 0.0;
  if (bb2[pick] >= 16777216.0) err2 = 3.0 * (double)jb.L * ldexp(1.0, (int)floor(log2(bb2[pick])) - 24);
  if (bb34[pick] >= 8388608.0) err3 = 3.0 * (double)jb.L * ldexp(1.0, (int)floor(log2(bb34[pick])) - 24);
  // Mhat = 2^28 S0 + 2^19 S1 + 2^10 S2 + 2 S3'; the Rayleigh quotient moves
  // by at most sqrt(3) ||dMhat||_F per unit |q|^2, and E by twice that
  jb.d34 = (float)(6.0 * sqrt(3.0) * (1024.0 * err2 + 2.0 * err3) * (1.0 + 1e-6));
  jb.scale_exp = jb.scale_base + pick;
  jb.u = ldexpf(1.0f, 2 * jb.scale_exp);
  if (jb.screen) {
    // The screen accumulates digits 0 and 1 only (levels 0 and 1, and e1 e1):
    // levels 0-1 are exact here; e1 e1 is exact below 2^24, otherwise its
    // half-ulp roundings (L steps per entry) are charged as an error of E.
    const double b11 = sqrt((double)jb.norm[pick][1]) * (jb.mode == 1 ? (double)jb.norm_b[1] : sqrt((double)jb.norm[pick][1]));
    double e11 = 0.0;
    if (b11 >= 16777216.0) e11 = (double)jb.L * ldexp(1.0, (int)floor(log2(b11)) - 24);
    jb.d34 = (float)(6.0 * sqrt(3.0) * 1024.0 * e11 * (1.0 + 1e-6));
    jb.layout = kAccScreen;
  }
}

// ---------------------------------------------------------------- digits
// Warp per structure, in chunks of 256 atoms.  Pass 1 reads a chunk's AoS
// coordinates coalesced and keeps the quantised values in shared memory
// (three rows of 256 ints: 3 KB per warp whatever the chain length); pass 2
// writes the chunk's digit rows 16 bytes at a time.
__device__ __forceinline__ uint32_t bf16x2(int lo, int hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn((float)lo, (float)hi);
  return *reinterpret_cast<const uint32_t *>(&v);
}
__device__ __forceinline__ uint32_t bf16x2s(int lo, int hi) {  // (d2/32) of both, from e2 = 16 d2
  const __nv_bfloat162 v = __floats2bfloat162_rn((float)lo * (1.0f / 512.0f), (float)hi * (1.0f / 512.0f));
  return *reinterpret_cast<const uint32_t *>(&v);
}

constexpr int kDigitWarps = 8;
constexpr int kChunkAtoms = 256;  // atoms staged per warp at a time: 768 coordinates, a multiple of 32

__global__ void __launch_bounds__(kDigitWarps * 32) k_mx_digits(PrepArgs p, int64_t nstructs) {
  __shared__ int qsm[kDigitWarps][3 * kChunkAtoms];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int64_t g = p.s_lo + (int64_t)blockIdx.x * kDigitWarps + wib;
  if (g >= nstructs) return;
  const Where w = locate(p, g);
  if (!w.valid) return;
  Job &jb = p.jobs[w.job];
  if (jb.err) return;
  const int L = jb.L, lp = jb.lp;
  int *q = qsm[wib];
  const double *x = jb.xyz + w.local * 3 * (int64_t)L;
  const long long C[3] = {p.ctr[3 * g], p.ctr[3 * g + 1], p.ctr[3 * g + 2]};
  const int t = jb.scale_exp + kFixBits;
  long long gsum = 0;
  float rsum = 0.f;  // |r| < 2^31 units; relative rounding charged below
  long long gt = 0;
  int d2s = 0;
  // The structure in chunks of kChunkAtoms atoms (the last one up to lp).  A
  // chunk's coordinates start at a multiple of 768, so each lane visits its
  // coordinates lane + 32 j in the same order as over the whole structure.
  for (int a0 = 0; a0 < lp; a0 += kChunkAtoms) {
    const int na = min(kChunkAtoms, lp - a0);         // atoms of the chunk, a multiple of 16
    const int nreal = max(0, min(na, L - a0));        // of which real atoms
    const double *xc = x + 3 * (int64_t)a0;
    // pass 1: coalesced reads, four loads in flight per lane; quantised
    // values staged by coordinate row
    int c = lane % 3;
    for (int i0 = lane; i0 < 3 * nreal; i0 += 128) {
      double xv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) xv[u] = i0 + 32 * u < 3 * nreal ? xc[i0 + 32 * u] : 0.0;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int i = i0 + 32 * u;
        if (i < 3 * nreal) {
          long long v;
          to_fix(xv[u], v);
          const long long y = v - (c == 0 ? C[0] : (c == 1 ? C[1] : C[2]));
          const int n = (int)((y + (1ll << (t - 1))) >> t);
          const long long r = y - ((long long)n << t);
          gsum += (long long)n * n;
          const float rf = (float)(int)r;
          rsum = fmaf(rf, rf, rsum);
          q[c * kChunkAtoms + i / 3] = n;
        }
        c = (c + 2) % 3;
      }
    }
    for (int i = nreal + lane; i < na; i += 32) {  // padding atoms
      q[i] = 0;
      q[kChunkAtoms + i] = 0;
      q[2 * kChunkAtoms + i] = 0;
    }
    __syncwarp();
    // pass 2: 8 atoms of one row per lane-step; also the truncated structure
    // t = n - d2 that levels 0 and 1 describe (sum of t^2, sum of d2^2)
    const int chunks = na / 8;
    for (int u = lane; u < 3 * chunks; u += 32) {
      const int r = u / chunks, k0 = (u - r * chunks) * 8;
      int e0[8], e1[8], e2[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int nv = q[r * kChunkAtoms + k0 + k];
        bsm::split_digits(nv, e0[k], e1[k], e2[k]);
        const int d2 = e2[k] >> 4, tv = nv - d2;
        gt += (long long)tv * tv;
        d2s += d2 * d2;
      }
      const int64_t off = digit_row(g, r) * p.pitch + a0 + k0;
      uint4 v0, v1, v2, v3;
      v0.x = bf16x2(e0[0], e0[1]); v0.y = bf16x2(e0[2], e0[3]); v0.z = bf16x2(e0[4], e0[5]); v0.w = bf16x2(e0[6], e0[7]);
      v1.x = bf16x2(e1[0], e1[1]); v1.y = bf16x2(e1[2], e1[3]); v1.z = bf16x2(e1[4], e1[5]); v1.w = bf16x2(e1[6], e1[7]);
      v2.x = bf16x2(e2[0], e2[1]); v2.y = bf16x2(e2[2], e2[3]); v2.z = bf16x2(e2[4], e2[5]); v2.w = bf16x2(e2[6], e2[7]);
      v3.x = bf16x2s(e2[0], e2[1]); v3.y = bf16x2s(e2[2], e2[3]); v3.z = bf16x2s(e2[4], e2[5]); v3.w = bf16x2s(e2[6], e2[7]);
      *reinterpret_cast<uint4 *>(p.dig[0] + off) = v0;
      *reinterpret_cast<uint4 *>(p.dig[1] + off) = v1;
      *reinterpret_cast<uint4 *>(p.dig[2] + off) = v2;
      *reinterpret_cast<uint4 *>(p.dig[3] + off) = v3;
    }
    __syncwarp();  // the next chunk overwrites the staged rows
  }
  gsum = warp_sum64(gsum);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) rsum += __shfl_xor_sync(0xffffffffu, rsum, o);
  if (lane == 0) {
    SInfo in;
    in.ghat = gsum;
    in.gf = (float)gsum;
    // RMS residual in Angstrom, rounded up: a sum of 3L non-negative FP32
    // terms (each rounded at most twice) is within (3L + 64) 2^-23 of the
    // exact sum; plus 2^-30 A for the fixed-point reading and the centroid
    // rounding (each below 2^-32 A per coordinate)
    const double up = 1.0 + (3.0 * L + 64.0) * 1.1920928955078125e-7;
    const double rms = sqrt((double)rsum * up / (double)L) * 2.3283064365386963e-10;  // 2^-32
    in.qres = (float)(rms * (1.0 + 1e-6) + 9.313225746154785e-10);
    p.info[g] = in;
    atomicMax(&jb.qres_max_bits, __float_as_uint(in.qres));
  }
  if (p.tinfo) {
    gt = warp_sum64(gt);
    d2s = (int)warp_sum32((unsigned)d2s);
    if (lane == 0) {
      // RMS of the omitted digit in Angstrom (2^scale_exp per unit), rounded up
      const double rt = sqrt((double)d2s / (double)L) * ldexp(1.0, jb.scale_exp);
      p.tinfo[g] = make_float2((float)gt, (float)(rt * (1.0 + 1e-6)));
    }
  }
}

// ------------------------------------------------------------ plain path
constexpr int kPlainThreads = 128;

template <int N>
__device__ __forceinline__ void block_sum_d(double (&v)[N], double *scratch /* [4][N] */) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
  if (lane == 0)
#pragma unroll
    for (int i = 0; i < N; ++i) scratch[warp * N + i] = v[i];
  __syncthreads();
#pragma unroll
  for (int i = 0; i < N; ++i) {
    double s = 0;
    for (int w = 0; w < kPlainThreads / 32; ++w) s += scratch[w * N + i];
    v[i] = s;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kPlainThreads) k_plain_center(const double *__restrict__ xyz, int L, double *ctr,
                                                                int *err) {
  __shared__ double red[4 * 3];
  const int64_t s = blockIdx.x;
  const double *x = xyz + s * 3 * (int64_t)L;
  double acc[3] = {0.0, 0.0, 0.0};
  int bad = 0;
  for (int i = threadIdx.x; i < 3 * L; i += kPlainThreads) {
    const double v = x[i];
    bad |= !isfinite(v);
    const int c = i % 3;
    acc[0] += (c == 0) ? v : 0.0;
    acc[1] += (c == 1) ? v : 0.0;
    acc[2] += (c == 2) ? v : 0.0;
  }
  block_sum_d<3>(acc, red);
  bad = __syncthreads_or(bad);
  if (threadIdx.x == 0) {
    const double inv = 1.0 / (double)L;
    ctr[3 * s + 0] = acc[0] * inv;
    ctr[3 * s + 1] = acc[1] * inv;
    ctr[3 * s + 2] = acc[2] * inv;
    if (bad) atomicOr(err, kErrNonFinite);
  }
}

__global__ void __launch_bounds__(kPlainThreads)
    k_prep_plain(const double *__restrict__ xyz, const double *__restrict__ ctr, int L, int lp,
                 double *__restrict__ y, double *__restrict__ g) {
  __shared__ double red[4];
  const int64_t s = blockIdx.x;
  const double *x = xyz + s * 3 * (int64_t)L;
  const double cc[3] = {ctr[3 * s], ctr[3 * s + 1], ctr[3 * s + 2]};
  double *ys = y + s * 3 * (int64_t)lp;
  double acc[1] = {0.0};
  for (int k = threadIdx.x; k < lp; k += kPlainThreads) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double v = (k < L) ? x[3 * k + c] - cc[c] : 0.0;
      ys[(int64_t)c * lp + k] = v;
      acc[0] += v * v;
    }
  }
  block_sum_d<1>(acc, red);
  if (threadIdx.x == 0) g[s] = acc[0];
}

}  // namespace

cudaError_t launch_prep_mixed(const PrepArgs &p, cudaStream_t st) {
  const int64_t total = p.nblocks * kBlockStructs;
  const int64_t hi = p.s_hi < 0 ? total : (p.s_hi < total ? p.s_hi : total);  // structures [s_lo, hi)
  const int64_t count = hi - p.s_lo;
  if (count <= 0) return cudaSuccess;
  int dev = 0, nsm = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int64_t per = count / ((int64_t)nsm * 32);
  const int run = per < 1 ? 1 : (per > 8 ? 8 : (int)per);
  const unsigned gw = (unsigned)((count + (int64_t)run * kWarpsPerBlock - 1) / ((int64_t)run * kWarpsPerBlock));
  k_mx_center<<<gw, kWarpsPerBlock * 32, 0, st>>>(p, hi, run);
  k_mx_scale<<<(p.njobs + 127) / 128, 128, 0, st>>>(p);
  k_mx_norms<<<gw, kWarpsPerBlock * 32, 0, st>>>(p, hi, run);
  k_mx_choose<<<(p.njobs + 127) / 128, 128, 0, st>>>(p);
  k_mx_digits<<<(unsigned)((count + kDigitWarps - 1) / kDigitWarps), kDigitWarps * 32, 0, st>>>(p, hi);
  return cudaGetLastError();
}

// Largest digit-row pitch (atoms) the preparation pass supports.
// The mixed path's longest chain (digit row pitch, atoms).
int prep_max_pitch() { return 16384; }

// Kernel attributes, set once per device before any launch or capture (the
// preparation kernels need none).
cudaError_t prep_prepare() { return cudaSuccess; }

cudaError_t launch_prep_plain(const double *xyz, int64_t n, int L, int lp, double *ctr, double *y, double *g,
                              int *err, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_plain_center<<<(unsigned)n, kPlainThreads, 0, st>>>(xyz, L, ctr, err);
  k_prep_plain<<<(unsigned)n, kPlainThreads, 0, st>>>(xyz, ctr, L, lp, y, g);
  return cudaGetLastError();
}

}  // namespace bs
