// refine.cu -- exact recomputation of flagged pairs, and the CUDA-core
// mixed path for explicit pair lists.
//
// Exact path: the quantised coordinates n = 2^14 e0 + 2^5 e1 + e2 / 16 are
// rebuilt from the digit matrices, the covariance Mhat = sum n_a n_b is
// accumulated in int64 (exact), and the FP64 QCP of crmsd_math.cuh finishes
// the pair.  One warp per pair, lanes striding over atoms.
#include "crmsd_math.cuh"
#include "kernels.h"

namespace bs {
namespace {

__device__ __forceinline__ int64_t tri_index(int64_t n, int64_t i, int64_t j) {
  return i * n - i * (i + 1) / 2 + (j - i - 1);
}

__device__ __forceinline__ void tri_pair(int64_t n, int64_t t, int64_t &i, int64_t &j) {
  // inverse of tri_index: row i holds n-1-i pairs
  const double b = 2.0 * (double)n - 1.0;
  int64_t r = (int64_t)floor((b - sqrt(b * b - 8.0 * (double)t)) * 0.5);
  if (r < 0) r = 0;
  while (r > 0 && r * n - r * (r + 1) / 2 > t) --r;
  while ((r + 1) * n - (r + 1) * (r + 2) / 2 <= t) ++r;
  i = r;
  j = t - (r * n - r * (r + 1) / 2) + r + 1;
}

__device__ __forceinline__ void store_pair(const OutDesc &o, int64_t i, int64_t j, double v) {
  if (o.layout == kLayoutNeighbors) {  // the pair's crmsd as the tensor-core path keeps it: f32
    const float f = (float)v;
    if (!(f <= o.eps)) return;
    const NbrSink *sk = static_cast<const NbrSink *>(o.ptr);
    const unsigned long long s = atomicAdd(sk->count, 2ull);
    if (s + 1 < sk->cap) {
      sk->ij[s] = make_int2((int)i, (int)j);
      sk->d[s] = f;
      sk->ij[s + 1] = make_int2((int)j, (int)i);
      sk->d[s + 1] = f;
    }
    return;
  }
  int64_t idx, idx2 = -1;
  if (o.layout == kLayoutTriangle) {
    idx = tri_index(o.n, i, j);
  } else if (o.layout == kLayoutRect) {
    idx = i * o.ld + j;
  } else {
    idx = i * o.ld + j;
    idx2 = j * o.ld + i;
  }
  if (o.out_type == 0) {
    static_cast<double *>(o.ptr)[idx] = v;
    if (idx2 >= 0) static_cast<double *>(o.ptr)[idx2] = v;
  } else {
    static_cast<float *>(o.ptr)[idx] = (float)v;
    if (idx2 >= 0) static_cast<float *>(o.ptr)[idx2] = (float)v;
  }
}

__device__ __forceinline__ int coord(const DigitsView &dg, int64_t s, int c, int k) {
  const int64_t off = digit_row(s, c) * dg.pitch + k;
  return bsm::join_digits((int)__bfloat162float(dg.d0[off]), (int)__bfloat162float(dg.d1[off]),
                          (int)__bfloat162float(dg.d2[off]));
}

// The FP64 finish of the exact path as one compiled function shared by
// every kernel here: inlined copies may contract multiply-adds differently,
// and a pair's exact value must not depend on which kernel recomputed it.
__device__ __noinline__ double exact_finish(const long long mh[9], long long ga, long long gb, int scale_exp, int L) {
  return bsm::pair_rmsd_exact(mh, ga, gb, scale_exp, L);
}

// Exact int64 covariance of pair (i on side A, j on side B), partial over
// atoms k = k0, k0+ks, ...
__device__ __forceinline__ void exact_cov_partial(const DigitsView &da, const DigitsView &db, int64_t i, int64_t j,
                                                  int L, int k0, int ks, long long mh[9]) {
#pragma unroll
  for (int e = 0; e < 9; ++e) mh[e] = 0;
  for (int k = k0; k < L; k += ks) {
    const int a0 = coord(da, i, 0, k), a1 = coord(da, i, 1, k), a2 = coord(da, i, 2, k);
    const int b0 = coord(db, j, 0, k), b1 = coord(db, j, 1, k), b2 = coord(db, j, 2, k);
    mh[0] += (long long)a0 * b0;
    mh[1] += (long long)a0 * b1;
    mh[2] += (long long)a0 * b2;
    mh[3] += (long long)a1 * b0;
    mh[4] += (long long)a1 * b1;
    mh[5] += (long long)a1 * b2;
    mh[6] += (long long)a2 * b0;
    mh[7] += (long long)a2 * b1;
    mh[8] += (long long)a2 * b2;
  }
}

__device__ __forceinline__ double exact_pair_warp(const RefineArgs &r, const Job &jb, int64_t ig, int64_t jg,
                                                  int lane) {
  long long mh[9];
  exact_cov_partial(r.da, r.db, ig, jg, jb.L, lane, 32, mh);
#pragma unroll
  for (int e = 0; e < 9; ++e)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mh[e] += __shfl_xor_sync(0xffffffffu, mh[e], o);
  return exact_finish(mh, r.info_a[ig].ghat, r.info_b[jg].ghat, jb.scale_exp, jb.L);
}

__global__ void k_refine_list(RefineArgs r) {
  const unsigned long long cnt = r.sc->flag_count < r.cap ? r.sc->flag_count : r.cap;
  const int64_t done = (int64_t)r.sc->flag_done;
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t w = done + (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < (int64_t)cnt;
       w += warps) {
    const unsigned long long f = r.flags[w];
    const int job = (int)(f >> 48);
    const int64_t ig = (int64_t)((f >> 24) & 0xffffffull), jg = (int64_t)(f & 0xffffffull);
    const Job &jb = r.jobs[job];
    const double v = exact_pair_warp(r, jb, ig, jg, lane);
    if (lane == 0) store_pair(jb.out, ig - jb.first_a, jg - jb.first_b, v);
  }
}

// After a band's recomputation: its queue entries are done.
__global__ void k_refine_mark(DevScalars *sc, unsigned long long cap) {
  sc->flag_done = sc->flag_count < cap ? sc->flag_count : cap;
}

// Fallback when the queue overflowed: every negative (sentinel) entry of the
// jobs' outputs is recomputed.  Returns at once when nothing overflowed.
__global__ void k_refine_scan(RefineArgs r) {
  if (r.sc->flag_count <= r.cap) return;
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t w0 = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  for (int job = 0; job < r.njobs; ++job) {
    const Job &jb = r.jobs[job];
    if (jb.err || jb.out.layout == kLayoutNeighbors) continue;  // no sentinels to find: the host reports it
    const OutDesc &out = jb.out;
    const bool sym = jb.mode == 0;
    const int64_t n = jb.n, nb = jb.n_b;
    int64_t total = sym ? n * (n - 1) / 2 : n * nb, first = 0;
    if (r.scan_hi >= 0) {
      if (job > 0) break;
      first = r.scan_lo;
      total = r.scan_hi < total ? r.scan_hi : total;
    }
    for (int64_t base = first + w0 * 32; base < total; base += warps * 32) {
      const int64_t t = base + lane;
      int64_t i = 0, j = 0;
      bool sent = false;
      if (t < total) {
        int64_t idx;
        if (sym) {
          tri_pair(n, t, i, j);
          idx = out.layout == kLayoutTriangle ? t : i * out.ld + j;
        } else {
          i = t / nb;
          j = t - i * nb;
          idx = i * out.ld + j;
        }
        const double v = out.out_type == 0 ? static_cast<const double *>(out.ptr)[idx]
                                           : (double)static_cast<const float *>(out.ptr)[idx];
        sent = v < 0.0;
      }
      unsigned m = __ballot_sync(0xffffffffu, sent);
      while (m) {
        const int src = __ffs(m) - 1;
        m &= m - 1;
        const int64_t si = __shfl_sync(0xffffffffu, i, src);
        const int64_t sj = __shfl_sync(0xffffffffu, j, src);
        const double v = exact_pair_warp(r, jb, si + jb.first_a, sj + jb.first_b, lane);
        if (lane == 0) store_pair(out, si, sj, v);
      }
    }
  }
}

// One pair (A structure ig, B structure jg) with exact level sums on CUDA
// cores, the fast epilogue, and the exact path when the pair is flagged.
// Level 3 carries S3 + S4/512 as the tensor cores accumulate it (here
// rounded once from the exact value).  levels_out (optional) receives the
// 36 level sums.
__device__ double certified_pair(const DigitsView &da, const DigitsView &db, int64_t ig, int64_t jg, const SInfo &ia,
                                 const SInfo &ib, const Job &jb, float *levels_out) {
  const int L = jb.L;
  int S[5][9];
#pragma unroll
  for (int l = 0; l < 5; ++l)
#pragma unroll
    for (int e = 0; e < 9; ++e) S[l][e] = 0;
  for (int k = 0; k < L; ++k) {
    int a[3][3], b[3][3];  // [coord][digit]
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int64_t oa = digit_row(ig, c) * da.pitch + k, ob = digit_row(jg, c) * db.pitch + k;
      a[c][0] = (int)__bfloat162float(da.d0[oa]);
      a[c][1] = (int)__bfloat162float(da.d1[oa]);
      a[c][2] = (int)__bfloat162float(da.d2[oa]);
      b[c][0] = (int)__bfloat162float(db.d0[ob]);
      b[c][1] = (int)__bfloat162float(db.d1[ob]);
      b[c][2] = (int)__bfloat162float(db.d2[ob]);
    }
#pragma unroll
    for (int x = 0; x < 3; ++x)
#pragma unroll
      for (int y = 0; y < 3; ++y) {
        const int e = 3 * x + y;
        S[0][e] += a[x][0] * b[y][0];
        S[1][e] += a[x][0] * b[y][1] + a[x][1] * b[y][0];
        S[2][e] += a[x][0] * b[y][2] + a[x][1] * b[y][1] + a[x][2] * b[y][0];
        S[3][e] += a[x][1] * b[y][2] + a[x][2] * b[y][1];
        S[4][e] += (a[x][2] >> 4) * (b[y][2] >> 4);  // sum d2a d2b; S4/512 = (sum d2a d2b) / 2
      }
  }
  bsm::EpilogueIn in;
#pragma unroll
  for (int e = 0; e < 9; ++e) {
    in.s0[e] = (float)S[0][e];
    in.s1[e] = (float)S[1][e];
    in.s2[e] = (float)S[2][e];
    in.s3[e] = (float)((double)S[3][e] + 0.5 * (double)S[4][e]);
  }
  in.ga = ia.ghat;
  in.gb = ib.ghat;
  in.gfa = ia.gf;
  in.gfb = ib.gf;
  in.qa = ia.qres;
  in.qb = ib.qres;
  if (levels_out) {
#pragma unroll
    for (int e = 0; e < 9; ++e) {
      levels_out[e] = in.s0[e];
      levels_out[9 + e] = in.s1[e];
      levels_out[18 + e] = in.s2[e];
      levels_out[27 + e] = in.s3[e];
    }
  }
  int flag = 0;
  const float r = bsm::pair_rmsd_fast(in, jb.u, jb.d34, L, jb.tol, flag);
  if (!flag) return (double)r;
  long long mh[9];
  exact_cov_partial(da, db, ig, jg, L, 0, 1, mh);
  return exact_finish(mh, in.ga, in.gb, jb.scale_exp, L);
}

// Thread per pair of job 0 (explicit pair lists, and the tensor-core path's
// independent check).
__global__ void k_mixed_pairs(DigitsView dg, const SInfo *__restrict__ info, const Job *job, DevScalars *sc,
                              const int64_t *__restrict__ ii, const int64_t *__restrict__ jj, int64_t np,
                              double *__restrict__ out, float *__restrict__ levels_out) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= np) return;
  const Job &jb = *job;
  if (jb.err) return;
  const int64_t i = ii[t] + jb.first_a, j = jj[t] + jb.first_a;
  if (i == j) {
    out[t] = 0.0;
    if (levels_out)
      for (int e = 0; e < 36; ++e) levels_out[t * 36 + e] = 0.f;
    return;
  }
  out[t] = certified_pair(dg, dg, i, j, info[i], info[j], jb, levels_out ? levels_out + t * 36 : nullptr);
}

// Block per query row; the row's candidates are split evenly over the eight
// warps, and a warp takes its share 32 at a time: for each candidate, all
// lanes accumulate the integer level sums over strided atoms and reduce
// them, and the candidate's lane keeps the totals; then every lane finishes
// its own candidate (the certified epilogue once per pair, not once per
// lane).  Integer sums do not depend on the order of accumulation, so every
// value is bit-identical to certified_pair's.
constexpr int kCandWarps = 8;
__global__ void __launch_bounds__(kCandWarps * 32)
    k_exact_candidates(DigitsView da, DigitsView db, const SInfo *__restrict__ info_a,
                       const SInfo *__restrict__ info_b, const Job *__restrict__ jobs,
                       const int *__restrict__ row_job, const int64_t *__restrict__ row_ig,
                       const int *__restrict__ cand_j, const int *__restrict__ cand_n, int cap,
                       float *__restrict__ cand_v) {
  const int64_t r = blockIdx.x;
  const Job &jb = jobs[row_job[r]];
  if (jb.err) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t ig = row_ig[r];
  const int n = min(cand_n[r], cap);
  const int L = jb.L;
  const int64_t ra = digit_row(ig, 0) * da.pitch;
  const int share = (n + kCandWarps - 1) / kCandWarps;
  const int cb = min(n, warp * share), ce = min(n, cb + share);
  for (int c0 = cb; c0 < ce; c0 += 32) {
    int mine[5][9];
#pragma unroll
    for (int l = 0; l < 5; ++l)
#pragma unroll
      for (int e = 0; e < 9; ++e) mine[l][e] = 0;
    const int cnt = min(32, ce - c0);
    for (int cc = 0; cc < cnt; ++cc) {
      const int64_t jg = (int64_t)cand_j[r * cap + c0 + cc] + jb.first_b;
      const int64_t rb = digit_row(jg, 0) * db.pitch;
      int S[5][9];
#pragma unroll
      for (int l = 0; l < 5; ++l)
#pragma unroll
        for (int e = 0; e < 9; ++e) S[l][e] = 0;
      for (int k = lane; k < L; k += 32) {
        int a[3][3], b[3][3];  // [coord][digit]
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const int64_t oa = ra + c * da.pitch + k, ob = rb + c * db.pitch + k;
          a[c][0] = (int)__bfloat162float(da.d0[oa]);
          a[c][1] = (int)__bfloat162float(da.d1[oa]);
          a[c][2] = (int)__bfloat162float(da.d2[oa]);
          b[c][0] = (int)__bfloat162float(db.d0[ob]);
          b[c][1] = (int)__bfloat162float(db.d1[ob]);
          b[c][2] = (int)__bfloat162float(db.d2[ob]);
        }
#pragma unroll
        for (int x = 0; x < 3; ++x)
#pragma unroll
          for (int y = 0; y < 3; ++y) {
            const int e = 3 * x + y;
            S[0][e] += a[x][0] * b[y][0];
            S[1][e] += a[x][0] * b[y][1] + a[x][1] * b[y][0];
            S[2][e] += a[x][0] * b[y][2] + a[x][1] * b[y][1] + a[x][2] * b[y][0];
            S[3][e] += a[x][1] * b[y][2] + a[x][2] * b[y][1];
            S[4][e] += (a[x][2] >> 4) * (b[y][2] >> 4);
          }
      }
#pragma unroll
      for (int l = 0; l < 5; ++l)
#pragma unroll
        for (int e = 0; e < 9; ++e) {
          const int t = __reduce_add_sync(0xffffffffu, S[l][e]);
          if (lane == cc) mine[l][e] = t;
        }
    }
    if (lane >= cnt) continue;
    const int64_t jg = (int64_t)cand_j[r * cap + c0 + lane] + jb.first_b;
    const SInfo ia = info_a[ig], ib = info_b[jg];
    bsm::EpilogueIn in;
#pragma unroll
    for (int e = 0; e < 9; ++e) {
      in.s0[e] = (float)mine[0][e];
      in.s1[e] = (float)mine[1][e];
      in.s2[e] = (float)mine[2][e];
      in.s3[e] = (float)((double)mine[3][e] + 0.5 * (double)mine[4][e]);
    }
    in.ga = ia.ghat;
    in.gb = ib.ghat;
    in.gfa = ia.gf;
    in.gfb = ib.gf;
    in.qa = ia.qres;
    in.qb = ib.qres;
    int flag = 0;
    float v = bsm::pair_rmsd_fast(in, jb.u, jb.d34, L, jb.tol, flag);
    if (flag) {  // rare: the exact path, on this lane alone
      long long mh[9];
      exact_cov_partial(da, db, ig, jg, L, 0, 1, mh);
      v = (float)exact_finish(mh, in.ga, in.gb, jb.scale_exp, L);
    }
    cand_v[r * cap + c0 + lane] = v;
  }
}

}  // namespace

cudaError_t launch_refine(const RefineArgs &r, cudaStream_t st) {
  k_refine_list<<<r.num_sms * 4, 256, 0, st>>>(r);
  if (r.mark) k_refine_mark<<<1, 1, 0, st>>>(r.sc, r.cap);
  k_refine_scan<<<r.num_sms * 4, 256, 0, st>>>(r);
  return cudaGetLastError();
}

cudaError_t launch_exact_candidates(const DigitsView &da, const DigitsView &db, const SInfo *info_a,
                                    const SInfo *info_b, const Job *jobs, const int *row_job, const int64_t *row_ig,
                                    int64_t rows, const int *cand_j, const int *cand_n, int cap, float *cand_v,
                                    cudaStream_t st) {
  if (rows <= 0) return cudaSuccess;
  k_exact_candidates<<<(unsigned)rows, kCandWarps * 32, 0, st>>>(da, db, info_a, info_b, jobs, row_job, row_ig, cand_j, cand_n,
                                                   cap, cand_v);
  return cudaGetLastError();
}

cudaError_t launch_mixed_pairs(const DigitsView &dg, const SInfo *info, const Job *job, DevScalars *sc,
                               const int64_t *ii, const int64_t *jj, int64_t np, double *out, float *levels_out,
                               cudaStream_t st) {
  if (np <= 0) return cudaSuccess;
  const int th = 128;
  k_mixed_pairs<<<(unsigned)((np + th - 1) / th), th, 0, st>>>(dg, info, job, sc, ii, jj, np, out, levels_out);
  return cudaGetLastError();
}

}  // namespace bs
