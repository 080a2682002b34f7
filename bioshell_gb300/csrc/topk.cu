// topk.cu -- the k nearest library structures of each query structure: the
// k smallest values of each row of a dense [rows][n] f32 crmsd block, in
// ascending (value, library index) order -- a total order, so the result
// does not depend on how the row is scanned or in which order candidates
// were appended.  The library index of column c is perm[c] when the library
// is stored in another order (perm), else c; candidate lists map their
// positions to columns first (col_map).
//
// One block of eight warps per row.  Each warp scans a strided share of the
// row and keeps its best k in a sorted list spread over its lanes (two
// entries per lane, entry e at lane e / 2, slot e % 2); a value enters only
// if it beats the warp's current k-th entry, so after the first few hundred
// values a 32-value chunk costs one compare and one ballot.  Warp 0 then
// folds the other warps' lists into its own.
#include <stdint.h>

#include "kernels.h"

namespace bs {
namespace {

constexpr int kTopkWarps = 8;
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ bool less_vi(float a, int ai, float b, int bi) { return a < b || (a == b && ai < bi); }

// Inserts (x, xi) into the warp's sorted list (lv, li); the last entry drops.
__device__ __forceinline__ void list_insert(float (&lv)[2], int (&li)[2], float x, int xi, int lane) {
  const bool gt0 = less_vi(x, xi, lv[0], li[0]);
  const bool gt1 = less_vi(x, xi, lv[1], li[1]);
  const int p = __popc(__ballot_sync(kFull, !gt0)) + __popc(__ballot_sync(kFull, !gt1));
  const float up_v = __shfl_up_sync(kFull, lv[1], 1);
  const int up_i = __shfl_up_sync(kFull, li[1], 1);
  const int e0 = 2 * lane, e1 = 2 * lane + 1;
  const float n0v = e0 < p ? lv[0] : (e0 == p ? x : up_v);
  const int n0i = e0 < p ? li[0] : (e0 == p ? xi : up_i);
  const float n1v = e1 < p ? lv[1] : (e1 == p ? x : lv[0]);
  const int n1i = e1 < p ? li[1] : (e1 == p ? xi : li[0]);
  lv[0] = n0v;
  li[0] = n0i;
  lv[1] = n1v;
  li[1] = n1i;
}

__device__ __forceinline__ void kth(const float (&lv)[2], const int (&li)[2], int k, float &tv, int &ti) {
  const int e = k - 1;
  tv = __shfl_sync(kFull, (e & 1) ? lv[1] : lv[0], e >> 1);
  ti = __shfl_sync(kFull, (e & 1) ? li[1] : li[0], e >> 1);
}

__device__ __forceinline__ void consider(float x, int xi, int lane, int k, float (&lv)[2], int (&li)[2], float &tv,
                                         int &ti, bool cand) {
  unsigned m = __ballot_sync(kFull, cand && less_vi(x, xi, tv, ti));
  while (m) {
    const int src = __ffs(m) - 1;
    m &= m - 1;
    const float xv = __shfl_sync(kFull, x, src);
    const int xii = __shfl_sync(kFull, xi, src);
    if (!less_vi(xv, xii, tv, ti)) continue;  // the threshold moved since the ballot
    list_insert(lv, li, xv, xii, lane);
    kth(lv, li, k, tv, ti);
  }
}

// The ordering key (library index) of position pos of row r.
struct KeyMap {
  const int *col_map;  // [rows][ld] candidate -> column, or null
  const int *perm;     // column -> library index, or null
  int64_t ld;
  __device__ __forceinline__ int key(int64_t r, int pos) const {
    const int c = col_map ? col_map[r * ld + pos] : pos;
    return perm ? perm[c] : c;
  }
};

// One warp's share of a row: 16-byte loads of four values per lane; a
// chunk of 128 values costs one compare and one ballot unless some lane
// holds a value below the warp's current k-th entry.
__device__ void warp_scan(const float *__restrict__ v, int64_t n, int warp, int lane, int k, float (&lv)[2],
                          int (&li)[2], float &tv, int &ti, const KeyMap &km, int64_t row) {
  const float inf = __int_as_float(0x7f800000);
  const int64_t mis = (int64_t)(((16 - ((uintptr_t)v & 15)) & 15) >> 2);  // values before 16-byte alignment
  const int64_t head = n < mis ? n : mis;
  if (warp == 0) {
    const bool ok = lane < head;
    consider(ok ? v[lane] : inf, ok ? km.key(row, lane) : 0x7fffffff, lane, k, lv, li, tv, ti, ok);
  }
  const float4 *v4 = reinterpret_cast<const float4 *>(v + head);
  const int64_t n4 = (n - head) >> 2;
  for (int64_t q = (int64_t)warp * 32; q < n4; q += kTopkWarps * 32) {
    const int64_t qi = q + lane;
    const float4 x = qi < n4 ? v4[qi] : make_float4(inf, inf, inf, inf);
    const float mn = fminf(fminf(x.x, x.y), fminf(x.z, x.w));
    if (!__any_sync(kFull, qi < n4 && mn <= tv)) continue;
    const int base = (int)(head + 4 * qi);
    const bool in = qi < n4;
    // keys only where a value can enter (the mapping reads global memory)
    const bool any = in && mn <= tv;
    consider(x.x, any ? km.key(row, base + 0) : 0x7fffffff, lane, k, lv, li, tv, ti, in);
    consider(x.y, any ? km.key(row, base + 1) : 0x7fffffff, lane, k, lv, li, tv, ti, in);
    consider(x.z, any ? km.key(row, base + 2) : 0x7fffffff, lane, k, lv, li, tv, ti, in);
    consider(x.w, any ? km.key(row, base + 3) : 0x7fffffff, lane, k, lv, li, tv, ti, in);
  }
  const int64_t tail0 = head + 4 * n4;
  if (warp == kTopkWarps - 1) {
    const int64_t j = tail0 + lane;
    const bool ok = j < n;
    consider(ok ? v[j] : inf, ok ? km.key(row, (int)j) : 0x7fffffff, lane, k, lv, li, tv, ti, ok);
  }
}

// Warp 0 folds the other warps' lists (in shared memory) into its own.
__device__ void merge_lists(float (*sv)[kTopkMax], int (*si)[kTopkMax], int lane, int k, float (&lv)[2], int (&li)[2],
                            float &tv, int &ti) {
  const float inf = __int_as_float(0x7f800000);
  for (int w = 1; w < kTopkWarps; ++w)
    for (int e0 = 0; e0 < k; e0 += 32) {
      const int e = e0 + lane;
      consider(e < k ? sv[w][e] : inf, e < k ? si[w][e] : 0x7fffffff, lane, k, lv, li, tv, ti, e < k);
    }
}

__global__ void __launch_bounds__(kTopkWarps * 32) k_topk(const float *__restrict__ vals, int64_t n_all, int64_t ld,
                                                          const int *__restrict__ row_n, KeyMap km, int k,
                                                          int64_t *__restrict__ out_idx,
                                                          float *__restrict__ out_val) {
  __shared__ float sv[kTopkWarps][kTopkMax];
  __shared__ int si[kTopkWarps][kTopkMax];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const float *v = vals + (int64_t)blockIdx.x * ld;
  const int64_t n = row_n ? (int64_t)min(row_n[blockIdx.x], (int)ld) : n_all;
  const float inf = __int_as_float(0x7f800000);
  float lv[2] = {inf, inf};
  int li[2] = {0x7fffffff, 0x7fffffff};
  float tv = inf;
  int ti = 0x7fffffff;
  warp_scan(v, n, warp, lane, k, lv, li, tv, ti, km, blockIdx.x);
  sv[warp][2 * lane] = lv[0];
  sv[warp][2 * lane + 1] = lv[1];
  si[warp][2 * lane] = li[0];
  si[warp][2 * lane + 1] = li[1];
  __syncthreads();
  if (warp != 0) return;
  merge_lists(sv, si, lane, k, lv, li, tv, ti);
  int64_t *oi = out_idx + (int64_t)blockIdx.x * k;
  float *ov = out_val + (int64_t)blockIdx.x * k;
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const int e = 2 * lane + s;
    if (e < k) {
      const bool real = li[s] != 0x7fffffff;
      oi[e] = real ? (int64_t)li[s] : -1;  // the key is the library index
      ov[e] = real ? lv[s] : -1.0f;
    }
  }
}

// ------------------------------------------------- screen candidates
// A row of packed brackets (ld a multiple of 4 words, rows 16-byte aligned)
// is read in chunks of kSelChunk words by blocks of 256 threads (grid:
// chunks x rows); each thread issues all eight of its 16-byte loads before
// using any.  Positive half-precision bit patterns order like the values,
// so a bin of hi is its top 12 bits (sign, exponent, six mantissa bits) and
// comparisons of lo run on the raw bits.
constexpr int kSelThreads = 256;
constexpr int kSelChunk = 8192;
constexpr int kSelPer = kSelChunk / 4 / kSelThreads;  // 16-byte loads per thread

__device__ __forceinline__ void load_chunk(const uint32_t *__restrict__ row, int64_t c0, uint4 (&w)[kSelPer],
                                           int64_t c1) {
  const uint4 *q = reinterpret_cast<const uint4 *>(row + c0);
#pragma unroll
  for (int u = 0; u < kSelPer; ++u) {
    const int64_t t = (int64_t)u * kSelThreads + threadIdx.x;
    w[u] = c0 + 4 * t < c1 ? q[t] : make_uint4(0, 0, 0, 0);
  }
}

__global__ void __launch_bounds__(kSelThreads) k_screen_hist(const uint32_t *__restrict__ packed, int64_t n,
                                                             int64_t ld, uint32_t *__restrict__ hist) {
  __shared__ uint32_t h[kScreenBins];
  for (int b = threadIdx.x; b < kScreenBins; b += kSelThreads) h[b] = 0;
  const int64_t r = blockIdx.y;
  const int64_t c0 = (int64_t)blockIdx.x * kSelChunk, c1 = min(n, c0 + kSelChunk);
  uint4 w[kSelPer];
  load_chunk(packed + r * ld, c0, w, c1);
  __syncthreads();
#pragma unroll
  for (int u = 0; u < kSelPer; ++u) {
    const int64_t c = c0 + 4 * ((int64_t)u * kSelThreads + threadIdx.x);
    if (c < c1) atomicAdd(&h[w[u].x >> 20], 1u);
    if (c + 1 < c1) atomicAdd(&h[w[u].y >> 20], 1u);
    if (c + 2 < c1) atomicAdd(&h[w[u].z >> 20], 1u);
    if (c + 3 < c1) atomicAdd(&h[w[u].w >> 20], 1u);
  }
  __syncthreads();
  uint32_t *gh = hist + r * kScreenBins;
  for (int b = threadIdx.x; b < kScreenBins; b += kSelThreads)
    if (h[b]) atomicAdd(&gh[b], h[b]);
}

// Block per row: the first bin at which the cumulative count reaches k; the
// threshold is that bin's top edge (all bins when the row has fewer than k).
__global__ void __launch_bounds__(kSelThreads) k_screen_thresh(const uint32_t *__restrict__ hist, int k,
                                                               uint32_t *__restrict__ thr) {
  constexpr int kPer = kScreenBins / kSelThreads;  // 16 consecutive bins per thread
  __shared__ uint32_t wsum[kSelThreads / 32];
  __shared__ uint32_t found;
  const int64_t r = blockIdx.x;
  const uint32_t *gh = hist + r * kScreenBins + threadIdx.x * kPer;
  uint32_t v[kPer], tot = 0;
#pragma unroll
  for (int i = 0; i < kPer; ++i) {
    v[i] = gh[i];
    tot += v[i];
  }
  if (threadIdx.x == 0) found = 0xffffffffu;
  // exclusive prefix of the per-thread totals across the block
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t inc = tot;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) wsum[warp] = inc;
  __syncthreads();
  uint32_t base = 0;
  for (int w = 0; w < warp; ++w) base += wsum[w];
  uint32_t cum = base + inc - tot;
  if (cum < (uint32_t)k && cum + tot >= (uint32_t)k) {
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
      cum += v[i];
      if (cum >= (uint32_t)k) {
        found = (uint32_t)(threadIdx.x * kPer + i);
        break;
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) thr[r] = found == 0xffffffffu ? 0xffffu : ((found << 4) | 0xfu);
}

__global__ void __launch_bounds__(kSelThreads) k_screen_extract(const uint32_t *__restrict__ packed, int64_t n,
                                                                int64_t ld, const uint32_t *__restrict__ thr,
                                                                int cap, int *__restrict__ cand_j,
                                                                int *__restrict__ cand_n) {
  const int64_t r = blockIdx.y;
  const int64_t c0 = (int64_t)blockIdx.x * kSelChunk, c1 = min(n, c0 + kSelChunk);
  uint4 w[kSelPer];
  load_chunk(packed + r * ld, c0, w, c1);
  const uint32_t t = thr[r];
  const int lane = threadIdx.x & 31;
  int *cj = cand_j + r * (int64_t)cap;
  // one atomic per warp and word position; every lane runs the same rounds
#pragma unroll
  for (int u = 0; u < kSelPer; ++u) {
    const int64_t c = c0 + 4 * ((int64_t)u * kSelThreads + threadIdx.x);
    const uint32_t v[4] = {w[u].x, w[u].y, w[u].z, w[u].w};
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const bool hit = c + e < c1 && (v[e] & 0xffffu) <= t;
      const unsigned m = __ballot_sync(0xffffffffu, hit);
      if (!m) continue;
      int base = 0;
      if (lane == 0) base = atomicAdd(&cand_n[r], __popc(m));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (hit) {
        const int slot = base + __popc(m & ((1u << lane) - 1u));
        if (slot < cap) cj[slot] = (int)(c + e);
      }
    }
  }
}

// The same two passes over a list of row-block segments only (pruned
// screens): segment s covers rows r0 .. r0 + nr - 1 and columns [c0, c1)
// (at most kSelChunk, c0 a multiple of 4); blockIdx.y picks the row.
__global__ void __launch_bounds__(kSelThreads) k_screen_hist_seg(const uint32_t *__restrict__ packed, int64_t ld,
                                                                 const SelSeg *__restrict__ segs,
                                                                 uint32_t *__restrict__ hist) {
  __shared__ uint32_t h[kScreenBins];
  const SelSeg sg = segs[blockIdx.x];
  if ((int)blockIdx.y >= sg.nr) return;  // the same for the whole block
  for (int b = threadIdx.x; b < kScreenBins; b += kSelThreads) h[b] = 0;
  const int64_t r = sg.r0 + blockIdx.y;
  const int64_t c0 = sg.c0, c1 = sg.c1;
  uint4 w[kSelPer];
  load_chunk(packed + r * ld, c0, w, c1);
  __syncthreads();
#pragma unroll
  for (int u = 0; u < kSelPer; ++u) {
    const int64_t c = c0 + 4 * ((int64_t)u * kSelThreads + threadIdx.x);
    if (c < c1) atomicAdd(&h[w[u].x >> 20], 1u);
    if (c + 1 < c1) atomicAdd(&h[w[u].y >> 20], 1u);
    if (c + 2 < c1) atomicAdd(&h[w[u].z >> 20], 1u);
    if (c + 3 < c1) atomicAdd(&h[w[u].w >> 20], 1u);
  }
  __syncthreads();
  uint32_t *gh = hist + r * kScreenBins;
  for (int b = threadIdx.x; b < kScreenBins; b += kSelThreads)
    if (h[b]) atomicAdd(&gh[b], h[b]);
}

__global__ void __launch_bounds__(kSelThreads) k_screen_extract_seg(const uint32_t *__restrict__ packed, int64_t ld,
                                                                    const SelSeg *__restrict__ segs,
                                                                    const uint32_t *__restrict__ thr, int cap,
                                                                    int *__restrict__ cand_j,
                                                                    int *__restrict__ cand_n) {
  const SelSeg sg = segs[blockIdx.x];
  if ((int)blockIdx.y >= sg.nr) return;
  const int64_t r = sg.r0 + blockIdx.y;
  const int64_t c0 = sg.c0, c1 = sg.c1;
  uint4 w[kSelPer];
  load_chunk(packed + r * ld, c0, w, c1);
  const uint32_t t = thr[r];
  const int lane = threadIdx.x & 31;
  int *cj = cand_j + r * (int64_t)cap;
#pragma unroll
  for (int u = 0; u < kSelPer; ++u) {
    const int64_t c = c0 + 4 * ((int64_t)u * kSelThreads + threadIdx.x);
    const uint32_t v[4] = {w[u].x, w[u].y, w[u].z, w[u].w};
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const bool hit = c + e < c1 && (v[e] & 0xffffu) <= t;
      const unsigned m = __ballot_sync(0xffffffffu, hit);
      if (!m) continue;
      int base = 0;
      if (lane == 0) base = atomicAdd(&cand_n[r], __popc(m));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (hit) {
        const int slot = base + __popc(m & ((1u << lane) - 1u));
        if (slot < cap) cj[slot] = (int)(c + e);
      }
    }
  }
}

}  // namespace

int screen_select_chunk() { return kSelChunk; }

cudaError_t launch_screen_select_seg(const uint32_t *packed, int64_t rows, int64_t ld, int k, int cap,
                                     const SelSeg *segs, int64_t nsegs, int max_rows, uint32_t *hist,
                                     uint32_t *thresholds, int *cand_j, int *cand_n, cudaStream_t st) {
  if (rows <= 0) return cudaSuccess;
  if (cap < 1 || k < 1 || (ld & 3) || ((uintptr_t)packed & 15) || max_rows < 1 || max_rows > 65535 ||
      nsegs > 0x7fffffff)
    return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(hist, 0, (size_t)rows * kScreenBins * 4, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(cand_n, 0, (size_t)rows * 4, st);
  if (e != cudaSuccess) return e;
  if (nsegs > 0) k_screen_hist_seg<<<dim3((unsigned)nsegs, (unsigned)max_rows), kSelThreads, 0, st>>>(packed, ld, segs,
                                                                                                    hist);
  k_screen_thresh<<<(unsigned)rows, kSelThreads, 0, st>>>(hist, k, thresholds);
  if (nsegs > 0)
    k_screen_extract_seg<<<dim3((unsigned)nsegs, (unsigned)max_rows), kSelThreads, 0, st>>>(packed, ld, segs,
                                                                                          thresholds, cap, cand_j,
                                                                                          cand_n);
  return cudaGetLastError();
}

cudaError_t launch_topk(const float *vals, int64_t rows, int64_t n, int64_t ld, int k, const int *perm,
                        int64_t *out_idx, float *out_val, cudaStream_t st) {
  if (rows <= 0) return cudaSuccess;
  if (k < 1 || k > kTopkMax || n > 0x7ffffffe) return cudaErrorInvalidValue;
  k_topk<<<(unsigned)rows, kTopkWarps * 32, 0, st>>>(vals, n, ld, nullptr, KeyMap{nullptr, perm, ld}, k, out_idx,
                                                      out_val);
  return cudaGetLastError();
}

cudaError_t launch_topk_rows(const float *vals, int64_t rows, const int *row_n, int64_t ld, int k,
                             const int *col_map, const int *perm, int64_t *out_idx, float *out_val, cudaStream_t st) {
  if (rows <= 0) return cudaSuccess;
  if (k < 1 || k > kTopkMax || ld > 0x7ffffffe) return cudaErrorInvalidValue;
  k_topk<<<(unsigned)rows, kTopkWarps * 32, 0, st>>>(vals, ld, ld, row_n, KeyMap{col_map, perm, ld}, k, out_idx,
                                                      out_val);
  return cudaGetLastError();
}

cudaError_t launch_screen_select(const uint32_t *packed, int64_t rows, int64_t n, int64_t ld, int k, int cap,
                                 uint32_t *hist, uint32_t *thresholds, int *cand_j, int *cand_n, cudaStream_t st) {
  if (rows <= 0) return cudaSuccess;
  if (n > 0x7ffffffe || n > ld || cap < 1 || k < 1 || rows > 65535 || (ld & 3) || ((uintptr_t)packed & 15))
    return cudaErrorInvalidValue;
  const unsigned chunks = (unsigned)((n + kSelChunk - 1) / kSelChunk);
  cudaError_t e = cudaMemsetAsync(hist, 0, (size_t)rows * kScreenBins * 4, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(cand_n, 0, (size_t)rows * 4, st);
  if (e != cudaSuccess) return e;
  if (chunks > 0) k_screen_hist<<<dim3(chunks, (unsigned)rows), kSelThreads, 0, st>>>(packed, n, ld, hist);
  k_screen_thresh<<<(unsigned)rows, kSelThreads, 0, st>>>(hist, k, thresholds);
  if (chunks > 0)
    k_screen_extract<<<dim3(chunks, (unsigned)rows), kSelThreads, 0, st>>>(packed, n, ld, thresholds, cap, cand_j,
                                                                         cand_n);
  return cudaGetLastError();
}

}  // namespace bs
