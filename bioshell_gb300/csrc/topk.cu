// topk.cu -- the k nearest library structures of each query structure: the
// k smallest values of each row of a dense [rows][n] f32 crmsd block, in
// ascending (value, column) order -- a total order, so the result does not
// depend on how the row is scanned.
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

// One warp's share of a row: 16-byte loads of four values per lane; a
// chunk of 128 values costs one compare and one ballot unless some lane
// holds a value below the warp's current k-th entry.
__device__ void warp_scan(const float *__restrict__ v, int64_t n, int warp, int lane, int k, float (&lv)[2],
                          int (&li)[2], float &tv, int &ti) {
  const float inf = __int_as_float(0x7f800000);
  const int64_t mis = (int64_t)(((16 - ((uintptr_t)v & 15)) & 15) >> 2);  // values before 16-byte alignment
  const int64_t head = n < mis ? n : mis;
  if (warp == 0) {
    const bool ok = lane < head;
    consider(ok ? v[lane] : inf, lane, lane, k, lv, li, tv, ti, ok);
  }
  const float4 *v4 = reinterpret_cast<const float4 *>(v + head);
  const int64_t n4 = (n - head) >> 2;
  for (int64_t q = (int64_t)warp * 32; q < n4; q += kTopkWarps * 32) {
    const int64_t qi = q + lane;
    const float4 x = qi < n4 ? v4[qi] : make_float4(inf, inf, inf, inf);
    const float mn = fminf(fminf(x.x, x.y), fminf(x.z, x.w));
    if (!__any_sync(kFull, qi < n4 && mn <= tv)) continue;
    const int base = (int)(head + 4 * qi);
    consider(x.x, base + 0, lane, k, lv, li, tv, ti, qi < n4);
    consider(x.y, base + 1, lane, k, lv, li, tv, ti, qi < n4);
    consider(x.z, base + 2, lane, k, lv, li, tv, ti, qi < n4);
    consider(x.w, base + 3, lane, k, lv, li, tv, ti, qi < n4);
  }
  const int64_t tail0 = head + 4 * n4;
  if (warp == kTopkWarps - 1) {
    const int64_t j = tail0 + lane;
    const bool ok = j < n;
    consider(ok ? v[j] : inf, (int)j, lane, k, lv, li, tv, ti, ok);
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
                                                          const int *__restrict__ row_n,
                                                          const int *__restrict__ col_map, int k,
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
  warp_scan(v, n, warp, lane, k, lv, li, tv, ti);
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
      int64_t col = -1;
      if (real) col = col_map ? (int64_t)col_map[(int64_t)blockIdx.x * ld + li[s]] : (int64_t)li[s];
      oi[e] = col;
      ov[e] = real ? lv[s] : -1.0f;
    }
  }
}

// Screen candidates of one row (block per row): the k-th smallest upper
// bound of the row (the scan of k_topk), then every column whose lower
// bound does not exceed it.
__global__ void __launch_bounds__(kTopkWarps * 32) k_screen_select(const float *__restrict__ hi,
                                                                   const float *__restrict__ lo, int64_t n,
                                                                   int64_t ld, int k, int cap,
                                                                   int *__restrict__ cand_j,
                                                                   int *__restrict__ cand_n) {
  __shared__ float sv[kTopkWarps][kTopkMax];
  __shared__ int si[kTopkWarps][kTopkMax];
  __shared__ float thr;
  __shared__ int count;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t r = blockIdx.x;
  const float inf = __int_as_float(0x7f800000);
  float lv[2] = {inf, inf};
  int li[2] = {0x7fffffff, 0x7fffffff};
  float tv = inf;
  int ti = 0x7fffffff;
  warp_scan(hi + r * ld, n, warp, lane, k, lv, li, tv, ti);
  sv[warp][2 * lane] = lv[0];
  sv[warp][2 * lane + 1] = lv[1];
  si[warp][2 * lane] = li[0];
  si[warp][2 * lane + 1] = li[1];
  if (threadIdx.x == 0) count = 0;
  __syncthreads();
  if (warp == 0) {
    merge_lists(sv, si, lane, k, lv, li, tv, ti);
    // fewer than k columns: every column is a candidate
    if (lane == 0) thr = ti == 0x7fffffff ? inf : tv;
  }
  __syncthreads();
  const float t = thr;
  const float *v = lo + r * ld;
  int *cj = cand_j + r * (int64_t)cap;
  for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
    if (v[j] <= t) {
      const int slot = atomicAdd(&count, 1);
      if (slot < cap) cj[slot] = (int)j;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) cand_n[r] = count;
}

}  // namespace

cudaError_t launch_topk(const float *vals, int64_t rows, int64_t n, int64_t ld, int k, int64_t *out_idx,
                        float *out_val, cudaStream_t st) {
  if (rows <= 0) return cudaSuccess;
  if (k < 1 || k > kTopkMax || n > 0x7ffffffe) return cudaErrorInvalidValue;
  k_topk<<<(unsigned)rows, kTopkWarps * 32, 0, st>>>(vals, n, ld, nullptr, nullptr, k, out_idx, out_val);
  return cudaGetLastError();
}

cudaError_t launch_topk_rows(const float *vals, int64_t rows, const int *row_n, int64_t ld, int k,
                             const int *col_map, int64_t *out_idx, float *out_val, cudaStream_t st) {
  if (rows <= 0) return cudaSuccess;
  if (k < 1 || k > kTopkMax || ld > 0x7ffffffe) return cudaErrorInvalidValue;
  k_topk<<<(unsigned)rows, kTopkWarps * 32, 0, st>>>(vals, ld, ld, row_n, col_map, k, out_idx, out_val);
  return cudaGetLastError();
}

cudaError_t launch_screen_select(const float *hi, const float *lo, int64_t rows, int64_t n, int64_t ld, int k,
                                 int cap, int *cand_j, int *cand_n, cudaStream_t st) {
  if (rows <= 0) return cudaSuccess;
  if (n > 0x7ffffffe || cap < 1 || k < 1 || k > kTopkMax) return cudaErrorInvalidValue;
  k_screen_select<<<(unsigned)rows, kTopkWarps * 32, 0, st>>>(hi, lo, n, ld, k, cap, cand_j, cand_n);
  return cudaGetLastError();
}

}  // namespace bs
