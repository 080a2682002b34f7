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

__global__ void __launch_bounds__(kTopkWarps * 32) k_topk(const float *__restrict__ vals, int64_t n, int64_t ld,
                                                          int k, int64_t *__restrict__ out_idx,
                                                          float *__restrict__ out_val) {
  __shared__ float sv[kTopkWarps][kTopkMax];
  __shared__ int si[kTopkWarps][kTopkMax];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const float *v = vals + (int64_t)blockIdx.x * ld;
  const float inf = __int_as_float(0x7f800000);
  float lv[2] = {inf, inf};
  int li[2] = {0x7fffffff, 0x7fffffff};
  float tv = inf;
  int ti = 0x7fffffff;
  for (int64_t base = (int64_t)warp * 32; base < n; base += kTopkWarps * 32) {
    const int64_t j = base + lane;
    const float x = j < n ? v[j] : inf;
    unsigned m = __ballot_sync(kFull, j < n && less_vi(x, (int)j, tv, ti));
    while (m) {
      const int src = __ffs(m) - 1;
      m &= m - 1;
      const float xv = __shfl_sync(kFull, x, src);
      const int xi = (int)(base + src);
      if (!less_vi(xv, xi, tv, ti)) continue;  // the threshold moved since the ballot
      list_insert(lv, li, xv, xi, lane);
      kth(lv, li, k, tv, ti);
    }
  }
  sv[warp][2 * lane] = lv[0];
  sv[warp][2 * lane + 1] = lv[1];
  si[warp][2 * lane] = li[0];
  si[warp][2 * lane + 1] = li[1];
  __syncthreads();
  if (warp != 0) return;
  for (int w = 1; w < kTopkWarps; ++w) {
    for (int e0 = 0; e0 < k; e0 += 32) {
      const int e = e0 + lane;
      const float x = e < k ? sv[w][e] : inf;
      const int xi = e < k ? si[w][e] : 0x7fffffff;
      unsigned m = __ballot_sync(kFull, e < k && less_vi(x, xi, tv, ti));
      while (m) {
        const int src = __ffs(m) - 1;
        m &= m - 1;
        const float xv = __shfl_sync(kFull, x, src);
        const int xii = __shfl_sync(kFull, xi, src);
        if (!less_vi(xv, xii, tv, ti)) continue;
        list_insert(lv, li, xv, xii, lane);
        kth(lv, li, k, tv, ti);
      }
    }
  }
  int64_t *oi = out_idx + (int64_t)blockIdx.x * k;
  float *ov = out_val + (int64_t)blockIdx.x * k;
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const int e = 2 * lane + s;
    if (e < k) {
      const bool real = li[s] != 0x7fffffff;
      oi[e] = real ? (int64_t)li[s] : -1;
      ov[e] = real ? lv[s] : -1.0f;
    }
  }
}

}  // namespace

cudaError_t launch_topk(const float *vals, int64_t rows, int64_t n, int64_t ld, int k, int64_t *out_idx,
                        float *out_val, cudaStream_t st) {
  if (rows <= 0) return cudaSuccess;
  if (k < 1 || k > kTopkMax || n > 0x7ffffffe) return cudaErrorInvalidValue;
  k_topk<<<(unsigned)rows, kTopkWarps * 32, 0, st>>>(vals, n, ld, k, out_idx, out_val);
  return cudaGetLastError();
}

}  // namespace bs
