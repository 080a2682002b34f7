// neighbors.cu -- sparse eps-neighbour lists from the neighbour layout of the
// tensor-core kernel: the unordered (i, j, d) entries it appended become CSR
// rows, each ordered by (d, j) -- the order CartesianPoints::neighbors_of
// returns (points_set.rs:150-169: stable sort by distance of an ascending-j
// scan), without the point itself.
//
//   count    per row, the entries appended for it;
//   scan     row_ptr = exclusive prefix sum (one block);
//   scatter  each entry to its row as the 64-bit key (d bits << 32 | j): d is
//            a non-negative float, so its bits order like its value, and the
//            keys of a row are distinct;
//   sort     per row: bitonic sort in shared memory up to kSmemSort keys,
//            otherwise merge passes in global memory (rank by binary search);
//   unpack   keys -> col (int32), dist (f32).
#include <stdint.h>

#include "kernels.h"

namespace bs {
namespace {

constexpr int kScanThreads = 1024;
constexpr int kSortThreads = 512;
constexpr int kSmemSort = 4096;

__global__ void k_nbr_count(const int2 *__restrict__ ij, int64_t cnt, unsigned long long *__restrict__ rc) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < cnt; t += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&rc[ij[t].x], 1ull);
}

// row_ptr[0] = 0, row_ptr[i + 1] = row_ptr[i] + rc[i]; also the scatter cursors.
__global__ void __launch_bounds__(kScanThreads) k_nbr_scan(const unsigned long long *__restrict__ rc, int64_t n,
                                                           int64_t *__restrict__ row_ptr,
                                                           unsigned long long *__restrict__ cur) {
  __shared__ unsigned long long part[kScanThreads];
  const int64_t per = (n + kScanThreads - 1) / kScanThreads;
  const int64_t b = threadIdx.x * per, e = min(n, b + per);
  unsigned long long s = 0;
  for (int64_t i = b; i < e; ++i) s += rc[i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int o = 1; o < kScanThreads; o <<= 1) {
    const unsigned long long v = threadIdx.x >= o ? part[threadIdx.x - o] : 0ull;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  unsigned long long run = part[threadIdx.x] - s;  // exclusive prefix of this thread's segment
  if (threadIdx.x == 0) row_ptr[0] = 0;
  for (int64_t i = b; i < e; ++i) {
    cur[i] = run;
    run += rc[i];
    row_ptr[i + 1] = (int64_t)run;
  }
}

__global__ void k_nbr_scatter(const int2 *__restrict__ ij, const float *__restrict__ d, int64_t cnt,
                              unsigned long long *__restrict__ cur, unsigned long long *__restrict__ key) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < cnt; t += (int64_t)gridDim.x * blockDim.x) {
    const int2 p = ij[t];
    const unsigned long long pos = atomicAdd(&cur[p.x], 1ull);
    key[pos] = ((unsigned long long)__float_as_uint(d[t]) << 32) | (unsigned)p.y;
  }
}

// Number of keys in v[0..len) below x (v sorted, keys distinct).
__device__ __forceinline__ int64_t rank_below(const unsigned long long *v, int64_t len, unsigned long long x) {
  int64_t lo = 0, hi = len;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (v[mid] < x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Block per row.  Short rows: bitonic sort in shared memory.  Long rows:
// bottom-up merge passes between `key` and `tmp` (the result ends in `key`).
__global__ void __launch_bounds__(kSortThreads) k_nbr_sort(const int64_t *__restrict__ row_ptr,
                                                           unsigned long long *__restrict__ key,
                                                           unsigned long long *__restrict__ tmp) {
  __shared__ unsigned long long s[kSmemSort];
  const int64_t r = blockIdx.x;
  const int64_t b = row_ptr[r], len = row_ptr[r + 1] - b;
  if (len < 2) return;
  unsigned long long *v = key + b;
  if (len <= kSmemSort) {
    int p2 = 2;
    while (p2 < len) p2 <<= 1;
    for (int i = threadIdx.x; i < p2; i += kSortThreads) s[i] = i < len ? v[i] : ~0ull;
    __syncthreads();
    for (int k = 2; k <= p2; k <<= 1)
      for (int jj = k >> 1; jj > 0; jj >>= 1) {
        for (int i = threadIdx.x; i < p2; i += kSortThreads) {
          const int l = i ^ jj;
          if (l > i) {
            const bool up = (i & k) == 0;
            const unsigned long long x = s[i], y = s[l];
            if ((x > y) == up) {
              s[i] = y;
              s[l] = x;
            }
          }
        }
        __syncthreads();
      }
    for (int i = threadIdx.x; i < len; i += kSortThreads) v[i] = s[i];
    return;
  }
  unsigned long long *src = v, *dst = tmp + b;
  for (int64_t w = 1; w < len; w <<= 1) {
    for (int64_t i = threadIdx.x; i < len; i += kSortThreads) {
      const int64_t run = i / (2 * w), a0 = run * 2 * w;
      const int64_t a1 = min(len, a0 + w), b1 = min(len, a0 + 2 * w);
      int64_t pos;
      if (i < a1) pos = (i - a0) + rank_below(src + a1, b1 - a1, src[i]);
      else pos = (i - a1) + rank_below(src + a0, a1 - a0, src[i]);
      dst[a0 + pos] = src[i];
    }
    __syncthreads();
    unsigned long long *t = src;
    src = dst;
    dst = t;
  }
  if (src != v)
    for (int64_t i = threadIdx.x; i < len; i += kSortThreads) v[i] = src[i];
}

__global__ void k_nbr_unpack(const unsigned long long *__restrict__ key, int64_t nnz, int32_t *__restrict__ col,
                             float *__restrict__ dist) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nnz; t += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long k = key[t];
    col[t] = (int32_t)(uint32_t)k;
    dist[t] = __uint_as_float((unsigned)(k >> 32));
  }
}

}  // namespace

cudaError_t launch_neighbors_csr(const int2 *ij, const float *d, int64_t cnt, int64_t n, int num_sms,
                                 int64_t *row_ptr, int32_t *col, float *dist, unsigned long long *scratch_rows,
                                 unsigned long long *key, unsigned long long *tmp, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  if (n > 0x7fffffff) return cudaErrorInvalidValue;
  unsigned long long *rc = scratch_rows, *cur = scratch_rows + n;
  cudaError_t e = cudaMemsetAsync(rc, 0, (size_t)n * 8, st);
  if (e != cudaSuccess) return e;
  const unsigned grid = (unsigned)num_sms * 8;
  if (cnt > 0) k_nbr_count<<<grid, 256, 0, st>>>(ij, cnt, rc);
  k_nbr_scan<<<1, kScanThreads, 0, st>>>(rc, n, row_ptr, cur);
  if (cnt > 0) {
    k_nbr_scatter<<<grid, 256, 0, st>>>(ij, d, cnt, cur, key);
    k_nbr_sort<<<(unsigned)n, kSortThreads, 0, st>>>(row_ptr, key, tmp);
    k_nbr_unpack<<<grid, 256, 0, st>>>(key, cnt, col, dist);
  }
  return cudaGetLastError();
}

}  // namespace bs
