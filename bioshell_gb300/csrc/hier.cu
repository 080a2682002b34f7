// hier.cu -- hierarchical agglomerative clustering on the GPU: the whole
// merge loop of hierarchical_clustering (hierarchical.rs:22-80) in one
// cooperative launch over a device-resident n x n f32 matrix, with the
// semantics of the host version in cluster.cpp bit for bit:
//   * the pair to merge is the first minimum of the reference's scan order
//     (clustering_matrix.rs:27-42), found from per-column minima kept up to
//     date (column j's minimum over rows r < j; ties: smallest r), the
//     smallest column winning ties;
//   * update_distances (clustering_matrix.rs:55-74) evaluates the merge rule
//     (strategies/mod.rs:101-167) with size_k = sizes[j] for every k, in the
//     same f32 operation order (no contraction: every product and sum below
//     is a correctly rounded intrinsic), and stores the merged cluster at i;
//   * replace_with_last (clustering_matrix.rs:47-53) swaps rows j and last,
//     copies column last into column j and leaves `sizes` where it was.
// The matrix stays exactly symmetric through these steps, so column scans
// read rows (coalesced).  Phases of a merge are separated by grid-wide
// barriers (the launch is cooperative, so every block is resident); every
// block recomputes the merge pair from the per-block partial minima, so no
// extra barrier is needed to broadcast it.  Each barrier wait is bounded: on
// a timeout, or if a merge pair ever falls outside the active matrix, the
// kernel records the phase in `err` and every block returns.
#include <float.h>
#include <stdint.h>

#include <algorithm>

#include "../../include/bioshell_crmsd.h"
#include "kernels.h"
#include "ptx.cuh"

namespace bs {
namespace {

constexpr int kHThreads = 512;

struct HierState {
  float *m;                 // [n][n]
  int64_t n;
  int rule;
  int64_t *sizes;           // [n] the matrix's size slots
  int64_t *ids;             // [n] tree node at each matrix index
  int64_t *node_size;       // [2n-1] leaves under each tree node
  float *cm_v;              // [n] column minima (columns 1 .. order-1)
  int64_t *cm_i;
  float *res;               // [n] scratch: the merged row
  float *part_v;            // [grid] per-block partial minima
  int64_t *part_j;
  int64_t *merges;          // [n-1][4]
  float *merge_dist;        // [n-1]
  unsigned *bar;            // [2] grid barrier: arrivals, generation (zeroed before the launch)
  int *err;                 // 0, or 1 + the phase that gave up
  uint64_t wait_ns;         // bound on each barrier wait
};

constexpr uint64_t kBarrierTimeoutNs = 2000000000ull;  // default bound

// Grid-wide barrier with a bounded wait.  Returns false, with *err set, when
// the other blocks did not arrive in time (or another block gave up).
__device__ bool grid_barrier(const HierState &s, int phase) {
  __syncthreads();
  int ok = 1;
  if (threadIdx.x == 0) {
    volatile unsigned *gen = s.bar + 1;
    const unsigned g = *gen;
    __threadfence();
    if (atomicAdd(s.bar, 1u) == gridDim.x - 1) {
      s.bar[0] = 0;
      __threadfence();
      atomicAdd(s.bar + 1, 1u);
    } else {
      const uint64_t t0 = ptx::globaltimer();
      while (*gen == g) {
        if (*(volatile int *)s.err || ptx::globaltimer() - t0 > s.wait_ns) {
          atomicCAS(s.err, 0, 1 + phase);
          ok = 0;
          break;
        }
      }
    }
    __threadfence();
  }
  return __syncthreads_and(ok) != 0;
}

__device__ __forceinline__ float rule_value(int rule, int64_t si, int64_t sj, int64_t sk, float dij, float dik,
                                            float djk) {
  switch (rule) {
    case BS_LINK_SINGLE:
      return djk < dik ? djk : dik;
    case BS_LINK_COMPLETE:
      return dik < djk ? djk : dik;
    case BS_LINK_AVERAGE: {
      const float d = __frcp_rn(__ll2float_rn(si + sj));
      return __fadd_rn(__fmul_rn(__fmul_rn(d, __ll2float_rn(si)), dik), __fmul_rn(__fmul_rn(d, __ll2float_rn(sj)), djk));
    }
    case BS_LINK_MEDIAN:
      return __fsub_rn(__fadd_rn(__fmul_rn(0.5f, dik), __fmul_rn(0.5f, djk)), __fmul_rn(0.25f, dij));
    case BS_LINK_CENTROID: {
      const float d = __frcp_rn(__ll2float_rn(si + sj));
      const float a = __fadd_rn(__fmul_rn(__fmul_rn(d, __ll2float_rn(si)), dik),
                                __fmul_rn(__fmul_rn(d, __ll2float_rn(sj)), djk));
      const float b = __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(__ll2float_rn(si), __ll2float_rn(sj)), d), d), dij);
      return __fsub_rn(a, b);
    }
    default: {  // Ward
      const float d = __frcp_rn(__ll2float_rn(si + sj + sk));
      const float a = __fadd_rn(__fmul_rn(__fmul_rn(d, __ll2float_rn(si + sk)), dik),
                                __fmul_rn(__fmul_rn(d, __ll2float_rn(sj + sk)), djk));
      return __fsub_rn(a, __fmul_rn(__fmul_rn(__ll2float_rn(sk), d), dij));
    }
  }
}

// (v, j) lexicographic minimum
__device__ __forceinline__ bool better(float v, int64_t j, float bv, int64_t bj) {
  return v < bv || (v == bv && j < bj);
}

// min over r < k of m[k][r] (= column k above the diagonal), first r on ties;
// the calling warp reduces.
__device__ void warp_colmin(const HierState &s, int64_t k, int lane, float &v, int64_t &idx) {
  const float *row = s.m + k * s.n;
  float bv = FLT_MAX;
  int64_t bi = 0;
  for (int64_t r = lane; r < k; r += 32) {
    const float x = row[r];
    if (x < bv) {  // r increases per lane: keeps the first
      bv = x;
      bi = r;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
    const int64_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
    if (better(ov, oi, bv, bi)) {
      bv = ov;
      bi = oi;
    }
  }
  if (bv == FLT_MAX) bi = 0;  // an empty or all-FLT_MAX column keeps the host's {FLT_MAX, 0}
  v = bv;
  idx = bi;
}

// After row/column x changed: column minima of x itself and of every column
// k > x whose minimum may have moved (warps over columns).
__device__ void refresh_columns(const HierState &s, int64_t x, int64_t order, int64_t gwarp, int64_t nwarps,
                                int lane) {
  for (int64_t k = x + gwarp; k < order; k += nwarps) {
    if (k == 0) continue;
    if (k == x) {
      float v;
      int64_t idx;
      warp_colmin(s, k, lane, v, idx);
      if (lane == 0) {
        s.cm_v[k] = v;
        s.cm_i[k] = idx;
      }
      continue;
    }
    const float v = s.m[x * s.n + k];
    const float cv = s.cm_v[k];
    const int64_t ci = s.cm_i[k];
    if (v < cv || (v == cv && x < ci)) {
      if (lane == 0) {
        s.cm_v[k] = v;
        s.cm_i[k] = x;
      }
    } else if (ci == x) {
      float nv;
      int64_t ni;
      warp_colmin(s, k, lane, nv, ni);
      if (lane == 0) {
        s.cm_v[k] = nv;
        s.cm_i[k] = ni;
      }
    }
  }
}

__global__ void __launch_bounds__(kHThreads) k_hier(HierState s) {
  __shared__ float sv[kHThreads / 32];
  __shared__ int64_t sj[kHThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  const int64_t gwarp = gtid >> 5, nwarps = nthreads >> 5;
  const int64_t n = s.n;
  // initial column minima
  for (int64_t k = 1 + gwarp; k < n; k += nwarps) {
    float v;
    int64_t idx;
    warp_colmin(s, k, lane, v, idx);
    if (lane == 0) {
      s.cm_v[k] = v;
      s.cm_i[k] = idx;
    }
  }
  if (!grid_barrier(s, 0)) return;
  int64_t order = n, cur = n;
  for (int64_t step = 0; step < n - 1; ++step) {
    // ---- 1: the merge pair (per-block partial minima of columns 1 .. order-1)
    float bv = FLT_MAX;
    int64_t bj = INT64_MAX;
    for (int64_t k = 1 + gtid; k < order; k += nthreads) {
      const float v = s.cm_v[k];
      if (better(v, k, bv, bj)) {
        bv = v;
        bj = k;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
      const int64_t oj = __shfl_xor_sync(0xffffffffu, bj, o);
      if (better(ov, oj, bv, bj)) {
        bv = ov;
        bj = oj;
      }
    }
    if (lane == 0) {
      sv[warp] = bv;
      sj[warp] = bj;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int w = 1; w < kHThreads / 32; ++w)
        if (better(sv[w], sj[w], bv, bj)) {
          bv = sv[w];
          bj = sj[w];
        }
      s.part_v[blockIdx.x] = bv;
      s.part_j[blockIdx.x] = bj;
    }
    if (!grid_barrier(s, 1)) return;
    if (threadIdx.x == 0) {
      bv = FLT_MAX;
      bj = INT64_MAX;
      for (unsigned b = 0; b < gridDim.x; ++b)
        if (better(s.part_v[b], s.part_j[b], bv, bj)) {
          bv = s.part_v[b];
          bj = s.part_j[b];
        }
      sj[0] = bj;
    }
    __syncthreads();
    const int64_t j = sj[0];
    const int64_t i = (j >= 1 && j < order) ? s.cm_i[j] : -1;
    if (!(i >= 0 && i < j)) {  // the same in every block: all return
      if (gtid == 0) atomicCAS(s.err, 0, 100);
      return;
    }
    const float dij = s.m[i * n + j];
    const int64_t si = s.sizes[i], szj = s.sizes[j];
    // ---- 2: the merged row from the old rows i and j
    for (int64_t k = gtid; k < order; k += nthreads)
      s.res[k] = rule_value(s.rule, si, szj, szj, dij, s.m[i * n + k], s.m[j * n + k]);
    if (!grid_barrier(s, 2)) return;
    for (int64_t k = gtid; k < order; k += nthreads) {
      const float r = k == i ? 0.0f : s.res[k];  // the diagonal is reset after the row is stored
      s.m[i * n + k] = r;
      s.m[k * n + i] = r;
    }
    if (gtid == 0) {
      const int64_t a = s.ids[i], b = s.ids[j];
      s.merges[4 * step + 0] = a;
      s.merges[4 * step + 1] = b;
      s.merges[4 * step + 2] = cur;
      s.node_size[cur] = s.node_size[a] + s.node_size[b];
      s.merges[4 * step + 3] = s.node_size[cur];
      s.merge_dist[step] = dij;
      s.sizes[i] = szj + si;
      s.ids[i] = cur;
    }
    if (!grid_barrier(s, 3)) return;
    // ---- 3: column minima touched by row/column i
    refresh_columns(s, i, order, gwarp, nwarps, lane);
    if (!grid_barrier(s, 4)) return;
    const int64_t last = order - 1;
    if (j < last) {
      // ---- 4: replace_with_last(j)
      for (int64_t k = gtid; k < n; k += nthreads) {
        const float a = s.m[j * n + k], b = s.m[last * n + k];
        s.m[j * n + k] = b;
        s.m[last * n + k] = a;
      }
      if (!grid_barrier(s, 5)) return;
      for (int64_t r = gtid; r < last; r += nthreads) s.m[r * n + j] = s.m[r * n + last];
      if (gtid == 0) s.ids[j] = s.ids[last];
      if (!grid_barrier(s, 6)) return;
      refresh_columns(s, j, last, gwarp, nwarps, lane);
      if (!grid_barrier(s, 7)) return;
    }
    order -= 1;
    cur += 1;
  }
}

// the square matrix from a packed upper triangle (f64 or f32), as f32
__global__ void k_hier_expand(const void *tri, int out_type, int64_t n, float *m) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t / n, c = t - r * n;
    float v = 0.0f;
    if (r != c) {
      const int64_t a = r < c ? r : c, b = r < c ? c : r;
      const int64_t k = a * n - a * (a + 1) / 2 + (b - a - 1);
      v = out_type == 0 ? (float)static_cast<const double *>(tri)[k] : static_cast<const float *>(tri)[k];
    }
    m[t] = v;
  }
}

__global__ void k_hier_init(int64_t n, int64_t *sizes, int64_t *ids, int64_t *node_size) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < 2 * n - 1; t += (int64_t)gridDim.x * blockDim.x) {
    if (t < n) {
      sizes[t] = 1;
      ids[t] = t;
    }
    node_size[t] = 1;
  }
}

}  // namespace

namespace {
size_t al(size_t b) { return (b + 255) & ~size_t(255); }
}  // namespace

size_t hier_workspace_bytes(int64_t n, int grid) {
  return al((size_t)n * n * 4) + 3 * al((size_t)n * 8) + al((size_t)(2 * n) * 8) + 2 * al((size_t)n * 4) +
         al((size_t)grid * 4) + al((size_t)grid * 8) + al(8) + al(4);
}

int hier_grid(int num_sms) {
  int per = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_hier, kHThreads, 0) != cudaSuccess || per < 1) {
    cudaGetLastError();
    per = 1;
  }
  return num_sms * std::min(per, 2);
}

cudaError_t launch_hierarchical(const void *tri, int out_type, int64_t n, int rule, void *ws, int grid,
                                int64_t *merges, float *merge_dist, int **err_out, uint64_t wait_ns, cudaStream_t st) {
  if (n < 2) return cudaSuccess;
  char *p = static_cast<char *>(ws);
  auto take = [&](size_t bytes) {
    void *r = p;
    p += (bytes + 255) & ~size_t(255);
    return r;
  };
  HierState s{};
  s.n = n;
  s.rule = rule;
  s.m = static_cast<float *>(take((size_t)n * n * 4));
  s.sizes = static_cast<int64_t *>(take((size_t)n * 8));
  s.ids = static_cast<int64_t *>(take((size_t)n * 8));
  s.node_size = static_cast<int64_t *>(take((size_t)(2 * n) * 8));
  s.cm_v = static_cast<float *>(take((size_t)n * 4));
  s.cm_i = static_cast<int64_t *>(take((size_t)n * 8));
  s.res = static_cast<float *>(take((size_t)n * 4));
  s.part_v = static_cast<float *>(take((size_t)grid * 4));
  s.part_j = static_cast<int64_t *>(take((size_t)grid * 8));
  s.bar = static_cast<unsigned *>(take(8));
  s.err = static_cast<int *>(take(4));
  s.merges = merges;
  s.merge_dist = merge_dist;
  s.wait_ns = wait_ns ? wait_ns : kBarrierTimeoutNs;
  *err_out = s.err;
  cudaError_t e = cudaMemsetAsync(s.bar, 0, 8, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(s.err, 0, 4, st);
  if (e != cudaSuccess) return e;
  k_hier_expand<<<1024, 256, 0, st>>>(tri, out_type, n, s.m);
  k_hier_init<<<256, 256, 0, st>>>(n, s.sizes, s.ids, s.node_size);
  void *args[] = {&s};
  return cudaLaunchCooperativeKernel((const void *)k_hier, dim3((unsigned)grid), dim3(kHThreads), args, 0, st);
}

}  // namespace bs
