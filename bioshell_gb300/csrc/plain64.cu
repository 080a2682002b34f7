// plain64.cu -- the plain FP64 all-vs-all crmsd (CUDA-core FP64).
//
// The honest FP64 method on the GPU: FP64 centred coordinates (prep.cu),
// the 3x3 covariance of every pair accumulated with FP64 FMAs, and the FP64
// QCP quartic solve of the same method as the CPU oracle.  This is the
// denominator the mixed path is compared against, so it is tiled for reuse:
// a block owns a 32 x 32 tile of structure pairs, stages K-major slices of
// both structure sets in shared memory, and each thread accumulates the
// covariances of one row structure against four column structures.
#include "crmsd_math.cuh"
#include "kernels.h"

namespace bs {
namespace {

constexpr int kT = 32;    // structures per tile side
constexpr int kKC = 16;   // atoms per shared-memory slice
constexpr int kThreads = 256;
constexpr int kJPer = 4;  // column structures per thread

__device__ __forceinline__ void tri_tile(int64_t t, int64_t nb, int64_t &I, int64_t &J) {
  // tiles (I, J), I <= J, row-major; row I starts at I*nb - I(I-1)/2
  const double b = 2.0 * (double)nb + 1.0;
  int64_t i = (int64_t)floor((b - sqrt(b * b - 8.0 * (double)t)) * 0.5);
  if (i < 0) i = 0;
  while (i > 0 && i * nb - i * (i - 1) / 2 > t) --i;
  while ((i + 1) * nb - (i + 1) * i / 2 <= t) ++i;
  I = i;
  J = i + (t - (i * nb - i * (i - 1) / 2));
}

__device__ __forceinline__ int64_t tri_index(int64_t n, int64_t i, int64_t j) {
  return i * n - i * (i + 1) / 2 + (j - i - 1);
}

__device__ __forceinline__ void store_pair(const OutDesc &o, int64_t i, int64_t j, double v) {
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

// SYM: tiles (I <= J) of the upper triangle of one set, pairs i < j;
// otherwise a grid of na/32 x nb/32 tiles of set A against set B, every pair.
template <bool SYM>
__global__ void __launch_bounds__(kThreads)
    k_plain64_tiles(const double *__restrict__ ya, const double *__restrict__ ga, int64_t na,
                    const double *__restrict__ yb, const double *__restrict__ gb, int64_t nb, int L, int lp,
                    OutDesc out) {
  __shared__ double sA[3][kKC][kT];
  __shared__ double sB[3][kKC][kT];
  int64_t I, J;
  if (SYM) {
    tri_tile(blockIdx.x, (na + kT - 1) / kT, I, J);
  } else {
    const int64_t tb_count = (nb + kT - 1) / kT;
    I = blockIdx.x / tb_count;
    J = blockIdx.x - I * tb_count;
  }
  const int ta = threadIdx.x / (kT / kJPer);            // 0..31 row structure
  const int tb = (threadIdx.x % (kT / kJPer)) * kJPer;  // first column structure
  double acc[kJPer][9];
#pragma unroll
  for (int q = 0; q < kJPer; ++q)
#pragma unroll
    for (int e = 0; e < 9; ++e) acc[q][e] = 0.0;
  for (int k0 = 0; k0 < L; k0 += kKC) {
    // stage: element (s, c, k) of both tiles; 2 * 32 * 3 * 16 = 3072 values
    for (int e = threadIdx.x; e < 2 * kT * 3 * kKC; e += kThreads) {
      const int side = e / (kT * 3 * kKC);
      const int r = e % (kT * 3 * kKC);
      const int s = r / (3 * kKC);
      const int c = (r / kKC) % 3;
      const int k = r % kKC;
      const int64_t gs = (side == 0 ? I : J) * kT + s;
      double v = 0.0;
      if (side == 0) {
        if (gs < na && k0 + k < lp) v = ya[(gs * 3 + c) * (int64_t)lp + k0 + k];
        sA[c][k][s] = v;
      } else {
        if (gs < nb && k0 + k < lp) v = yb[(gs * 3 + c) * (int64_t)lp + k0 + k];
        sB[c][k][s] = v;
      }
    }
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < kKC; ++k) {
      const double a0 = sA[0][k][ta], a1 = sA[1][k][ta], a2 = sA[2][k][ta];
#pragma unroll
      for (int q = 0; q < kJPer; ++q) {
        const double b0 = sB[0][k][tb + q], b1 = sB[1][k][tb + q], b2 = sB[2][k][tb + q];
        acc[q][0] = fma(a0, b0, acc[q][0]);
        acc[q][1] = fma(a0, b1, acc[q][1]);
        acc[q][2] = fma(a0, b2, acc[q][2]);
        acc[q][3] = fma(a1, b0, acc[q][3]);
        acc[q][4] = fma(a1, b1, acc[q][4]);
        acc[q][5] = fma(a1, b2, acc[q][5]);
        acc[q][6] = fma(a2, b0, acc[q][6]);
        acc[q][7] = fma(a2, b1, acc[q][7]);
        acc[q][8] = fma(a2, b2, acc[q][8]);
      }
    }
    __syncthreads();
  }
  const int64_t i = I * kT + ta;
  if (i >= na) return;
  const double gi = ga[i];
#pragma unroll
  for (int q = 0; q < kJPer; ++q) {
    const int64_t j = J * kT + tb + q;
    if (j >= nb || (SYM && j <= i)) continue;
    store_pair(out, i, j, bsm::qcp_rmsd_f64(acc[q], gi + gb[j], L));
  }
}

__global__ void k_plain64_pairs(const double *__restrict__ y, const double *__restrict__ g, int64_t n, int L,
                                int lp, const int64_t *__restrict__ ii, const int64_t *__restrict__ jj,
                                int64_t np, double *__restrict__ out) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= np) return;
  const int64_t i = ii[t], j = jj[t];
  const double *a = y + i * 3 * (int64_t)lp;
  const double *b = y + j * 3 * (int64_t)lp;
  double s[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int k = 0; k < L; ++k) {
    const double a0 = a[k], a1 = a[lp + k], a2 = a[2 * lp + k];
    const double b0 = b[k], b1 = b[lp + k], b2 = b[2 * lp + k];
    s[0] = fma(a0, b0, s[0]);
    s[1] = fma(a0, b1, s[1]);
    s[2] = fma(a0, b2, s[2]);
    s[3] = fma(a1, b0, s[3]);
    s[4] = fma(a1, b1, s[4]);
    s[5] = fma(a1, b2, s[5]);
    s[6] = fma(a2, b0, s[6]);
    s[7] = fma(a2, b1, s[7]);
    s[8] = fma(a2, b2, s[8]);
  }
  out[t] = (i == j) ? 0.0 : bsm::qcp_rmsd_f64(s, g[i] + g[j], L);
}

}  // namespace

cudaError_t launch_plain64_all(const double *y, const double *g, int64_t n, int L, int lp, OutDesc out,
                               cudaStream_t st) {
  if (n < 2) return cudaSuccess;
  const int64_t nb = (n + kT - 1) / kT;
  const int64_t ntiles = nb * (nb + 1) / 2;
  if (ntiles > 0x7fffffffLL) return cudaErrorInvalidValue;
  k_plain64_tiles<true><<<(unsigned)ntiles, kThreads, 0, st>>>(y, g, n, y, g, n, L, lp, out);
  return cudaGetLastError();
}

cudaError_t launch_plain64_rect(const double *ya, const double *ga, int64_t na, const double *yb, const double *gb,
                                int64_t nb, int L, int lp, OutDesc out, cudaStream_t st) {
  if (na < 1 || nb < 1) return cudaSuccess;
  const int64_t ntiles = ((na + kT - 1) / kT) * ((nb + kT - 1) / kT);
  if (ntiles > 0x7fffffffLL) return cudaErrorInvalidValue;
  k_plain64_tiles<false><<<(unsigned)ntiles, kThreads, 0, st>>>(ya, ga, na, yb, gb, nb, L, lp, out);
  return cudaGetLastError();
}

cudaError_t launch_plain64_pairs(const double *y, const double *g, int64_t n, int L, int lp, const int64_t *ii,
                                 const int64_t *jj, int64_t np, double *out, cudaStream_t st) {
  if (np <= 0) return cudaSuccess;
  const int th = 128;
  k_plain64_pairs<<<(unsigned)((np + th - 1) / th), th, 0, st>>>(y, g, n, L, lp, ii, jj, np, out);
  return cudaGetLastError();
}

}  // namespace bs
