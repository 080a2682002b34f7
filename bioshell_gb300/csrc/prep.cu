// prep.cu -- streaming preparation pass over the input coordinates.
//
// Per structure: centroid (arithmetic mean, as bioshell-pdb's
// SubstructureAxis centres, calc/substructures.rs:26-31), largest centred
// coordinate, then either
//   - mixed path: quantisation onto the grid 2^e, balanced digits (9, 9 and
//     5 bits) written as bf16 rows of the digit matrices (plus the low digit
//     scaled by 1/32, the operand of the level-4 product), exact squared norm
//     Ghat, the RMS quantisation residual and digit norms for the exactness
//     bound; or
//   - plain path: the centred f64 coordinates in K-major [n][3][lp] and G.
// One block per structure; the [L][3] AoS input of a structure is one
// contiguous range, read coalesced.
#include <math.h>

#include "crmsd_math.cuh"
#include "kernels.h"

namespace bs {
namespace {

constexpr int kPrepThreads = 128;

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Block-wide sum of N values held per thread; result valid in all threads.
template <typename T, int N>
__device__ __forceinline__ void block_sum(T (&v)[N], T *scratch /* [4][N] */) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int i = 0; i < N; ++i) v[i] = warp_sum(v[i]);
  if (lane == 0)
#pragma unroll
    for (int i = 0; i < N; ++i) scratch[warp * N + i] = v[i];
  __syncthreads();
#pragma unroll
  for (int i = 0; i < N; ++i) {
    T s = 0;
    for (int w = 0; w < kPrepThreads / 32; ++w) s += scratch[w * N + i];
    v[i] = s;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kPrepThreads) k_prep_stats(const double *__restrict__ xyz, int L,
                                                             double *__restrict__ ctr, DevScalars *sc) {
  __shared__ double red[4 * 3];
  __shared__ double redm[4];
  const int64_t s = blockIdx.x;
  const double *x = xyz + s * 3 * (int64_t)L;
  double acc[3] = {0.0, 0.0, 0.0};
  int bad = 0;
  for (int i = threadIdx.x; i < 3 * L; i += kPrepThreads) {
    const double v = x[i];
    bad |= !isfinite(v);
    const int c = i % 3;
    acc[0] += (c == 0) ? v : 0.0;
    acc[1] += (c == 1) ? v : 0.0;
    acc[2] += (c == 2) ? v : 0.0;
  }
  block_sum<double, 3>(acc, red);
  const double inv = 1.0 / (double)L;
  const double c0 = acc[0] * inv, c1 = acc[1] * inv, c2 = acc[2] * inv;
  double m = 0.0;
  for (int i = threadIdx.x; i < 3 * L; i += kPrepThreads) {
    const int c = i % 3;
    const double v = x[i] - (c == 0 ? c0 : (c == 1 ? c1 : c2));
    m = fmax(m, fabs(v));
  }
  m = warp_max(m);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) redm[warp] = m;
  bad = __syncthreads_or(bad);
  if (threadIdx.x == 0) {
    double mm = 0.0;
    for (int w = 0; w < kPrepThreads / 32; ++w) mm = fmax(mm, redm[w]);
    ctr[3 * s + 0] = c0;
    ctr[3 * s + 1] = c1;
    ctr[3 * s + 2] = c2;
    if (bad || !isfinite(mm)) {
      atomicOr(&sc->err, kErrNonFinite);
    } else {
      atomicMax(&sc->maxabs_bits, (unsigned long long)__double_as_longlong(mm));
    }
  }
}

// Smallest e >= scale_min with max|y| <= (2^22 - 1) 2^e, so that every
// quantised coordinate fits the three balanced digits.
__global__ void k_prep_scale(DevScalars *sc) {
  const double maxabs = __longlong_as_double((long long)sc->maxabs_bits);
  const double lim = 4194303.0;  // 2^22 - 1
  int e = -40;
  if (maxabs > 0.0) {
    e = (int)ceil(log2(maxabs / lim));
    while (ldexp(lim, e) < maxabs) ++e;
    while (ldexp(lim, e - 1) >= maxabs) --e;
  }
  if (e < sc->scale_min) e = sc->scale_min;
  sc->scale_exp = e;
}

__global__ void __launch_bounds__(kPrepThreads)
    k_prep_digits(const double *__restrict__ xyz, const double *__restrict__ ctr, int L, int lp,
                  __nv_bfloat16 *__restrict__ d0, __nv_bfloat16 *__restrict__ d1, __nv_bfloat16 *__restrict__ d2,
                  __nv_bfloat16 *__restrict__ d2s, SInfo *__restrict__ info, DevScalars *sc) {
  __shared__ long long red[4 * 10];
  __shared__ double redd[4];
  const int64_t s = blockIdx.x;
  const int e = sc->scale_exp;
  const double r = ldexp(1.0, e), inv_r = ldexp(1.0, -e);
  const double *x = xyz + s * 3 * (int64_t)L;
  const double cc[3] = {ctr[3 * s], ctr[3 * s + 1], ctr[3 * s + 2]};
  int64_t row[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) row[c] = digit_row(s, c) * lp;
  // acc[0] = Ghat, acc[1 + 3*i + c] = sum of e_i^2 for coordinate c
  long long acc[10];
#pragma unroll
  for (int i = 0; i < 10; ++i) acc[i] = 0;
  double res[1] = {0.0};  // sum of squared quantisation residuals
  for (int k = threadIdx.x; k < L; k += kPrepThreads) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double y = x[3 * k + c] - cc[c];
      const int q = __double2int_rn(y * inv_r);
      const double dq = y - (double)q * r;
      res[0] += dq * dq;
      int a, b, d;
      bsm::split_digits(q, a, b, d);
      d0[row[c] + k] = __float2bfloat16_rn((float)a);
      d1[row[c] + k] = __float2bfloat16_rn((float)b);
      d2[row[c] + k] = __float2bfloat16_rn((float)d);
      d2s[row[c] + k] = __float2bfloat16_rn((float)d * (1.0f / 512.0f));  // d2 / 32 = e2 / 512
      acc[0] += (long long)q * q;
      acc[1 + c] += (long long)(a * a);
      acc[4 + c] += (long long)(b * b);
      acc[7 + c] += (long long)(d * d);
    }
  }
  block_sum<long long, 10>(acc, red);
  block_sum<double, 1>(res, redd);
  if (threadIdx.x == 0) {
    SInfo in;
    in.ghat = acc[0];
    in.gf = (float)acc[0];
    // rounded up so that the Minkowski bound stays a bound
    in.qres = (float)(sqrt(res[0] / (double)L) * (1.0 + 1e-6)) + 1e-12f;
    info[s] = in;
    atomicMax(&sc->qres_max_bits, (unsigned long long)__float_as_uint(in.qres));
    for (int i = 0; i < 3; ++i) {
      long long mx = acc[1 + 3 * i];
      mx = acc[2 + 3 * i] > mx ? acc[2 + 3 * i] : mx;
      mx = acc[3 + 3 * i] > mx ? acc[3 + 3 * i] : mx;
      atomicMax(&sc->norm_max[i], (unsigned long long)mx);
    }
  }
}

__global__ void __launch_bounds__(kPrepThreads)
    k_prep_plain(const double *__restrict__ xyz, const double *__restrict__ ctr, int L, int lp,
                 double *__restrict__ y, double *__restrict__ g) {
  __shared__ double red[4];
  const int64_t s = blockIdx.x;
  const double *x = xyz + s * 3 * (int64_t)L;
  const double cc[3] = {ctr[3 * s], ctr[3 * s + 1], ctr[3 * s + 2]};
  double *ys = y + s * 3 * (int64_t)lp;
  double acc[1] = {0.0};
  for (int k = threadIdx.x; k < lp; k += kPrepThreads) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double v = (k < L) ? x[3 * k + c] - cc[c] : 0.0;
      ys[(int64_t)c * lp + k] = v;
      acc[0] += v * v;
    }
  }
  block_sum<double, 1>(acc, red);
  if (threadIdx.x == 0) g[s] = acc[0];
}

}  // namespace

cudaError_t launch_prep_stats(const double *xyz, int64_t n, int L, double *ctr, DevScalars *sc,
                              cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_prep_stats<<<(unsigned)n, kPrepThreads, 0, st>>>(xyz, L, ctr, sc);
  return cudaGetLastError();
}

cudaError_t launch_prep_scale(DevScalars *sc, cudaStream_t st) {
  k_prep_scale<<<1, 1, 0, st>>>(sc);
  return cudaGetLastError();
}

cudaError_t launch_prep_digits(const double *xyz, const double *ctr, int64_t n, int L, int lp,
                               __nv_bfloat16 *const *dig, SInfo *info, DevScalars *sc, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_prep_digits<<<(unsigned)n, kPrepThreads, 0, st>>>(xyz, ctr, L, lp, dig[0], dig[1], dig[2], dig[3], info, sc);
  return cudaGetLastError();
}

cudaError_t launch_prep_plain(const double *xyz, const double *ctr, int64_t n, int L, int lp, double *y,
                              double *g, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_prep_plain<<<(unsigned)n, kPrepThreads, 0, st>>>(xyz, ctr, L, lp, y, g);
  return cudaGetLastError();
}

}  // namespace bs
