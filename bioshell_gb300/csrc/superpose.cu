// superpose.cu -- the optimal superposition of explicit pairs as a
// rototranslation: for pair (i, j), the proper rotation R (3x3 row-major)
// and translation t with R x_j,k + t ~ x_i,k in the least-squares sense, and
// the RMSD of that superposition.  It is the output the reference's
// Rototranslation (bioshell-pdb/src/calc/transformation.rs:22-37, applied as
// R v + t by apply_mut, :171-174) carries.
//
// FP64 throughout: per pair the centroids and the covariance of the centred
// coordinates with lanes striding over atoms (XOR-butterfly sums, so every
// lane holds the same totals), the QCP key matrix's top eigenvector by
// Jacobi (crmsd_math.cuh: rotation_from_cov), then the residual of the
// superposition itself, so the returned RMSD is that of the returned
// transform.  This path is not the certified crmsd path: it works on the raw
// coordinates, with no quantisation.
#include "crmsd_math.cuh"
#include "kernels.h"

namespace bs {
namespace {

template <int N>
__device__ __forceinline__ void warp_sum(double (&v)[N]) {
#pragma unroll
  for (int e = 0; e < N; ++e)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[e] += __shfl_xor_sync(0xffffffffu, v[e], o);
}

// One warp per batch of 32 pairs.  The atom sums of pair t run over the
// lanes and land in lane t; the eigenproblems then run one pair per lane (an
// FP64 instruction costs a warp issue whether one lane or 32 are active, so
// a lane-0 eigensolver per pair would cost 32 times as much); the residual
// of pair t runs over the lanes again with its transform broadcast from
// lane t.
__global__ void k_superpose(const double *__restrict__ xyz, int64_t n, int L, const int64_t *__restrict__ pi,
                            const int64_t *__restrict__ pj, int64_t np, double *__restrict__ rot,
                            double *__restrict__ trans, double *__restrict__ rmsd, int *err) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t base = ((int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; base < np;
       base += warps * 32) {
    const int cnt = np - base < 32 ? (int)(np - base) : 32;
    double my_m[9], my_c[6];
#pragma unroll
    for (int e = 0; e < 9; ++e) my_m[e] = 0.0;
#pragma unroll
    for (int e = 0; e < 6; ++e) my_c[e] = 0.0;
    bool my_ok = false;
    for (int t = 0; t < cnt; ++t) {
      const int64_t i = pi[base + t], j = pj[base + t];
      if (i < 0 || i >= n || j < 0 || j >= n) {  // the same for the whole warp
        if (lane == 0) atomicOr(err, kErrBounds);
        continue;
      }
      const double *a = xyz + (size_t)i * L * 3, *b = xyz + (size_t)j * L * 3;
      double c[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
      for (int k = lane; k < L; k += 32)
#pragma unroll
        for (int x = 0; x < 3; ++x) {
          c[x] += a[3 * k + x];
          c[3 + x] += b[3 * k + x];
        }
      warp_sum(c);
#pragma unroll
      for (int x = 0; x < 6; ++x) c[x] /= (double)L;
      double m[9] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
      for (int k = lane; k < L; k += 32) {
        const double u0 = a[3 * k] - c[0], u1 = a[3 * k + 1] - c[1], u2 = a[3 * k + 2] - c[2];
        const double v0 = b[3 * k] - c[3], v1 = b[3 * k + 1] - c[4], v2 = b[3 * k + 2] - c[5];
        m[0] += u0 * v0;
        m[1] += u0 * v1;
        m[2] += u0 * v2;
        m[3] += u1 * v0;
        m[4] += u1 * v1;
        m[5] += u1 * v2;
        m[6] += u2 * v0;
        m[7] += u2 * v1;
        m[8] += u2 * v2;
      }
      warp_sum(m);
      if (lane == t) {
#pragma unroll
        for (int e = 0; e < 9; ++e) my_m[e] = m[e];
#pragma unroll
        for (int e = 0; e < 6; ++e) my_c[e] = c[e];
        my_ok = true;
      }
    }
    // this lane's pair: R and t = ca - R cb
    double r[9] = {1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0}, tv[3] = {0.0, 0.0, 0.0};
    if (my_ok) {
      bsm::rotation_from_cov(my_m, r);
#pragma unroll
      for (int x = 0; x < 3; ++x)
        tv[x] = my_c[x] - (r[3 * x] * my_c[3] + r[3 * x + 1] * my_c[4] + r[3 * x + 2] * my_c[5]);
    }
    double my_ss = 0.0;
    for (int t = 0; t < cnt; ++t) {
      const int64_t i = pi[base + t], j = pj[base + t];
      if (i < 0 || i >= n || j < 0 || j >= n) continue;
      double rr[9], tt[3];
#pragma unroll
      for (int e = 0; e < 9; ++e) rr[e] = __shfl_sync(0xffffffffu, r[e], t);
#pragma unroll
      for (int x = 0; x < 3; ++x) tt[x] = __shfl_sync(0xffffffffu, tv[x], t);
      const double *a = xyz + (size_t)i * L * 3, *b = xyz + (size_t)j * L * 3;
      double ss[1] = {0.0};
      for (int k = lane; k < L; k += 32) {
        const double b0 = b[3 * k], b1 = b[3 * k + 1], b2 = b[3 * k + 2];
#pragma unroll
        for (int x = 0; x < 3; ++x) {
          const double d = rr[3 * x] * b0 + rr[3 * x + 1] * b1 + rr[3 * x + 2] * b2 + tt[x] - a[3 * k + x];
          ss[0] += d * d;
        }
      }
      warp_sum(ss);
      if (lane == t) my_ss = ss[0];
    }
    if (my_ok) {
      const int64_t p = base + lane;
      bool fin = isfinite(my_ss);
#pragma unroll
      for (int e = 0; e < 9; ++e) fin = fin && isfinite(my_m[e]);
      if (!fin) atomicOr(err, kErrNonFinite);
#pragma unroll
      for (int e = 0; e < 9; ++e) rot[p * 9 + e] = r[e];
#pragma unroll
      for (int x = 0; x < 3; ++x) trans[p * 3 + x] = tv[x];
      if (rmsd) rmsd[p] = sqrt(my_ss / (double)L);
    }
  }
}

}  // namespace

cudaError_t launch_superpose(const double *xyz, int64_t n, int L, const int64_t *pi, const int64_t *pj, int64_t np,
                             double *rot, double *trans, double *rmsd, int *err, int num_sms, cudaStream_t st) {
  if (np <= 0) return cudaSuccess;
  const int64_t want = (np + 255) / 256;  // 8 warps of 32 pairs per block
  const unsigned grid = (unsigned)(want < (int64_t)num_sms * 16 ? want : (int64_t)num_sms * 16);
  k_superpose<<<grid, 256, 0, st>>>(xyz, n, L, pi, pj, np, rot, trans, rmsd, err);
  return cudaGetLastError();
}

}  // namespace bs
