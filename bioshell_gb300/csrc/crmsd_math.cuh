// crmsd_math.cuh -- per-pair arithmetic of the crmsd engine, shared by the
// GPU kernels and the host-side self-test hooks (same source, __host__
// __device__).
//
// Notation (one pair of structures a, b with L index-matched atoms):
//   centred coordinates are quantised to integers n = rint(y / 2^e),
//   |n| < 2^22, and split into balanced digits
//       n = d0 2^14 + d1 2^5 + d2,   |d0| <= 256, |d1| <= 256, |d2| <= 16,
//   stored as the bf16 values e0 = d0, e1 = d1, e2 = 16 d2 (all exact in bf16),
//   so that n = 2^14 (e0 + 2^-9 e1 + 2^-18 e2): three digits one 2^9 step apart.
//   S_l[x][y]  level sums of digit products, l = i + j:
//     S0 = sum e0a e0b                    S1 = sum e0a e1b + e1a e0b
//     S2 = sum e0a e2b + e1a e1b + e2a e0b S3 = sum e1a e2b + e2a e1b
//   The level-4 term sum e2a e2b = 256 sum d2a d2b rides in the level-3
//   accumulator as sum (d2a/32) e2b, i.e. the accumulator holds
//     S3' = S3 + S4 / 512,
//   which is exact while its partial sums stay below 2^23 (half-integers) and
//   otherwise carries a small, bounded FP32 rounding error.
//   Mhat = 2^28 S0 + 2^19 S1 + 2^10 S2 + 2 S3'           (units u = 2^(2e))
//   Ghat = sum n^2 (exact)                               (units u)
//   K(S) 4x4 quaternion key matrix, lambda0 = (Ga + Gb)/2,
//   E = Ga + Gb - 2 lambda_max(K) = 2 min_q q'(lambda0 I - K)q / |q|^2,
//   RMSD = sqrt(E / L).
// With the row-major convention S[3x+y] = sum a_x b_y used here,
//   q' K(S) q = sum_xy T(q)_xy S_xy,  T(q) = R(q)^T (transposed rotation).
//
// Levels 0-2 are exact: the host picks e so that every partial sum of those
// levels stays below 2^24 in magnitude, which FP32 accumulation represents
// exactly.
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define BS_HD __host__ __device__ __forceinline__
#else
#define BS_HD static inline
#endif

// Division where a few ulps do not matter (Halley steps, normalisations):
// the device uses the fast reciprocal-based divide, the host plain IEEE.
#if defined(__CUDA_ARCH__)
#define BS_FDIV(a, b) __fdividef((a), (b))
#else
#define BS_FDIV(a, b) ((a) / (b))
#endif

namespace bsm {

// ---------------------------------------------------------------- FP32 QCP
struct Key {
  float k00, k01, k02, k03, k11, k12, k13, k22, k23, k33;
};

BS_HD Key key_from_s(const float s[9]) {
  Key k;
  const float sxx = s[0], sxy = s[1], sxz = s[2];
  const float syx = s[3], syy = s[4], syz = s[5];
  const float szx = s[6], szy = s[7], szz = s[8];
  k.k00 = sxx + syy + szz;
  k.k01 = syz - szy;
  k.k02 = szx - sxz;
  k.k03 = sxy - syx;
  k.k11 = sxx - syy - szz;
  k.k12 = sxy + syx;
  k.k13 = szx + sxz;
  k.k22 = -sxx + syy - szz;
  k.k23 = syz + szy;
  k.k33 = -sxx - syy + szz;
  return k;
}

BS_HD float det3f(const float m[9]) {
  return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
         m[2] * (m[3] * m[7] - m[4] * m[6]);
}

// det of the symmetric 4x4 with entries b_ij; Laplace over 2x2 minors of
// rows (0,1) and their complements in rows (2,3).
BS_HD float det4_sym(float b00, float b01, float b02, float b03, float b11, float b12, float b13, float b22,
                     float b23, float b33) {
  // rows 0,1
  const float s01 = b00 * b11 - b01 * b01;
  const float s02 = b00 * b12 - b02 * b01;
  const float s03 = b00 * b13 - b03 * b01;
  const float s12 = b01 * b12 - b02 * b11;
  const float s13 = b01 * b13 - b03 * b11;
  const float s23 = b02 * b13 - b03 * b12;
  // rows 2,3 (row2 = b02 b12 b22 b23, row3 = b03 b13 b23 b33)
  const float c23 = b22 * b33 - b23 * b23;
  const float c13 = b12 * b33 - b23 * b13;
  const float c12 = b12 * b23 - b22 * b13;
  const float c03 = b02 * b33 - b23 * b03;
  const float c02 = b02 * b23 - b22 * b03;
  const float c01 = b02 * b13 - b12 * b03;
  return s01 * c23 - s02 * c13 + s03 * c12 + s12 * c03 - s13 * c02 + s23 * c01;
}

// 4-D generalised cross product of three row vectors (null vector of the
// 3x4 matrix they form).
BS_HD void gcross4(const float a[4], const float b[4], const float c[4], float v[4]) {
  const float m01 = b[0] * c[1] - b[1] * c[0];
  const float m02 = b[0] * c[2] - b[2] * c[0];
  const float m03 = b[0] * c[3] - b[3] * c[0];
  const float m12 = b[1] * c[2] - b[2] * c[1];
  const float m13 = b[1] * c[3] - b[3] * c[1];
  const float m23 = b[2] * c[3] - b[3] * c[2];
  v[0] = a[1] * m23 - a[2] * m13 + a[3] * m12;
  v[1] = -(a[0] * m23 - a[2] * m03 + a[3] * m02);
  v[2] = a[0] * m13 - a[1] * m03 + a[3] * m01;
  v[3] = -(a[0] * m12 - a[1] * m02 + a[2] * m01);
}

// Largest eigenvalue x and an eigenvector q (unnormalised) of K(s), for s
// scaled so that (Ga+Gb)/2 == 1 (then x <= 1).  Newton on the QCP quartic
// from x = 1, then the adjugate column of K - xI with the largest diagonal
// cofactor.  Returns |q|^2 relative to the scale of the cofactors; a tiny
// value means the top eigenvalue is (nearly) degenerate.
BS_HD float qcp_top_eig(const float s[9], float &xout, float q[4]) {
  const Key k = key_from_s(s);
  float fro2 = 0.f;
#pragma unroll
  for (int i = 0; i < 9; ++i) fro2 = fmaf(s[i], s[i], fro2);
  const float c2 = -2.f * fro2;
  const float c1 = -8.f * det3f(s);
  const float c0 = det4_sym(k.k00, k.k01, k.k02, k.k03, k.k11, k.k12, k.k13, k.k22, k.k23, k.k33);
  // Halley iterations from the upper bound x = 1 (the largest root is <= 1
  // and P is convex above it); five steps reach FP32 precision for every
  // root in (0, 1] met in practice, and a fixed count keeps warps converged.
  float x = 1.0f;
#pragma unroll
  for (int it = 0; it < 5; ++it) {
    const float x2 = x * x;
    const float p = fmaf(fmaf(x2 + c2, x, c1), x, c0);  // ((x^2+c2)x + c1)x + c0
    const float dp = fmaf(fmaf(4.f, x2, 2.f * c2), x, c1);
    const float ddp = fmaf(12.f, x2, 2.f * c2);
    const float den = fmaf(2.f * dp, dp, -p * ddp);
    const float step = BS_FDIV(2.f * p * dp, den);
    x = (den > 0.f) ? x - step : x;
  }
  xout = x;
  const float b00 = k.k00 - x, b11 = k.k11 - x, b22 = k.k22 - x, b33 = k.k33 - x;
  const float r0[4] = {b00, k.k01, k.k02, k.k03};
  const float r1[4] = {k.k01, b11, k.k12, k.k13};
  const float r2[4] = {k.k02, k.k12, b22, k.k23};
  const float r3[4] = {k.k03, k.k13, k.k23, b33};
  // diagonal cofactors
  const float C0 = b11 * (b22 * b33 - k.k23 * k.k23) - k.k12 * (k.k12 * b33 - k.k23 * k.k13) +
                   k.k13 * (k.k12 * k.k23 - b22 * k.k13);
  const float C1 = b00 * (b22 * b33 - k.k23 * k.k23) - k.k02 * (k.k02 * b33 - k.k23 * k.k03) +
                   k.k03 * (k.k02 * k.k23 - b22 * k.k03);
  const float C2 = b00 * (b11 * b33 - k.k13 * k.k13) - k.k01 * (k.k01 * b33 - k.k13 * k.k03) +
                   k.k03 * (k.k01 * k.k13 - b11 * k.k03);
  const float C3 = b00 * (b11 * b22 - k.k12 * k.k12) - k.k01 * (k.k01 * b22 - k.k12 * k.k02) +
                   k.k02 * (k.k01 * k.k12 - b11 * k.k02);
  const float a0 = fabsf(C0), a1 = fabsf(C1), a2 = fabsf(C2), a3 = fabsf(C3);
  int j = 0;
  float best = a0;
  if (a1 > best) { best = a1; j = 1; }
  if (a2 > best) { best = a2; j = 2; }
  if (a3 > best) { best = a3; j = 3; }
  float sa[4], sb[4], sc[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    sa[i] = (j == 0) ? r1[i] : r0[i];
    sb[i] = (j <= 1) ? r2[i] : r1[i];
    sc[i] = (j <= 2) ? r3[i] : r2[i];
  }
  gcross4(sa, sb, sc, q);
  return best;
}

// Screen of one pair from digits 0 and 1 only: m = S0 + 2^-9 S1 + 2^-18 S11
// (S11 = sum e1 e1; units 2^28 u) is the covariance of the truncated
// structures t = n - d2 (digit 2 dropped), gsum_f their G_a + G_b (units
// u), de a bound on the FP32 rounding of the accumulated S11 as an error of
// E (units u; 0 when it is exact).  Returns a bracket
// lo <= crmsd(n_a, n_b) <= hi without the eigenvector.
//
// P(x), the QCP quartic of t normalised by lambda0 = gsum/2, has four real
// roots (the eigenvalues of the symmetric key matrix over lambda0) and the
// top one is 0 <= x* <= 1.  Above its largest root a real-rooted polynomial is
// increasing and convex, so Newton's method from x = 1 decreases
// monotonically towards x*: every iterate x satisfies x - P(x)/P'(x) >= x*.
// And since P'/P = sum 1 / (x - x_i) over the four roots, the root nearest
// to x -- here x* -- lies within 4 P(x)/P'(x) of x.  With eP >= |computed P -
// P| and eD >= |computed P' - P'|, for x >= x*:
//     x - max(P - eP, 0) / (P' + eD)  >=  x*  >=  x - 4 (P + eP) / (P' - eD).
// The bracket holds whether or not the iteration has converged: near pairs
// converge in two or three steps, far pairs only need a loose bracket, and
// where the top root is nearly double (P' small) the bracket widens instead
// of failing.
//
// The error bounds (u = 2^-24): a forward error analysis of the operations
// below in the manner of Higham (Accuracy and Stability of Numerical
// Algorithms, ch. 3), every rounding bounded by u times the magnitude it
// rounds, with the magnitudes bounded as follows.  Let s = M / lambda0 be the
// exact normalised covariance of the truncated pair: ||M||_F <= sqrt(Ga Gb)
// <= lambda0 gives ||s||_F <= 1, and the eigenvalues of K(s) are sign
// combinations of the singular values of s, so ||K(s)||_2 <= ||s||_* <= 1
// (nuclear norm of A B^T <= ||A||_F ||B||_F).  Hence every row of K has norm
// <= 1, the singular values of adj(K) are <= 1 (||adj K||_F <= 2), any two
// distinct products of a 2x2 minor sum to <= 1/2 (s) or <= 1 (K) in
// magnitude (AM-GM), the six 2x2 minors of two rows have squares summing to
// <= 1 (Lagrange's identity), and |c2| <= 2, |c1| <= 8 / 3^1.5, |c0| <= 1.
//   * input: the computed sn differs from s by at most 8.1u |s_i| + 0.01u
//     per entry (the two FMAs forming m, gsum_f from two rounded G's, the fast
//     reciprocal (2 ulp), the product), so ||sn - s||_F <= 8.1u and, by Weyl
//     with ||K(D)||_2 <= sqrt(3) ||D||_F, the top root moves by at most
//     14u < 2^-19: the bracket is widened by 2^-19 on both sides;
//   * coefficients from sn: c2 (a 9-term FMA chain) within 18.1u; c1 = -8
//     det3 within 8 x 4.35u = 35u; c0 = det4 within 31.5u (15.9u for the
//     expansion in 2x2 minors, 15.6u for the rounded key-matrix entries,
//     ||dK||_F <= 7.8u, through the cofactors);
//   * evaluation by Horner at 0 <= x <= 1: P within 14.1u, P' within 21.5u.
// So |computed P - P| <= 99u and |computed P' - P'| <= 93u, below the
// eP = eD = 2^-16 (256u) used.  The final steps' roundings are covered by
// 2^-20 on x and a relative 2^-20 on the two RMSD bounds.  Finally crmsd(t)
// is within dr = rms(d2_a) + rms(d2_b) (Angstrom) of crmsd(n) (Minkowski:
// each structure moves by the RMS of its dropped digit), and the rounding of
// an inexact S11 enters through de as an error of E.
BS_HD void screen_bracket(const float m[9], float gsum_f, float de, float dr, float u, int L, float &lo,
                          float &hi) {
  if (!(gsum_f > 0.f)) {
    lo = 0.f;
    hi = dr;
    return;
  }
  const float lam0 = gsum_f * 1.862645149230957e-09f;  // 2^-29: gsum/2 in units of m
  const float inv = BS_FDIV(1.0f, lam0);
  float sn[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) sn[i] = m[i] * inv;
  const Key k = key_from_s(sn);
  float fro2 = 0.f;
#pragma unroll
  for (int i = 0; i < 9; ++i) fro2 = fmaf(sn[i], sn[i], fro2);
  const float c2 = -2.f * fro2;
  const float c1 = -8.f * det3f(sn);
  const float c0 = det4_sym(k.k00, k.k01, k.k02, k.k03, k.k11, k.k12, k.k13, k.k22, k.k23, k.k33);
  constexpr float eP = 1.52587890625e-05f, eD = 1.52587890625e-05f;  // 2^-16 (see above)
  constexpr float mx = 2.86102294921875e-06f;                        // 2^-19 + 2^-20 on x
  float x = 1.0f, p = 0.f, dp = 0.f;
#pragma unroll
  for (int it = 0; it < 4; ++it) {
    const float x2 = x * x;
    p = fmaf(fmaf(x2 + c2, x, c1), x, c0);
    dp = fmaf(fmaf(4.f, x2, 2.f * c2), x, c1);
    if (it < 3) x -= BS_FDIV(fmaxf(p - eP, 0.f), fmaxf(dp + eD, eD));  // P' >= 0 for x >= x*
  }
  const float xhi = fminf(x - BS_FDIV(fmaxf(p - eP, 0.f), fmaxf(dp + eD, eD)) + mx, 1.0f);  // >= x*
  const float xlo = dp > eD ? fmaxf(x - BS_FDIV(4.f * (p + eP), dp - eD) - mx, 0.f) : 0.f;
  const float scale = BS_FDIV(u, (float)L);
  lo = fmaxf(sqrtf(fmaxf(fmaf(gsum_f, 1.0f - xhi, -de), 0.f) * scale) * 0.99999904632568359375f - dr, 0.f);
  hi = sqrtf(fmaf(gsum_f, 1.0f - xlo, de) * scale) * 1.00000095367431640625f + dr;
}

#if defined(__CUDACC__)
// Two pairs at once on the packed FP32x2 pipe (sm_100 and later): each
// operation below is one instruction for both lanes of the pair, rounded as
// the scalar operation (a - b is fma(b, -1, a): one rounding).  Division,
// maxima and square roots stay per component.
struct F2 {
  float2 v;
};
__device__ __forceinline__ F2 f2(float a) { return F2{make_float2(a, a)}; }
__device__ __forceinline__ F2 f2(float a, float b) { return F2{make_float2(a, b)}; }
__device__ __forceinline__ F2 operator+(F2 a, F2 b) { return F2{__fadd2_rn(a.v, b.v)}; }
__device__ __forceinline__ F2 operator*(F2 a, F2 b) { return F2{__fmul2_rn(a.v, b.v)}; }
__device__ __forceinline__ F2 operator-(F2 a, F2 b) { return F2{__ffma2_rn(b.v, make_float2(-1.f, -1.f), a.v)}; }
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c) { return F2{__ffma2_rn(a.v, b.v, c.v)}; }
__device__ __forceinline__ F2 max2(F2 a, F2 b) { return F2{make_float2(fmaxf(a.v.x, b.v.x), fmaxf(a.v.y, b.v.y))}; }
__device__ __forceinline__ F2 div2(F2 a, F2 b) {
  return F2{make_float2(__fdividef(a.v.x, b.v.x), __fdividef(a.v.y, b.v.y))};
}

// screen_bracket for two pairs (the same bracket, the same margins).
__device__ __forceinline__ void screen_bracket2(const F2 m[9], F2 gsum, float de, F2 dr, float u, int L, F2 &lo,
                                                F2 &hi) {
  const F2 lam0 = gsum * f2(1.862645149230957e-09f);  // 2^-29: gsum/2 in units of m
  const F2 inv = div2(f2(1.0f), lam0);
  F2 sn[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) sn[i] = m[i] * inv;
  const F2 sxx = sn[0], sxy = sn[1], sxz = sn[2], syx = sn[3], syy = sn[4], syz = sn[5], szx = sn[6], szy = sn[7],
           szz = sn[8];
  const F2 k00 = sxx + syy + szz, k01 = syz - szy, k02 = szx - sxz, k03 = sxy - syx;
  const F2 k11 = sxx - syy - szz, k12 = sxy + syx, k13 = szx + sxz;
  const F2 k22 = syy - sxx - szz, k23 = syz + szy, k33 = szz - sxx - syy;
  F2 fro2 = f2(0.f);
#pragma unroll
  for (int i = 0; i < 9; ++i) fro2 = fma2(sn[i], sn[i], fro2);
  const F2 c2 = f2(-2.f) * fro2;
  const F2 det3 = sxx * (syy * szz - syz * szy) - sxy * (syx * szz - syz * szx) + sxz * (syx * szy - syy * szx);
  const F2 c1 = f2(-8.f) * det3;
  const F2 s01 = k00 * k11 - k01 * k01, s02 = k00 * k12 - k02 * k01, s03 = k00 * k13 - k03 * k01;
  const F2 s12 = k01 * k12 - k02 * k11, s13 = k01 * k13 - k03 * k11, s23 = k02 * k13 - k03 * k12;
  const F2 t23 = k22 * k33 - k23 * k23, t13 = k12 * k33 - k23 * k13, t12 = k12 * k23 - k22 * k13;
  const F2 t03 = k02 * k33 - k23 * k03, t02 = k02 * k23 - k22 * k03, t01 = k02 * k13 - k12 * k03;
  const F2 c0 = s01 * t23 - s02 * t13 + s03 * t12 + s12 * t03 - s13 * t02 + s23 * t01;
  const F2 eP = f2(1.52587890625e-05f), eD = eP;  // 2^-16, as screen_bracket
  F2 x = f2(1.0f), p = f2(0.f), dp = f2(0.f);
#pragma unroll
  for (int it = 0; it < 4; ++it) {
    const F2 x2 = x * x;
    p = fma2(fma2(x2 + c2, x, c1), x, c0);
    dp = fma2(fma2(f2(4.f), x2, f2(2.f) * c2), x, c1);
    if (it < 3) x = x - div2(max2(p - eP, f2(0.f)), max2(dp + eD, eD));  // P' >= 0 for x >= x*
  }
  const F2 d1 = div2(max2(p - eP, f2(0.f)), max2(dp + eD, eD));
  const F2 d4 = div2(f2(4.f) * (p + eP), dp - eD);
  const float scale = __fdividef(u, (float)L);
  float lx[2], hx[2];
  const float xs[2] = {x.v.x, x.v.y}, d1s[2] = {d1.v.x, d1.v.y}, d4s[2] = {d4.v.x, d4.v.y};
  const float dps[2] = {dp.v.x, dp.v.y}, gs[2] = {gsum.v.x, gsum.v.y}, drs[2] = {dr.v.x, dr.v.y};
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    if (!(gs[c] > 0.f)) {
      lx[c] = 0.f;
      hx[c] = drs[c];
      continue;
    }
    const float xhi = fminf(xs[c] - d1s[c] + 2.86102294921875e-06f, 1.0f);  // >= x*
    const float xlo = dps[c] > 1.52587890625e-05f ? fmaxf(xs[c] - d4s[c] - 2.86102294921875e-06f, 0.f) : 0.f;
    lx[c] = fmaxf(sqrtf(fmaxf(fmaf(gs[c], 1.0f - xhi, -de), 0.f) * scale) * 0.99999904632568359375f - drs[c], 0.f);
    hx[c] = sqrtf(fmaf(gs[c], 1.0f - xlo, de) * scale) * 1.00000095367431640625f + drs[c];
  }
  lo = f2(lx[0], lx[1]);
  hi = f2(hx[0], hx[1]);
}
#endif

// ------------------------------------------------- quaternion -> T = R^T
// T(q) with q = (w, x, y, z); quadratic, homogeneous.
template <typename V>
BS_HD void t_of_q(const V q[4], V t[9]) {
  const V w = q[0], x = q[1], y = q[2], z = q[3];
  const V ww = w * w, xx = x * x, yy = y * y, zz = z * z;
  const V wx = w * x, wy = w * y, wz = w * z, xy = x * y, xz = x * z, yz = y * z;
  t[0] = ww + xx - yy - zz;
  t[1] = 2 * (xy + wz);
  t[2] = 2 * (xz - wy);
  t[3] = 2 * (xy - wz);
  t[4] = ww - xx + yy - zz;
  t[5] = 2 * (yz + wx);
  t[6] = 2 * (xz + wy);
  t[7] = 2 * (yz - wx);
  t[8] = ww - xx - yy + zz;
}

// Symmetric bilinear form T(q, p):  T(q+p) = T(q) + 2 T(q,p) + T(p).
BS_HD void t_bilinear(const float q[4], const float p[4], float t[9]) {
  const float w = q[0], x = q[1], y = q[2], z = q[3];
  const float W = p[0], X = p[1], Y = p[2], Z = p[3];
  const float ww = w * W, xx = x * X, yy = y * Y, zz = z * Z;
  const float xy = x * Y + y * X, wz = w * Z + z * W, xz = x * Z + z * X;
  const float wy = w * Y + y * W, yz = y * Z + z * Y, wx = w * X + x * W;
  t[0] = ww + xx - yy - zz;
  t[1] = xy + wz;
  t[2] = xz - wy;
  t[3] = xy - wz;
  t[4] = ww - xx + yy - zz;
  t[5] = yz + wx;
  t[6] = xz + wy;
  t[7] = yz - wx;
  t[8] = ww - xx - yy + zz;
}

// int128 -> float from three 32-bit pieces (|v| < 2^95); 32-bit integer
// conversions avoid the 64-bit ones, which run on the slow FP64 pipe.
BS_HD float i128_to_f32(__int128 v) {
  const int top = (int)(long long)(v >> 64);
  const unsigned mid = (unsigned)((unsigned long long)v >> 32);
  const unsigned low = (unsigned)(unsigned long long)v;
  return fmaf((float)top, 18446744073709551616.0f, fmaf((float)mid, 4294967296.0f, (float)low));
}

// int64 -> float from two 32-bit pieces (|v| < 2^63).
BS_HD float i64_to_f32(long long v) {
  return fmaf((float)(int)(v >> 32), 4294967296.0f, (float)(unsigned)(unsigned long long)v);
}

// ----------------------------------------------------- fast-path epilogue
// The fast path runs in three phases so that the tensor-core epilogue can
// stream one TMEM level accumulator at a time:
//   1. fast_begin: FP32 covariance m (from all levels) -> FP32 QCP eigenpair,
//      unit eigenvector split q = q_h + q_l with q_h on the 2^-17 grid
//      (Q_h = 2^17 q_h integers, |T(Q_h)| <= |Q_h|^2 <= 2^34), exact int64
//      T(Q_h), and the small FP32 terms 4 B(q_h,q_l) + 2 F(q_l);
//   2. fast_level (l = 0..3): U_l += sum_xy T_xy S_l,xy, exactly in int64 for
//      l = 0, 1, 2 and in FP32 for l = 3;
//   3. fast_finish: 2 F(q_h) exactly in int128, E = 2 F(q) / |q|^2, RMSD and
//      the error bound that decides whether the pair is recomputed.
// m is the covariance in units of 2^28 u:  m = S0 + 2^-9 S1 + 2^-18 S2 + 2^-27 S3.
BS_HD float m_from_levels(float s0, float s1, float s2, float s3) {
  return fmaf(s3, 7.450580596923828125e-9f, fmaf(s2, 3.814697265625e-6f, fmaf(s1, 0.001953125f, s0)));
}

struct FastState {
  long long T[9];
  long long U0, U1, U2;
  float U3;
  float rest;    // 4 B(q_h,q_l) + 2 F(q_l), units 2^28 u
  float qq;      // |q|^2 of the (unit) eigenvector as represented
  long long q2;  // |Q_h|^2
  float qh[4];   // q_h as floats (exact), for the level-3 term
  int flag;      // 1: degenerate eigenvector, recompute exactly
};

BS_HD void fast_begin(const float m[9], float gsum_f, FastState &st) {
  st.U0 = st.U1 = st.U2 = 0;
  st.U3 = 0.f;
  st.flag = 0;
  st.rest = 0.f;
  st.qq = 1.f;
  st.q2 = 0;
#pragma unroll
  for (int i = 0; i < 9; ++i) st.T[i] = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) st.qh[i] = 0.f;
  if (!(gsum_f > 0.f)) return;  // both structures collapse onto one point: E = 0
  const float lam0 = gsum_f * 1.862645149230957e-9f;  // (Ga+Gb)/2 in units 2^28 u: 2^-29
  const float inv = BS_FDIV(1.0f, lam0);
  float sn[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) sn[i] = m[i] * inv;
  float x, q[4];
  const float cof = qcp_top_eig(sn, x, q);
  const float qsq = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
  if (!(qsq > 1e-30f) || !(cof > 1e-6f)) {
    st.flag = 1;
    return;
  }
  const float qs = rsqrtf(qsq) * 0.99999f;  // unit length (a hair below, so |Q_h|^2 <= 2^34)
  float qn[4], qh[4], ql[4];
  long long Q[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    qn[i] = q[i] * qs;
    const float h = rintf(qn[i] * 131072.f);
    Q[i] = (long long)(int)h;
    qh[i] = h * 7.62939453125e-6f;  // 2^-17
    ql[i] = qn[i] - qh[i];
  }
  t_of_q<long long>(Q, st.T);
  st.q2 = Q[0] * Q[0] + Q[1] * Q[1] + Q[2] * Q[2] + Q[3] * Q[3];
#pragma unroll
  for (int i = 0; i < 4; ++i) st.qh[i] = qh[i];
  float tb[9], tl[9];
  t_bilinear(qh, ql, tb);
  t_of_q<float>(ql, tl);
  const float dot_hl = qh[0] * ql[0] + qh[1] * ql[1] + qh[2] * ql[2] + qh[3] * ql[3];
  const float dot_ll = ql[0] * ql[0] + ql[1] * ql[1] + ql[2] * ql[2] + ql[3] * ql[3];
  float sb = 0.f, sl = 0.f;
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    sb = fmaf(tb[i], m[i], sb);
    sl = fmaf(tl[i], m[i], sl);
  }
  st.rest = 4.f * (lam0 * dot_hl - sb) + 2.f * (lam0 * dot_ll - sl);
  float qq = 0.f;
#pragma unroll
  for (int i = 0; i < 4; ++i) qq = fmaf(qn[i], qn[i], qq);
  st.qq = qq;
}

#if defined(__CUDACC__)
// fast_begin for two pairs at once: the FP32 parts (QCP, eigenvector, the
// small bilinear terms) on the packed FP32x2 pipe, the integer parts per
// pair.  The same steps and margins as fast_begin.
__device__ __forceinline__ void fast_begin2(const F2 m[9], F2 gsum, FastState &s0, FastState &s1) {
  FastState *st[2] = {&s0, &s1};
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    FastState &t = *st[c];
    t.U0 = t.U1 = t.U2 = 0;
    t.U3 = 0.f;
    t.flag = 0;
    t.rest = 0.f;
    t.qq = 1.f;
    t.q2 = 0;
#pragma unroll
    for (int i = 0; i < 9; ++i) t.T[i] = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) t.qh[i] = 0.f;
  }
  const F2 lam0 = gsum * f2(1.862645149230957e-9f);
  const F2 inv = div2(f2(1.0f), lam0);
  F2 sn[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) sn[i] = m[i] * inv;
  const F2 sxx = sn[0], sxy = sn[1], sxz = sn[2], syx = sn[3], syy = sn[4], syz = sn[5], szx = sn[6], szy = sn[7],
           szz = sn[8];
  const F2 k00 = sxx + syy + szz, k01 = syz - szy, k02 = szx - sxz, k03 = sxy - syx;
  const F2 k11 = sxx - syy - szz, k12 = sxy + syx, k13 = szx + sxz;
  const F2 k22 = syy - sxx - szz, k23 = syz + szy, k33 = szz - sxx - syy;
  F2 fro2 = f2(0.f);
#pragma unroll
  for (int i = 0; i < 9; ++i) fro2 = fma2(sn[i], sn[i], fro2);
  const F2 c2 = f2(-2.f) * fro2;
  const F2 c1 = f2(-8.f) * (sxx * (syy * szz - syz * szy) - sxy * (syx * szz - syz * szx) + sxz * (syx * szy - syy * szx));
  const F2 s01 = k00 * k11 - k01 * k01, s02 = k00 * k12 - k02 * k01, s03 = k00 * k13 - k03 * k01;
  const F2 s12 = k01 * k12 - k02 * k11, s13 = k01 * k13 - k03 * k11, s23 = k02 * k13 - k03 * k12;
  const F2 t23 = k22 * k33 - k23 * k23, t13 = k12 * k33 - k23 * k13, t12 = k12 * k23 - k22 * k13;
  const F2 t03 = k02 * k33 - k23 * k03, t02 = k02 * k23 - k22 * k03, t01 = k02 * k13 - k12 * k03;
  const F2 c0 = s01 * t23 - s02 * t13 + s03 * t12 + s12 * t03 - s13 * t02 + s23 * t01;
  // Halley from x = 1, five steps (qcp_top_eig)
  F2 x = f2(1.0f);
#pragma unroll
  for (int it = 0; it < 5; ++it) {
    const F2 x2 = x * x;
    const F2 p = fma2(fma2(x2 + c2, x, c1), x, c0);
    const F2 dp = fma2(fma2(f2(4.f), x2, f2(2.f) * c2), x, c1);
    const F2 ddp = fma2(f2(12.f), x2, f2(2.f) * c2);
    const F2 den = fma2(f2(2.f) * dp, dp, f2(0.f) - p * ddp);
    const F2 nx = x - div2(f2(2.f) * p * dp, den);
    x = f2(den.v.x > 0.f ? nx.v.x : x.v.x, den.v.y > 0.f ? nx.v.y : x.v.y);
  }
  const F2 b00 = k00 - x, b11 = k11 - x, b22 = k22 - x, b33 = k33 - x;
  const F2 C0 = b11 * (b22 * b33 - k23 * k23) - k12 * (k12 * b33 - k23 * k13) + k13 * (k12 * k23 - b22 * k13);
  const F2 C1 = b00 * (b22 * b33 - k23 * k23) - k02 * (k02 * b33 - k23 * k03) + k03 * (k02 * k23 - b22 * k03);
  const F2 C2 = b00 * (b11 * b33 - k13 * k13) - k01 * (k01 * b33 - k13 * k03) + k03 * (k01 * k13 - b11 * k03);
  const F2 C3 = b00 * (b11 * b22 - k12 * k12) - k01 * (k01 * b22 - k12 * k02) + k02 * (k01 * k12 - b11 * k02);
  const F2 r0[4] = {b00, k01, k02, k03}, r1[4] = {k01, b11, k12, k13};
  const F2 r2[4] = {k02, k12, b22, k23}, r3[4] = {k03, k13, k23, b33};
  // per pair: the diagonal cofactor of largest magnitude picks the three rows
  float best[2];
  F2 sa[4], sb[4], sc[4];
  {
    int jj[2];
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const float a0 = fabsf(c ? C0.v.y : C0.v.x), a1 = fabsf(c ? C1.v.y : C1.v.x);
      const float a2 = fabsf(c ? C2.v.y : C2.v.x), a3 = fabsf(c ? C3.v.y : C3.v.x);
      int j = 0;
      float b = a0;
      if (a1 > b) { b = a1; j = 1; }
      if (a2 > b) { b = a2; j = 2; }
      if (a3 > b) { b = a3; j = 3; }
      best[c] = b;
      jj[c] = j;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const F2 A = r0[i], B = r1[i], Cc = r2[i], D = r3[i];
      sa[i] = f2(jj[0] == 0 ? B.v.x : A.v.x, jj[1] == 0 ? B.v.y : A.v.y);
      sb[i] = f2(jj[0] <= 1 ? Cc.v.x : B.v.x, jj[1] <= 1 ? Cc.v.y : B.v.y);
      sc[i] = f2(jj[0] <= 2 ? D.v.x : Cc.v.x, jj[1] <= 2 ? D.v.y : Cc.v.y);
    }
  }
  // q = generalised cross product of the three rows (gcross4)
  F2 q[4];
  {
    const F2 m01 = sb[0] * sc[1] - sb[1] * sc[0], m02 = sb[0] * sc[2] - sb[2] * sc[0];
    const F2 m03 = sb[0] * sc[3] - sb[3] * sc[0], m12 = sb[1] * sc[2] - sb[2] * sc[1];
    const F2 m13 = sb[1] * sc[3] - sb[3] * sc[1], m23 = sb[2] * sc[3] - sb[3] * sc[2];
    q[0] = sa[1] * m23 - sa[2] * m13 + sa[3] * m12;
    q[1] = f2(0.f) - (sa[0] * m23 - sa[2] * m03 + sa[3] * m02);
    q[2] = sa[0] * m13 - sa[1] * m03 + sa[3] * m01;
    q[3] = f2(0.f) - (sa[0] * m12 - sa[1] * m02 + sa[2] * m01);
  }
  const F2 qsq = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
  const float gs[2] = {gsum.v.x, gsum.v.y}, qs2[2] = {qsq.v.x, qsq.v.y};
  bool live[2];
  float qsc[2];
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    live[c] = gs[c] > 0.f;
    if (live[c] && (!(qs2[c] > 1e-30f) || !(best[c] > 1e-6f))) {
      st[c]->flag = 1;
      live[c] = false;
    }
    qsc[c] = rsqrtf(qs2[c]) * 0.99999f;  // unit length (a hair below, so |Q_h|^2 <= 2^34)
  }
  const F2 qs = f2(qsc[0], qsc[1]);
  F2 qn[4], qh[4], ql[4];
  long long Q[2][4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    qn[i] = q[i] * qs;
    const F2 hs = qn[i] * f2(131072.f);
    const float h0 = rintf(hs.v.x), h1 = rintf(hs.v.y);
    Q[0][i] = (long long)(int)h0;
    Q[1][i] = (long long)(int)h1;
    qh[i] = f2(h0, h1) * f2(7.62939453125e-6f);  // 2^-17
    ql[i] = qn[i] - qh[i];
  }
  // T(q_h, q_l) and T(q_l) (t_bilinear, t_of_q), packed
  F2 tb[9], tl[9];
  {
    const F2 w = qh[0], xx_ = qh[1], y = qh[2], z = qh[3];
    const F2 W = ql[0], X = ql[1], Y = ql[2], Z = ql[3];
    const F2 ww = w * W, xx = xx_ * X, yy = y * Y, zz = z * Z;
    const F2 xy = fma2(xx_, Y, y * X), wz = fma2(w, Z, z * W), xz = fma2(xx_, Z, z * X);
    const F2 wy = fma2(w, Y, y * W), yz = fma2(y, Z, z * Y), wx = fma2(w, X, xx_ * W);
    tb[0] = ww + xx - yy - zz;
    tb[1] = xy + wz;
    tb[2] = xz - wy;
    tb[3] = xy - wz;
    tb[4] = ww - xx + yy - zz;
    tb[5] = yz + wx;
    tb[6] = xz + wy;
    tb[7] = yz - wx;
    tb[8] = ww - xx - yy + zz;
    const F2 lww = W * W, lxx = X * X, lyy = Y * Y, lzz = Z * Z;
    const F2 lwx = W * X, lwy = W * Y, lwz = W * Z, lxy = X * Y, lxz = X * Z, lyz = Y * Z;
    const F2 two = f2(2.f);
    tl[0] = lww + lxx - lyy - lzz;
    tl[1] = two * (lxy + lwz);
    tl[2] = two * (lxz - lwy);
    tl[3] = two * (lxy - lwz);
    tl[4] = lww - lxx + lyy - lzz;
    tl[5] = two * (lyz + lwx);
    tl[6] = two * (lxz + lwy);
    tl[7] = two * (lyz - lwx);
    tl[8] = lww - lxx - lyy + lzz;
  }
  const F2 dot_hl = qh[0] * ql[0] + qh[1] * ql[1] + qh[2] * ql[2] + qh[3] * ql[3];
  const F2 dot_ll = ql[0] * ql[0] + ql[1] * ql[1] + ql[2] * ql[2] + ql[3] * ql[3];
  F2 sbv = f2(0.f), slv = f2(0.f);
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    sbv = fma2(tb[i], m[i], sbv);
    slv = fma2(tl[i], m[i], slv);
  }
  const F2 rest = f2(4.f) * (lam0 * dot_hl - sbv) + f2(2.f) * (lam0 * dot_ll - slv);
  F2 qq = f2(0.f);
#pragma unroll
  for (int i = 0; i < 4; ++i) qq = fma2(qn[i], qn[i], qq);
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    if (!live[c]) continue;
    FastState &t = *st[c];
    t_of_q<long long>(Q[c], t.T);
    t.q2 = Q[c][0] * Q[c][0] + Q[c][1] * Q[c][1] + Q[c][2] * Q[c][2] + Q[c][3] * Q[c][3];
#pragma unroll
    for (int i = 0; i < 4; ++i) t.qh[i] = c ? qh[i].v.y : qh[i].v.x;
    t.rest = c ? rest.v.y : rest.v.x;
    t.qq = c ? qq.v.y : qq.v.x;
  }
}
#endif

BS_HD void fast_level(FastState &st, int level, const float s[9]) {
  if (level < 3) {
    long long u = 0;
#pragma unroll
    for (int i = 0; i < 9; ++i) u += st.T[i] * (long long)(int)s[i];
    if (level == 0) st.U0 += u;
    else if (level == 1) st.U1 += u;
    else st.U2 += u;
  } else {
    // level 3 weighs 2^-27 of level 0: T(q_h) in FP32 is accurate enough
    float t[9];
    t_of_q<float>(st.qh, t);
    float u = 0.f;
#pragma unroll
    for (int i = 0; i < 9; ++i) u = fmaf(t[i], s[i], u);
    st.U3 += u * 17179869184.0f;  // T(Q_h) = 2^34 T(q_h)
  }
}

// The same from staged values: levels 0-2 arrive as int32 bit patterns (the
// exact integer sums, possibly of two atom ranges), level 3 as a float.
BS_HD void fast_level_staged(FastState &st, int level, const float s[9]) {
  if (level < 3) {
    long long u = 0;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
      int v;
      memcpy(&v, &s[i], 4);
      u += st.T[i] * (long long)v;
    }
    if (level == 0) st.U0 += u;
    else if (level == 1) st.U1 += u;
    else st.U2 += u;
  } else {
    fast_level(st, 3, s);
  }
}

// gsum: exact Ga + Gb (units u); gsum_f: the same as float; qsum: the two
// structures' quantisation residual RMS (Angstrom) -- by Minkowski, the
// crmsd of the quantised pair is within qsum of the exact one; d34: bound on
// the level-3 accumulator's rounding, as an error of E (units u); u:
// Angstrom^2 per unit; tol: certified |dRMSD| budget per pair.
BS_HD float fast_finish(const FastState &st, long long gsum, float gsum_f, float qsum, float d34, float u, int L,
                        float tol, int &flag) {
  flag = st.flag;
  if (gsum <= 0 || st.flag) return 0.f;
  // 2 F(q_h) 2^34 in units u = gsum |Q_h|^2 - 2 (2^28 U0 + 2^19 U1 + 2^10 U2 + 2 U3)
  __int128 c = (__int128)gsum * (__int128)st.q2;
  c -= ((__int128)st.U0 << 29) + ((__int128)st.U1 << 20) + ((__int128)st.U2 << 11);
  const float twoFh = (i128_to_f32(c) - 4.f * st.U3) * 5.820766091346741e-11f;  // 2^-34 -> u
  const float twoF = twoFh + st.rest * 268435456.0f;                              // 2^28 -> u
  const float e_u = BS_FDIV(twoF, st.qq);
  const float e_a2 = fmaxf(e_u, 0.f) * u;
  const float rmsd = sqrtf(BS_FDIV(e_a2, (float)L));
  // error bound on E: level-3 accumulator rounding plus the FP32 arithmetic
  // of the fast path: the rounding of m and of the bilinear sum against
  // |q_l| <= 2^-18 stays below 2^-34.8 (Ga+Gb); bounded by 2^-34
  const float darith = gsum_f * 5.820766091346741e-11f;  // 2^-34 (Ga+Gb)
  const float de_a2 = (d34 + darith) * u;
  const float elo = fmaxf(e_a2 - de_a2, 0.f);
  // the fast path gets what quantisation leaves of the budget (at least 1e-5)
  const float tf = fmaxf(tol - qsum, 1e-5f);
  // |dRMSD| <= dE / (sqrt(L) sqrt(E_lo)): recompute when dE^2 > tf^2 L E_lo
  if (de_a2 * de_a2 > tf * tf * (float)L * elo) flag = 1;
  return rmsd;
}

// All three phases for one pair whose level sums are at hand.
struct EpilogueIn {
  float s0[9], s1[9], s2[9], s3[9];  // s3 holds S3 + S4/512
  long long ga, gb;                  // exact Ghat
  float gfa, gfb;                    // Ghat as float
  float qa, qb;                      // quantisation residual RMS (Angstrom)
};

BS_HD float pair_rmsd_fast(const EpilogueIn &in, float u, float d34, int L, float tol, int &flag) {
  const float gsum_f = in.gfa + in.gfb;
  float m[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) m[i] = m_from_levels(in.s0[i], in.s1[i], in.s2[i], in.s3[i]);
  FastState st;
  fast_begin(m, gsum_f, st);
  fast_level(st, 0, in.s0);
  fast_level(st, 1, in.s1);
  fast_level(st, 2, in.s2);
  fast_level(st, 3, in.s3);
  return fast_finish(st, in.ga + in.gb, gsum_f, in.qa + in.qb, d34, u, L, tol, flag);
}

// Bits of the double nearest to a non-negative float, built with integer
// operations (the float -> double conversion runs on the slow FP64 pipe).
BS_HD unsigned long long f32_to_f64_bits(float f) {
  unsigned b;
  memcpy(&b, &f, 4);
  if ((b & 0x7f800000u) == 0u) return (unsigned long long)(b & 0x80000000u) << 32;  // zero (flushes subnormals)
  return ((unsigned long long)(b & 0x80000000u) << 32) | (((unsigned long long)(b & 0x7fffffffu) << 29) +
                                                         ((unsigned long long)896 << 52));
}

// ------------------------------------------------------------ FP64 QCP
// Largest eigenvalue of K(sn) for sn = S / lambda0 (so the root is <= 1),
// by Newton on the quartic from 1; returns the deficit 1 - x.  Then
// E = (Ga + Gb) (1 - x).
BS_HD double qcp_deficit_f64(const double sn[9]) {
  const double sxx = sn[0], sxy = sn[1], sxz = sn[2], syx = sn[3], syy = sn[4], syz = sn[5], szx = sn[6],
               szy = sn[7], szz = sn[8];
  const double k00 = sxx + syy + szz, k01 = syz - szy, k02 = szx - sxz, k03 = sxy - syx;
  const double k11 = sxx - syy - szz, k12 = sxy + syx, k13 = szx + sxz;
  const double k22 = -sxx + syy - szz, k23 = syz + szy, k33 = -sxx - syy + szz;
  double fro2 = 0.0;
  for (int i = 0; i < 9; ++i) fro2 += sn[i] * sn[i];
  const double c2 = -2.0 * fro2;
  const double det3 = sxx * (syy * szz - syz * szy) - sxy * (syx * szz - syz * szx) + sxz * (syx * szy - syy * szx);
  const double c1 = -8.0 * det3;
  const double s01 = k00 * k11 - k01 * k01, s02 = k00 * k12 - k02 * k01, s03 = k00 * k13 - k03 * k01;
  const double s12 = k01 * k12 - k02 * k11, s13 = k01 * k13 - k03 * k11, s23 = k02 * k13 - k03 * k12;
  const double t23 = k22 * k33 - k23 * k23, t13 = k12 * k33 - k23 * k13, t12 = k12 * k23 - k22 * k13;
  const double t03 = k02 * k33 - k23 * k03, t02 = k02 * k23 - k22 * k03, t01 = k02 * k13 - k12 * k03;
  const double c0 = s01 * t23 - s02 * t13 + s03 * t12 + s12 * t03 - s13 * t02 + s23 * t01;
  // Halley iterations from the upper bound 1 (cubic convergence; the
  // largest root is simple and P is convex above it)
  double x = 1.0;
  for (int it = 0; it < 12; ++it) {
    const double x2 = x * x;
    const double p = ((x2 + c2) * x + c1) * x + c0;
    const double dp = (4.0 * x2 + 2.0 * c2) * x + c1;
    const double ddp = 12.0 * x2 + 2.0 * c2;
    const double den = 2.0 * dp * dp - p * ddp;
    if (!(den > 0.0)) break;
    const double dx = 2.0 * p * dp / den;
    x -= dx;
    if (fabs(dx) <= 1e-17) break;
  }
  return 1.0 - x;
}

// RMSD from an FP64 covariance S (S[3x+y] = sum a_x b_y) and G_a + G_b.
BS_HD double qcp_rmsd_f64(const double s[9], double gsum, int L) {
  if (!(gsum > 0.0)) return 0.0;
  const double inv = 2.0 / gsum;
  double sn[9];
  for (int i = 0; i < 9; ++i) sn[i] = s[i] * inv;
  const double e = gsum * qcp_deficit_f64(sn);
  return e > 0.0 ? sqrt(e / (double)L) : 0.0;
}

// ------------------------------------------------------- exact recompute
// FP64 eigenvector of K(sn) for the eigenvalue x: adjugate column of
// K - xI with the largest diagonal cofactor.  Returns that cofactor's size.
BS_HD double top_vec_f64(const double sn[9], double x, double q[4]) {
  const double sxx = sn[0], sxy = sn[1], sxz = sn[2], syx = sn[3], syy = sn[4], syz = sn[5], szx = sn[6],
               szy = sn[7], szz = sn[8];
  const double k01 = syz - szy, k02 = szx - sxz, k03 = sxy - syx;
  const double k12 = sxy + syx, k13 = szx + sxz, k23 = syz + szy;
  const double b00 = sxx + syy + szz - x, b11 = sxx - syy - szz - x, b22 = -sxx + syy - szz - x,
               b33 = -sxx - syy + szz - x;
  const double C0 = b11 * (b22 * b33 - k23 * k23) - k12 * (k12 * b33 - k23 * k13) + k13 * (k12 * k23 - b22 * k13);
  const double C1 = b00 * (b22 * b33 - k23 * k23) - k02 * (k02 * b33 - k23 * k03) + k03 * (k02 * k23 - b22 * k03);
  const double C2 = b00 * (b11 * b33 - k13 * k13) - k01 * (k01 * b33 - k13 * k03) + k03 * (k01 * k13 - b11 * k03);
  const double C3 = b00 * (b11 * b22 - k12 * k12) - k01 * (k01 * b22 - k12 * k02) + k02 * (k01 * k12 - b11 * k02);
  const double a0 = fabs(C0), a1 = fabs(C1), a2 = fabs(C2), a3 = fabs(C3);
  int j = 0;
  double best = a0;
  if (a1 > best) { best = a1; j = 1; }
  if (a2 > best) { best = a2; j = 2; }
  if (a3 > best) { best = a3; j = 3; }
  const double r0[4] = {b00, k01, k02, k03}, r1[4] = {k01, b11, k12, k13};
  const double r2[4] = {k02, k12, b22, k23}, r3[4] = {k03, k13, k23, b33};
  double A[4], B[4], C[4];
  for (int i = 0; i < 4; ++i) {
    A[i] = (j == 0) ? r1[i] : r0[i];
    B[i] = (j <= 1) ? r2[i] : r1[i];
    C[i] = (j <= 2) ? r3[i] : r2[i];
  }
  const double m01 = B[0] * C[1] - B[1] * C[0], m02 = B[0] * C[2] - B[2] * C[0], m03 = B[0] * C[3] - B[3] * C[0];
  const double m12 = B[1] * C[2] - B[2] * C[1], m13 = B[1] * C[3] - B[3] * C[1], m23 = B[2] * C[3] - B[3] * C[2];
  q[0] = A[1] * m23 - A[2] * m13 + A[3] * m12;
  q[1] = -(A[0] * m23 - A[2] * m03 + A[3] * m02);
  q[2] = A[0] * m13 - A[1] * m03 + A[3] * m01;
  q[3] = -(A[0] * m12 - A[1] * m02 + A[2] * m01);
  return best;
}

// Exact recomputation from the integer covariance Mhat of the quantised
// coordinates (units u = 2^(2e)).  Mhat and Ghat are exact integers below
// 2^53, so they are exact in FP64.  The FP64 QCP root gives the eigenvector
// q, and E is its Rayleigh quotient against the exact matrix:
//   E = 2 (lambda0 |q|^2 - sum_xy T(q)_xy Mhat_xy) / |q|^2,
// whose error is second order in the eigenvector error plus FP64 rounding
// of terms of size lambda0.  A degenerate top eigenvalue falls back to
// E = (Ga + Gb)(1 - x).  Used for the (rare) pairs the fast path flags.
BS_HD double pair_rmsd_exact(const long long mh[9], long long ga, long long gb, int scale_exp, int L) {
  const long long gsum = ga + gb;
  if (gsum <= 0) return 0.0;
  const double g = (double)gsum;
  const double inv = 2.0 / g;
  double sn[9];
  for (int i = 0; i < 9; ++i) sn[i] = (double)mh[i] * inv;
  const double deficit = qcp_deficit_f64(sn);
  double e_u = g * deficit;
  double q[4];
  const double cof = top_vec_f64(sn, 1.0 - deficit, q);
  if (cof > 1e-12) {
    double t[9];
    t_of_q<double>(q, t);
    const double qq = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
    double acc = 0.5 * g * qq;
    for (int i = 0; i < 9; ++i) acc -= t[i] * (double)mh[i];
    e_u = 2.0 * acc / qq;
  }
  const double e_a2 = (e_u > 0.0 ? e_u : 0.0) * ldexp(1.0, 2 * scale_exp);
  return sqrt(e_a2 / (double)L);
}

// ------------------------------------------------------------- digits
// Balanced digits of a quantised coordinate |n| < 2^22:
//   n = d0 2^14 + d1 2^5 + d2,  d2 in [-16, 15], d1 in [-256, 255], |d0| <= 256;
// returned as the stored values e0 = d0, e1 = d1, e2 = 16 d2.
BS_HD void split_digits(int n, int &e0, int &e1, int &e2) {
  const int d2 = ((n + 16) & 31) - 16;
  const int n1 = (n - d2) >> 5;
  e1 = ((n1 + 256) & 511) - 256;
  e0 = (n1 - e1) >> 9;
  e2 = 16 * d2;
}

// The quantised coordinate back from its stored digits.
BS_HD int join_digits(int e0, int e1, int e2) { return e0 * 16384 + e1 * 32 + (e2 >> 4); }

// ------------------------------------------------------- superposition
// The eigenpair of the largest eigenvalue of a symmetric 4x4 matrix k
// (row-major) by the cyclic Jacobi method (Golub & Van Loan, Matrix
// Computations, sec. 8.5): sweeps of plane rotations, each zeroing one
// off-diagonal entry, until the off-diagonal mass is below 1e-30 of the
// whole (at most 24 sweeps).  Unlike an adjugate column it stays well defined
// when the top eigenvalue is (nearly) repeated, where any unit vector of its
// eigenspace is returned.  q is a unit vector.
BS_HD double sym4_top_eig(const double k[16], double q[4]) {
  // (every index below is a compile-time constant once unrolled, so the
  // matrices stay in registers)
  double a[4][4], v[4][4];
  double total = 0.0;
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      a[r][c] = k[4 * r + c];
      v[r][c] = r == c ? 1.0 : 0.0;
      total += a[r][c] * a[r][c];
    }
  for (int sweep = 0; sweep < 24; ++sweep) {
    double off = 0.0;
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = r + 1; c < 4; ++c) off += a[r][c] * a[r][c];
    if (!(off > 1e-30 * total)) break;
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
      for (int r = p + 1; r < 4; ++r) {
        const double apr = a[p][r];
        if (apr == 0.0) continue;
        // rotation J (c at (p,p), (r,r); s at (p,r); -s at (r,p)) with
        // (J^T A J)_pr = 0: t = tan = sgn(th) / (|th| + sqrt(th^2 + 1))
        const double th = (a[r][r] - a[p][p]) / (2.0 * apr);
        const double t = (th >= 0.0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
#pragma unroll
        for (int i = 0; i < 4; ++i) {  // A J
          const double x = a[i][p], y = a[i][r];
          a[i][p] = c * x - s * y;
          a[i][r] = s * x + c * y;
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {  // J^T (A J)
          const double x = a[p][i], y = a[r][i];
          a[p][i] = c * x - s * y;
          a[r][i] = s * x + c * y;
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {  // V J
          const double x = v[i][p], y = v[i][r];
          v[i][p] = c * x - s * y;
          v[i][r] = s * x + c * y;
        }
      }
  }
  double top = a[0][0];
#pragma unroll
  for (int i = 0; i < 4; ++i) q[i] = v[i][0];
#pragma unroll
  for (int c = 1; c < 4; ++c)
    if (a[c][c] > top) {
      top = a[c][c];
#pragma unroll
      for (int i = 0; i < 4; ++i) q[i] = v[i][c];
    }
  const double inv = 1.0 / sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
#pragma unroll
  for (int i = 0; i < 4; ++i) q[i] *= inv;
  return top;
}

// The proper rotation R (row-major) that best superposes b onto a, from the
// covariance of the centred structures m_xy = sum_k (a_k - ca)_x (b_k - cb)_y:
// R maximises sum_xy R_xy m_xy = sum_k (a_k - ca) . R (b_k - cb); it is T(q)
// of the unit top eigenvector q of the QCP key matrix of m.
BS_HD void rotation_from_cov(const double m[9], double rot[9]) {
  const double sxx = m[0], sxy = m[1], sxz = m[2], syx = m[3], syy = m[4], syz = m[5], szx = m[6], szy = m[7],
               szz = m[8];
  const double k[16] = {sxx + syy + szz, syz - szy,       szx - sxz,        sxy - syx,
                        syz - szy,       sxx - syy - szz, sxy + syx,        szx + sxz,
                        szx - sxz,       sxy + syx,       -sxx + syy - szz, syz + szy,
                        sxy - syx,       szx + sxz,       syz + szy,        -sxx - syy + szz};
  double q[4];
  sym4_top_eig(k, q);
  t_of_q<double>(q, rot);
}

}  // namespace bsm
