// 3x3 SVD and its clamped backward on the device.
//
// Forward: cyclic Jacobi eigen-decomposition of A^T A with symmetric Schur
// rotations (Golub & Van Loan, "Matrix Computations", Sec. 8.5.2), columns
// sorted by eigenvalue, then U from Gram-Schmidt on B = A V.  Output follows
// the convention of ti.svd used by plb/engine/mpm_simulator.py:127-129:
// A = U diag(s) V^T, det U = det V = +1, s0 >= s1 >= |s2|, s2 may be negative.
//
// Backward: backward_svd of plb/engine/mpm_simulator.py:137-156 with the
// +-1e-6 clamp of clamp() (184-192) on s_j^2 - s_i^2.
#pragma once
#include "mpm_math.cuh"

namespace mpm {

template <typename T>
struct SvdIters;
template <>
struct SvdIters<float> {
  static constexpr int max_sweeps = 6;
  static constexpr float tol = 1e-14f;  // on off^2 / diag^2
};
template <>
struct SvdIters<double> {
  static constexpr int max_sweeps = 12;
  static constexpr double tol = 1e-32;
};

// rotation tangent t = sgn(theta) / (|theta| + sqrt(theta^2 + 1)) and cosine c;
// FP32 uses the approximate reciprocal, square root and rsqrt: the error only
// moves the rotation angle, and c and s = t c come from the same rsqrt, so the
// rotation stays orthogonal to rounding
MPM_DI void rot_tc(double theta, double& t, double& c) {
  t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
  c = 1.0 / sqrt(t * t + 1.0);
}
MPM_DI void rot_tc(float theta, float& t, float& c) {
  const float at = fabsf(theta);
  // for huge |theta|, t ~ 1/(2 theta) (avoids theta^2 overflow)
  const float y = fmaf(theta, theta, 1.0f);
  const float den = at < 1e18f ? at + y * rsqrtf(y) : 2.0f * at;
  t = copysignf(__fdividef(1.0f, den), theta);
  c = rsqrtf(fmaf(t, t, 1.0f));
}

// a / b; FP32 by the approximate reciprocal (|b| < 2^126 here).  Used for the
// Jacobi angle, and for the SVD backward's 1 / (s_j^2 - s_i^2), whose divisor
// is clamped to |b| >= 1e-6.  The substep kernels are built with -ftz=true, so
// a subnormal s_pq compares equal to 0 and is never a divisor.
MPM_DI double fast_div(double a, double b) { return a / b; }
MPM_DI float fast_div(float a, float b) { return __fdividef(a, b); }

// one Jacobi rotation zeroing s_pq of the symmetric matrix held as
// (s_pp, s_qq, s_pq, s_rp, s_rq); V columns p, q rotated alongside
template <typename T>
MPM_DI void jacobi_rot(T& app, T& aqq, T& apq, T& arp, T& arq, T* V, int p, int q) {
  if (apq == T(0)) return;
  T theta = fast_div(aqq - app, T(2) * apq);
  T t, c;
  rot_tc(theta, t, c);
  T s = t * c;
  app = app - t * apq;
  aqq = aqq + t * apq;
  apq = T(0);
  T rp = c * arp - s * arq;
  T rq = s * arp + c * arq;
  arp = rp;
  arq = rq;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    T vp = V[k * 3 + p], vq = V[k * 3 + q];
    V[k * 3 + p] = c * vp - s * vq;
    V[k * 3 + q] = s * vp + c * vq;
  }
}

template <typename T>
MPM_DI void swap_cols(T* V, T* ev, int a, int b) {
  T t = ev[a];
  ev[a] = ev[b];
  ev[b] = t;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    T x = V[k * 3 + a];
    V[k * 3 + a] = V[k * 3 + b];
    V[k * 3 + b] = x;
  }
}

template <typename T>
MPM_DI void svd3(const T* A, T* U, T* s, T* V) {
  T S[9];
  mTm(A, A, S);
  T a00 = S[0], a11 = S[4], a22 = S[8], a01 = S[1], a02 = S[2], a12 = S[5];
#pragma unroll
  for (int k = 0; k < 9; ++k) V[k] = (k % 4 == 0) ? T(1) : T(0);
  for (int sweep = 0; sweep < SvdIters<T>::max_sweeps; ++sweep) {
    T off = a01 * a01 + a02 * a02 + a12 * a12;
    T dg = a00 * a00 + a11 * a11 + a22 * a22;
    if (off <= SvdIters<T>::tol * dg) break;
    jacobi_rot(a00, a11, a01, a02, a12, V, 0, 1);  // r = 2: (s_20, s_21)
    jacobi_rot(a00, a22, a02, a01, a12, V, 0, 2);  // r = 1: (s_10, s_12)
    jacobi_rot(a11, a22, a12, a01, a02, V, 1, 2);  // r = 0: (s_01, s_02)
  }
  // descending eigenvalues; each swap flips det V
  T ev[3] = {a00, a11, a22};
  bool flip = false;
  if (ev[0] < ev[1]) { swap_cols(V, ev, 0, 1); flip = !flip; }
  if (ev[0] < ev[2]) { swap_cols(V, ev, 0, 2); flip = !flip; }
  if (ev[1] < ev[2]) { swap_cols(V, ev, 1, 2); flip = !flip; }
  if (flip) {
#pragma unroll
    for (int k = 0; k < 3; ++k) V[k * 3 + 2] = -V[k * 3 + 2];
  }
  T B[9];
  mm(A, V, B);
  T b0[3] = {B[0], B[3], B[6]}, b1[3] = {B[1], B[4], B[7]}, b2[3] = {B[2], B[5], B[8]};
  T u0[3], u1[3], u2[3];
  // column norms from one reciprocal square root each: |b| = b.b / sqrt(b.b)
  T d0 = dot3(b0, b0);
  T n0 = T(0);
  if (d0 > T(0)) {
    T inv = inv_len(d0);
    n0 = d0 * inv;
#pragma unroll
    for (int k = 0; k < 3; ++k) u0[k] = b0[k] * inv;
  } else {
    u0[0] = T(1); u0[1] = T(0); u0[2] = T(0);
  }
  T pr = dot3(u0, b1);
  T r1[3] = {b1[0] - pr * u0[0], b1[1] - pr * u0[1], b1[2] - pr * u0[2]};
  T d1 = dot3(r1, r1);
  if (d1 > T(0)) {
    T inv = inv_len(d1);
#pragma unroll
    for (int k = 0; k < 3; ++k) u1[k] = r1[k] * inv;
  } else {
    // any unit vector orthogonal to u0 (A of rank <= 1)
    int m = (mabs(u0[0]) < mabs(u0[1])) ? 0 : 1;
    if (mabs(u0[2]) < mabs(u0[m])) m = 2;
    T e[3] = {T(0), T(0), T(0)};
    e[m] = T(1);
    T pe = dot3(u0, e);
#pragma unroll
    for (int k = 0; k < 3; ++k) r1[k] = e[k] - pe * u0[k];
    T inv = T(1) / msqrt(dot3(r1, r1));
#pragma unroll
    for (int k = 0; k < 3; ++k) u1[k] = r1[k] * inv;
  }
  cross3(u0, u1, u2);
  s[0] = n0;
  s[1] = dot3(u1, b1);
  s[2] = dot3(u2, b2);
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    U[r * 3 + 0] = u0[r];
    U[r * 3 + 1] = u1[r];
    U[r * 3 + 2] = u2[r];
  }
}

// FP32 SVD of A = I + D given the displacement D = A - I (not A itself), so
// that the strain information (of size |D|, typically 1e-4 .. 1e-2) keeps
// FP32's relative precision instead of the absolute precision of numbers
// near 1.  The same cyclic Jacobi rotations as svd3 act on the shifted
// symmetric matrix M = A^T A - I = D + D^T + D^T D (same eigenvectors V,
// eigenvalues s^2 - 1), converged relative to M itself.  Returns U, V, s and
// sm1 = s - 1 (from (s^2 - 1) / (1 + s), exact as s -> 1).  Same conventions
// as svd3: det U = det V = +1, s0 >= s1 >= |s2|, s2 may be negative.
// convergence of the shifted sweeps: off-diagonal^2 <= kShiftedTol * diagonal^2 of M
constexpr float kShiftedTol = 1e-14f;
MPM_DI void svd3_shifted(const float* D, float* U, float* s, float* sm1, float* V) {
  float M[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      M[i * 3 + j] = D[i * 3 + j] + D[j * 3 + i] + (D[i] * D[j] + D[3 + i] * D[3 + j] + D[6 + i] * D[6 + j]);
  float a00 = M[0], a11 = M[4], a22 = M[8], a01 = M[1], a02 = M[2], a12 = M[5];
#pragma unroll
  for (int k = 0; k < 9; ++k) V[k] = (k % 4 == 0) ? 1.f : 0.f;
  for (int sweep = 0; sweep < SvdIters<float>::max_sweeps; ++sweep) {
    const float off = a01 * a01 + a02 * a02 + a12 * a12;
    const float dg = a00 * a00 + a11 * a11 + a22 * a22;
    // relative to M; the absolute floor stops sweeps on rounding noise (rigid rotations, M ~ 0)
    if (off <= kShiftedTol * dg + 1e-30f) break;
    jacobi_rot(a00, a11, a01, a02, a12, V, 0, 1);
    jacobi_rot(a00, a22, a02, a01, a12, V, 0, 2);
    jacobi_rot(a11, a22, a12, a01, a02, V, 1, 2);
  }
  float ev[3] = {a00, a11, a22};
  bool flip = false;
  if (ev[0] < ev[1]) { swap_cols(V, ev, 0, 1); flip = !flip; }
  if (ev[0] < ev[2]) { swap_cols(V, ev, 0, 2); flip = !flip; }
  if (ev[1] < ev[2]) { swap_cols(V, ev, 1, 2); flip = !flip; }
  if (flip) {
#pragma unroll
    for (int k = 0; k < 3; ++k) V[k * 3 + 2] = -V[k * 3 + 2];
  }
  // B = A V = V + D V, U by Gram-Schmidt as in svd3
  float B[9];
  mm(D, V, B);
#pragma unroll
  for (int k = 0; k < 9; ++k) B[k] += V[k];
  float b0[3] = {B[0], B[3], B[6]}, b1[3] = {B[1], B[4], B[7]}, b2[3] = {B[2], B[5], B[8]};
  float u0[3], u1[3], u2[3];
  const float d0 = dot3(b0, b0);
  if (d0 > 0.f) {
    const float inv = inv_len(d0);
#pragma unroll
    for (int k = 0; k < 3; ++k) u0[k] = b0[k] * inv;
  } else {
    u0[0] = 1.f; u0[1] = 0.f; u0[2] = 0.f;
  }
  const float pr = dot3(u0, b1);
  float r1[3] = {b1[0] - pr * u0[0], b1[1] - pr * u0[1], b1[2] - pr * u0[2]};
  const float d1 = dot3(r1, r1);
  if (d1 > 0.f) {
    const float inv = inv_len(d1);
#pragma unroll
    for (int k = 0; k < 3; ++k) u1[k] = r1[k] * inv;
  } else {
    int m = (fabsf(u0[0]) < fabsf(u0[1])) ? 0 : 1;
    if (fabsf(u0[2]) < fabsf(u0[m])) m = 2;
    float e[3] = {0.f, 0.f, 0.f};
    e[m] = 1.f;
    const float pe = dot3(u0, e);
#pragma unroll
    for (int k = 0; k < 3; ++k) r1[k] = e[k] - pe * u0[k];
    const float inv = 1.f / sqrtf(dot3(r1, r1));
#pragma unroll
    for (int k = 0; k < 3; ++k) u1[k] = r1[k] * inv;
  }
  cross3(u0, u1, u2);
  // s_i - 1 = (s_i^2 - 1) / (1 + s_i), s_i^2 - 1 the eigenvalue of M; the sign
  // of s2 (an inverted element) from u2 . b2 as in svd3
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float q = fmaxf(1.f + ev[i], 0.f);
    const float r = sqrtf(q);
    sm1[i] = ev[i] / (1.f + r);
    s[i] = r;
  }
  if (dot3(u2, b2) < 0.f) {
    s[2] = -s[2];
    sm1[2] = s[2] - 1.f;
  }
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    U[r * 3 + 0] = u0[r];
    U[r * 3 + 1] = u1[r];
    U[r * 3 + 2] = u2[r];
  }
}

template <typename T>
MPM_DI T svd_clamp(T a) {
  return a >= T(0) ? (a > T(1e-6) ? a : T(1e-6)) : (a < T(-1e-6) ? a : T(-1e-6));
}

// gA = U [ (F o (U^T gU - gU^T U)) S + S (F o (V^T gV - gV^T V)) + diag(gs) ] V^T
template <typename T>
MPM_DI void svd3_bwd(const T* U, const T* s, const T* V, const T* gU, const T* gs, const T* gV, T* gA) {
  T ss[3] = {s[0] * s[0], s[1] * s[1], s[2] * s[2]};
  T UtgU[9], VtgV[9];
  mTm(U, gU, UtgU);
  mTm(V, gV, VtgV);
  T X[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      if (i == j) {
        X[i * 3 + j] = gs[i];
      } else {
        T Fij = fast_div(T(1), svd_clamp(ss[j] - ss[i]));
        T au = UtgU[i * 3 + j] - UtgU[j * 3 + i];  // (U^T gU - gU^T U)_ij
        T av = VtgV[i * 3 + j] - VtgV[j * 3 + i];
        X[i * 3 + j] = Fij * (au * s[j] + s[i] * av);
      }
    }
  T T1[9];
  mm(U, X, T1);
  mmT(T1, V, gA);
}

// Divided difference D = (e_j - e_i) / (s_j - s_i) of the return map's new
// singular values e = exp((1 - k) log s + k mean(log s)) (mpm_simulator.py:
// 172-180; k = delta_gamma / |eps_hat|, a = 1 - k), exact as s_j -> s_i:
//   e_j / e_i = (s_j / s_i)^a, so D = e_i a / s_i * E1(a L) * L / u
// with u = (s_j - s_i) / s_i, L = log1p(u) and E1(z) = expm1(z) / z.  For
// |u| < 1/64 both factors come from their Taylor series (L / u = 1 - u/2 +
// u^2/3 - u^3/4 + u^4/5, E1 = 1 + z/2 + z^2/6 + z^3/24 + z^4/120; truncation
// below 3e-11 and 2e-11); otherwise |s_j - s_i| is well above the rounding
// of s and the plain quotient is exact enough, as it is when a singular value
// sits at the return map's 0.05 floor.  ds = s_j - s_i and e_j - e_i are
// formed from s - 1 and e - 1.
MPM_DI float ret_map_dd(float si, float sj, float ds, float ei, float em1i, float em1j, float a) {
  if (si > 0.05f && sj > 0.05f) {
    const float u = ds / si;
    if (fabsf(u) < 0.015625f) {
      const float lg = fmaf(u, fmaf(u, fmaf(u, fmaf(u, 0.2f, -0.25f), 1.f / 3.f), -0.5f), 1.f);
      const float z = a * u * lg;
      const float e1 = fmaf(z, fmaf(z, fmaf(z, fmaf(z, 1.f / 120.f, 1.f / 24.f), 1.f / 6.f), 0.5f), 1.f);
      return ei * a / si * e1 * lg;
    }
  }
  return ds != 0.f ? (em1j - em1i) / ds : 0.f;
}

// backward_svd (mpm_simulator.py:137-156, clamp 184-192) of the two functions
// p2g takes of the trial F's SVD, in a form without cancellation (FP32):
// the rotation R = U V^T (gradient gR) and, when the return map yields,
// newF = U diag(e) V^T (gradient gN).  Then gU = gR V + gN V diag(e),
// gV = gR^T U + gN^T U diag(e), and with M_R = U^T gR V, M_N = U^T gN V the
// reference's off-diagonal term
//   X_ij = (au_ij s_j + s_i av_ij) / clamp(s_j^2 - s_i^2)
// (au = U^T gU - gU^T U, av = V^T gV - gV^T V) is, identically,
//   X_ij = K_ij (s_j - s_i) / clamp((s_j - s_i)(s_j + s_i)),
//   K_ij = (M_R,ij - M_R,ji) + 1/2 [M_N,ij (D S + E) + M_N,ji (D S - E)]
// with S = s_i + s_j, E = e_i + e_j and D the divided difference of e
// (ret_map_dd); s_j - s_i is taken from sm1 = s - 1.  The reference's numerator is a difference of terms of size
// |g| that leaves a value of size |g| (s_j - s_i), so in FP32 its rounding
// error is amplified by 1 / (s_j^2 - s_i^2), up to 1e6 at the clamp, whenever
// two singular values nearly coincide (near-isotropic deformation); K has no
// such cancellation.  The diagonal X_ii = gs_i (sigma_term) is unchanged.
// Returns X, the gradient of the SVD's input in the bases U, V (gA =
// U X V^T).  M_N, e and e - 1 (em1) are read only when `yield`.
MPM_DI void svd3_bwd_factored_basis(const float* s, const float* sm1, const float* MR, const float* MN,
                                    const float* e, const float* em1, float a, bool yield, const float* gs, float* X) {
#pragma unroll
  for (int i = 0; i < 3; ++i) X[i * 4] = gs[i];
  // each unordered pair (i, j) once: D and the clamped factor are symmetric in i, j
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const int i = q == 2 ? 1 : 0, j = q == 0 ? 1 : 2;
    const float ds = sm1[j] - sm1[i], sm = s[j] + s[i];  // s_j - s_i from s - 1: exact as s_j -> s_i
    const float f = fast_div(ds, svd_clamp(ds * sm));    // ds / clamp(s_j^2 - s_i^2); swapping i, j keeps it
    float Kij = MR[i * 3 + j] - MR[j * 3 + i];
    float Kji = -Kij;
    if (yield) {
      const float D = ret_map_dd(s[i], s[j], ds, e[i], em1[i], em1[j], a);
      const float se = e[i] + e[j];
      const float p = 0.5f * (D * sm + se), m = 0.5f * (D * sm - se);
      Kij += MN[i * 3 + j] * p + MN[j * 3 + i] * m;
      Kji += MN[j * 3 + i] * p + MN[i * 3 + j] * m;
    }
    X[i * 3 + j] = Kij * f;
    X[j * 3 + i] = Kji * f;
  }
}

}  // namespace mpm
