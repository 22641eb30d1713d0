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

}  // namespace mpm
