// Device math for the MPM substep: small vectors, 3x3 matrices, quaternions
// and their vector-Jacobian products, templated on the scalar type.
//
// Quaternion conventions follow plb/engine/primitive/utils.py:9-54
// (w, x, y, z); autodiff conventions follow the reference's taichi source
// transform: branch decisions frozen, max(a,b) sends the gradient to a iff
// b < a, min(a,b) to a iff a < b, abs' = sgn with sgn(0) = 0.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#define MPM_DI __device__ __forceinline__
#define MPM_HD __host__ __device__

namespace mpm {

MPM_DI float msqrt(float x) { return sqrtf(x); }
MPM_DI double msqrt(double x) { return sqrt(x); }
// exp and log of the return map (log of singular values near 1, exp of the
// projected strains): the accurate library functions.  __logf's error near 1
// is absolute (about 2^-21), i.e. hundreds of ulp of a strain of 1e-3.
MPM_DI float mexp(float x) { return expf(x); }
MPM_DI double mexp(double x) { return exp(x); }
MPM_DI float mlog(float x) { return logf(x); }
MPM_DI double mlog(double x) { return log(x); }
// log(1 + x) and exp(x) - 1 for the FP32 strains (x = s - 1 of a singular
// value, or a projected log-strain), accurate to the result's own precision:
// for |x| < 1/64 by their Taylor series (truncation below 3e-12 and 2e-13
// relative), otherwise by the library's log1pf / expm1f.
MPM_DI float log1p_strain(float x) {
  if (fabsf(x) < 0.015625f)
    return x * fmaf(x, fmaf(x, fmaf(x, fmaf(x, fmaf(x, -1.f / 6.f, 0.2f), -0.25f), 1.f / 3.f), -0.5f), 1.f);
  return log1pf(x);
}
MPM_DI float expm1_strain(float x) {
  if (fabsf(x) < 0.015625f)
    return x * fmaf(x, fmaf(x, fmaf(x, fmaf(x, fmaf(x, 1.f / 720.f, 1.f / 120.f), 1.f / 24.f), 1.f / 6.f), 0.5f), 1.f);
  return expm1f(x);
}
// exp of the contact softness exp(-dist * softness) (primive_base.py:99), FP32
// by the hardware approximation: its relative error (a few ulp over the
// influence range exp(x) > 0.1) stays below the substep's rounding noise
MPM_DI float mexp_fast(float x) { return __expf(x); }
MPM_DI double mexp_fast(double x) { return exp(x); }
MPM_DI float msin(float x) { return sinf(x); }
MPM_DI double msin(double x) { return sin(x); }
MPM_DI float mcos(float x) { return cosf(x); }
MPM_DI double mcos(double x) { return cos(x); }
MPM_DI float mabs(float x) { return fabsf(x); }
MPM_DI double mabs(double x) { return fabs(x); }
template <typename T>
MPM_DI T sgn(T x) {
  return x > T(0) ? T(1) : (x < T(0) ? T(-1) : T(0));
}
template <typename T>
MPM_DI bool finite(T x) {
  return isfinite(x);
}

template <typename T>
MPM_DI T dot3(const T* a, const T* b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
template <typename T>
MPM_DI void cross3(const T* a, const T* b, T* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
template <typename T>
MPM_DI void add_cross3(const T* a, const T* b, T* c) {
  c[0] += a[1] * b[2] - a[2] * b[1];
  c[1] += a[2] * b[0] - a[0] * b[2];
  c[2] += a[0] * b[1] - a[1] * b[0];
}
// C = A B
template <typename T>
MPM_DI void mm(const T* A, const T* B, T* C) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) C[i * 3 + j] = A[i * 3] * B[j] + A[i * 3 + 1] * B[3 + j] + A[i * 3 + 2] * B[6 + j];
}
// C = A B^T
template <typename T>
MPM_DI void mmT(const T* A, const T* B, T* C) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      C[i * 3 + j] = A[i * 3] * B[j * 3] + A[i * 3 + 1] * B[j * 3 + 1] + A[i * 3 + 2] * B[j * 3 + 2];
}
// C = A^T B
template <typename T>
MPM_DI void mTm(const T* A, const T* B, T* C) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) C[i * 3 + j] = A[i] * B[j] + A[3 + i] * B[3 + j] + A[6 + i] * B[6 + j];
}
template <typename T>
MPM_DI T det3(const T* A) {
  return A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
         A[2] * (A[3] * A[7] - A[4] * A[6]);
}
// cofactor matrix = d det / d A
template <typename T>
MPM_DI void cof3(const T* A, T* Cf) {
  Cf[0] = A[4] * A[8] - A[5] * A[7];
  Cf[1] = A[5] * A[6] - A[3] * A[8];
  Cf[2] = A[3] * A[7] - A[4] * A[6];
  Cf[3] = A[2] * A[7] - A[1] * A[8];
  Cf[4] = A[0] * A[8] - A[2] * A[6];
  Cf[5] = A[1] * A[6] - A[0] * A[7];
  Cf[6] = A[1] * A[5] - A[2] * A[4];
  Cf[7] = A[2] * A[3] - A[0] * A[5];
  Cf[8] = A[0] * A[4] - A[1] * A[3];
}

// length() with the eps of plb/engine/primitive/primitives.py:13-15
template <typename T>
MPM_DI T len14(const T* a) {
  return msqrt(dot3(a, a) + T(1e-14));
}
// length() with the eps of plb/engine/primitive/utils.py:4-6
template <typename T>
MPM_DI T len8(const T* a) {
  return msqrt(dot3(a, a) + T(1e-8));
}
// d(u/len14(u))^T g
template <typename T>
MPM_DI void unit14_vjp(const T* u, const T* g, T* gu) {
  T L = len14(u);
  T ug = dot3(u, g);
  T iL = T(1) / L;
  T c = ug * iL * iL * iL;
#pragma unroll
  for (int k = 0; k < 3; ++k) gu[k] = g[k] * iL - u[k] * c;
}

// ---------------------------------------------------------------------------
// quaternions
// ---------------------------------------------------------------------------
// qrot (utils.py:9-15)
template <typename T>
MPM_DI void qrot(const T* q, const T* v, T* out) {
  const T qv[3] = {q[1], q[2], q[3]};
  T uv[3], uuv[3];
  cross3(qv, v, uv);
  cross3(qv, uv, uuv);
#pragma unroll
  for (int d = 0; d < 3; ++d) out[d] = v[d] + T(2) * (q[0] * uv[d] + uuv[d]);
}
// accumulates gq (may be null) and gv (may be null)
template <typename T>
MPM_DI void qrot_vjp(const T* q, const T* v, const T* g, T* gq, T* gv) {
  const T qv[3] = {q[1], q[2], q[3]};
  T uv[3];
  cross3(qv, v, uv);
  T g_uv[3], g_uuv[3], g_qv[3] = {T(0), T(0), T(0)};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    g_uv[d] = T(2) * q[0] * g[d];
    g_uuv[d] = T(2) * g[d];
  }
  add_cross3(uv, g_uuv, g_qv);
  add_cross3(g_uuv, qv, g_uv);
  add_cross3(v, g_uv, g_qv);
  if (gv) {
#pragma unroll
    for (int d = 0; d < 3; ++d) gv[d] += g[d];
    add_cross3(g_uv, qv, gv);
  }
  if (gq) {
    gq[0] += T(2) * dot3(g, uv);
    gq[1] += g_qv[0];
    gq[2] += g_qv[1];
    gq[3] += g_qv[2];
  }
}
// normalized() of the conjugate (utils.py:53, primive_base.py:89-90)
template <typename T>
MPM_DI void conj_unit(const T* r, T* iq) {
  T L = msqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + r[3] * r[3]);
  T inv = T(1) / L;
  iq[0] = r[0] * inv;
  iq[1] = -r[1] * inv;
  iq[2] = -r[2] * inv;
  iq[3] = -r[3] * inv;
}
template <typename T>
MPM_DI void conj_unit_vjp(const T* r, const T* g_iq, T* g_r) {
  const T c[4] = {r[0], -r[1], -r[2], -r[3]};
  T L = msqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2] + c[3] * c[3]);
  T inv = T(1) / L;
  T ng = (c[0] * g_iq[0] + c[1] * g_iq[1] + c[2] * g_iq[2] + c[3] * g_iq[3]) * inv;
  T gc[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) gc[i] = (g_iq[i] - c[i] * inv * ng) * inv;
  g_r[0] += gc[0];
  g_r[1] -= gc[1];
  g_r[2] -= gc[2];
  g_r[3] -= gc[3];
}
// inv_trans (utils.py:50-54)
template <typename T>
MPM_DI void inv_trans(const T* p, const T* pos, const T* rot, T* out) {
  T iq[4];
  conj_unit(rot, iq);
  const T d[3] = {p[0] - pos[0], p[1] - pos[1], p[2] - pos[2]};
  qrot(iq, d, out);
}
template <typename T>
MPM_DI void inv_trans_vjp(const T* p, const T* pos, const T* rot, const T* g, T* g_p, T* g_pos, T* g_rot) {
  T iq[4];
  conj_unit(rot, iq);
  const T d[3] = {p[0] - pos[0], p[1] - pos[1], p[2] - pos[2]};
  T g_iq[4] = {T(0), T(0), T(0), T(0)}, g_d[3] = {T(0), T(0), T(0)};
  qrot_vjp(iq, d, g, g_iq, g_d);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (g_p) g_p[k] += g_d[k];
    g_pos[k] -= g_d[k];
  }
  conj_unit_vjp(rot, g_iq, g_rot);
}
// qmul (utils.py:23-31): Hamilton product q*r, normalised
template <typename T>
MPM_DI void qmul_raw(const T* q, const T* r, T* o) {
  o[0] = r[0] * q[0] - r[1] * q[1] - r[2] * q[2] - r[3] * q[3];
  o[1] = r[0] * q[1] + r[1] * q[0] - r[2] * q[3] + r[3] * q[2];
  o[2] = r[0] * q[2] + r[1] * q[3] + r[2] * q[0] - r[3] * q[1];
  o[3] = r[0] * q[3] - r[1] * q[2] + r[2] * q[1] + r[3] * q[0];
}
// 1 / sqrt(L2) through rsqrt: FP64 within 1 ulp (FP64 divide and square root
// are long instruction sequences on GB300's FP64 pipe), FP32 by the hardware
// approximation
MPM_DI double inv_len(double L2) { return rsqrt(L2); }
MPM_DI float inv_len(float L2) { return rsqrtf(L2); }
template <typename T>
MPM_DI void qmul(const T* q, const T* r, T* out) {
  T o[4];
  qmul_raw(q, r, o);
  T inv = inv_len(o[0] * o[0] + o[1] * o[1] + o[2] * o[2] + o[3] * o[3]);
#pragma unroll
  for (int i = 0; i < 4; ++i) out[i] = o[i] * inv;
}
template <typename T>
MPM_DI void qmul_vjp(const T* q, const T* r, const T* g, T* gq, T* gr) {
  T o[4];
  qmul_raw(q, r, o);
  T iL = inv_len(o[0] * o[0] + o[1] * o[1] + o[2] * o[2] + o[3] * o[3]);
  T on = (o[0] * g[0] + o[1] * g[1] + o[2] * g[2] + o[3] * g[3]) * iL * iL;
  T go[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) go[i] = (g[i] - o[i] * on) * iL;
  gq[0] += go[0] * r[0] + go[1] * r[1] + go[2] * r[2] + go[3] * r[3];
  gq[1] += -go[0] * r[1] + go[1] * r[0] - go[2] * r[3] + go[3] * r[2];
  gq[2] += -go[0] * r[2] + go[1] * r[3] + go[2] * r[0] - go[3] * r[1];
  gq[3] += -go[0] * r[3] - go[1] * r[2] + go[2] * r[1] + go[3] * r[0];
  gr[0] += go[0] * q[0] + go[1] * q[1] + go[2] * q[2] + go[3] * q[3];
  gr[1] += -go[0] * q[1] + go[1] * q[0] + go[2] * q[3] - go[3] * q[2];
  gr[2] += -go[0] * q[2] - go[1] * q[3] + go[2] * q[0] + go[3] * q[1];
  gr[3] += -go[0] * q[3] + go[1] * q[2] - go[2] * q[1] + go[3] * q[0];
}
// w2quat (utils.py:34-47)
template <typename T>
MPM_DI void w2quat(const T* aa, T* out) {
  T w = msqrt(dot3(aa, aa) + T(1e-16));
  out[0] = T(1);
  out[1] = out[2] = out[3] = T(0);
  if (w > T(1e-9)) {
    T s = msin(w / T(2));
    out[0] = mcos(w / T(2));
#pragma unroll
    for (int k = 0; k < 3; ++k) out[k + 1] = (aa[k] / w) * s;
  }
}
template <typename T>
MPM_DI void w2quat_vjp(const T* aa, const T* g, T* gaa) {
  T w = msqrt(dot3(aa, aa) + T(1e-16));
  if (!(w > T(1e-9))) return;
  T s = msin(w / T(2)), c = mcos(w / T(2));
  T gw = T(-0.5) * s * g[0];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    gaa[k] += g[k + 1] * s / w;
    gw += g[k + 1] * aa[k] * (-s / (w * w) + T(0.5) * c / w);
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) gaa[k] += gw * aa[k] / w;
}

}  // namespace mpm
