// Rigid tools on the device: SDFs, normals, collider velocity, the soft
// contact response of grid_op, and the vector-Jacobian products of each.
//
// Restates plb/engine/primitive/primive_base.py:75-120 (sdf, normal,
// collider_v, collide) and the shapes of plb/engine/primitive/primitives.py:
// Sphere 23-40, Capsule 55-66 (also the shape of RollingPin 101-117,
// RollingPinExt 120-135 and the fingers of Gripper2 576-697), Chopsticks
// 248-266, Cylinder 300-321, Torus 336-350, Box 375-393, Prism 712-730,
// Knife 770-807, Gripper 471-536.
#pragma once
#include "../../include/mpm_gb300.h"
#include "mpm_math.cuh"

namespace mpm {

enum {
  TOOL_SPHERE = 0,
  TOOL_CAPSULE = 1,
  TOOL_BOX = 2,
  TOOL_KNIFE = 3,
  TOOL_GRIPPER = 4,
  TOOL_ROLLINGPIN = 5,
  TOOL_ROLLINGPINEXT = 6,
  TOOL_CHOPSTICKS = 7,
  TOOL_CYLINDER = 8,
  TOOL_TORUS = 9,
  TOOL_GRIPPER2 = 10
};
// shapes that are a Capsule in their local frame
MPM_HD inline bool capsule_shape(int type) {
  return type == TOOL_CAPSULE || type == TOOL_ROLLINGPIN || type == TOOL_ROLLINGPINEXT || type == TOOL_GRIPPER2;
}
// tools made of two fingers at pos +- qrot(rot, (gap/2, 0, 0)), collided one after the other
MPM_HD inline bool fingered(int type) { return type == TOOL_GRIPPER || type == TOOL_GRIPPER2; }
// shapes whose SDF / normal adjoints come from forward-mode dual numbers
MPM_HD inline bool dual_shape(int type) {
  return type == TOOL_CHOPSTICKS || type == TOOL_CYLINDER || type == TOOL_TORUS;
}
enum { MAX_TOOLS_PER_SCENE = 8 };

// Tool parameters in the compute precision (built from MpmToolDesc).
template <typename T>
struct Tool {
  int type;
  int action_dim;
  T friction, softness;
  T radius, cap_h, cap_r;
  T size[3];
  T prism_h[2];
  T prot_inv[4];  // normalized conjugate of the prism rotation (Prism._sdf)
  T torus[2];     // tx, ty
};

// Pose of one tool at one frame in the compute precision.
template <typename T>
struct Pose {
  T pos[3];
  T rot[4];
  T gap;
};
template <typename T>
struct PoseGrad {
  T pos[3];
  T rot[4];
  T gap;
  MPM_DI void zero() {
#pragma unroll
    for (int k = 0; k < 3; ++k) pos[k] = T(0);
#pragma unroll
    for (int k = 0; k < 4; ++k) rot[k] = T(0);
    gap = T(0);
  }
};

template <typename T>
MPM_DI T fd_step() {
  return T((float)1e-4);  // d = ti.cast(1e-4, ti.float32) (primitives.py:385)
}

// tool and pose of the C ABI in the compute precision
template <typename T>
MPM_DI void to_tool(const MpmToolDesc& d, Tool<T>& t) {
  t.type = d.type;
  t.action_dim = d.action_dim;
  t.friction = T(d.friction);
  t.softness = T(d.softness);
  t.radius = T(d.radius);
  t.cap_h = T(d.cap_h);
  t.cap_r = T(d.cap_r);
#pragma unroll
  for (int k = 0; k < 3; ++k) t.size[k] = T(d.size[k]);
  t.prism_h[0] = T(d.prism_h[0]);
  t.prism_h[1] = T(d.prism_h[1]);
  T pr[4] = {T(d.prot[0]), T(d.prot[1]), T(d.prot[2]), T(d.prot[3])};
  conj_unit(pr, t.prot_inv);
  t.torus[0] = T(d.torus[0]);
  t.torus[1] = T(d.torus[1]);
}
template <typename T>
MPM_DI void to_pose(const double* src, Pose<T>& P) {
#pragma unroll
  for (int k = 0; k < 3; ++k) P.pos[k] = T(src[k]);
#pragma unroll
  for (int k = 0; k < 4; ++k) P.rot[k] = T(src[3 + k]);
  P.gap = T(src[7]);
}

// ------------------- forward-mode dual numbers (4 tangents) -------------------
// Tangents 0..2 are the local point q, tangent 3 is the gap.  Comparisons use
// the values, so branches are those of the forward pass, as in the
// reference's autodiff.
template <typename T>
struct Dual4 {
  T v, d[4];
  MPM_DI Dual4(T c = T(0)) : v(c) {
#pragma unroll
    for (int k = 0; k < 4; ++k) d[k] = T(0);
  }
};
template <typename T>
MPM_DI Dual4<T> dvar(T c, int k) {
  Dual4<T> r(c);
  r.d[k] = T(1);
  return r;
}
template <typename T>
MPM_DI T val(T x) {
  return x;
}
template <typename T>
MPM_DI T val(const Dual4<T>& x) {
  return x.v;
}
template <typename T>
MPM_DI Dual4<T> operator+(const Dual4<T>& a, const Dual4<T>& b) {
  Dual4<T> r(a.v + b.v);
#pragma unroll
  for (int k = 0; k < 4; ++k) r.d[k] = a.d[k] + b.d[k];
  return r;
}
template <typename T>
MPM_DI Dual4<T> operator-(const Dual4<T>& a, const Dual4<T>& b) {
  Dual4<T> r(a.v - b.v);
#pragma unroll
  for (int k = 0; k < 4; ++k) r.d[k] = a.d[k] - b.d[k];
  return r;
}
template <typename T>
MPM_DI Dual4<T> operator*(const Dual4<T>& a, const Dual4<T>& b) {
  Dual4<T> r(a.v * b.v);
#pragma unroll
  for (int k = 0; k < 4; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
template <typename T>
MPM_DI Dual4<T> operator/(const Dual4<T>& a, const Dual4<T>& b) {
  const T ib = T(1) / b.v;
  Dual4<T> r(a.v * ib);
#pragma unroll
  for (int k = 0; k < 4; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
  return r;
}
template <typename T>
MPM_DI Dual4<T> operator+(const Dual4<T>& a, T b) {
  return a + Dual4<T>(b);
}
template <typename T>
MPM_DI Dual4<T> operator-(const Dual4<T>& a, T b) {
  return a - Dual4<T>(b);
}
template <typename T>
MPM_DI Dual4<T> operator*(const Dual4<T>& a, T b) {
  return a * Dual4<T>(b);
}
template <typename T>
MPM_DI Dual4<T> operator/(const Dual4<T>& a, T b) {
  return a / Dual4<T>(b);
}
template <typename T>
MPM_DI Dual4<T> msqrt(const Dual4<T>& a) {
  Dual4<T> r(msqrt(a.v));
  const T h = T(0.5) / r.v;
#pragma unroll
  for (int k = 0; k < 4; ++k) r.d[k] = a.d[k] * h;
  return r;
}
// |x| with derivative sgn(x) (0 at 0)
template <typename T>
MPM_DI Dual4<T> mabs(const Dual4<T>& a) {
  const T s = sgn(a.v);
  Dual4<T> r(mabs(a.v));
#pragma unroll
  for (int k = 0; k < 4; ++k) r.d[k] = a.d[k] * s;
  return r;
}
template <typename S>
MPM_DI S sel(bool c, const S& a, const S& b) {
  return c ? a : b;
}

// generic (scalar S = T or Dual4<T>) shapes of primitives.py, length() with +1e-14
template <typename T, typename S>
MPM_DI S g_len2(const S& a, const S& b) {
  return msqrt(a * a + b * b + S(T(1e-14)));
}
template <typename T, typename S>
MPM_DI S g_len3(const S& a, const S& b, const S& c) {
  return msqrt(a * a + b * b + c * c + S(T(1e-14)));
}
// Capsule._sdf / _normal (primitives.py:55-66) on a point (x, y, z)
template <typename T, typename S>
MPM_DI void g_capsule_p2(T h, const S& y, S& p1) {
  const S a = y + S(h / T(2));
  const S m1 = sel(T(0) < val(a), a, S(T(0)));
  const S m2 = sel(val(m1) < h, m1, S(h));
  p1 = a - m2;
}
template <typename T, typename S>
MPM_DI S g_capsule_sdf(T h, T r, const S& x, const S& y, const S& z) {
  S p1;
  g_capsule_p2<T, S>(h, y, p1);
  return g_len3<T, S>(x, p1, z) - S(r);
}
template <typename T, typename S>
MPM_DI void g_capsule_normal(T h, const S& x, const S& y, const S& z, S* n) {
  S p1;
  g_capsule_p2<T, S>(h, y, p1);
  const S L = g_len3<T, S>(x, p1, z);
  n[0] = x / L;
  n[1] = p1 / L;
  n[2] = z / L;
}
// Chopsticks._sdf / _normal (primitives.py:248-266): two capsules at
// (+-gap/2, 0, 0) around p = q + (0, h/2, 0); min SDF, normal of the nearer
template <typename T, typename S>
MPM_DI S g_chop_sdf(T h, T r, const S* q, const S& gap) {
  const S half = gap / S(T(2));
  const S y = q[1] + S(h / T(2));
  const S a = g_capsule_sdf<T, S>(h, r, q[0] - half, y, q[2]);
  const S b = g_capsule_sdf<T, S>(h, r, q[0] + half, y, q[2]);
  return sel(val(a) < val(b), a, b);
}
template <typename T, typename S>
MPM_DI void g_chop_normal(T h, T r, const S* q, const S& gap, S* n) {
  const S half = gap / S(T(2));
  const S y = q[1] + S(h / T(2));
  const S a = g_capsule_sdf<T, S>(h, r, q[0] - half, y, q[2]);
  const S b = g_capsule_sdf<T, S>(h, r, q[0] + half, y, q[2]);
  g_capsule_normal<T, S>(h, val(a) <= val(b) ? q[0] - half : q[0] + half, y, q[2], n);
}
// Cylinder._sdf / _normal (primitives.py:300-321): d = (|len(x,z)|, |y|) - (h, r)
template <typename T, typename S>
MPM_DI S g_cyl_sdf(T h, T r, const S* q) {
  const S d0 = mabs(g_len2<T, S>(q[0], q[2])) - S(h), d1 = mabs(q[1]) - S(r);
  const S mx = sel(val(d1) < val(d0), d0, d1);
  const S in = sel(val(mx) < T(0), mx, S(T(0)));
  const S e0 = sel(T(0) < val(d0), d0, S(T(0))), e1 = sel(T(0) < val(d1), d1, S(T(0)));
  return in + g_len2<T, S>(e0, e1);
}
template <typename T, typename S>
MPM_DI void g_cyl_normal(T h, T r, const S* q, S* n) {
  const S l = g_len2<T, S>(q[0], q[2]);
  const S d0 = l - S(h), d1 = mabs(q[1]) - S(r);
  const T f = (val(d0) > val(d1)) ? T(1) : T(0);
  const T inside = (((val(d1) < val(d0)) ? val(d0) : val(d1)) <= T(0)) ? T(1) : T(0);
  const S a0 = sel(T(0) < val(d0), d0, S(T(0))) + S(inside * f);
  const S a1 = sel(T(0) < val(d1), d1, S(T(0))) + S(inside * (T(1) - f));
  const S L2 = g_len2<T, S>(a0, a1);
  const S n0 = a0 / L2, n1 = a1 / L2;
  const T sy = (val(q[1]) >= T(0)) ? T(1) : T(-1);
  const S m0 = (q[0] / l) * n0, m1 = n1 * S(sy), m2 = (q[2] / l) * n0;
  const S L3 = g_len3<T, S>(m0, m1, m2);
  n[0] = m0 / L3;
  n[1] = m1 / L3;
  n[2] = m2 / L3;
}
// Torus._sdf / _normal (primitives.py:336-350)
template <typename T, typename S>
MPM_DI S g_torus_sdf(T tx, T ty, const S* q) {
  return g_len2<T, S>(g_len2<T, S>(q[0], q[2]) - S(tx), q[1]) - S(ty);
}
template <typename T, typename S>
MPM_DI void g_torus_normal(T tx, const S* q, S* n) {
  const S l = g_len2<T, S>(q[0], q[2]);
  const S qa = l - S(tx);
  const S Lq = g_len2<T, S>(qa, q[1]);
  const S n0 = qa / Lq, n1 = q[1] / Lq;
  const S m0 = (q[0] / l) * n0, m2 = (q[2] / l) * n0;
  const S L3 = g_len3<T, S>(m0, n1, m2);
  n[0] = m0 / L3;
  n[1] = n1 / L3;
  n[2] = m2 / L3;
}
template <typename T, typename S>
MPM_DI S g_shape_sdf(const Tool<T>& t, const S* q, const S& gap) {
  if (t.type == TOOL_CHOPSTICKS) return g_chop_sdf<T, S>(t.cap_h, t.cap_r, q, gap);
  if (t.type == TOOL_CYLINDER) return g_cyl_sdf<T, S>(t.cap_h, t.cap_r, q);
  return g_torus_sdf<T, S>(t.torus[0], t.torus[1], q);
}
template <typename T, typename S>
MPM_DI void g_shape_normal(const Tool<T>& t, const S* q, const S& gap, S* n) {
  if (t.type == TOOL_CHOPSTICKS) g_chop_normal<T, S>(t.cap_h, t.cap_r, q, gap, n);
  else if (t.type == TOOL_CYLINDER) g_cyl_normal<T, S>(t.cap_h, t.cap_r, q, n);
  else g_torus_normal<T, S>(t.torus[0], q, n);
}
// out-of-line so the hot grid kernels do not carry their registers
template <typename T>
__device__ __noinline__ T dual_sdf(const Tool<T>& t, const T* q, T gap) {
  return g_shape_sdf<T, T>(t, q, gap);
}
template <typename T>
__device__ __noinline__ void dual_sdf_grad(const Tool<T>& t, const T* q, T gap, T g, T* gq, T* ggap) {
  const Dual4<T> qd[3] = {dvar(q[0], 0), dvar(q[1], 1), dvar(q[2], 2)};
  const Dual4<T> r = g_shape_sdf<T, Dual4<T>>(t, qd, dvar(gap, 3));
#pragma unroll
  for (int k = 0; k < 3; ++k) gq[k] += g * r.d[k];
  if (ggap) *ggap += g * r.d[3];
}
template <typename T>
__device__ __noinline__ void dual_normal(const Tool<T>& t, const T* q, T gap, T* n) {
  g_shape_normal<T, T>(t, q, gap, n);
}
template <typename T>
__device__ __noinline__ void dual_normal_vjp(const Tool<T>& t, const T* q, T gap, const T* gn, T* gq, T* ggap) {
  const Dual4<T> qd[3] = {dvar(q[0], 0), dvar(q[1], 1), dvar(q[2], 2)};
  Dual4<T> n[3];
  g_shape_normal<T, Dual4<T>>(t, qd, dvar(gap, 3), n);
#pragma unroll
  for (int k = 0; k < 3; ++k) gq[k] += gn[0] * n[0].d[k] + gn[1] * n[1].d[k] + gn[2] * n[2].d[k];
  if (ggap) *ggap += gn[0] * n[0].d[3] + gn[1] * n[1].d[3] + gn[2] * n[2].d[3];
}

// ------------------------------- local SDFs -------------------------------
// Capsule: p2 = q with p2.y += h/2; p2.y -= min(max(p2.y, 0), h)
template <typename T>
MPM_DI void capsule_p2(const Tool<T>& t, const T* q, T* p2, T* dp1) {
  p2[0] = q[0];
  p2[2] = q[2];
  T a = q[1] + t.cap_h / T(2);
  T m1 = (T(0) < a) ? a : T(0);
  T m2 = (m1 < t.cap_h) ? m1 : t.cap_h;
  p2[1] = a - m2;
  *dp1 = (T(0) < a && m1 < t.cap_h) ? T(0) : T(1);
}
template <typename T>
MPM_DI T box_sdf(const T* size, const T* q) {
  T qq[3], mq[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    qq[k] = mabs(q[k]) - size[k];
    mq[k] = (T(0) < qq[k]) ? qq[k] : T(0);
  }
  T t = (qq[2] < qq[1]) ? qq[1] : qq[2];
  T u = (t < qq[0]) ? qq[0] : t;
  return len14(mq) + ((u < T(0)) ? u : T(0));
}
template <typename T>
MPM_DI void box_sdf_grad(const T* size, const T* q, T g, T* gq) {
  T qq[3], mq[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    qq[k] = mabs(q[k]) - size[k];
    mq[k] = (T(0) < qq[k]) ? qq[k] : T(0);
  }
  T iL = T(1) / len14(mq);
  T gqq[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) gqq[k] = (T(0) < qq[k]) ? g * mq[k] * iL : T(0);
  T t = (qq[2] < qq[1]) ? qq[1] : qq[2];
  T u = (t < qq[0]) ? qq[0] : t;
  if (u < T(0)) {
    if (t < qq[0]) gqq[0] += g;
    else if (qq[2] < qq[1]) gqq[1] += g;
    else gqq[2] += g;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) gq[k] += gqq[k] * sgn(q[k]);
}
template <typename T>
MPM_DI T prism_sdf(const Tool<T>& t, const T* q) {
  T qq[3];
  qrot(t.prot_inv, q, qq);
  T A = mabs(qq[2]) - t.prism_h[1];
  T C = mabs(qq[0]) * T(0.866025) + qq[1] * T(0.5), D = -qq[1];
  T B = ((D < C) ? C : D) - t.prism_h[0] * T(0.5);
  return (B < A) ? A : B;
}
template <typename T>
MPM_DI void prism_sdf_grad(const Tool<T>& t, const T* q, T g, T* gq) {
  T qq[3];
  qrot(t.prot_inv, q, qq);
  T A = mabs(qq[2]) - t.prism_h[1];
  T C = mabs(qq[0]) * T(0.866025) + qq[1] * T(0.5), D = -qq[1];
  T B = ((D < C) ? C : D) - t.prism_h[0] * T(0.5);
  T gA = (B < A) ? g : T(0);
  T gB = (B < A) ? T(0) : g;
  T gC = (D < C) ? gB : T(0);
  T gD = (D < C) ? T(0) : gB;
  const T gqq[3] = {gC * T(0.866025) * sgn(qq[0]), gC * T(0.5) - gD, gA * sgn(qq[2])};
  qrot_vjp(t.prot_inv, q, gqq, (T*)nullptr, gq);
}
// gap: the pose's gap (only the Chopsticks shape depends on it)
template <typename T>
MPM_DI T local_sdf(const Tool<T>& t, const T* q, T gap) {
  if (capsule_shape(t.type)) {
    T p2[3], dp;
    capsule_p2(t, q, p2, &dp);
    return len14(p2) - t.cap_r;
  }
  if (t.type == TOOL_KNIFE) {
    T a = prism_sdf(t, q), b = box_sdf(t.size, q);
    return (b < a) ? a : b;
  }
  if (dual_shape(t.type)) return dual_sdf(t, q, gap);
  return box_sdf(t.size, q);  // Box and Gripper fingers
}
// accumulates gq and, if ggap is not NULL, the gap gradient
template <typename T>
MPM_DI void local_sdf_grad(const Tool<T>& t, const T* q, T gap, T g, T* gq, T* ggap) {
  if (dual_shape(t.type)) {
    dual_sdf_grad(t, q, gap, g, gq, ggap);
    return;
  }
  if (capsule_shape(t.type)) {
    T p2[3], dp;
    capsule_p2(t, q, p2, &dp);
    T iL = g / len14(p2);
    gq[0] += p2[0] * iL;
    gq[1] += p2[1] * iL * dp;
    gq[2] += p2[2] * iL;
    return;
  }
  if (t.type == TOOL_KNIFE) {
    T a = prism_sdf(t, q), b = box_sdf(t.size, q);
    if (b < a) prism_sdf_grad(t, q, g, gq);
    else box_sdf_grad(t.size, q, g, gq);
    return;
  }
  box_sdf_grad(t.size, q, g, gq);
}
// finite-difference normal before normalisation (Box._normal, Knife._normal);
// only box-type shapes (Box, Gripper fingers) and the Knife come here.  The
// shape test is taken once, so the six SDF evaluations are straight-line code
// that the compiler can interleave.
template <typename T>
MPM_DI T knife_sdf(const Tool<T>& t, const T* q) {
  T a = prism_sdf(t, q), b = box_sdf(t.size, q);
  return (b < a) ? a : b;
}
template <typename T>
MPM_DI void fd_normal_raw(const Tool<T>& t, const T* q, T* r) {
  const T d = fd_step<T>();
  const T h = T(0.5) / d;
  if (t.type == TOOL_KNIFE) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      T inc[3] = {q[0], q[1], q[2]}, dec[3] = {q[0], q[1], q[2]};
      inc[i] += d;
      dec[i] -= d;
      r[i] = h * (knife_sdf(t, inc) - knife_sdf(t, dec));
    }
  } else {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      T inc[3] = {q[0], q[1], q[2]}, dec[3] = {q[0], q[1], q[2]};
      inc[i] += d;
      dec[i] -= d;
      r[i] = h * (box_sdf(t.size, inc) - box_sdf(t.size, dec));
    }
  }
}
// r_out (may be null): the vector before normalisation, for local_normal_vjp
template <typename T>
MPM_DI void local_normal(const Tool<T>& t, const T* q, T gap, T* n, T* r_out = nullptr) {
  if (dual_shape(t.type)) {
    dual_normal(t, q, gap, n);
    return;
  }
  T r[3];
  if (capsule_shape(t.type)) {
    T dp;
    capsule_p2(t, q, r, &dp);
  } else {
    fd_normal_raw(t, q, r);
  }
  T iL = T(1) / len14(r);
#pragma unroll
  for (int k = 0; k < 3; ++k) n[k] = r[k] * iL;
  if (r_out) {
#pragma unroll
    for (int k = 0; k < 3; ++k) r_out[k] = r[k];
  }
}
// r_in (may be null): the r_out of local_normal at the same q (saves the six
// SDF evaluations of a finite-difference normal)
template <typename T>
MPM_DI void local_normal_vjp(const Tool<T>& t, const T* q, T gap, const T* gn, T* gq, T* ggap,
                             const T* r_in = nullptr) {
  if (dual_shape(t.type)) {
    dual_normal_vjp(t, q, gap, gn, gq, ggap);
    return;
  }
  T r[3], gr[3];
  if (capsule_shape(t.type)) {
    T dp;
    capsule_p2(t, q, r, &dp);
    unit14_vjp(r, gn, gr);
    gq[0] += gr[0];
    gq[1] += gr[1] * dp;
    gq[2] += gr[2];
    return;
  }
  if (r_in) {
#pragma unroll
    for (int k = 0; k < 3; ++k) r[k] = r_in[k];
  } else {
    fd_normal_raw(t, q, r);
  }
  unit14_vjp(r, gn, gr);
  const T d = fd_step<T>();
  const T h = T(0.5) / d;
  if (t.type == TOOL_KNIFE) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      T inc[3] = {q[0], q[1], q[2]}, dec[3] = {q[0], q[1], q[2]};
      inc[i] += d;
      dec[i] -= d;
      local_sdf_grad(t, inc, T(0), h * gr[i], gq, (T*)nullptr);
      local_sdf_grad(t, dec, T(0), -h * gr[i], gq, (T*)nullptr);
    }
  } else {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      T inc[3] = {q[0], q[1], q[2]}, dec[3] = {q[0], q[1], q[2]};
      inc[i] += d;
      dec[i] -= d;
      box_sdf_grad(t.size, inc, h * gr[i], gq);
      box_sdf_grad(t.size, dec, -h * gr[i], gq);
    }
  }
}

// ------------------------------ world space --------------------------------
// "rigid" pose = (pos, rot); Sphere ignores rot (primitives.py:28-34)
template <typename T>
MPM_DI T shape_sdf(const Tool<T>& t, const T* pos, const T* rot, T gap, const T* p) {
  if (t.type == TOOL_SPHERE) {
    const T d[3] = {p[0] - pos[0], p[1] - pos[1], p[2] - pos[2]};
    return len14(d) - t.radius;
  }
  T q[3];
  inv_trans(p, pos, rot, q);
  return local_sdf(t, q, gap);
}
template <typename T>
MPM_DI void shape_sdf_vjp(const Tool<T>& t, const T* pos, const T* rot, T gap, const T* p, T g, T* gp, T* gpos,
                          T* grot, T* ggap) {
  if (t.type == TOOL_SPHERE) {
    const T d[3] = {p[0] - pos[0], p[1] - pos[1], p[2] - pos[2]};
    T c = g / len14(d);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (gp) gp[k] += c * d[k];
      gpos[k] -= c * d[k];
    }
    return;
  }
  T q[3], gq[3] = {T(0), T(0), T(0)};
  inv_trans(p, pos, rot, q);
  local_sdf_grad(t, q, gap, g, gq, ggap);
  inv_trans_vjp(p, pos, rot, gq, gp, gpos, grot);
}
// r_out (may be null): the local normal before normalisation, for shape_normal_vjp
template <typename T>
MPM_DI void shape_normal(const Tool<T>& t, const T* pos, const T* rot, T gap, const T* p, T* n,
                         T* r_out = nullptr) {
  if (t.type == TOOL_SPHERE) {
    const T d[3] = {p[0] - pos[0], p[1] - pos[1], p[2] - pos[2]};
    T iL = T(1) / len14(d);
#pragma unroll
    for (int k = 0; k < 3; ++k) n[k] = d[k] * iL;
    return;
  }
  T q[3], nl[3];
  inv_trans(p, pos, rot, q);
  local_normal(t, q, gap, nl, r_out);
  qrot(rot, nl, n);
}
// gp (the point's gradient) and ggap may be NULL; r_in (may be null): the
// r_out of shape_normal at the same pose and point
template <typename T>
MPM_DI void shape_normal_vjp(const Tool<T>& t, const T* pos, const T* rot, T gap, const T* p, const T* gn, T* gp,
                             T* gpos, T* grot, T* ggap, const T* r_in = nullptr) {
  if (t.type == TOOL_SPHERE) {
    const T d[3] = {p[0] - pos[0], p[1] - pos[1], p[2] - pos[2]};
    T gd[3];
    unit14_vjp(d, gn, gd);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      gpos[k] -= gd[k];
      if (gp) gp[k] += gd[k];
    }
    return;
  }
  T q[3], nl[3], r[3];
  inv_trans(p, pos, rot, q);
  if (r_in && !dual_shape(t.type)) {  // the normal from r exactly as local_normal forms it
#pragma unroll
    for (int k = 0; k < 3; ++k) r[k] = r_in[k];
    T iL = T(1) / len14(r);
#pragma unroll
    for (int k = 0; k < 3; ++k) nl[k] = r[k] * iL;
  } else {
    local_normal(t, q, gap, nl, r);
  }
  T gnl[3] = {T(0), T(0), T(0)}, gq[3] = {T(0), T(0), T(0)};
  qrot_vjp(rot, nl, gn, grot, gnl);
  local_normal_vjp(t, q, gap, gnl, gq, ggap, r);
  inv_trans_vjp(p, pos, rot, gq, gp, gpos, grot);
}
// collider_v (primive_base.py:87-94)
template <typename T>
MPM_DI void collider_v(const T* pos0, const T* rot0, const T* pos1, const T* rot1, const T* p, T dt, T* cv) {
  T rel[3], nw[3];
  inv_trans(p, pos0, rot0, rel);
  qrot(rot1, rel, nw);
  T idt = T(1) / dt;
#pragma unroll
  for (int k = 0; k < 3; ++k) cv[k] = (nw[k] + pos1[k] - p[k]) * idt;
}
template <typename T>
MPM_DI void collider_v_vjp(const T* pos0, const T* rot0, const T* pos1, const T* rot1, const T* p, T dt, const T* g,
                           T* gpos0, T* grot0, T* gpos1, T* grot1) {
  T rel[3];
  inv_trans(p, pos0, rot0, rel);
  T idt = T(1) / dt;
  const T gnw[3] = {g[0] * idt, g[1] * idt, g[2] * idt};
#pragma unroll
  for (int k = 0; k < 3; ++k) gpos1[k] += gnw[k];
  T grel[3] = {T(0), T(0), T(0)};
  qrot_vjp(rot1, rel, gnw, grot1, grel);
  inv_trans_vjp(p, pos0, rot0, grel, (T*)nullptr, gpos0, grot0);
}

// Primitive.collide (primive_base.py:96-120).  Returns whether the contact
// branch ran; vout = vin otherwise.
template <typename T>
MPM_DI bool collide_fwd(const Tool<T>& t, const T* pos0, const T* rot0, T gap0, const T* pos1, const T* rot1,
                        const T* p, T dt, const T* vin, T* vout) {
  T dist = shape_sdf(t, pos0, rot0, gap0, p);
  T e = mexp_fast(-dist * t.softness);
  T infl = (e < T(1)) ? e : T(1);
#pragma unroll
  for (int k = 0; k < 3; ++k) vout[k] = vin[k];
  if (!((t.softness > T(0) && infl > T(0.1)) || dist <= T(0))) return false;
  T D[3], cv[3], iv[3], vt[3];
  shape_normal(t, pos0, rot0, gap0, p, D);
  collider_v(pos0, rot0, pos1, rot1, p, dt, cv);
#pragma unroll
  for (int k = 0; k < 3; ++k) iv[k] = vin[k] - cv[k];
  T nc = dot3(iv, D);
  T mn = (nc < T(0)) ? nc : T(0);
#pragma unroll
  for (int k = 0; k < 3; ++k) vt[k] = iv[k] - mn * D[k];
  T vtn = len8(vt);
  T a = vtn + nc * t.friction;
  T m = (a < T(0)) ? T(0) : a;
  T flag = (nc < T(0) && msqrt(dot3(vt, vt)) > T(1e-30)) ? T(1) : T(0);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    T vtf = vt[k] / vtn * m;
    T vt2 = vtf * flag + vt[k] * (T(1) - flag);
    vout[k] = cv[k] + iv[k] * (T(1) - infl) + vt2 * infl;
  }
  return true;
}
template <typename T>
MPM_DI void collide_vjp(const Tool<T>& t, const T* pos0, const T* rot0, T gap0, const T* pos1, const T* rot1,
                        const T* p, T dt, const T* vin, const T* gout, T* gvin, T* gpos0, T* grot0, T* ggap0,
                        T* gpos1, T* grot1) {
  T dist = shape_sdf(t, pos0, rot0, gap0, p);
  T e = mexp_fast(-dist * t.softness);
  T infl = (e < T(1)) ? e : T(1);
  if (!((t.softness > T(0) && infl > T(0.1)) || dist <= T(0))) {
#pragma unroll
    for (int k = 0; k < 3; ++k) gvin[k] = gout[k];
    return;
  }
  T D[3], Dr[3], cv[3], iv[3], vt[3];
  shape_normal(t, pos0, rot0, gap0, p, D, Dr);  // Dr reused by the normal's adjoint
  collider_v(pos0, rot0, pos1, rot1, p, dt, cv);
#pragma unroll
  for (int k = 0; k < 3; ++k) iv[k] = vin[k] - cv[k];
  T nc = dot3(iv, D);
  T mn = (nc < T(0)) ? nc : T(0);
#pragma unroll
  for (int k = 0; k < 3; ++k) vt[k] = iv[k] - mn * D[k];
  T vtn = len8(vt);
  T a = vtn + nc * t.friction;
  T m = (a < T(0)) ? T(0) : a;
  T flag = (nc < T(0) && msqrt(dot3(vt, vt)) > T(1e-30)) ? T(1) : T(0);
  T g_cv[3], g_iv[3], g_vt[3], g_vtf[3], g_infl = T(0);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    T vtf = vt[k] / vtn * m;
    T vt2 = vtf * flag + vt[k] * (T(1) - flag);
    g_cv[k] = gout[k];
    g_iv[k] = gout[k] * (T(1) - infl);
    g_infl += gout[k] * (vt2 - iv[k]);
    g_vtf[k] = gout[k] * infl * flag;
    g_vt[k] = gout[k] * infl * (T(1) - flag);
  }
  T gvtf_vt = dot3(g_vtf, vt);
  T g_vtn = -gvtf_vt * m / (vtn * vtn);
  T g_m = gvtf_vt / vtn;
  T g_nc = T(0);
  if (!(a < T(0))) {
    g_vtn += g_m;
    g_nc += g_m * t.friction;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) g_vt[k] += g_vtf[k] * m / vtn + g_vtn * vt[k] / vtn;
  T g_D[3] = {T(0), T(0), T(0)};
#pragma unroll
  for (int k = 0; k < 3; ++k) g_iv[k] += g_vt[k];
  if (nc < T(0)) {
    g_nc -= dot3(g_vt, D);
#pragma unroll
    for (int k = 0; k < 3; ++k) g_D[k] -= nc * g_vt[k];
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    g_iv[k] += g_nc * D[k];
    g_D[k] += g_nc * iv[k];
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    gvin[k] = g_iv[k];
    g_cv[k] -= g_iv[k];
  }
  T g_dist = (e < T(1)) ? g_infl * e * (-t.softness) : T(0);
  shape_sdf_vjp(t, pos0, rot0, gap0, p, g_dist, (T*)nullptr, gpos0, grot0, ggap0);
  shape_normal_vjp(t, pos0, rot0, gap0, p, g_D, (T*)nullptr, gpos0, grot0, ggap0, Dr);
  collider_v_vjp(pos0, rot0, pos1, rot1, p, dt, g_cv, gpos0, grot0, gpos1, grot1);
}

// Gripper finger position (primitives.py:475-477)
template <typename T>
MPM_DI void finger_pos(const Pose<T>& P, T flag, T* fpos) {
  const T lv[3] = {P.gap / T(2) * flag, T(0), T(0)};
  T off[3];
  qrot(P.rot, lv, off);
#pragma unroll
  for (int k = 0; k < 3; ++k) fpos[k] = P.pos[k] + off[k];
}
template <typename T>
MPM_DI void finger_pos_vjp(const Pose<T>& P, T flag, const T* gfpos, PoseGrad<T>& gP) {
  const T lv[3] = {P.gap / T(2) * flag, T(0), T(0)};
  T glv[3] = {T(0), T(0), T(0)};
#pragma unroll
  for (int k = 0; k < 3; ++k) gP.pos[k] += gfpos[k];
  qrot_vjp(P.rot, lv, gfpos, gP.rot, glv);
  gP.gap += glv[0] * flag / T(2);
}

// grid_op's call of primitives[i].collide (mpm_simulator.py:237-239)
// returns whether the contact response was applied (else v passes unchanged,
// and so does its adjoint, with zero pose gradients)
template <typename T>
MPM_DI bool tool_collide(const Tool<T>& t, const Pose<T>& P0, const Pose<T>& P1, const T* p, T dt, T* v) {
  T out[3];
  if (fingered(t.type)) {
    bool hit = false;
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      T flag = side == 0 ? T(-1) : T(1);
      T f0[3], f1[3];
      finger_pos(P0, flag, f0);
      finger_pos(P1, flag, f1);
      hit = collide_fwd(t, f0, P0.rot, T(0), f1, P1.rot, p, dt, v, out) || hit;
#pragma unroll
      for (int k = 0; k < 3; ++k) v[k] = out[k];
    }
    return hit;
  }
  const bool hit = collide_fwd(t, P0.pos, P0.rot, P0.gap, P1.pos, P1.rot, p, dt, v, out);
#pragma unroll
  for (int k = 0; k < 3; ++k) v[k] = out[k];
  return hit;
}
// g: in = d/d vout, out = d/d vin
template <typename T>
MPM_DI void tool_collide_vjp(const Tool<T>& t, const Pose<T>& P0, const Pose<T>& P1, const T* p, T dt,
                             const T* vin, T* g, PoseGrad<T>& g0, PoseGrad<T>& g1) {
  T gin[3];
  if (fingered(t.type)) {
    T fa0[3], fa1[3], fb0[3], fb1[3], mid[3];
    finger_pos(P0, T(-1), fa0);
    finger_pos(P1, T(-1), fa1);
    finger_pos(P0, T(1), fb0);
    finger_pos(P1, T(1), fb1);
    collide_fwd(t, fa0, P0.rot, T(0), fa1, P1.rot, p, dt, vin, mid);
    T gf0[3] = {T(0), T(0), T(0)}, gf1[3] = {T(0), T(0), T(0)};
    collide_vjp(t, fb0, P0.rot, T(0), fb1, P1.rot, p, dt, mid, g, gin, gf0, g0.rot, (T*)nullptr, gf1, g1.rot);
    finger_pos_vjp(P0, T(1), gf0, g0);
    finger_pos_vjp(P1, T(1), gf1, g1);
    T gin2[3];
    T ga0[3] = {T(0), T(0), T(0)}, ga1[3] = {T(0), T(0), T(0)};
    collide_vjp(t, fa0, P0.rot, T(0), fa1, P1.rot, p, dt, vin, gin, gin2, ga0, g0.rot, (T*)nullptr, ga1, g1.rot);
    finger_pos_vjp(P0, T(-1), ga0, g0);
    finger_pos_vjp(P1, T(-1), ga1, g1);
#pragma unroll
    for (int k = 0; k < 3; ++k) g[k] = gin2[k];
    return;
  }
  collide_vjp(t, P0.pos, P0.rot, P0.gap, P1.pos, P1.rot, p, dt, vin, g, gin, g0.pos, g0.rot, &g0.gap, g1.pos,
              g1.rot);
#pragma unroll
  for (int k = 0; k < 3; ++k) g[k] = gin[k];
}

// world SDF (Gripper.sdf = min of fingers, primitives.py:486-487)
template <typename T>
MPM_DI T tool_sdf(const Tool<T>& t, const Pose<T>& P, const T* p) {
  if (fingered(t.type)) {
    T fa[3], fb[3];
    finger_pos(P, T(-1), fa);
    finger_pos(P, T(1), fb);
    T a = shape_sdf(t, fa, P.rot, T(0), p), b = shape_sdf(t, fb, P.rot, T(0), p);
    return (a < b) ? a : b;
  }
  return shape_sdf(t, P.pos, P.rot, P.gap, p);
}
template <typename T>
MPM_DI void tool_sdf_vjp(const Tool<T>& t, const Pose<T>& P, const T* p, T g, T* gp, PoseGrad<T>& gP) {
  if (fingered(t.type)) {
    T fa[3], fb[3];
    finger_pos(P, T(-1), fa);
    finger_pos(P, T(1), fb);
    T a = shape_sdf(t, fa, P.rot, T(0), p), b = shape_sdf(t, fb, P.rot, T(0), p);
    T gf[3] = {T(0), T(0), T(0)};
    if (a < b) {
      shape_sdf_vjp(t, fa, P.rot, T(0), p, g, gp, gf, gP.rot, (T*)nullptr);
      finger_pos_vjp(P, T(-1), gf, gP);
    } else {
      shape_sdf_vjp(t, fb, P.rot, T(0), p, g, gp, gf, gP.rot, (T*)nullptr);
      finger_pos_vjp(P, T(1), gf, gP);
    }
    return;
  }
  shape_sdf_vjp(t, P.pos, P.rot, P.gap, p, g, gp, gP.pos, gP.rot, &gP.gap);
}
// world normal (Primitive.normal, primive_base.py:81-85; Gripper/Gripper2
// take the finger with the smaller SDF, ties to finger -1, primitives.py:489-496, 621-628)
template <typename T>
MPM_DI void tool_normal(const Tool<T>& t, const Pose<T>& P, const T* p, T* n) {
  if (fingered(t.type)) {
    T fa[3], fb[3];
    finger_pos(P, T(-1), fa);
    finger_pos(P, T(1), fb);
    T a = shape_sdf(t, fa, P.rot, T(0), p), b = shape_sdf(t, fb, P.rot, T(0), p);
    shape_normal(t, a <= b ? fa : fb, P.rot, T(0), p, n);
    return;
  }
  shape_normal(t, P.pos, P.rot, P.gap, p, n);
}
template <typename T>
MPM_DI void tool_normal_vjp(const Tool<T>& t, const Pose<T>& P, const T* p, const T* gn, T* gp, PoseGrad<T>& gP) {
  if (fingered(t.type)) {
    T fa[3], fb[3];
    finger_pos(P, T(-1), fa);
    finger_pos(P, T(1), fb);
    T a = shape_sdf(t, fa, P.rot, T(0), p), b = shape_sdf(t, fb, P.rot, T(0), p);
    T gf[3] = {T(0), T(0), T(0)};
    shape_normal_vjp(t, a <= b ? fa : fb, P.rot, T(0), p, gn, gp, gf, gP.rot, (T*)nullptr);
    finger_pos_vjp(P, a <= b ? T(-1) : T(1), gf, gP);
    return;
  }
  shape_normal_vjp(t, P.pos, P.rot, P.gap, p, gn, gp, gP.pos, gP.rot, &gP.gap);
}

}  // namespace mpm
