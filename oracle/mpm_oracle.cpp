// FP64 CPU oracle for the differentiable MLS-MPM substep of DiffSkill.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity oracle and the timed CPU
// baseline.  The product package (diffskill_gb300) never links, loads or calls
// it; only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg do.
//
// Parity status: PARTIALLY PINNED.  The reference runs on taichi==0.7.26
// (environment.yml:22), which cannot be imported here, so no substep output of
// the reference can be reproduced.  What is pinned: grid mass conservation,
// p_mass, the 64^3 C-order density layout and the quadratic B-spline moments
// (against the reference's plb/envs/assets/*3D-v*.npy density grids), and the
// SDF normal consistency property of plb/engine/primitive/test_primitives.py:67.
// Everything else restates the reference code line by line (cited below) and
// the hand-written adjoint is checked against FP64 central differences.
//
// Semantics copied from the reference's autodiff (taichi source transform):
//   * branch decisions are frozen at their forward values;
//   * max(a, b) sends the gradient to a iff b < a (ties go to b);
//   * min(a, b) sends the gradient to a iff a < b (ties go to b);
//   * abs'(x) = sgn(x) with sgn(0) = 0;
//   * the SVD gradient is the clamped formula of mpm_simulator.py:137-156.
//
// State layout (AoS, one row of 24 doubles per particle):
//   x[0..2] v[3..5] C[6..14] F[15..23], matrices row-major.
// Tool pose layout (8 doubles): pos[3] rot[4] (w,x,y,z) gap.
// Tool velocity layout (8 doubles): v[3] w[3] gap_vel pad.
// Grid layout: node (i,j,k) at (i*n + j)*n + k, as the reference's 64^3 fields.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

struct OracleSim {
  int32_t n_grid;
  int32_t pad0;
  double dx, inv_dx, dt, p_vol, p_mass;
  double mu, lam, yield_stress;
  double gravity[3];
  double ground_friction;
  double lower_bound;
};

struct OracleTool {
  int32_t type;  // 0 sphere, 1 capsule, 2 box, 3 knife, 4 gripper, 5 rolling pin, 6 rolling pin ext,
                 // 7 chopsticks, 8 cylinder, 9 torus, 10 gripper2
  int32_t action_dim;
  double friction;
  double softness;
  double radius;        // sphere
  double cap_h, cap_r;  // capsule
  double size[3];       // box / knife box / gripper finger half extents
  double prism_h[2];    // knife prism
  double prot[4];       // knife prism rotation
  double min_gap, max_gap;
  double lower[3], upper[3];
  double action_scale[7];
  double torus[2];         // Torus tx, ty
  int32_t collision_mask;  // bit j: projected out of tool j (collision_group[j] > 0)
  int32_t pad1;
};

}  // extern "C"

namespace {

enum {
  T_SPHERE = 0,
  T_CAPSULE = 1,
  T_BOX = 2,
  T_KNIFE = 3,
  T_GRIPPER = 4,
  T_ROLLINGPIN = 5,
  T_ROLLINGPINEXT = 6,
  T_CHOPSTICKS = 7,
  T_CYLINDER = 8,
  T_TORUS = 9,
  T_GRIPPER2 = 10
};
inline bool is_fingered(int type) { return type == T_GRIPPER || type == T_GRIPPER2; }
inline bool has_gap_vel(int type) { return type == T_GRIPPER || type == T_CHOPSTICKS || type == T_GRIPPER2; }

// ----------------------------------------------------------------------------
// small linear algebra
// ----------------------------------------------------------------------------
inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
inline void cross3(const double* a, const double* b, double* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
inline void add_cross3(const double* a, const double* b, double* c) {  // c += a x b
  c[0] += a[1] * b[2] - a[2] * b[1];
  c[1] += a[2] * b[0] - a[0] * b[2];
  c[2] += a[0] * b[1] - a[1] * b[0];
}
inline void mm(const double* A, const double* B, double* C) {  // C = A B
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) C[i * 3 + j] = A[i * 3] * B[j] + A[i * 3 + 1] * B[3 + j] + A[i * 3 + 2] * B[6 + j];
}
inline void mmT(const double* A, const double* B, double* C) {  // C = A B^T
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      C[i * 3 + j] = A[i * 3] * B[j * 3] + A[i * 3 + 1] * B[j * 3 + 1] + A[i * 3 + 2] * B[j * 3 + 2];
}
inline void mTm(const double* A, const double* B, double* C) {  // C = A^T B
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) C[i * 3 + j] = A[i] * B[j] + A[3 + i] * B[3 + j] + A[6 + i] * B[6 + j];
}
inline double det3(const double* A) {
  return A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
         A[2] * (A[3] * A[7] - A[4] * A[6]);
}
inline void cof3(const double* A, double* Cf) {  // d det / d A
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
inline double sgn(double x) { return x > 0 ? 1.0 : (x < 0 ? -1.0 : 0.0); }

// length() of plb/engine/primitive/primitives.py:13-15 (eps 1e-14)
inline double len14(const double* a) { return std::sqrt(dot3(a, a) + 1e-14); }
// length() of plb/engine/primitive/utils.py:4-6 (eps 1e-8)
inline double len8(const double* a) { return std::sqrt(dot3(a, a) + 1e-8); }

// ----------------------------------------------------------------------------
// quaternions: plb/engine/primitive/utils.py:9-54
// ----------------------------------------------------------------------------
// qrot (utils.py:9-15): v + 2 (q0 (qv x v) + qv x (qv x v))
inline void qrot(const double* q, const double* v, double* out) {
  const double qv[3] = {q[1], q[2], q[3]};
  double uv[3], uuv[3];
  cross3(qv, v, uv);
  cross3(qv, uv, uuv);
  for (int d = 0; d < 3; ++d) out[d] = v[d] + 2.0 * (q[0] * uv[d] + uuv[d]);
}
// accumulate gq (4) and gv (3) given upstream g (3); either may be null
inline void qrot_vjp(const double* q, const double* v, const double* g, double* gq, double* gv) {
  const double qv[3] = {q[1], q[2], q[3]};
  double uv[3];
  cross3(qv, v, uv);
  double g_uv[3], g_uuv[3], g_qv[3] = {0, 0, 0};
  for (int d = 0; d < 3; ++d) {
    g_uv[d] = 2.0 * q[0] * g[d];
    g_uuv[d] = 2.0 * g[d];
  }
  // uuv = qv x uv
  add_cross3(uv, g_uuv, g_qv);
  add_cross3(g_uuv, qv, g_uv);
  // uv = qv x v
  add_cross3(v, g_uv, g_qv);
  if (gv) {
    for (int d = 0; d < 3; ++d) gv[d] += g[d];
    add_cross3(g_uv, qv, gv);
  }
  if (gq) {
    gq[0] += 2.0 * dot3(g, uv);
    gq[1] += g_qv[0];
    gq[2] += g_qv[1];
    gq[3] += g_qv[2];
  }
}
// Vector.normalized(): q * (1/sqrt(q.q))
inline void normalize4(const double* q, double* n) {
  double L = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  double inv = 1.0 / L;
  for (int i = 0; i < 4; ++i) n[i] = q[i] * inv;
}
inline void normalize4_vjp(const double* q, const double* gn, double* gq) {
  double L = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  double n[4];
  for (int i = 0; i < 4; ++i) n[i] = q[i] / L;
  double ng = n[0] * gn[0] + n[1] * gn[1] + n[2] * gn[2] + n[3] * gn[3];
  for (int i = 0; i < 4; ++i) gq[i] += (gn[i] - n[i] * ng) / L;
}
inline void conj_normalized(const double* rot, double* iq) {
  const double c[4] = {rot[0], -rot[1], -rot[2], -rot[3]};
  normalize4(c, iq);
}
inline void conj_normalized_vjp(const double* rot, const double* g_iq, double* g_rot) {
  const double c[4] = {rot[0], -rot[1], -rot[2], -rot[3]};
  double gc[4] = {0, 0, 0, 0};
  normalize4_vjp(c, g_iq, gc);
  g_rot[0] += gc[0];
  g_rot[1] -= gc[1];
  g_rot[2] -= gc[2];
  g_rot[3] -= gc[3];
}
// inv_trans (utils.py:50-54)
inline void inv_trans(const double* p, const double* pos, const double* rot, double* out) {
  double iq[4];
  conj_normalized(rot, iq);
  const double d[3] = {p[0] - pos[0], p[1] - pos[1], p[2] - pos[2]};
  qrot(iq, d, out);
}
inline void inv_trans_vjp(const double* p, const double* pos, const double* rot, const double* g, double* g_p,
                          double* g_pos, double* g_rot) {
  double iq[4];
  conj_normalized(rot, iq);
  const double d[3] = {p[0] - pos[0], p[1] - pos[1], p[2] - pos[2]};
  double g_iq[4] = {0, 0, 0, 0}, g_d[3] = {0, 0, 0};
  qrot_vjp(iq, d, g, g_iq, g_d);
  for (int k = 0; k < 3; ++k) {
    if (g_p) g_p[k] += g_d[k];
    if (g_pos) g_pos[k] -= g_d[k];
  }
  if (g_rot) conj_normalized_vjp(rot, g_iq, g_rot);
}
// qmul (utils.py:23-31), Hamilton product q*r then normalised
inline void qmul_raw(const double* q, const double* r, double* o) {
  o[0] = r[0] * q[0] - r[1] * q[1] - r[2] * q[2] - r[3] * q[3];
  o[1] = r[0] * q[1] + r[1] * q[0] - r[2] * q[3] + r[3] * q[2];
  o[2] = r[0] * q[2] + r[1] * q[3] + r[2] * q[0] - r[3] * q[1];
  o[3] = r[0] * q[3] - r[1] * q[2] + r[2] * q[1] + r[3] * q[0];
}
inline void qmul(const double* q, const double* r, double* out) {
  double o[4];
  qmul_raw(q, r, o);
  double L = std::sqrt(o[0] * o[0] + o[1] * o[1] + o[2] * o[2] + o[3] * o[3]);
  for (int i = 0; i < 4; ++i) out[i] = o[i] / L;
}
inline void qmul_vjp(const double* q, const double* r, const double* g, double* gq, double* gr) {
  double o[4];
  qmul_raw(q, r, o);
  double L = std::sqrt(o[0] * o[0] + o[1] * o[1] + o[2] * o[2] + o[3] * o[3]);
  double go[4];
  double on = (o[0] * g[0] + o[1] * g[1] + o[2] * g[2] + o[3] * g[3]) / (L * L);
  for (int i = 0; i < 4; ++i) go[i] = g[i] / L - o[i] * on / L;
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
inline void w2quat(const double* aa, double* out) {
  double w = std::sqrt(dot3(aa, aa) + 1e-16);
  out[0] = 1.0;
  out[1] = out[2] = out[3] = 0.0;
  if (w > 1e-9) {
    double s = std::sin(w / 2);
    out[0] = std::cos(w / 2);
    for (int k = 0; k < 3; ++k) out[k + 1] = (aa[k] / w) * s;
  }
}
inline void w2quat_vjp(const double* aa, const double* g, double* gaa) {
  double w = std::sqrt(dot3(aa, aa) + 1e-16);
  if (!(w > 1e-9)) return;
  double s = std::sin(w / 2), c = std::cos(w / 2);
  double gw = -0.5 * s * g[0];
  for (int k = 0; k < 3; ++k) {
    gaa[k] += g[k + 1] * s / w;
    gw += g[k + 1] * aa[k] * (-s / (w * w) + 0.5 * c / w);
  }
  for (int k = 0; k < 3; ++k) gaa[k] += gw * aa[k] / w;
}

// ----------------------------------------------------------------------------
// local shape SDFs: plb/engine/primitive/primitives.py
// ----------------------------------------------------------------------------
enum { K_SPHERE = 0, K_CAPSULE = 1, K_BOX = 2, K_KNIFE = 3, K_CHOPSTICKS = 4, K_CYLINDER = 5, K_TORUS = 6 };
const double kFdStep = (double)(float)1e-4;  // d = ti.cast(1e-4, ti.float32) (primitives.py:385)

// Capsule (primitives.py:55-66)
inline void capsule_p2(const OracleTool& t, const double* q, double* p2, double* dp1) {
  p2[0] = q[0];
  p2[2] = q[2];
  double a = q[1] + t.cap_h / 2;
  double m1 = (0.0 < a) ? a : 0.0;
  double m2 = (m1 < t.cap_h) ? m1 : t.cap_h;
  p2[1] = a - m2;
  *dp1 = 1.0 - ((0.0 < a && m1 < t.cap_h) ? 1.0 : 0.0);
}
// Box (primitives.py:375-380)
inline double box_sdf(const double* size, const double* q) {
  double qq[3], mq[3];
  for (int k = 0; k < 3; ++k) {
    qq[k] = std::fabs(q[k]) - size[k];
    mq[k] = (0.0 < qq[k]) ? qq[k] : 0.0;
  }
  double out = len14(mq);
  double t = (qq[2] < qq[1]) ? qq[1] : qq[2];
  double u = (t < qq[0]) ? qq[0] : t;
  out += (u < 0.0) ? u : 0.0;
  return out;
}
inline void box_sdf_grad(const double* size, const double* q, double g, double* gq) {
  double qq[3], mq[3];
  for (int k = 0; k < 3; ++k) {
    qq[k] = std::fabs(q[k]) - size[k];
    mq[k] = (0.0 < qq[k]) ? qq[k] : 0.0;
  }
  double L = len14(mq);
  double gqq[3];
  for (int k = 0; k < 3; ++k) gqq[k] = (0.0 < qq[k]) ? g * mq[k] / L : 0.0;
  double t = (qq[2] < qq[1]) ? qq[1] : qq[2];
  double u = (t < qq[0]) ? qq[0] : t;
  if (u < 0.0) {
    if (t < qq[0]) gqq[0] += g;
    else if (qq[2] < qq[1]) gqq[1] += g;
    else gqq[2] += g;
  }
  for (int k = 0; k < 3; ++k) gq[k] += gqq[k] * sgn(q[k]);
}
// Prism (primitives.py:712-718)
inline double prism_sdf(const OracleTool& t, const double* q) {
  double iq[4], qq[3];
  conj_normalized(t.prot, iq);
  qrot(iq, q, qq);
  double A = std::fabs(qq[2]) - t.prism_h[1];
  double C = std::fabs(qq[0]) * 0.866025 + qq[1] * 0.5, D = -qq[1];
  double B = ((D < C) ? C : D) - t.prism_h[0] * 0.5;
  return (B < A) ? A : B;
}
inline void prism_sdf_grad(const OracleTool& t, const double* q, double g, double* gq) {
  double iq[4], qq[3];
  conj_normalized(t.prot, iq);
  qrot(iq, q, qq);
  double A = std::fabs(qq[2]) - t.prism_h[1];
  double C = std::fabs(qq[0]) * 0.866025 + qq[1] * 0.5, D = -qq[1];
  double B = ((D < C) ? C : D) - t.prism_h[0] * 0.5;
  double gA = 0, gB = 0;
  if (B < A) gA = g; else gB = g;
  double gC = 0, gD = 0;
  if (D < C) gC = gB; else gD = gB;
  double gqq[3] = {gC * 0.866025 * sgn(qq[0]), gC * 0.5 - gD, gA * sgn(qq[2])};
  qrot_vjp(iq, q, gqq, nullptr, gq);
}
// Knife (primitives.py:770-773): intersection of prism and box
inline double knife_sdf(const OracleTool& t, const double* q) {
  double a = prism_sdf(t, q), b = box_sdf(t.size, q);
  return (b < a) ? a : b;
}
inline void knife_sdf_grad(const OracleTool& t, const double* q, double g, double* gq) {
  double a = prism_sdf(t, q), b = box_sdf(t.size, q);
  if (b < a) prism_sdf_grad(t, q, g, gq);
  else box_sdf_grad(t.size, q, g, gq);
}

// Chopsticks, Cylinder and Torus: value and derivatives by forward-mode dual
// numbers with tangents (q0, q1, q2, gap).  Branches compare values, as the
// reference's autodiff freezes them.
struct Dual {
  double v;
  double d[4];
  Dual(double c = 0.0) : v(c), d{0, 0, 0, 0} {}
};
inline Dual seed(double c, int k) {
  Dual r(c);
  r.d[k] = 1.0;
  return r;
}
inline Dual operator+(const Dual& a, const Dual& b) {
  Dual r(a.v + b.v);
  for (int k = 0; k < 4; ++k) r.d[k] = a.d[k] + b.d[k];
  return r;
}
inline Dual operator-(const Dual& a, const Dual& b) {
  Dual r(a.v - b.v);
  for (int k = 0; k < 4; ++k) r.d[k] = a.d[k] - b.d[k];
  return r;
}
inline Dual operator*(const Dual& a, const Dual& b) {
  Dual r(a.v * b.v);
  for (int k = 0; k < 4; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
inline Dual operator/(const Dual& a, const Dual& b) {
  Dual r(a.v / b.v);
  for (int k = 0; k < 4; ++k) r.d[k] = (a.d[k] * b.v - a.v * b.d[k]) / (b.v * b.v);
  return r;
}
inline Dual dsqrt(const Dual& a) {
  Dual r(std::sqrt(a.v));
  for (int k = 0; k < 4; ++k) r.d[k] = a.d[k] / (2.0 * r.v);
  return r;
}
inline Dual dabs(const Dual& a) {  // abs' = sgn, 0 at 0
  Dual r(std::fabs(a.v));
  for (int k = 0; k < 4; ++k) r.d[k] = a.d[k] * sgn(a.v);
  return r;
}
inline Dual dlen(const Dual& a, const Dual& b) { return dsqrt(a * a + b * b + Dual(1e-14)); }
inline Dual dlen(const Dual& a, const Dual& b, const Dual& c) { return dsqrt(a * a + b * b + c * c + Dual(1e-14)); }
inline Dual dmax0(const Dual& a) { return (0.0 < a.v) ? a : Dual(0.0); }  // max(a, 0)

// Capsule._sdf on (x, y, z) with the segment [-h/2, h/2] on y (primitives.py:55-60)
inline Dual capsule_y(double h, const Dual& y) {
  Dual a = y + Dual(h / 2);
  Dual m1 = (0.0 < a.v) ? a : Dual(0.0);
  Dual m2 = (m1.v < h) ? m1 : Dual(h);
  return a - m2;
}
// Chopsticks._sdf (primitives.py:248-254): min of capsules at x -+ gap/2 around q + (0, h/2, 0)
inline Dual chop_sdf(const OracleTool& t, const Dual* q, const Dual& gap, bool* first) {
  Dual half = gap / Dual(2.0);
  Dual y = capsule_y(t.cap_h, q[1] + Dual(t.cap_h / 2));
  Dual xa = q[0] - half, xb = q[0] + half;
  Dual a = dlen(xa, y, q[2]) - Dual(t.cap_r), b = dlen(xb, y, q[2]) - Dual(t.cap_r);
  if (first) *first = a.v <= b.v;
  return (a.v < b.v) ? a : b;
}
inline void chop_normal(const OracleTool& t, const Dual* q, const Dual& gap, Dual* n) {
  bool first;
  chop_sdf(t, q, gap, &first);  // Chopsticks._normal (256-266): normal of the capsule with a <= b
  Dual half = gap / Dual(2.0);
  Dual x = first ? q[0] - half : q[0] + half;
  Dual y = capsule_y(t.cap_h, q[1] + Dual(t.cap_h / 2));
  Dual L = dlen(x, y, q[2]);
  n[0] = x / L;
  n[1] = y / L;
  n[2] = q[2] / L;
}
// Cylinder._sdf (primitives.py:300-303)
inline Dual cyl_sdf(const OracleTool& t, const Dual* q) {
  Dual d0 = dabs(dlen(q[0], q[2])) - Dual(t.cap_h);
  Dual d1 = dabs(q[1]) - Dual(t.cap_r);
  Dual mx = (d1.v < d0.v) ? d0 : d1;
  Dual in = (mx.v < 0.0) ? mx : Dual(0.0);
  return in + dlen(dmax0(d0), dmax0(d1));
}
// Cylinder._normal (primitives.py:306-321)
inline void cyl_normal(const OracleTool& t, const Dual* q, Dual* n) {
  Dual l = dlen(q[0], q[2]);
  Dual d0 = l - Dual(t.cap_h), d1 = dabs(q[1]) - Dual(t.cap_r);
  double f = (d0.v > d1.v) ? 1.0 : 0.0;
  double inside = (std::max(d0.v, d1.v) <= 0.0) ? 1.0 : 0.0;
  Dual a0 = dmax0(d0) + Dual(inside * f), a1 = dmax0(d1) + Dual(inside * (1.0 - f));
  Dual L2 = dlen(a0, a1);
  Dual n0 = a0 / L2, n1 = a1 / L2;
  double sy = (q[1].v >= 0.0) ? 1.0 : -1.0;
  Dual m0 = q[0] / l * n0, m1 = n1 * Dual(sy), m2 = q[2] / l * n0;
  Dual L3 = dlen(m0, m1, m2);
  n[0] = m0 / L3;
  n[1] = m1 / L3;
  n[2] = m2 / L3;
}
// Torus._sdf / _normal (primitives.py:336-350)
inline Dual torus_sdf(const OracleTool& t, const Dual* q) {
  return dlen(dlen(q[0], q[2]) - Dual(t.torus[0]), q[1]) - Dual(t.torus[1]);
}
inline void torus_normal(const OracleTool& t, const Dual* q, Dual* n) {
  Dual l = dlen(q[0], q[2]);
  Dual qa = dlen(q[0], q[2]) - Dual(t.torus[0]);
  Dual Lq = dlen(qa, q[1]);
  Dual n0 = qa / Lq, n1 = q[1] / Lq;
  Dual m0 = q[0] / l * n0, m2 = q[2] / l * n0;
  Dual L3 = dlen(m0, n1, m2);
  n[0] = m0 / L3;
  n[1] = n1 / L3;
  n[2] = m2 / L3;
}
inline Dual dual_sdf(const OracleTool& t, int kind, const double* q, double gap) {
  Dual qd[3] = {seed(q[0], 0), seed(q[1], 1), seed(q[2], 2)};
  Dual g = seed(gap, 3);
  if (kind == K_CHOPSTICKS) return chop_sdf(t, qd, g, nullptr);
  if (kind == K_CYLINDER) return cyl_sdf(t, qd);
  return torus_sdf(t, qd);
}
inline void dual_normal(const OracleTool& t, int kind, const double* q, double gap, Dual* n) {
  Dual qd[3] = {seed(q[0], 0), seed(q[1], 1), seed(q[2], 2)};
  Dual g = seed(gap, 3);
  if (kind == K_CHOPSTICKS) chop_normal(t, qd, g, n);
  else if (kind == K_CYLINDER) cyl_normal(t, qd, n);
  else torus_normal(t, qd, n);
}
inline bool is_dual_kind(int kind) { return kind == K_CHOPSTICKS || kind == K_CYLINDER || kind == K_TORUS; }

inline double local_sdf(const OracleTool& t, int kind, const double* q, double gap) {
  if (is_dual_kind(kind)) return dual_sdf(t, kind, q, gap).v;
  switch (kind) {
    case K_CAPSULE: {
      double p2[3], dp;
      capsule_p2(t, q, p2, &dp);
      return len14(p2) - t.cap_r;
    }
    case K_BOX: return box_sdf(t.size, q);
    default: return knife_sdf(t, q);
  }
}
inline void local_sdf_grad(const OracleTool& t, int kind, const double* q, double gap, double g, double* gq,
                           double* ggap) {
  if (is_dual_kind(kind)) {
    Dual r = dual_sdf(t, kind, q, gap);
    for (int k = 0; k < 3; ++k) gq[k] += g * r.d[k];
    if (ggap) *ggap += g * r.d[3];
    return;
  }
  switch (kind) {
    case K_CAPSULE: {
      double p2[3], dp;
      capsule_p2(t, q, p2, &dp);
      double L = len14(p2);
      gq[0] += g * p2[0] / L;
      gq[1] += g * p2[1] / L * dp;
      gq[2] += g * p2[2] / L;
      return;
    }
    case K_BOX: box_sdf_grad(t.size, q, g, gq); return;
    default: knife_sdf_grad(t, q, g, gq); return;
  }
}
// finite-difference normal of box / knife (primitives.py:383-393, 797-807)
inline void fd_normal_raw(const OracleTool& t, int kind, const double* q, double* n) {
  for (int i = 0; i < 3; ++i) {
    double inc[3] = {q[0], q[1], q[2]}, dec[3] = {q[0], q[1], q[2]};
    inc[i] += kFdStep;
    dec[i] -= kFdStep;
    n[i] = (0.5 / kFdStep) * (local_sdf(t, kind, inc, 0.0) - local_sdf(t, kind, dec, 0.0));
  }
}
inline void local_normal(const OracleTool& t, int kind, const double* q, double gap, double* n) {
  if (is_dual_kind(kind)) {
    Dual nd[3];
    dual_normal(t, kind, q, gap, nd);
    for (int k = 0; k < 3; ++k) n[k] = nd[k].v;
    return;
  }
  if (kind == K_CAPSULE) {
    double p2[3], dp;
    capsule_p2(t, q, p2, &dp);
    double L = len14(p2);
    for (int k = 0; k < 3; ++k) n[k] = p2[k] / L;
    return;
  }
  double r[3];
  fd_normal_raw(t, kind, q, r);
  double L = len14(r);
  for (int k = 0; k < 3; ++k) n[k] = r[k] / L;
}
// VJP of u / len14(u) w.r.t. u
inline void unit14_vjp(const double* u, const double* g, double* gu) {
  double L = len14(u);
  double ug = dot3(u, g);
  for (int k = 0; k < 3; ++k) gu[k] = g[k] / L - u[k] * ug / (L * L * L);
}
inline void local_normal_vjp(const OracleTool& t, int kind, const double* q, double gap, const double* gn,
                             double* gq, double* ggap) {
  if (is_dual_kind(kind)) {
    Dual nd[3];
    dual_normal(t, kind, q, gap, nd);
    for (int k = 0; k < 3; ++k) gq[k] += gn[0] * nd[0].d[k] + gn[1] * nd[1].d[k] + gn[2] * nd[2].d[k];
    if (ggap) *ggap += gn[0] * nd[0].d[3] + gn[1] * nd[1].d[3] + gn[2] * nd[2].d[3];
    return;
  }
  if (kind == K_CAPSULE) {
    double p2[3], dp;
    capsule_p2(t, q, p2, &dp);
    double gp2[3];
    unit14_vjp(p2, gn, gp2);
    gq[0] += gp2[0];
    gq[1] += gp2[1] * dp;
    gq[2] += gp2[2];
    return;
  }
  double r[3];
  fd_normal_raw(t, kind, q, r);
  double gr[3];
  unit14_vjp(r, gn, gr);
  for (int i = 0; i < 3; ++i) {
    double inc[3] = {q[0], q[1], q[2]}, dec[3] = {q[0], q[1], q[2]};
    inc[i] += kFdStep;
    dec[i] -= kFdStep;
    double c = (0.5 / kFdStep) * gr[i];
    local_sdf_grad(t, kind, inc, 0.0, c, gq, nullptr);
    local_sdf_grad(t, kind, dec, 0.0, -c, gq, nullptr);
  }
}

// ----------------------------------------------------------------------------
// world-space shapes with a rigid pose (pos, rot)
// ----------------------------------------------------------------------------
struct Pose {
  double pos[3];
  double rot[4];
  double gap = 0.0;  // only the Chopsticks shape depends on it
};
struct PoseGrad {
  double pos[3] = {0, 0, 0};
  double rot[4] = {0, 0, 0, 0};
  double gap = 0.0;
};

// Sphere.sdf / Sphere.normal (primitives.py:28-34): no rotation
// Primitive.sdf / Primitive.normal (primive_base.py:75-85) otherwise
inline double shape_sdf(const OracleTool& t, int kind, const Pose& P, const double* p) {
  if (kind == K_SPHERE) {
    const double d[3] = {p[0] - P.pos[0], p[1] - P.pos[1], p[2] - P.pos[2]};
    return len14(d) - t.radius;
  }
  double q[3];
  inv_trans(p, P.pos, P.rot, q);
  return local_sdf(t, kind, q, P.gap);
}
inline void shape_sdf_vjp(const OracleTool& t, int kind, const Pose& P, const double* p, double g, double* gp,
                          PoseGrad* gP) {
  if (kind == K_SPHERE) {
    const double d[3] = {p[0] - P.pos[0], p[1] - P.pos[1], p[2] - P.pos[2]};
    double L = len14(d);
    for (int k = 0; k < 3; ++k) {
      if (gp) gp[k] += g * d[k] / L;
      if (gP) gP->pos[k] -= g * d[k] / L;
    }
    return;
  }
  double q[3];
  inv_trans(p, P.pos, P.rot, q);
  double gq[3] = {0, 0, 0};
  local_sdf_grad(t, kind, q, P.gap, g, gq, gP ? &gP->gap : nullptr);
  inv_trans_vjp(p, P.pos, P.rot, gq, gp, gP ? gP->pos : nullptr, gP ? gP->rot : nullptr);
}
inline void shape_normal(const OracleTool& t, int kind, const Pose& P, const double* p, double* n) {
  if (kind == K_SPHERE) {
    const double d[3] = {p[0] - P.pos[0], p[1] - P.pos[1], p[2] - P.pos[2]};
    double L = len14(d);
    for (int k = 0; k < 3; ++k) n[k] = d[k] / L;
    return;
  }
  double q[3], nl[3];
  inv_trans(p, P.pos, P.rot, q);
  local_normal(t, kind, q, P.gap, nl);
  qrot(P.rot, nl, n);
}
// gp (the point's gradient) may be null
inline void shape_normal_vjp(const OracleTool& t, int kind, const Pose& P, const double* p, const double* gn,
                             PoseGrad* gP, double* gp = nullptr) {
  if (kind == K_SPHERE) {
    const double d[3] = {p[0] - P.pos[0], p[1] - P.pos[1], p[2] - P.pos[2]};
    double gd[3];
    unit14_vjp(d, gn, gd);
    for (int k = 0; k < 3; ++k) {
      gP->pos[k] -= gd[k];
      if (gp) gp[k] += gd[k];
    }
    return;
  }
  double q[3], nl[3];
  inv_trans(p, P.pos, P.rot, q);
  local_normal(t, kind, q, P.gap, nl);
  double gnl[3] = {0, 0, 0};
  qrot_vjp(P.rot, nl, gn, gP->rot, gnl);
  double gq[3] = {0, 0, 0};
  local_normal_vjp(t, kind, q, P.gap, gnl, gq, &gP->gap);
  inv_trans_vjp(p, P.pos, P.rot, gq, gp, gP->pos, gP->rot);
}
// collider_v (primive_base.py:87-94; Gripper.collider_v primitives.py:498-505)
inline void collider_v(const Pose& P0, const Pose& P1, const double* p, double dt, double* cv) {
  double iq[4], rel[3], nw[3];
  conj_normalized(P0.rot, iq);
  const double d[3] = {p[0] - P0.pos[0], p[1] - P0.pos[1], p[2] - P0.pos[2]};
  qrot(iq, d, rel);
  qrot(P1.rot, rel, nw);
  for (int k = 0; k < 3; ++k) cv[k] = (nw[k] + P1.pos[k] - p[k]) / dt;
}
inline void collider_v_vjp(const Pose& P0, const Pose& P1, const double* p, double dt, const double* g, PoseGrad* g0,
                           PoseGrad* g1) {
  double iq[4], rel[3];
  conj_normalized(P0.rot, iq);
  const double d[3] = {p[0] - P0.pos[0], p[1] - P0.pos[1], p[2] - P0.pos[2]};
  qrot(iq, d, rel);
  double gnw[3] = {g[0] / dt, g[1] / dt, g[2] / dt};
  for (int k = 0; k < 3; ++k) g1->pos[k] += gnw[k];
  double grel[3] = {0, 0, 0};
  qrot_vjp(P1.rot, rel, gnw, g1->rot, grel);
  double giq[4] = {0, 0, 0, 0}, gd[3] = {0, 0, 0};
  qrot_vjp(iq, d, grel, giq, gd);
  for (int k = 0; k < 3; ++k) g0->pos[k] -= gd[k];
  conj_normalized_vjp(P0.rot, giq, g0->rot);
}

// Primitive.collide (primive_base.py:96-120) / Gripper.collide2 (primitives.py:513-536)
struct CollideTape {
  bool active;
  double dist, infl, e;
  double D[3], cv[3], iv[3], nc, vt[3], vtn, a, flag;
};
inline void collide_fwd(const OracleTool& t, int kind, const Pose& P0, const Pose& P1, const double* p, double dt,
                        const double* vin, double* vout, CollideTape* tp) {
  CollideTape T;
  T.dist = shape_sdf(t, kind, P0, p);
  T.e = std::exp(-T.dist * t.softness);
  T.infl = (T.e < 1.0) ? T.e : 1.0;
  T.active = (t.softness > 0 && T.infl > 0.1) || T.dist <= 0;
  for (int k = 0; k < 3; ++k) vout[k] = vin[k];
  if (T.active) {
    shape_normal(t, kind, P0, p, T.D);
    collider_v(P0, P1, p, dt, T.cv);
    for (int k = 0; k < 3; ++k) T.iv[k] = vin[k] - T.cv[k];
    T.nc = dot3(T.iv, T.D);
    double mn = (T.nc < 0.0) ? T.nc : 0.0;
    for (int k = 0; k < 3; ++k) T.vt[k] = T.iv[k] - mn * T.D[k];
    T.vtn = len8(T.vt);
    T.a = T.vtn + T.nc * t.friction;
    double m = (T.a < 0.0) ? 0.0 : T.a;  // max(0, a): the constant 0 wins iff a < 0
    T.flag = (T.nc < 0 && std::sqrt(dot3(T.vt, T.vt)) > 1e-30) ? 1.0 : 0.0;
    for (int k = 0; k < 3; ++k) {
      double vtf = T.vt[k] / T.vtn * m;
      double vt2 = vtf * T.flag + T.vt[k] * (1 - T.flag);
      vout[k] = T.cv[k] + T.iv[k] * (1 - T.infl) + vt2 * T.infl;
    }
  }
  if (tp) *tp = T;
}
inline void collide_vjp(const OracleTool& t, int kind, const Pose& P0, const Pose& P1, const double* p, double dt,
                        const double* vin, const double* gout, double* gvin, PoseGrad* g0, PoseGrad* g1) {
  CollideTape T;
  double vout[3];
  collide_fwd(t, kind, P0, P1, p, dt, vin, vout, &T);
  if (!T.active) {
    for (int k = 0; k < 3; ++k) gvin[k] = gout[k];
    return;
  }
  double m = (T.a < 0.0) ? 0.0 : T.a;
  double g_cv[3], g_iv[3], g_vt2[3], g_infl = 0;
  for (int k = 0; k < 3; ++k) {
    double vtf = T.vt[k] / T.vtn * m;
    double vt2 = vtf * T.flag + T.vt[k] * (1 - T.flag);
    g_cv[k] = gout[k];
    g_iv[k] = gout[k] * (1 - T.infl);
    g_infl += gout[k] * (vt2 - T.iv[k]);
    g_vt2[k] = gout[k] * T.infl;
  }
  double g_vt[3], g_vtf[3];
  for (int k = 0; k < 3; ++k) {
    g_vtf[k] = g_vt2[k] * T.flag;
    g_vt[k] = g_vt2[k] * (1 - T.flag);
  }
  // vtf = vt / vtn * m
  double g_vtn = 0, g_nc = 0;
  double gvtf_vt = dot3(g_vtf, T.vt);
  for (int k = 0; k < 3; ++k) g_vt[k] += g_vtf[k] * m / T.vtn;
  g_vtn += -gvtf_vt * m / (T.vtn * T.vtn);
  double g_m = gvtf_vt / T.vtn;
  if (!(T.a < 0.0)) {
    g_vtn += g_m;
    g_nc += g_m * t.friction;
  }
  // vtn = sqrt(vt.vt + 1e-8)
  for (int k = 0; k < 3; ++k) g_vt[k] += g_vtn * T.vt[k] / T.vtn;
  // vt = iv - min(nc, 0) D
  double g_D[3] = {0, 0, 0};
  for (int k = 0; k < 3; ++k) g_iv[k] += g_vt[k];
  if (T.nc < 0.0) {
    g_nc -= dot3(g_vt, T.D);
    for (int k = 0; k < 3; ++k) g_D[k] -= T.nc * g_vt[k];
  }
  // nc = iv . D
  for (int k = 0; k < 3; ++k) {
    g_iv[k] += g_nc * T.D[k];
    g_D[k] += g_nc * T.iv[k];
  }
  // iv = vin - cv
  for (int k = 0; k < 3; ++k) {
    gvin[k] = g_iv[k];
    g_cv[k] -= g_iv[k];
  }
  // infl = min(exp(-dist s), 1)
  double g_dist = 0;
  if (T.e < 1.0) g_dist = g_infl * T.e * (-t.softness);
  shape_sdf_vjp(t, kind, P0, p, g_dist, nullptr, g0);
  shape_normal_vjp(t, kind, P0, p, g_D, g0);
  collider_v_vjp(P0, P1, p, dt, g_cv, g0, g1);
}

// Gripper finger pose (primitives.py:475-477): pos + qrot(rot, (gap/2*flag, 0, 0))
inline Pose finger_pose(const double* pose8, double flag) {
  Pose F;
  const double lv[3] = {pose8[7] / 2 * flag, 0, 0};
  double off[3];
  qrot(pose8 + 3, lv, off);
  for (int k = 0; k < 3; ++k) F.pos[k] = pose8[k] + off[k];
  for (int k = 0; k < 4; ++k) F.rot[k] = pose8[3 + k];
  return F;
}
inline void finger_pose_vjp(const double* pose8, double flag, const PoseGrad& gF, double* gpose8) {
  const double lv[3] = {pose8[7] / 2 * flag, 0, 0};
  double glv[3] = {0, 0, 0};
  for (int k = 0; k < 3; ++k) gpose8[k] += gF.pos[k];
  for (int k = 0; k < 4; ++k) gpose8[3 + k] += gF.rot[k];
  qrot_vjp(pose8 + 3, lv, gF.pos, gpose8 + 3, glv);
  gpose8[7] += glv[0] * flag / 2;
}
inline Pose rigid_pose(const double* pose8) {
  Pose P;
  for (int k = 0; k < 3; ++k) P.pos[k] = pose8[k];
  for (int k = 0; k < 4; ++k) P.rot[k] = pose8[3 + k];
  P.gap = pose8[7];
  return P;
}
inline void add_pose_grad(const PoseGrad& g, double* gpose8) {
  for (int k = 0; k < 3; ++k) gpose8[k] += g.pos[k];
  for (int k = 0; k < 4; ++k) gpose8[3 + k] += g.rot[k];
  gpose8[7] += g.gap;
}
inline int tool_kind(const OracleTool& t) {
  switch (t.type) {
    case T_SPHERE: return K_SPHERE;
    case T_CAPSULE:
    case T_ROLLINGPIN:
    case T_ROLLINGPINEXT:
    case T_GRIPPER2: return K_CAPSULE;  // Gripper2 fingers are capsules
    case T_KNIFE: return K_KNIFE;
    case T_CHOPSTICKS: return K_CHOPSTICKS;
    case T_CYLINDER: return K_CYLINDER;
    case T_TORUS: return K_TORUS;
    default: return K_BOX;  // box and gripper fingers
  }
}

// full tool collide in world space (grid_op, mpm_simulator.py:237-239)
inline void tool_collide(const OracleTool& t, const double* pose0, const double* pose1, const double* p, double dt,
                         const double* vin, double* vout) {
  int kind = tool_kind(t);
  if (is_fingered(t.type)) {
    double mid[3];
    collide_fwd(t, kind, finger_pose(pose0, -1), finger_pose(pose1, -1), p, dt, vin, mid, nullptr);
    collide_fwd(t, kind, finger_pose(pose0, 1), finger_pose(pose1, 1), p, dt, mid, vout, nullptr);
  } else {
    collide_fwd(t, kind, rigid_pose(pose0), rigid_pose(pose1), p, dt, vin, vout, nullptr);
  }
}
inline void tool_collide_vjp(const OracleTool& t, const double* pose0, const double* pose1, const double* p, double dt,
                             const double* vin, const double* gout, double* gvin, double* gpose0, double* gpose1) {
  int kind = tool_kind(t);
  if (is_fingered(t.type)) {
    double mid[3];
    Pose A0 = finger_pose(pose0, -1), A1 = finger_pose(pose1, -1);
    Pose B0 = finger_pose(pose0, 1), B1 = finger_pose(pose1, 1);
    collide_fwd(t, kind, A0, A1, p, dt, vin, mid, nullptr);
    double gmid[3];
    PoseGrad gB0, gB1, gA0, gA1;
    collide_vjp(t, kind, B0, B1, p, dt, mid, gout, gmid, &gB0, &gB1);
    collide_vjp(t, kind, A0, A1, p, dt, vin, gmid, gvin, &gA0, &gA1);
    finger_pose_vjp(pose0, 1, gB0, gpose0);
    finger_pose_vjp(pose1, 1, gB1, gpose1);
    finger_pose_vjp(pose0, -1, gA0, gpose0);
    finger_pose_vjp(pose1, -1, gA1, gpose1);
  } else {
    PoseGrad g0, g1;
    collide_vjp(t, kind, rigid_pose(pose0), rigid_pose(pose1), p, dt, vin, gout, gvin, &g0, &g1);
    add_pose_grad(g0, gpose0);
    add_pose_grad(g1, gpose1);
  }
}
// world SDF of a tool (Gripper.sdf = min of fingers, primitives.py:486-487)
inline double tool_sdf(const OracleTool& t, const double* pose, const double* p) {
  int kind = tool_kind(t);
  if (is_fingered(t.type)) {
    double a = shape_sdf(t, kind, finger_pose(pose, -1), p);
    double b = shape_sdf(t, kind, finger_pose(pose, 1), p);
    return (a < b) ? a : b;
  }
  return shape_sdf(t, kind, rigid_pose(pose), p);
}
inline void tool_sdf_vjp(const OracleTool& t, const double* pose, const double* p, double g, double* gp,
                         double* gpose) {
  int kind = tool_kind(t);
  if (is_fingered(t.type)) {
    Pose A = finger_pose(pose, -1), B = finger_pose(pose, 1);
    double a = shape_sdf(t, kind, A, p), b = shape_sdf(t, kind, B, p);
    PoseGrad gF;
    if (a < b) {
      shape_sdf_vjp(t, kind, A, p, g, gp, &gF);
      finger_pose_vjp(pose, -1, gF, gpose);
    } else {
      shape_sdf_vjp(t, kind, B, p, g, gp, &gF);
      finger_pose_vjp(pose, 1, gF, gpose);
    }
    return;
  }
  PoseGrad gP;
  shape_sdf_vjp(t, kind, rigid_pose(pose), p, g, gp, &gP);
  if (gpose) add_pose_grad(gP, gpose);
}
// world normal (Gripper.normal picks the nearer finger, primitives.py:489-496)
inline void tool_normal(const OracleTool& t, const double* pose, const double* p, double* n) {
  int kind = tool_kind(t);
  if (is_fingered(t.type)) {
    Pose A = finger_pose(pose, -1), B = finger_pose(pose, 1);
    double a = shape_sdf(t, kind, A, p), b = shape_sdf(t, kind, B, p);
    double na[3], nb[3];
    shape_normal(t, kind, A, p, na);
    shape_normal(t, kind, B, p, nb);
    double m = (a <= b) ? 1.0 : 0.0;
    for (int k = 0; k < 3; ++k) n[k] = m * na[k] + (1 - m) * nb[k];
    return;
  }
  shape_normal(t, kind, rigid_pose(pose), p, n);
}
inline void tool_normal_vjp(const OracleTool& t, const double* pose, const double* p, const double* gn, double* gp,
                            double* gpose) {
  int kind = tool_kind(t);
  if (is_fingered(t.type)) {
    Pose A = finger_pose(pose, -1), B = finger_pose(pose, 1);
    double a = shape_sdf(t, kind, A, p), b = shape_sdf(t, kind, B, p);
    PoseGrad gF;
    shape_normal_vjp(t, kind, a <= b ? A : B, p, gn, &gF, gp);
    finger_pose_vjp(pose, a <= b ? -1.0 : 1.0, gF, gpose);
    return;
  }
  PoseGrad gP;
  shape_normal_vjp(t, kind, rigid_pose(pose), p, gn, &gP, gp);
  add_pose_grad(gP, gpose);
}

// ----------------------------------------------------------------------------
// 3x3 SVD: one-sided Jacobi on A^T A (Golub & Van Loan, Alg. 8.4.3 style
// symmetric Schur rotations), then U by Gram-Schmidt of A V.
// Convention (that of ti.svd): A = U diag(s) V^T, det U = det V = +1,
// s0 >= s1 >= |s2|, s2 carries the sign of det A.
// ----------------------------------------------------------------------------
void svd3(const double* A, double* U, double* s, double* V) {
  double S[9];
  mTm(A, A, S);
  double Vm[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  for (int sweep = 0; sweep < 40; ++sweep) {
    double off = S[1] * S[1] + S[2] * S[2] + S[5] * S[5];
    double diag = S[0] * S[0] + S[4] * S[4] + S[8] * S[8];
    if (off <= 1e-40 * diag || off == 0.0) break;
    static const int P[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (int r = 0; r < 3; ++r) {
      int p = P[r][0], q = P[r][1];
      double apq = S[p * 3 + q];
      if (apq == 0.0) continue;
      double app = S[p * 3 + p], aqq = S[q * 3 + q];
      double theta = (aqq - app) / (2.0 * apq);
      double tt = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
      double c = 1.0 / std::sqrt(tt * tt + 1.0), sn = tt * c;
      // S <- J^T S J, J = rotation in (p,q)
      for (int k = 0; k < 3; ++k) {
        double skp = S[k * 3 + p], skq = S[k * 3 + q];
        S[k * 3 + p] = c * skp - sn * skq;
        S[k * 3 + q] = sn * skp + c * skq;
      }
      for (int k = 0; k < 3; ++k) {
        double spk = S[p * 3 + k], sqk = S[q * 3 + k];
        S[p * 3 + k] = c * spk - sn * sqk;
        S[q * 3 + k] = sn * spk + c * sqk;
      }
      for (int k = 0; k < 3; ++k) {
        double vkp = Vm[k * 3 + p], vkq = Vm[k * 3 + q];
        Vm[k * 3 + p] = c * vkp - sn * vkq;
        Vm[k * 3 + q] = sn * vkp + c * vkq;
      }
    }
  }
  // sort eigenvalues descending, permuting columns of V
  int idx[3] = {0, 1, 2};
  double ev[3] = {S[0], S[4], S[8]};
  std::sort(idx, idx + 3, [&](int a, int b) { return ev[a] > ev[b]; });
  double Vs[9];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) Vs[r * 3 + c] = Vm[r * 3 + idx[c]];
  if (det3(Vs) < 0)
    for (int r = 0; r < 3; ++r) Vs[r * 3 + 2] = -Vs[r * 3 + 2];
  double B[9];
  mm(A, Vs, B);
  double b0[3] = {B[0], B[3], B[6]}, b1[3] = {B[1], B[4], B[7]}, b2[3] = {B[2], B[5], B[8]};
  double u0[3], u1[3], u2[3];
  double n0 = std::sqrt(dot3(b0, b0));
  if (n0 > 1e-300) {
    for (int k = 0; k < 3; ++k) u0[k] = b0[k] / n0;
  } else {
    u0[0] = 1; u0[1] = 0; u0[2] = 0;
  }
  double pr = dot3(u0, b1);
  double r1[3] = {b1[0] - pr * u0[0], b1[1] - pr * u0[1], b1[2] - pr * u0[2]};
  double n1 = std::sqrt(dot3(r1, r1));
  if (n1 > 1e-300) {
    for (int k = 0; k < 3; ++k) u1[k] = r1[k] / n1;
  } else {
    // any unit vector orthogonal to u0
    double e[3] = {0, 0, 0};
    int m = (std::fabs(u0[0]) < std::fabs(u0[1])) ? 0 : 1;
    if (std::fabs(u0[2]) < std::fabs(u0[m])) m = 2;
    e[m] = 1;
    double pe = dot3(u0, e);
    for (int k = 0; k < 3; ++k) r1[k] = e[k] - pe * u0[k];
    double ne = std::sqrt(dot3(r1, r1));
    for (int k = 0; k < 3; ++k) u1[k] = r1[k] / ne;
  }
  cross3(u0, u1, u2);
  s[0] = n0;
  s[1] = dot3(u1, b1);
  s[2] = dot3(u2, b2);
  for (int r = 0; r < 3; ++r) {
    U[r * 3 + 0] = u0[r];
    U[r * 3 + 1] = u1[r];
    U[r * 3 + 2] = u2[r];
  }
  std::memcpy(V, Vs, sizeof(Vs));
}

// clamp (mpm_simulator.py:184-192)
inline double svd_clamp(double a) { return a >= 0 ? std::max(a, 1e-6) : std::min(a, -1e-6); }

// backward_svd (mpm_simulator.py:137-156); gs is the diagonal of sig.grad
void svd3_bwd(const double* U, const double* s, const double* V, const double* gU, const double* gs,
              const double* gV, double* gA) {
  double ss[3] = {s[0] * s[0], s[1] * s[1], s[2] * s[2]};
  double Fm[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Fm[i * 3 + j] = (i == j) ? 0.0 : 1.0 / svd_clamp(ss[j] - ss[i]);
  double UtgU[9], gUtU[9], VtgV[9], gVtV[9];
  mTm(U, gU, UtgU);
  mTm(gU, U, gUtU);
  mTm(V, gV, VtgV);
  mTm(gV, V, gVtV);
  double X[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      int k = i * 3 + j;
      // ((F o (U^T gU - gU^T U)) sig)_ij + (sig (F o (V^T gV - gV^T V)))_ij
      X[k] = Fm[k] * (UtgU[k] - gUtU[k]) * s[j] + s[i] * Fm[k] * (VtgV[k] - gVtV[k]);
    }
  for (int i = 0; i < 3; ++i) X[i * 3 + i] += gs[i];
  double T1[9];
  mm(U, X, T1);
  mmT(T1, V, gA);
}

// ----------------------------------------------------------------------------
// particle stages
// ----------------------------------------------------------------------------
struct Stencil {
  int base[3];
  double fx[3];
  double w[3][3];   // w[k][d]
  double dw[3][3];  // d w[k][d] / d fx[d]
};
inline void make_stencil(const OracleSim& S, const double* x, Stencil& st) {
  for (int d = 0; d < 3; ++d) {
    double t = x[d] * S.inv_dx - 0.5;
    st.base[d] = (int)t;  // cast(int) truncates toward zero
    st.fx[d] = x[d] * S.inv_dx - (double)st.base[d];
    double f = st.fx[d];
    st.w[0][d] = 0.5 * (1.5 - f) * (1.5 - f);
    st.w[1][d] = 0.75 - (f - 1) * (f - 1);
    st.w[2][d] = 0.5 * (f - 0.5) * (f - 0.5);
    st.dw[0][d] = -(1.5 - f);
    st.dw[1][d] = -2.0 * (f - 1);
    st.dw[2][d] = (f - 0.5);
  }
}
inline bool stencil_ok(const OracleSim& S, const Stencil& st) {
  for (int d = 0; d < 3; ++d)
    if (st.base[d] < 0 || st.base[d] + 2 >= S.n_grid) return false;
  return true;
}
inline int64_t node_index(int n, int i, int j, int k) { return ((int64_t)i * n + j) * n + k; }

// p2g particle math (mpm_simulator.py:122-129, 166-182, 199-215)
struct P2GTape {
  double Ftmp[9], U[9], s[3], V[9];
  double sigc[3], eps[3], ehat[3], nrm, dg, k, e[3];
  bool yield;
  double newF[9], J, R[9], affine[9];
};
inline void p2g_particle(const OracleSim& S, const double* row, P2GTape& T) {
  const double* C = row + 6;
  const double* F = row + 15;
  double IC[9];
  for (int i = 0; i < 9; ++i) IC[i] = S.dt * C[i];
  IC[0] += 1;
  IC[4] += 1;
  IC[8] += 1;
  mm(IC, F, T.Ftmp);
  svd3(T.Ftmp, T.U, T.s, T.V);
  double sum = 0;
  for (int i = 0; i < 3; ++i) {
    T.sigc[i] = (0.05 < T.s[i]) ? T.s[i] : 0.05;
    T.eps[i] = std::log(T.sigc[i]);
    sum += T.eps[i];
  }
  for (int i = 0; i < 3; ++i) T.ehat[i] = T.eps[i] - sum / 3.0;
  T.nrm = std::sqrt(dot3(T.ehat, T.ehat) + 1e-8);
  T.dg = T.nrm - S.yield_stress / (2 * S.mu);
  T.yield = T.dg > 0;
  if (T.yield) {
    T.k = T.dg / T.nrm;
    double UD[9];
    for (int i = 0; i < 3; ++i) T.e[i] = std::exp(T.eps[i] - T.k * T.ehat[i]);
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) UD[r * 3 + c] = T.U[r * 3 + c] * T.e[c];
    mmT(UD, T.V, T.newF);
  } else {
    T.k = 0;
    std::memcpy(T.newF, T.Ftmp, sizeof(T.newF));
  }
  T.J = det3(T.newF);
  mmT(T.U, T.V, T.R);
  double A[9], st[9];
  for (int i = 0; i < 9; ++i) A[i] = T.newF[i] - T.R[i];
  mmT(A, T.newF, st);
  double ks = -S.dt * S.p_vol * 4 * S.inv_dx * S.inv_dx;
  for (int i = 0; i < 9; ++i) {
    double v = 2 * S.mu * st[i];
    if (i % 4 == 0) v += S.lam * T.J * (T.J - 1);
    T.affine[i] = ks * v + S.p_mass * C[i];
  }
}
// adjoint of p2g_particle given g_affine and g_newF; accumulates g_C and g_F
inline void p2g_particle_vjp(const OracleSim& S, const double* row, const P2GTape& T, const double* g_affine,
                             const double* g_newF_in, double* g_C, double* g_F) {
  const double* C = row + 6;
  const double* F = row + 15;
  double ks = -S.dt * S.p_vol * 4 * S.inv_dx * S.inv_dx;
  double g_raw[9];
  for (int i = 0; i < 9; ++i) {
    g_raw[i] = ks * g_affine[i];
    g_C[i] += S.p_mass * g_affine[i];
  }
  double A[9];
  for (int i = 0; i < 9; ++i) A[i] = T.newF[i] - T.R[i];
  double g_newF[9], g_R[9], tmp[9];
  // (A newF^T): g_A = g newF, g_newF = g^T A
  mm(g_raw, T.newF, tmp);
  double g_A[9];
  for (int i = 0; i < 9; ++i) g_A[i] = 2 * S.mu * tmp[i];
  mTm(g_raw, A, tmp);
  for (int i = 0; i < 9; ++i) {
    g_newF[i] = 2 * S.mu * tmp[i] + g_A[i] + g_newF_in[i];
    g_R[i] = -g_A[i];
  }
  double g_J = S.lam * (2 * T.J - 1) * (g_raw[0] + g_raw[4] + g_raw[8]);
  double cf[9];
  cof3(T.newF, cf);
  for (int i = 0; i < 9; ++i) g_newF[i] += g_J * cf[i];
  double gU[9] = {0}, gV[9] = {0}, gs[3] = {0, 0, 0}, g_Ftmp[9] = {0};
  // R = U V^T
  mm(g_R, T.V, tmp);
  for (int i = 0; i < 9; ++i) gU[i] += tmp[i];
  mTm(g_R, T.U, tmp);
  for (int i = 0; i < 9; ++i) gV[i] += tmp[i];
  if (T.yield) {
    // newF = U diag(e) V^T
    double GV[9], GtU[9], UtGV[9];
    mm(g_newF, T.V, GV);
    mTm(g_newF, T.U, GtU);
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        gU[r * 3 + c] += GV[r * 3 + c] * T.e[c];
        gV[r * 3 + c] += GtU[r * 3 + c] * T.e[c];
      }
    mTm(T.U, GV, UtGV);
    double g_eps2[3], g_eps[3], g_ehat[3];
    for (int i = 0; i < 3; ++i) g_eps2[i] = UtGV[i * 4] * T.e[i];
    double g_k = 0;
    for (int i = 0; i < 3; ++i) {
      g_eps[i] = g_eps2[i];
      g_k -= g_eps2[i] * T.ehat[i];
      g_ehat[i] = -T.k * g_eps2[i];
    }
    double g_dg = g_k / T.nrm;
    double g_nrm = -g_k * T.dg / (T.nrm * T.nrm) + g_dg;
    for (int i = 0; i < 3; ++i) g_ehat[i] += g_nrm * T.ehat[i] / T.nrm;
    double sh = (g_ehat[0] + g_ehat[1] + g_ehat[2]) / 3.0;
    for (int i = 0; i < 3; ++i) {
      g_eps[i] += g_ehat[i] - sh;
      double g_sigc = g_eps[i] / T.sigc[i];
      gs[i] = (0.05 < T.s[i]) ? g_sigc : 0.0;
    }
  } else {
    for (int i = 0; i < 9; ++i) g_Ftmp[i] += g_newF[i];
  }
  double gA[9];
  svd3_bwd(T.U, T.s, T.V, gU, gs, gV, gA);
  for (int i = 0; i < 9; ++i) g_Ftmp[i] += gA[i];
  // Ftmp = (I + dt C) F
  mmT(g_Ftmp, F, tmp);
  for (int i = 0; i < 9; ++i) g_C[i] += S.dt * tmp[i];
  double IC[9];
  for (int i = 0; i < 9; ++i) IC[i] = S.dt * C[i];
  IC[0] += 1;
  IC[4] += 1;
  IC[8] += 1;
  mTm(IC, g_Ftmp, tmp);
  for (int i = 0; i < 9; ++i) g_F[i] += tmp[i];
}

// Deterministic scatter: particles bucketed by base x; each x-plane of the
// grid is written by exactly one task, in bucket order, so the sums do not
// depend on the thread count.
struct Buckets {
  std::vector<int64_t> start, order;
};
void bucket_by_x(int n_grid, int64_t n, const std::vector<Stencil>& st, Buckets& B) {
  B.start.assign(n_grid + 1, 0);
  for (int64_t p = 0; p < n; ++p) B.start[st[p].base[0] + 1]++;
  for (int i = 0; i < n_grid; ++i) B.start[i + 1] += B.start[i];
  std::vector<int64_t> fill(B.start.begin(), B.start.end() - 1);
  B.order.resize(n);
  for (int64_t p = 0; p < n; ++p) B.order[fill[st[p].base[0]]++] = p;
}
template <class Fn>
void scatter_planes(int n_grid, const Buckets& B, Fn&& fn) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int X = 0; X < n_grid; ++X) {
    for (int bx = X - 2; bx <= X; ++bx) {
      if (bx < 0 || bx >= n_grid) continue;
      int ox = X - bx;
      for (int64_t i = B.start[bx]; i < B.start[bx + 1]; ++i) fn(B.order[i], ox);
    }
  }
}

// grid_op (mpm_simulator.py:230-262) for one node; optional per-stage tape
struct NodeTape {
  double v_tools[9][3];  // velocity entering tool t (index t), and after last tool
  double v_pre[3][3];    // before lower wall test of dim d
  double v_mid[3][3];    // after lower, before upper test of dim d
  bool low[3], up[3];
};
inline void grid_node(const OracleSim& S, const OracleTool* tools, int T, const double* pose_f, const double* pose_f1,
                      const int* I, const double* mv, double m, double* vout, NodeTape* tp) {
  double v[3];
  for (int k = 0; k < 3; ++k) v[k] = (1.0 / m) * mv[k] + S.dt * S.gravity[k] * 30;
  const double p[3] = {I[0] * S.dx, I[1] * S.dx, I[2] * S.dx};
  for (int t = 0; t < T; ++t) {
    if (tp) std::memcpy(tp->v_tools[t], v, sizeof(v));
    double nv[3];
    tool_collide(tools[t], pose_f + 8 * t, pose_f1 + 8 * t, p, S.dt, v, nv);
    std::memcpy(v, nv, sizeof(v));
  }
  if (tp) std::memcpy(tp->v_tools[T], v, sizeof(v));
  const int bound = 3;
  for (int d = 0; d < 3; ++d) {
    if (tp) std::memcpy(tp->v_pre[d], v, sizeof(v));
    bool low = I[d] < bound && v[d] < 0;
    if (tp) tp->low[d] = low;
    if (low) {
      if (d != 1 || S.ground_friction == 0) {
        v[d] = 0;
      } else if (S.ground_friction < 10) {
        double lin = v[1] + 1e-30;
        double vit[3] = {v[0] - I[0] * 1e-30, v[1] - lin - I[1] * 1e-30, v[2] - I[2] * 1e-30};
        double lit = std::sqrt(dot3(vit, vit) + 1e-8);
        double a = 1.0 + S.ground_friction * lin / lit;
        double fac = (0.0 < a) ? a : 0.0;
        for (int k = 0; k < 3; ++k) v[k] = fac * (vit[k] + I[k] * 1e-30);
        v[1] = 0;
      } else {
        v[0] = v[1] = v[2] = 0;
      }
    }
    if (tp) std::memcpy(tp->v_mid[d], v, sizeof(v));
    bool up = I[d] > S.n_grid - bound && v[d] > 0;
    if (tp) tp->up[d] = up;
    if (up) v[d] = 0;
  }
  std::memcpy(vout, v, sizeof(v));
}
inline void grid_node_vjp(const OracleSim& S, const OracleTool* tools, int T, const double* pose_f,
                          const double* pose_f1, const int* I, const double* mv, double m, const double* gout,
                          double* g_mv, double* g_m, double* g_pose_f, double* g_pose_f1) {
  NodeTape tp;
  double vout[3];
  grid_node(S, tools, T, pose_f, pose_f1, I, mv, m, vout, &tp);
  double g[3] = {gout[0], gout[1], gout[2]};
  for (int d = 2; d >= 0; --d) {
    if (tp.up[d]) g[d] = 0;
    if (tp.low[d]) {
      if (d != 1 || S.ground_friction == 0) {
        g[d] = 0;
      } else if (S.ground_friction < 10) {
        const double* v = tp.v_pre[d];
        double lin = v[1] + 1e-30;
        double vit[3] = {v[0] - I[0] * 1e-30, v[1] - lin - I[1] * 1e-30, v[2] - I[2] * 1e-30};
        double lit = std::sqrt(dot3(vit, vit) + 1e-8);
        double a = 1.0 + S.ground_friction * lin / lit;
        double fac = (0.0 < a) ? a : 0.0;
        double go[3] = {g[0], 0.0, g[2]};  // v[1] = 0 overwrote the y output
        double w[3] = {vit[0] + I[0] * 1e-30, vit[1] + I[1] * 1e-30, vit[2] + I[2] * 1e-30};
        double g_fac = dot3(go, w);
        double g_vit[3] = {fac * go[0], fac * go[1], fac * go[2]};
        double g_lin = 0, g_lit = 0;
        if (0.0 < a) {
          g_lin += g_fac * S.ground_friction / lit;
          g_lit += -g_fac * S.ground_friction * lin / (lit * lit);
        }
        for (int k = 0; k < 3; ++k) g_vit[k] += g_lit * vit[k] / lit;
        double gv[3] = {g_vit[0], g_vit[1], g_vit[2]};
        g_lin -= g_vit[1];
        gv[1] += g_lin;
        std::memcpy(g, gv, sizeof(g));
      } else {
        g[0] = g[1] = g[2] = 0;
      }
    }
  }
  const double p[3] = {I[0] * S.dx, I[1] * S.dx, I[2] * S.dx};
  for (int t = T - 1; t >= 0; --t) {
    double gin[3];
    tool_collide_vjp(tools[t], pose_f + 8 * t, pose_f1 + 8 * t, p, S.dt, tp.v_tools[t], g, gin, g_pose_f + 8 * t,
                     g_pose_f1 + 8 * t);
    std::memcpy(g, gin, sizeof(g));
  }
  double inv = 1.0 / m;
  for (int k = 0; k < 3; ++k) g_mv[k] = g[k] * inv;
  *g_m = -dot3(g, mv) / (m * m);
}

void check_stencils(const OracleSim& S, const std::vector<Stencil>& st, int* err) {
  for (size_t p = 0; p < st.size(); ++p)
    if (!stencil_ok(S, st[p])) *err = 1;
}

}  // namespace

// ============================================================================
// C ABI (ctypes) -- oracle entry points
// ============================================================================
extern "C" {

int oracle_num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void oracle_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

void oracle_svd(const double* A, double* U, double* s, double* V) { svd3(A, U, s, V); }
void oracle_svd_bwd(const double* U, const double* s, const double* V, const double* gU, const double* gs,
                    const double* gV, double* gA) {
  svd3_bwd(U, s, V, gU, gs, gV, gA);
}

// SDF and normal of one tool at m points (tests, contact loss)
void oracle_tool_sdf(const OracleTool* tool, const double* pose, int64_t m, const double* pts, double* sdf,
                     double* normal) {
  for (int64_t i = 0; i < m; ++i) {
    if (sdf) sdf[i] = tool_sdf(*tool, pose, pts + 3 * i);
    if (normal) tool_normal(*tool, pose, pts + 3 * i, normal + 3 * i);
  }
}
void oracle_tool_sdf_vjp(const OracleTool* tool, const double* pose, int64_t m, const double* pts, const double* g,
                         double* g_pts, double* g_pose) {
  for (int64_t i = 0; i < m; ++i) tool_sdf_vjp(*tool, pose, pts + 3 * i, g[i], g_pts + 3 * i, g_pose);
}
// per-point distance columns of one tool (GradModel.compute_min_dist,
// function.py:79-89): Gripper -> two columns (sdf_2 with flag -1, +1,
// primitives.py:479-483), other tools -> one column (sdf).  out: [m][ncol].
int oracle_tool_distance_cols(const OracleTool* tool) { return is_fingered(tool->type) ? 2 : 1; }
void oracle_tool_distance(const OracleTool* tool, const double* pose, int64_t m, const double* pts, double* out) {
  const int nc = oracle_tool_distance_cols(tool);
  for (int64_t i = 0; i < m; ++i) {
    if (is_fingered(tool->type)) {
      out[i * nc] = shape_sdf(*tool, tool_kind(*tool), finger_pose(pose, -1), pts + 3 * i);
      out[i * nc + 1] = shape_sdf(*tool, tool_kind(*tool), finger_pose(pose, 1), pts + 3 * i);
    } else {
      out[i * nc] = tool_sdf(*tool, pose, pts + 3 * i);
    }
  }
}
void oracle_tool_distance_vjp(const OracleTool* tool, const double* pose, int64_t m, const double* pts,
                              const double* g, double* g_pts, double* g_pose) {
  const int nc = oracle_tool_distance_cols(tool);
  for (int64_t i = 0; i < m; ++i) {
    if (is_fingered(tool->type)) {
      for (int side = 0; side < 2; ++side) {
        double flag = side == 0 ? -1.0 : 1.0;
        PoseGrad gF;
        shape_sdf_vjp(*tool, tool_kind(*tool), finger_pose(pose, flag), pts + 3 * i, g[i * nc + side], g_pts + 3 * i,
                      &gF);
        finger_pose_vjp(pose, flag, gF, g_pose);
      }
    } else {
      tool_sdf_vjp(*tool, pose, pts + 3 * i, g[i * nc], g_pts + 3 * i, g_pose);
    }
  }
}
// one tool's collide at m points (tests)
void oracle_tool_collide(const OracleTool* tool, const double* pose0, const double* pose1, double dt, int64_t m,
                         const double* pts, const double* vin, double* vout) {
  for (int64_t i = 0; i < m; ++i) tool_collide(*tool, pose0, pose1, pts + 3 * i, dt, vin + 3 * i, vout + 3 * i);
}
void oracle_tool_collide_vjp(const OracleTool* tool, const double* pose0, const double* pose1, double dt, int64_t m,
                             const double* pts, const double* vin, const double* gout, double* gvin, double* gpose0,
                             double* gpose1) {
  for (int64_t i = 0; i < m; ++i)
    tool_collide_vjp(*tool, pose0, pose1, pts + 3 * i, dt, vin + 3 * i, gout + 3 * i, gvin + 3 * i, gpose0, gpose1);
}

// Primitive.set_velocity (primive_base.py:260-268; Gripper primitives.py:463-469,
// Chopsticks 238-245, Gripper2 595-601) followed by forward_kinematics
// (primive_base.py:153-156; RollingPin primitives.py:104-117, RollingPinExt
// 122-135, Chopsticks 231-235, Gripper 457-460, Gripper2 589-592) and, when
// tools have collision masks, the collision projection of every substep
// (mpm_simulator.py:287-305, 316-319) for the n_sub substeps of one action.
// pose: [(n_sub+1)][T][8] with frame 0 given.  vel: [n_sub][T][8] written.
// action: [T][7] (already clipped to [-1, 1]).  pts: [n_pairs][600][3] random
// numbers (rand_num); coll: [n_sub][n_pairs][4] written (index or -1, point).
}  // extern "C"
namespace {
const int kSurfacePoints = 600;
struct Pair {
  int i, j;
};
std::vector<Pair> collision_pairs(const OracleTool* tools, int T) {
  std::vector<Pair> pr;
  for (int i = 0; i < T; ++i)
    for (int j = 0; j < T; ++j)
      if ((tools[i].collision_mask >> j) & 1) pr.push_back({i, j});
  return pr;
}
inline void clamp_xyz(const OracleTool& tl, const double* p0, const double* dv, double* p1, bool* pass) {
  for (int k = 0; k < 3; ++k) {
    double a = p0[k] + dv[k];
    double mn = (a < tl.upper[k]) ? a : tl.upper[k];
    p1[k] = (tl.lower[k] < mn) ? mn : tl.lower[k];
    pass[k] = (a < tl.upper[k]) && (tl.lower[k] < mn);
  }
}
// RollingPin(Ext): x_dir = (0,1,0) x qrot(rot, (0,-1,0)) * (dw*0.03 [+ w0]), x_dir.y = dy
inline void rolling_terms(const OracleTool& tl, const double* p0, const double* vv, double* yd, double* s,
                          double* xd) {
  const double down[3] = {0, -1, 0};
  qrot(p0 + 3, down, yd);
  *s = vv[0] * 0.03 + (tl.type == T_ROLLINGPINEXT ? vv[3] : 0.0);
  const double up[3] = {0, 1, 0};
  cross3(up, yd, xd);
  for (int k = 0; k < 3; ++k) xd[k] *= *s;
  xd[1] = vv[2];
}
void fk(const OracleTool& tl, const double* p0, const double* vv, double* p1) {
  bool pass[3];
  if (tl.type == T_ROLLINGPIN || tl.type == T_ROLLINGPINEXT) {
    double yd[3], s, xd[3];
    rolling_terms(tl, p0, vv, yd, &s, xd);
    clamp_xyz(tl, p0, xd, p1, pass);
    const double wa[3] = {0, -vv[1], 0}, wb[3] = {0, vv[0], 0};
    double qa[4], qb[4], t[4];
    w2quat(wa, qa);
    w2quat(wb, qb);
    qmul(p0 + 3, qb, t);
    qmul(qa, t, p1 + 3);
    p1[7] = p0[7];
    return;
  }
  clamp_xyz(tl, p0, vv, p1, pass);
  double wq[4];
  w2quat(vv + 3, wq);
  if (has_gap_vel(tl.type)) {
    qmul(p0 + 3, wq, p1 + 3);
    double a = p0[7] - vv[6];
    double mx = (tl.min_gap < a) ? a : tl.min_gap;
    p1[7] = (tl.type == T_CHOPSTICKS) ? mx : ((mx < tl.max_gap) ? mx : tl.max_gap);
  } else {
    qmul(wq, p0 + 3, p1 + 3);
    p1[7] = p0[7];
  }
}
void fk_vjp(const OracleTool& tl, const double* p0, const double* vv, const double* g1, double* g0, double* gvv) {
  bool pass[3];
  double tmp[8];
  if (tl.type == T_ROLLINGPIN || tl.type == T_ROLLINGPINEXT) {
    double yd[3], s, xd[3];
    rolling_terms(tl, p0, vv, yd, &s, xd);
    clamp_xyz(tl, p0, xd, tmp, pass);
    double gxd[3];
    for (int k = 0; k < 3; ++k) {
      gxd[k] = pass[k] ? g1[k] : 0.0;
      g0[k] += gxd[k];
    }
    gvv[2] += gxd[1];
    // xd0 = yd2 s, xd2 = -yd0 s
    double gs = gxd[0] * yd[2] - gxd[2] * yd[0];
    const double gyd[3] = {-gxd[2] * s, 0.0, gxd[0] * s};
    const double down[3] = {0, -1, 0};
    qrot_vjp(p0 + 3, down, gyd, g0 + 3, nullptr);
    gvv[0] += gs * 0.03;
    if (tl.type == T_ROLLINGPINEXT) gvv[3] += gs;
    const double wa[3] = {0, -vv[1], 0}, wb[3] = {0, vv[0], 0};
    double qa[4], qb[4], t[4];
    w2quat(wa, qa);
    w2quat(wb, qb);
    qmul(p0 + 3, qb, t);
    double gqa[4] = {0, 0, 0, 0}, gt[4] = {0, 0, 0, 0}, gqb[4] = {0, 0, 0, 0};
    qmul_vjp(qa, t, g1 + 3, gqa, gt);
    qmul_vjp(p0 + 3, qb, gt, g0 + 3, gqb);
    double gwa[3] = {0, 0, 0}, gwb[3] = {0, 0, 0};
    w2quat_vjp(wa, gqa, gwa);
    w2quat_vjp(wb, gqb, gwb);
    gvv[1] -= gwa[1];
    gvv[0] += gwb[1];
    g0[7] += g1[7];
    return;
  }
  clamp_xyz(tl, p0, vv, tmp, pass);
  for (int k = 0; k < 3; ++k)
    if (pass[k]) {
      g0[k] += g1[k];
      gvv[k] += g1[k];
    }
  double wq[4], gwq[4] = {0, 0, 0, 0};
  w2quat(vv + 3, wq);
  if (has_gap_vel(tl.type)) {
    qmul_vjp(p0 + 3, wq, g1 + 3, g0 + 3, gwq);
    double a = p0[7] - vv[6];
    double mx = (tl.min_gap < a) ? a : tl.min_gap;
    bool ok = (tl.min_gap < a) && (tl.type == T_CHOPSTICKS || mx < tl.max_gap);
    if (ok) {
      g0[7] += g1[7];
      gvv[6] -= g1[7];
    }
  } else {
    qmul_vjp(wq, p0 + 3, g1 + 3, gwq, g0 + 3);
    g0[7] += g1[7];
  }
  w2quat_vjp(vv + 3, gwq, gvv + 3);
}
// Box._project of rand * size, moved to the box pose (get_surface_pos, primive_base.py:285-287)
inline void surface_pt(const OracleTool& box, const double* pose8, const double* rn, double* local, double* w) {
  for (int k = 0; k < 3; ++k) local[k] = std::max(std::min(rn[k] * box.size[k], box.size[k]), -box.size[k]);
  qrot(pose8 + 3, local, w);
  for (int k = 0; k < 3; ++k) w[k] += pose8[k];
}
void project(const OracleTool* tools, int T, const std::vector<Pair>& pr, const double* pts, double* pose1,
             double* coll) {
  for (size_t c = 0; c < pr.size(); ++c) {  // set_surface_points + set_collision_idx
    const Pair& P = pr[c];
    double min_dist = 0.0;
    int idx = -1;
    double best[3] = {0, 0, 0};
    for (int k = 0; k < kSurfacePoints; ++k) {
      double local[3], w[3];
      surface_pt(tools[P.j], pose1 + 8 * P.j, pts + 3 * (c * kSurfacePoints + k), local, w);
      double d = tool_sdf(tools[P.i], pose1 + 8 * P.i, w);
      if (d < min_dist) {
        min_dist = d;
        idx = k;
        std::memcpy(best, w, sizeof(best));
      }
    }
    coll[4 * c] = idx;
    coll[4 * c + 1] = best[0];
    coll[4 * c + 2] = best[1];
    coll[4 * c + 3] = best[2];
  }
  for (size_t c = 0; c < pr.size(); ++c) {  // apply_collision_projection
    if (coll[4 * c] < 0) continue;
    const Pair& P = pr[c];
    const double* w = coll + 4 * c + 1;
    double d = tool_sdf(tools[P.i], pose1 + 8 * P.i, w), n[3];
    tool_normal(tools[P.i], pose1 + 8 * P.i, w, n);
    double L = std::sqrt(dot3(n, n));
    for (int k = 0; k < 3; ++k) pose1[8 * P.i + k] += n[k] / L * d;
  }
}
// apply_collision_projection.grad + set_surface_points.grad at the stored
// (projected) poses and stored points, pairs in reverse
void project_vjp(const OracleTool* tools, int T, const std::vector<Pair>& pr, const double* pts, const double* pose1,
                 const double* coll, double* g1) {
  for (int c = (int)pr.size() - 1; c >= 0; --c) {
    if (coll[4 * c] < 0) continue;
    const Pair& P = pr[c];
    const double* w = coll + 4 * c + 1;
    const double* pi = pose1 + 8 * P.i;
    double d = tool_sdf(tools[P.i], pi, w), n[3];
    tool_normal(tools[P.i], pi, w, n);
    double L = std::sqrt(dot3(n, n));
    double nn[3] = {n[0] / L, n[1] / L, n[2] / L};
    const double gs[3] = {g1[8 * P.i], g1[8 * P.i + 1], g1[8 * P.i + 2]};
    double gd = dot3(gs, nn);
    double gnn[3] = {gs[0] * d, gs[1] * d, gs[2] * d};
    double dn = dot3(nn, gnn);
    double gn[3];
    for (int k = 0; k < 3; ++k) gn[k] = (gnn[k] - nn[k] * dn) / L;
    double gp[3] = {0, 0, 0};
    tool_sdf_vjp(tools[P.i], pi, w, gd, gp, g1 + 8 * P.i);
    tool_normal_vjp(tools[P.i], pi, w, gn, gp, g1 + 8 * P.i);
    double local[3], ww[3];
    surface_pt(tools[P.j], pose1 + 8 * P.j, pts + 3 * (c * kSurfacePoints + (int)coll[4 * c]), local, ww);
    for (int k = 0; k < 3; ++k) g1[8 * P.j + k] += gp[k];
    qrot_vjp(pose1 + 8 * P.j + 3, local, gp, g1 + 8 * P.j + 3, nullptr);
  }
}
}  // namespace
extern "C" {
int oracle_collision_pairs(const OracleTool* tools, int T) { return (int)collision_pairs(tools, T).size(); }
void oracle_tools_action(const OracleTool* tools, int T, int n_sub, const double* action, double* vel, double* pose,
                         const double* pts, double* coll) {
  const std::vector<Pair> pr = collision_pairs(tools, T);
  const int np = (int)pr.size();
  for (int t = 0; t < T; ++t) {
    const OracleTool& tl = tools[t];
    double vv[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (tl.action_dim > 0) {
      for (int k = 0; k < 3; ++k) vv[k] = action[t * 7 + k] * tl.action_scale[k] / n_sub;
      if (tl.action_dim > 3)
        for (int k = 0; k < 3; ++k) vv[3 + k] = action[t * 7 + 3 + k] * tl.action_scale[3 + k] / n_sub;
      if (has_gap_vel(tl.type)) vv[6] = action[t * 7 + 6] * tl.action_scale[6] / n_sub;
    }
    for (int j = 0; j < n_sub; ++j) std::memcpy(vel + ((int64_t)j * T + t) * 8, vv, sizeof(vv));
  }
  for (int j = 0; j < n_sub; ++j) {
    for (int t = 0; t < T; ++t)
      fk(tools[t], pose + ((int64_t)j * T + t) * 8, vel + ((int64_t)j * T + t) * 8,
         pose + ((int64_t)(j + 1) * T + t) * 8);
    if (np) project(tools, T, pr, pts, pose + (int64_t)(j + 1) * T * 8, coll + (int64_t)j * np * 4);
  }
}
// Adjoint of oracle_tools_action.  g_pose [(n_sub+1)][T][8] holds the
// accumulated gradients of every frame on entry; on exit g_pose[0] also holds
// the gradient reaching frame 0, and g_action [T][7] the action gradient
// (set_velocity.grad, primive_base.py:260-268, without the clip mask, as
// GradModel.backward returns it).
void oracle_tools_action_bwd(const OracleTool* tools, int T, int n_sub, const double* action, const double* vel,
                             const double* pose, const double* pts, const double* coll, double* g_pose,
                             double* g_action) {
  (void)action;
  const std::vector<Pair> pr = collision_pairs(tools, T);
  const int np = (int)pr.size();
  for (int j = n_sub - 1; j >= 0; --j) {
    if (np)
      project_vjp(tools, T, pr, pts, pose + (int64_t)(j + 1) * T * 8, coll + (int64_t)j * np * 4,
                  g_pose + (int64_t)(j + 1) * T * 8);
    for (int t = 0; t < T; ++t) {
      const OracleTool& tl = tools[t];
      double gvv[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      fk_vjp(tl, pose + ((int64_t)j * T + t) * 8, vel + ((int64_t)j * T + t) * 8,
             g_pose + ((int64_t)(j + 1) * T + t) * 8, g_pose + ((int64_t)j * T + t) * 8, gvv);
      if (tl.action_dim > 0) {
        for (int k = 0; k < 3; ++k) g_action[t * 7 + k] += gvv[k] * tl.action_scale[k] / n_sub;
        if (tl.action_dim > 3)
          for (int k = 0; k < 3; ++k) g_action[t * 7 + 3 + k] += gvv[3 + k] * tl.action_scale[3 + k] / n_sub;
        if (has_gap_vel(tl.type)) g_action[t * 7 + 6] += gvv[6] * tl.action_scale[6] / n_sub;
      }
    }
  }
}

// One substep (mpm_simulator.py:307-323 without forward_kinematics, which
// oracle_tools_action has done): clear_grid, F_tmp, svd, p2g, grid_op, g2p.
// Returns 0, or 1 if a particle stencil leaves the grid (nothing written).
int oracle_substep(const OracleSim* Sp, const OracleTool* tools, int T, const double* pose_f, const double* pose_f1,
                   int64_t n, const double* state_f, double* state_f1) {
  const OracleSim& S = *Sp;
  const int ng = S.n_grid;
  const int64_t G = (int64_t)ng * ng * ng;
  std::vector<Stencil> st(n);
  for (int64_t p = 0; p < n; ++p) make_stencil(S, state_f + 24 * p, st[p]);
  int err = 0;
  check_stencils(S, st, &err);
  if (err) return 1;
  std::vector<double> affine(9 * n), newF(9 * n);
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < n; ++p) {
    P2GTape tp;
    p2g_particle(S, state_f + 24 * p, tp);
    std::memcpy(&affine[9 * p], tp.affine, sizeof(tp.affine));
    std::memcpy(&newF[9 * p], tp.newF, sizeof(tp.newF));
  }
  std::vector<double> gmv(3 * G, 0.0), gm(G, 0.0), gvo(3 * G, 0.0);
  Buckets B;
  bucket_by_x(ng, n, st, B);
  scatter_planes(ng, B, [&](int64_t p, int ox) {
    const Stencil& s = st[p];
    const double* v = state_f + 24 * p + 3;
    const double* af = &affine[9 * p];
    for (int oy = 0; oy < 3; ++oy)
      for (int oz = 0; oz < 3; ++oz) {
        double wgt = s.w[ox][0] * s.w[oy][1] * s.w[oz][2];
        double dpos[3] = {(ox - s.fx[0]) * S.dx, (oy - s.fx[1]) * S.dx, (oz - s.fx[2]) * S.dx};
        int64_t id = node_index(ng, s.base[0] + ox, s.base[1] + oy, s.base[2] + oz);
        for (int k = 0; k < 3; ++k)
          gmv[3 * id + k] += wgt * (S.p_mass * v[k] + af[3 * k] * dpos[0] + af[3 * k + 1] * dpos[1] +
                                    af[3 * k + 2] * dpos[2]);
        gm[id] += wgt * S.p_mass;
      }
  });
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t id = 0; id < G; ++id) {
    if (!(gm[id] > 1e-12)) continue;
    int I[3] = {(int)(id / ((int64_t)ng * ng)), (int)((id / ng) % ng), (int)(id % ng)};
    grid_node(S, tools, T, pose_f, pose_f1, I, &gmv[3 * id], gm[id], &gvo[3 * id], nullptr);
  }
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < n; ++p) {
    const Stencil& s = st[p];
    const double* row = state_f + 24 * p;
    double* out = state_f1 + 24 * p;
    double nv[3] = {0, 0, 0}, nC[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int ox = 0; ox < 3; ++ox)
      for (int oy = 0; oy < 3; ++oy)
        for (int oz = 0; oz < 3; ++oz) {
          double wgt = s.w[ox][0] * s.w[oy][1] * s.w[oz][2];
          double dpos[3] = {ox - s.fx[0], oy - s.fx[1], oz - s.fx[2]};
          int64_t id = node_index(ng, s.base[0] + ox, s.base[1] + oy, s.base[2] + oz);
          const double* gv = &gvo[3 * id];
          for (int i = 0; i < 3; ++i) {
            nv[i] += wgt * gv[i];
            for (int j = 0; j < 3; ++j) nC[i * 3 + j] += 4 * S.inv_dx * wgt * gv[i] * dpos[j];
          }
        }
    for (int i = 0; i < 3; ++i) {
      double t = row[i] + S.dt * nv[i];
      double hi = 1.0 - 3 * S.dx, lo = S.lower_bound * S.dx;
      double mn = (t < hi) ? t : hi;
      out[i] = (lo < mn) ? mn : lo;
      out[3 + i] = nv[i];
    }
    std::memcpy(out + 6, nC, sizeof(nC));
    std::memcpy(out + 15, &newF[9 * p], 9 * sizeof(double));
  }
  return 0;
}

// Adjoint of oracle_substep (substep_grad, mpm_simulator.py:325-345).
// g_f1: [n][24] gradient of frame f+1; g_f: [n][24] written (overwritten).
// g_pose_f / g_pose_f1: [T][8] accumulated.
int oracle_substep_bwd(const OracleSim* Sp, const OracleTool* tools, int T, const double* pose_f,
                       const double* pose_f1, int64_t n, const double* state_f, const double* g_f1, double* g_f,
                       double* g_pose_f, double* g_pose_f1) {
  const OracleSim& S = *Sp;
  const int ng = S.n_grid;
  const int64_t G = (int64_t)ng * ng * ng;
  std::vector<Stencil> st(n);
  for (int64_t p = 0; p < n; ++p) make_stencil(S, state_f + 24 * p, st[p]);
  int err = 0;
  check_stencils(S, st, &err);
  if (err) return 1;
  // ---- recompute forward grid
  std::vector<double> affine(9 * n);
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < n; ++p) {
    P2GTape tp;
    p2g_particle(S, state_f + 24 * p, tp);
    std::memcpy(&affine[9 * p], tp.affine, sizeof(tp.affine));
  }
  std::vector<double> gmv(3 * G, 0.0), gm(G, 0.0), gvo(3 * G, 0.0);
  Buckets B;
  bucket_by_x(ng, n, st, B);
  scatter_planes(ng, B, [&](int64_t p, int ox) {
    const Stencil& s = st[p];
    const double* v = state_f + 24 * p + 3;
    const double* af = &affine[9 * p];
    for (int oy = 0; oy < 3; ++oy)
      for (int oz = 0; oz < 3; ++oz) {
        double wgt = s.w[ox][0] * s.w[oy][1] * s.w[oz][2];
        double dpos[3] = {(ox - s.fx[0]) * S.dx, (oy - s.fx[1]) * S.dx, (oz - s.fx[2]) * S.dx};
        int64_t id = node_index(ng, s.base[0] + ox, s.base[1] + oy, s.base[2] + oz);
        for (int k = 0; k < 3; ++k)
          gmv[3 * id + k] += wgt * (S.p_mass * v[k] + af[3 * k] * dpos[0] + af[3 * k + 1] * dpos[1] +
                                    af[3 * k + 2] * dpos[2]);
        gm[id] += wgt * S.p_mass;
      }
  });
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t id = 0; id < G; ++id) {
    if (!(gm[id] > 1e-12)) continue;
    int I[3] = {(int)(id / ((int64_t)ng * ng)), (int)((id / ng) % ng), (int)(id % ng)};
    grid_node(S, tools, T, pose_f, pose_f1, I, &gmv[3 * id], gm[id], &gvo[3 * id], nullptr);
  }
  // ---- g2p adjoint (g2p.grad): particle-local part first
  std::vector<double> gnv(3 * n), gC1(9 * n);
  for (int64_t p = 0; p < n; ++p) {
    const double* row = state_f + 24 * p;
    const double* g1 = g_f1 + 24 * p;
    double* g0 = g_f + 24 * p;
    std::memset(g0, 0, 24 * sizeof(double));
    const Stencil& s = st[p];
    // recompute new v for the clamp mask
    double nv[3] = {0, 0, 0};
    for (int ox = 0; ox < 3; ++ox)
      for (int oy = 0; oy < 3; ++oy)
        for (int oz = 0; oz < 3; ++oz) {
          double wgt = s.w[ox][0] * s.w[oy][1] * s.w[oz][2];
          int64_t id = node_index(ng, s.base[0] + ox, s.base[1] + oy, s.base[2] + oz);
          for (int i = 0; i < 3; ++i) nv[i] += wgt * gvo[3 * id + i];
        }
    for (int i = 0; i < 3; ++i) {
      double t = row[i] + S.dt * nv[i];
      double hi = 1.0 - 3 * S.dx, lo = S.lower_bound * S.dx;
      double mn = (t < hi) ? t : hi;
      bool pass = (t < hi) && (lo < mn);
      double gt = pass ? g1[i] : 0.0;
      g0[i] += gt;
      gnv[3 * p + i] = g1[3 + i] + S.dt * gt;
    }
    std::memcpy(&gC1[9 * p], g1 + 6, 9 * sizeof(double));
  }
  std::vector<double> g_gvo(3 * G, 0.0);
  scatter_planes(ng, B, [&](int64_t p, int ox) {
    const Stencil& s = st[p];
    const double* gv_ = &gnv[3 * p];
    const double* gC = &gC1[9 * p];
    for (int oy = 0; oy < 3; ++oy)
      for (int oz = 0; oz < 3; ++oz) {
        double wgt = s.w[ox][0] * s.w[oy][1] * s.w[oz][2];
        double dpos[3] = {ox - s.fx[0], oy - s.fx[1], oz - s.fx[2]};
        int64_t id = node_index(ng, s.base[0] + ox, s.base[1] + oy, s.base[2] + oz);
        for (int i = 0; i < 3; ++i)
          g_gvo[3 * id + i] += wgt * gv_[i] +
                               4 * S.inv_dx * wgt * (gC[3 * i] * dpos[0] + gC[3 * i + 1] * dpos[1] + gC[3 * i + 2] * dpos[2]);
      }
  });
  // g2p: gradient w.r.t. x through weights and dpos
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < n; ++p) {
    const Stencil& s = st[p];
    const double* gv_ = &gnv[3 * p];
    const double* gC = &gC1[9 * p];
    double gw[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    double gfx[3] = {0, 0, 0};
    for (int ox = 0; ox < 3; ++ox)
      for (int oy = 0; oy < 3; ++oy)
        for (int oz = 0; oz < 3; ++oz) {
          int o[3] = {ox, oy, oz};
          double wgt = s.w[ox][0] * s.w[oy][1] * s.w[oz][2];
          double dpos[3] = {ox - s.fx[0], oy - s.fx[1], oz - s.fx[2]};
          int64_t id = node_index(ng, s.base[0] + ox, s.base[1] + oy, s.base[2] + oz);
          const double* gv = &gvo[3 * id];
          double gCd[3];
          for (int i = 0; i < 3; ++i) gCd[i] = gC[3 * i] * dpos[0] + gC[3 * i + 1] * dpos[1] + gC[3 * i + 2] * dpos[2];
          double g_wgt = dot3(gv, gv_) + 4 * S.inv_dx * dot3(gv, gCd);
          for (int j = 0; j < 3; ++j) {
            double gd = 4 * S.inv_dx * wgt * (gC[j] * gv[0] + gC[3 + j] * gv[1] + gC[6 + j] * gv[2]);
            gfx[j] -= gd;
          }
          for (int d = 0; d < 3; ++d) {
            double other = 1.0;
            for (int e = 0; e < 3; ++e)
              if (e != d) other *= s.w[o[e]][e];
            gw[o[d]][d] += g_wgt * other;
          }
        }
    for (int d = 0; d < 3; ++d) {
      for (int k = 0; k < 3; ++k) gfx[d] += gw[k][d] * s.dw[k][d];
      g_f[24 * p + d] += S.inv_dx * gfx[d];
    }
  }
  // ---- grid_op adjoint; tool pose gradients reduced in a fixed chunk order
  std::vector<double> g_gmv(3 * G, 0.0), g_gm(G, 0.0);
  const int64_t chunk = 4096;
  const int64_t n_chunks = (G + chunk - 1) / chunk;
  std::vector<double> part0((size_t)n_chunks * T * 8, 0.0), part1((size_t)n_chunks * T * 8, 0.0);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t c = 0; c < n_chunks; ++c) {
    double* p0 = &part0[(size_t)c * T * 8];
    double* p1 = &part1[(size_t)c * T * 8];
    for (int64_t id = c * chunk; id < std::min(G, (c + 1) * chunk); ++id) {
      if (!(gm[id] > 1e-12)) continue;
      const double* go = &g_gvo[3 * id];
      if (go[0] == 0 && go[1] == 0 && go[2] == 0) continue;
      int I[3] = {(int)(id / ((int64_t)ng * ng)), (int)((id / ng) % ng), (int)(id % ng)};
      grid_node_vjp(S, tools, T, pose_f, pose_f1, I, &gmv[3 * id], gm[id], go, &g_gmv[3 * id], &g_gm[id], p0, p1);
    }
  }
  for (int64_t c = 0; c < n_chunks; ++c)
    for (int i = 0; i < T * 8; ++i) {
      g_pose_f[i] += part0[(size_t)c * T * 8 + i];
      g_pose_f1[i] += part1[(size_t)c * T * 8 + i];
    }
  // ---- p2g adjoint (p2g.grad, svd_grad, compute_F_tmp.grad): gather
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < n; ++p) {
    const double* row = state_f + 24 * p;
    const double* v = row + 3;
    double* g0 = g_f + 24 * p;
    const Stencil& s = st[p];
    P2GTape tp;
    p2g_particle(S, row, tp);
    double g_aff[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    double gw[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    double gfx[3] = {0, 0, 0};
    for (int ox = 0; ox < 3; ++ox)
      for (int oy = 0; oy < 3; ++oy)
        for (int oz = 0; oz < 3; ++oz) {
          int o[3] = {ox, oy, oz};
          double wgt = s.w[ox][0] * s.w[oy][1] * s.w[oz][2];
          double dpos[3] = {(ox - s.fx[0]) * S.dx, (oy - s.fx[1]) * S.dx, (oz - s.fx[2]) * S.dx};
          int64_t id = node_index(ng, s.base[0] + ox, s.base[1] + oy, s.base[2] + oz);
          const double* gv = &g_gmv[3 * id];
          double gmm = g_gm[id];
          double contrib[3];
          for (int k = 0; k < 3; ++k)
            contrib[k] = S.p_mass * v[k] + tp.affine[3 * k] * dpos[0] + tp.affine[3 * k + 1] * dpos[1] +
                         tp.affine[3 * k + 2] * dpos[2];
          double g_wgt = dot3(gv, contrib) + gmm * S.p_mass;
          for (int k = 0; k < 3; ++k) {
            g0[3 + k] += wgt * S.p_mass * gv[k];
            for (int j = 0; j < 3; ++j) g_aff[3 * k + j] += wgt * gv[k] * dpos[j];
          }
          for (int j = 0; j < 3; ++j) {
            double gd = wgt * (tp.affine[j] * gv[0] + tp.affine[3 + j] * gv[1] + tp.affine[6 + j] * gv[2]);
            gfx[j] -= S.dx * gd;
          }
          for (int d = 0; d < 3; ++d) {
            double other = 1.0;
            for (int e = 0; e < 3; ++e)
              if (e != d) other *= s.w[o[e]][e];
            gw[o[d]][d] += g_wgt * other;
          }
        }
    for (int d = 0; d < 3; ++d) {
      for (int k = 0; k < 3; ++k) gfx[d] += gw[k][d] * s.dw[k][d];
      g0[d] += S.inv_dx * gfx[d];
    }
    p2g_particle_vjp(S, row, tp, g_aff, g_f1 + 24 * p + 15, g0 + 6, g0 + 15);
  }
  return 0;
}

// compute_grid_m_kernel (mpm_simulator.py:456-466) on a cleared grid.
int oracle_grid_mass(const OracleSim* Sp, int64_t n, const double* state, double* grid_m) {
  const OracleSim& S = *Sp;
  const int ng = S.n_grid;
  const int64_t G = (int64_t)ng * ng * ng;
  std::vector<Stencil> st(n);
  for (int64_t p = 0; p < n; ++p) make_stencil(S, state + 24 * p, st[p]);
  int err = 0;
  check_stencils(S, st, &err);
  if (err) return 1;
  std::memset(grid_m, 0, G * sizeof(double));
  Buckets B;
  bucket_by_x(ng, n, st, B);
  scatter_planes(ng, B, [&](int64_t p, int ox) {
    const Stencil& s = st[p];
    for (int oy = 0; oy < 3; ++oy)
      for (int oz = 0; oz < 3; ++oz) {
        double wgt = s.w[ox][0] * s.w[oy][1] * s.w[oz][2];
        grid_m[node_index(ng, s.base[0] + ox, s.base[1] + oy, s.base[2] + oz)] += wgt * S.p_mass;
      }
  });
  return 0;
}
// compute_grid_m_kernel.grad: accumulates into the x part of g_state [n][24]
int oracle_grid_mass_bwd(const OracleSim* Sp, int64_t n, const double* state, const double* g_grid_m,
                         double* g_state) {
  const OracleSim& S = *Sp;
  const int ng = S.n_grid;
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < n; ++p) {
    Stencil s;
    make_stencil(S, state + 24 * p, s);
    if (!stencil_ok(S, s)) continue;
    double gw[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int ox = 0; ox < 3; ++ox)
      for (int oy = 0; oy < 3; ++oy)
        for (int oz = 0; oz < 3; ++oz) {
          int o[3] = {ox, oy, oz};
          double g = g_grid_m[node_index(ng, s.base[0] + ox, s.base[1] + oy, s.base[2] + oz)] * S.p_mass;
          for (int d = 0; d < 3; ++d) {
            double other = 1.0;
            for (int e = 0; e < 3; ++e)
              if (e != d) other *= s.w[o[e]][e];
            gw[o[d]][d] += g * other;
          }
        }
    for (int d = 0; d < 3; ++d) {
      double gfx = 0;
      for (int k = 0; k < 3; ++k) gfx += gw[k][d] * s.dw[k][d];
      g_state[24 * p + d] += S.inv_dx * gfx;
    }
  }
  return 0;
}
// compute_density_loss_kernel (loss.py:172-175): sum |m - target|, grad sgn
double oracle_density_l1(int64_t G, const double* grid_m, const double* target, double* g_grid_m) {
  double loss = 0;
  for (int64_t i = 0; i < G; ++i) {
    double d = grid_m[i] - target[i];
    loss += std::fabs(d);
    if (g_grid_m) g_grid_m[i] = sgn(d);
  }
  return loss;
}
// soft contact loss (loss.py:143-167) for one tool at one frame:
// returns min_dist = sum_i d_i w_i / sum_i w_i, d_i = max(sdf(x_i), 0),
// w_i = 1/(1 + 1e4 d_i^2).  With g_min != 0 accumulates the x part of
// g_state and g_pose.
double oracle_soft_contact(const OracleTool* tool, const double* pose, int64_t n, const double* state, double g_min,
                           double* g_state, double* g_pose) {
  std::vector<double> d(n), sdf(n), w(n);
  double norm = 0, num = 0;
  for (int64_t i = 0; i < n; ++i) {
    sdf[i] = tool_sdf(*tool, pose, state + 24 * i);
    d[i] = (0.0 < sdf[i]) ? sdf[i] : 0.0;
    w[i] = 1.0 / (1.0 + d[i] * d[i] * 10000);
    norm += w[i];
    num += d[i] * w[i];
  }
  double md = num / norm;
  if (g_min != 0 && g_state) {
    double g_norm = -g_min * md / norm;
    for (int64_t i = 0; i < n; ++i) {
      double g_w = g_min * d[i] / norm + g_norm;
      double g_d = g_min * w[i] / norm + g_w * (-2e4 * d[i] * w[i] * w[i]);
      if (0.0 < sdf[i]) tool_sdf_vjp(*tool, pose, state + 24 * i, g_d, g_state + 24 * i, g_pose);
    }
  }
  return md;
}

// update_target (loss.py:129-134): the copy is filled with inf = 1000, then
// update_target_sdf (loss.py:105-124) runs n_iters times.  Every node reads
// only the previous iteration's copy; offsets are visited in the order of
// ti.ndrange((-3,3),(-3,3),(-3,3)) and the first strict minimum of
// norm(grid_pos - nearest) = sqrt(|d|^2 + 1e-8) wins.  T is the simulator's
// float type; each operation is rounded to T (built with -ffp-contract=off).
// Nodes whose sdf stays inf get nearest = 0.
}  // extern "C"
template <typename T>
static void target_sdf_impl(int n, double dx, int n_iters, const T* dens, T* sdf, T* nearest) {
  const int64_t G = (int64_t)n * n * n;
  const T inf = T(1000.0);
  std::vector<T> sc(G, inf), nc(3 * G, T(0));
  for (int64_t i = 0; i < G; ++i) {
    sdf[i] = inf;
    nearest[3 * i] = nearest[3 * i + 1] = nearest[3 * i + 2] = T(0);
  }
  for (int it = 0; it < n_iters; ++it) {
#pragma omp parallel for schedule(static)
    for (int64_t id = 0; id < G; ++id) {
      const int i0 = (int)(id / ((int64_t)n * n)), i1 = (int)((id / n) % n), i2 = (int)(id % n);
      const T gp[3] = {T(double(i0) * dx), T(double(i1) * dx), T(double(i2) * dx)};
      T best = inf, bn[3] = {T(0), T(0), T(0)};
      if (double(dens[id]) > 1e-4) {
        best = T(0);
        bn[0] = gp[0];
        bn[1] = gp[1];
        bn[2] = gp[2];
      } else {
        for (int a = -3; a < 3; ++a)
          for (int b = -3; b < 3; ++b)
            for (int c = -3; c < 3; ++c) {
              const int v0 = i0 + a, v1 = i1 + b, v2 = i2 + c;
              if (std::min(v0, std::min(v1, v2)) < 0 || std::max(v0, std::max(v1, v2)) >= n) continue;
              if (std::abs(a) + std::abs(b) + std::abs(c) == 0) continue;
              const int64_t v = ((int64_t)v0 * n + v1) * n + v2;
              if (!(sc[v] < inf)) continue;
              const T d0 = gp[0] - nc[3 * v], d1 = gp[1] - nc[3 * v + 1], d2 = gp[2] - nc[3 * v + 2];
              const T dist = std::sqrt(T(T(T(d0 * d0) + T(d1 * d1)) + T(d2 * d2)) + T(1e-8));
              if (dist < best) {
                best = dist;
                bn[0] = nc[3 * v];
                bn[1] = nc[3 * v + 1];
                bn[2] = nc[3 * v + 2];
              }
            }
      }
      sdf[id] = best;
      nearest[3 * id] = bn[0];
      nearest[3 * id + 1] = bn[1];
      nearest[3 * id + 2] = bn[2];
    }
    std::copy(sdf, sdf + G, sc.begin());
    std::copy(nearest, nearest + 3 * G, nc.begin());
  }
}
extern "C" {
void oracle_target_sdf_f64(int n, double dx, int n_iters, const double* dens, double* sdf, double* nearest) {
  target_sdf_impl<double>(n, dx, n_iters, dens, sdf, nearest);
}
void oracle_target_sdf_f32(int n, double dx, int n_iters, const float* dens, float* sdf, float* nearest) {
  target_sdf_impl<float>(n, dx, n_iters, dens, sdf, nearest);
}

// hard contact distance (compute_contact_distance_kernel, loss.py:151-155)
// of one movable tool, started from 100000 (loss.py:243-244):
// min(100000, min_i max(sdf(x_i), 0)); *argmin = lowest index attaining it or
// -1.  With g_min != 0 the gradient goes to that particle (x part of g_state)
// and to g_pose, where sdf > 0.
double oracle_contact_min(const OracleTool* tool, const double* pose, int64_t n, const double* state, double g_min,
                          double* g_state, double* g_pose, int64_t* argmin) {
  double md = 100000.0;
  int64_t am = -1;
  for (int64_t i = 0; i < n; ++i) {
    const double sd = tool_sdf(*tool, pose, state + 24 * i);
    const double d = (0.0 < sd) ? sd : 0.0;
    if (d < md) {
      md = d;
      am = i;
    } else if (d == md && am < 0) {
      am = i;
    }
  }
  if (argmin) *argmin = am;
  if (g_min != 0 && g_state && am >= 0 && 0.0 < tool_sdf(*tool, pose, state + 24 * am))
    tool_sdf_vjp(*tool, pose, state + 24 * am, g_min, g_state + 24 * am, g_pose);
  return md;
}

// ----------------------------------------------------------------------------
// Particle-SDF renderer (taichi_three/tina/core/particle_sdf.py), FP32 as the
// reference's f32 fields; every operation rounded on its own.
// ----------------------------------------------------------------------------
}  // extern "C"
namespace {
struct F3 {
  float x, y, z;
};
inline F3 f3(float a, float b, float c) { return F3{a, b, c}; }
inline F3 fadd(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline F3 fsub(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline F3 fmul(F3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
inline float fdot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float fcomp(F3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
inline F3 fnormalized(F3 a) {  // taichi: (1 / norm) * v
  float inv = 1.0f / std::sqrt(fdot(a, a));
  return fmul(a, inv);
}
// mapply_pos (tina/common.py:169-183), M row-major 4x4
inline F3 fmapply(const float* M, F3 p) {
  float r[3];
  for (int i = 0; i < 3; ++i) r[i] = M[4 * i + 3] + M[4 * i] * p.x + M[4 * i + 1] * p.y + M[4 * i + 2] * p.z;
  float w = M[15] + M[12] * p.x + M[13] * p.y + M[14] * p.z;
  return f3(r[0] / w, r[1] / w, r[2] / w);
}
struct RVol {
  const float* sdf;
  const float* color;
  float b0[3], b1[3];
  int res[3];
  float thr;
};
// sample_tex (particle_sdf.py:271-290)
void rsample_tex(const float* tex, int nc, const int* res, const float* q, float* out) {
  float pos[3], fx[3];
  int b[3], b1[3];
  for (int c = 0; c < 3; ++c) {
    pos[c] = q[c] * (float)res[c];
    int t = (int)pos[c];
    b[c] = std::min(t, res[c] - 1);
    fx[c] = pos[c] - (float)b[c];
    b1[c] = std::min(b[c] + 1, res[c] - 1);
  }
  auto at = [&](int x, int y, int z, int ch) { return tex[(((int64_t)x * res[1] + y) * res[2] + z) * nc + ch]; };
  for (int ch = 0; ch < nc; ++ch) {
    float c00 = at(b[0], b[1], b[2], ch) * (1 - fx[0]) + at(b1[0], b[1], b[2], ch) * fx[0];
    float c01 = at(b[0], b[1], b1[2], ch) * (1 - fx[0]) + at(b1[0], b[1], b1[2], ch) * fx[0];
    float c10 = at(b[0], b1[1], b[2], ch) * (1 - fx[0]) + at(b1[0], b1[1], b[2], ch) * fx[0];
    float c11 = at(b[0], b1[1], b1[2], ch) * (1 - fx[0]) + at(b1[0], b1[1], b1[2], ch) * fx[0];
    float c0 = c00 * (1 - fx[1]) + c10 * fx[1];
    float c1 = c01 * (1 - fx[1]) + c11 * fx[1];
    out[ch] = c0 * (1 - fx[2]) + c1 * fx[2];
  }
}
bool rcoord(const RVol& V, F3 p, float* q) {
  for (int c = 0; c < 3; ++c) q[c] = (fcomp(p, c) - V.b0[c]) / (V.b1[c] - V.b0[c]);
  return std::min(q[0], std::min(q[1], q[2])) >= 0.0f && std::max(q[0], std::max(q[1], q[2])) <= 1.0f;
}
float rsdf(const RVol& V, F3 p) {
  float q[3], s = 0.0f;
  if (rcoord(V, p, q)) {
    rsample_tex(V.sdf, 1, V.res, q, &s);
    s = s - V.thr;
  }
  return s;
}
F3 rcolor(const RVol& V, F3 p) {
  float q[3], c[3] = {0, 0, 0};
  if (rcoord(V, p, q)) rsample_tex(V.color, 3, V.res, q, c);
  return f3(c[0], c[1], c[2]);
}
F3 rnormal(const RVol& V, F3 p) {
  const float d = 1e-3f;
  float n[3];
  for (int i = 0; i < 3; ++i) {
    F3 inc = p, dec = p;
    if (i == 0) { inc.x += d; dec.x -= d; }
    if (i == 1) { inc.y += d; dec.y -= d; }
    if (i == 2) { inc.z += d; dec.z -= d; }
    n[i] = (0.5f / d) * (rsdf(V, inc) - rsdf(V, dec));
  }
  return fnormalized(f3(n[0], n[1], n[2]));
}
}  // namespace
extern "C" {
// plb_set_particles + build_sdf_from_particles (particle_sdf.py:548-568, 237-265).
// x: double[n][3] (cast to f32); colors: uint32[n] 0xRRGGBB or null (white).
// sdf: float[res], color: float[res][3], bbox: float[6].  Returns 1 if the
// particles' box exceeds the volume (the reference asserts), else 0.
int oracle_render_bake(int64_t n, const double* x, const uint32_t* colors, const int* res, int bake_size, double dx,
                       float* sdf, float* color, float* bbox) {
  const float dxf = (float)dx, inv_dx = (float)(1.0 / dx);
  float lo[3] = {1e10f, 1e10f, 1e10f}, hi[3] = {-1e10f, -1e10f, -1e10f};
  for (int64_t i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) {
      float v = (std::floor((float)x[3 * i + c] * inv_dx) - 6.0f) * dxf;
      lo[c] = std::min(lo[c], v);
      hi[c] = std::max(hi[c], v);
    }
  int over = 0;
  for (int c = 0; c < 3; ++c) {
    if (!(((double)hi[c] - (double)lo[c]) / dx < (double)res[c])) over = 1;
    bbox[c] = lo[c];
    bbox[3 + c] = (float)((double)lo[c] + (double)res[c] * dx);
  }
  if (n == 0) over = 1;
  const int64_t nv = (int64_t)res[0] * res[1] * res[2];
  std::vector<int64_t> vol(nv, (int64_t)0xFFFFFFFF);  // (((1 << 31) - 1) + 1) * 2 - 1
  for (int64_t i = 0; i < n; ++i) {
    float p[3];
    int coord[3];
    for (int c = 0; c < 3; ++c) {
      p[c] = ((float)x[3 * i + c] - bbox[c]) * inv_dx;
      coord[c] = (int)p[c];
    }
    const int64_t col = colors ? (int64_t)colors[i] : 0xFFFFFF;
    for (int a = -bake_size - 1; a < bake_size + 1; ++a)
      for (int b = -bake_size - 1; b < bake_size + 1; ++b)
        for (int c = -bake_size - 1; c < bake_size + 1; ++c) {
          int ix = coord[0] + a, iy = coord[1] + b, iz = coord[2] + c;
          if (ix < 0 || iy < 0 || iz < 0 || ix >= res[0] || iy >= res[1] || iz >= res[2]) continue;
          float d0 = (float)ix - p[0], d1 = (float)iy - p[1], d2 = (float)iz - p[2];
          float dist = std::sqrt(d0 * d0 + d1 * d1 + d2 * d2);
          float q = std::min(std::max(0.0f, 51.0f * dist), 255.0f);
          int64_t v = ((int64_t)q << 24) + col;
          int64_t& t = vol[((int64_t)ix * res[1] + iy) * res[2] + iz];
          if (v < t) t = v;
        }
  }
  std::vector<float> s0(nv), s1(nv);
  for (int64_t i = 0; i < nv; ++i) {
    int64_t c = vol[i];
    for (int j = 2; j >= 0; --j) {
      color[3 * i + j] = (float)(c & 255) / 255.0f;
      c >>= 8;
    }
    s0[i] = (float)(c & 255) / 255.0f;
  }
  auto smooth = [&](const std::vector<float>& in, float* out) {
    for (int x0 = 0; x0 < res[0]; ++x0)
      for (int y0 = 0; y0 < res[1]; ++y0)
        for (int z0 = 0; z0 < res[2]; ++z0) {
          int64_t id = ((int64_t)x0 * res[1] + y0) * res[2] + z0;
          if (x0 >= 1 && y0 >= 1 && z0 >= 1 && x0 < res[0] - 1 && y0 < res[1] - 1 && z0 < res[2] - 1) {
            float sum = 0.0f;
            for (int a = -1; a < 2; ++a)
              for (int b = -1; b < 2; ++b)
                for (int c = -1; c < 2; ++c) sum += in[((int64_t)(x0 + a) * res[1] + (y0 + b)) * res[2] + (z0 + c)];
            out[id] = sum / 27.0f;
          } else {
            out[id] = 1.0f;
          }
        }
  };
  smooth(s0, s1.data());
  smooth(s1, sdf);
  return over;
}
// render_color + next_hit (particle_sdf.py:185-217, 353-440) per pixel; cam =
// V2W[16] then W2V[16]; tools at pose; tool_color [T][3].  Outputs as
// mpm_render_trace: depth [rx][ry], normal / color / image [rx][ry][3].
void oracle_render_trace(const float* sdf, const float* color, const float* bbox, const int* res, float thr,
                         const float* cam, int rx, int ry, float biasx, float biasy, const OracleTool* tools, int T,
                         const double* pose, const float* tool_color, int show_particles, float* depth, float* normal,
                         float* color_out, float* image) {
  RVol V;
  V.sdf = sdf;
  V.color = color;
  for (int c = 0; c < 3; ++c) {
    V.b0[c] = bbox[c];
    V.b1[c] = bbox[3 + c];
    V.res[c] = res[c];
  }
  V.thr = thr;
  const float* V2W = cam;
  const float* W2V = cam + 16;
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t pix = 0; pix < (int64_t)rx * ry; ++pix) {
    int px = (int)(pix / ry), py = (int)(pix % ry);
    float u = ((float)px + biasx) / (float)rx * 2.0f - 1.0f;
    float w = ((float)py + biasy) / (float)ry * 2.0f - 1.0f;
    F3 Pl = fmapply(V2W, f3(u, w, 1.0f)), o = fmapply(V2W, f3(u, w, 0.0f));
    F3 d = fnormalized(fsub(Pl, o));
    float closest = 0.99f;
    F3 nrm = f3(0, 1, 0), col = f3(0.3f * 0.3f, 0.5f * 0.3f, 0.7f * 0.3f);
    if (T > 0) {
      int j = 0, sid = 0;
      float dist = 0.0f, sval = 1e10f;
      F3 pp = o;
      while (j < 200 && dist < 100.0f && sval > 1e-8f) {
        pp = fadd(o, fmul(d, dist));
        sval = 1e10f;
        for (int i = 0; i < T; ++i) {
          const double q[3] = {pp.x, pp.y, pp.z};
          float dd = (float)tool_sdf(tools[i], pose + 8 * i, q);
          if (dd < sval) {
            sval = dd;
            sid = i;
          }
        }
        dist += sval;
        ++j;
      }
      float dz = fmapply(W2V, pp).z;
      if (dz < closest && dz < 100.0f) {
        closest = dz;
        F3 h = fadd(o, fmul(d, dist));
        const double q[3] = {h.x, h.y, h.z};
        double n[3];
        tool_normal(tools[sid], pose + 8 * sid, q, n);
        nrm = f3((float)n[0], (float)n[1], (float)n[2]);
        col = f3(tool_color[3 * sid], tool_color[3 * sid + 1], tool_color[3 * sid + 2]);
      }
    }
    if (show_particles) {
      // ray_aabb_intersection (renderer_utils.py:53-73)
      bool hit = true;
      float tn = -1e10f, tf = 1e10f;
      for (int i = 0; i < 3; ++i) {
        float oi = fcomp(o, i), di = fcomp(d, i);
        if (di == 0.0f) {
          if (oi < V.b0[i] || oi > V.b1[i]) hit = false;
        } else {
          float i1 = (V.b0[i] - oi) / di, i2 = (V.b1[i] - oi) / di;
          float nf = (i2 < i1) ? i1 : i2, nn = (i1 < i2) ? i1 : i2;
          tf = (nf < tf) ? nf : tf;
          tn = (tn < nn) ? nn : tn;
        }
      }
      if (tn > tf) hit = false;
      if (hit) {
        tn = (0.0f < tn) ? tn : 0.0f;
        F3 pos = fadd(o, fmul(d, tn + 1e-4f)), step = f3(0, 0, 0);
        for (int j = 0; j < 500; ++j) {
          float s = rsdf(V, pos);
          if (s < 0.0f) {
            F3 back = step;
            for (int k = 0; k < 20; ++k) {
              back = fmul(back, 0.5f);
              if (rsdf(V, fsub(pos, back)) < 0.0f) pos = fsub(pos, back);
            }
            float dz = fmapply(W2V, pos).z;
            if (dz < closest) {
              closest = dz;
              nrm = rnormal(V, pos);
              col = rcolor(V, pos);
            }
            break;
          }
          float a = s * 0.005f;
          step = fmul(d, (a < 0.002f) ? 0.002f : a);
          pos = fadd(pos, step);
        }
      }
    }
    col = fmul(col, 3.0f);
    depth[pix] = closest;
    normal[3 * pix] = nrm.x;
    normal[3 * pix + 1] = nrm.y;
    normal[3 * pix + 2] = nrm.z;
    color_out[3 * pix] = col.x;
    color_out[3 * pix + 1] = col.y;
    color_out[3 * pix + 2] = col.z;
    if (image) {
      float il = 1.0f / std::sqrt(14.0f);
      float cos_i = nrm.x * il + nrm.y * (2.0f * il) + nrm.z * (3.0f * il);
      float lam = cos_i > 0.0f ? cos_i * 0.9f * (1.0f / 3.14159265358979f) : 0.0f;
      image[3 * pix] = 0.1f * col.x + lam * col.x;
      image[3 * pix + 1] = 0.1f * col.y + lam * col.y;
      image[3 * pix + 2] = 0.1f * col.z + lam * col.z;
    }
  }
}

}  // extern "C"
