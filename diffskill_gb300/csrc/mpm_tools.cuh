// Rigid tools on the device: SDFs, normals, collider velocity, the soft
// contact response of grid_op, and the vector-Jacobian products of each.
//
// Restates plb/engine/primitive/primive_base.py:75-120 (sdf, normal,
// collider_v, collide) and the shapes of plb/engine/primitive/primitives.py:
// Sphere 23-40, Capsule 55-66, Box 375-393, Prism 712-730, Knife 770-807,
// Gripper 471-536.
#pragma once
#include "mpm_math.cuh"

namespace mpm {

enum { TOOL_SPHERE = 0, TOOL_CAPSULE = 1, TOOL_BOX = 2, TOOL_KNIFE = 3, TOOL_GRIPPER = 4 };
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
template <typename T>
MPM_DI T local_sdf(const Tool<T>& t, const T* q) {
  if (t.type == TOOL_CAPSULE) {
    T p2[3], dp;
    capsule_p2(t, q, p2, &dp);
    return len14(p2) - t.cap_r;
  }
  if (t.type == TOOL_KNIFE) {
    T a = prism_sdf(t, q), b = box_sdf(t.size, q);
    return (b < a) ? a : b;
  }
  return box_sdf(t.size, q);  // Box and Gripper fingers
}
template <typename T>
MPM_DI void local_sdf_grad(const Tool<T>& t, const T* q, T g, T* gq) {
  if (t.type == TOOL_CAPSULE) {
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
// finite-difference normal before normalisation (Box._normal, Knife._normal)
template <typename T>
MPM_DI void fd_normal_raw(const Tool<T>& t, const T* q, T* r) {
  const T d = fd_step<T>();
  const T h = T(0.5) / d;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    T inc[3] = {q[0], q[1], q[2]}, dec[3] = {q[0], q[1], q[2]};
    inc[i] += d;
    dec[i] -= d;
    r[i] = h * (local_sdf(t, inc) - local_sdf(t, dec));
  }
}
template <typename T>
MPM_DI void local_normal(const Tool<T>& t, const T* q, T* n) {
  T r[3];
  if (t.type == TOOL_CAPSULE) {
    T dp;
    capsule_p2(t, q, r, &dp);
  } else {
    fd_normal_raw(t, q, r);
  }
  T iL = T(1) / len14(r);
#pragma unroll
  for (int k = 0; k < 3; ++k) n[k] = r[k] * iL;
}
template <typename T>
MPM_DI void local_normal_vjp(const Tool<T>& t, const T* q, const T* gn, T* gq) {
  T r[3], gr[3];
  if (t.type == TOOL_CAPSULE) {
    T dp;
    capsule_p2(t, q, r, &dp);
    unit14_vjp(r, gn, gr);
    gq[0] += gr[0];
    gq[1] += gr[1] * dp;
    gq[2] += gr[2];
    return;
  }
  fd_normal_raw(t, q, r);
  unit14_vjp(r, gn, gr);
  const T d = fd_step<T>();
  const T h = T(0.5) / d;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    T inc[3] = {q[0], q[1], q[2]}, dec[3] = {q[0], q[1], q[2]};
    inc[i] += d;
    dec[i] -= d;
    local_sdf_grad(t, inc, h * gr[i], gq);
    local_sdf_grad(t, dec, -h * gr[i], gq);
  }
}

// ------------------------------ world space --------------------------------
// "rigid" pose = (pos, rot); Sphere ignores rot (primitives.py:28-34)
template <typename T>
MPM_DI T shape_sdf(const Tool<T>& t, const T* pos, const T* rot, const T* p) {
  if (t.type == TOOL_SPHERE) {
    const T d[3] = {p[0] - pos[0], p[1] - pos[1], p[2] - pos[2]};
    return len14(d) - t.radius;
  }
  T q[3];
  inv_trans(p, pos, rot, q);
  return local_sdf(t, q);
}
template <typename T>
MPM_DI void shape_sdf_vjp(const Tool<T>& t, const T* pos, const T* rot, const T* p, T g, T* gp, T* gpos, T* grot) {
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
  local_sdf_grad(t, q, g, gq);
  inv_trans_vjp(p, pos, rot, gq, gp, gpos, grot);
}
template <typename T>
MPM_DI void shape_normal(const Tool<T>& t, const T* pos, const T* rot, const T* p, T* n) {
  if (t.type == TOOL_SPHERE) {
    const T d[3] = {p[0] - pos[0], p[1] - pos[1], p[2] - pos[2]};
    T iL = T(1) / len14(d);
#pragma unroll
    for (int k = 0; k < 3; ++k) n[k] = d[k] * iL;
    return;
  }
  T q[3], nl[3];
  inv_trans(p, pos, rot, q);
  local_normal(t, q, nl);
  qrot(rot, nl, n);
}
template <typename T>
MPM_DI void shape_normal_vjp(const Tool<T>& t, const T* pos, const T* rot, const T* p, const T* gn, T* gpos,
                             T* grot) {
  if (t.type == TOOL_SPHERE) {
    const T d[3] = {p[0] - pos[0], p[1] - pos[1], p[2] - pos[2]};
    T gd[3];
    unit14_vjp(d, gn, gd);
#pragma unroll
    for (int k = 0; k < 3; ++k) gpos[k] -= gd[k];
    return;
  }
  T q[3], nl[3];
  inv_trans(p, pos, rot, q);
  local_normal(t, q, nl);
  T gnl[3] = {T(0), T(0), T(0)}, gq[3] = {T(0), T(0), T(0)};
  qrot_vjp(rot, nl, gn, grot, gnl);
  local_normal_vjp(t, q, gnl, gq);
  inv_trans_vjp(p, pos, rot, gq, (T*)nullptr, gpos, grot);
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
MPM_DI bool collide_fwd(const Tool<T>& t, const T* pos0, const T* rot0, const T* pos1, const T* rot1, const T* p,
                        T dt, const T* vin, T* vout) {
  T dist = shape_sdf(t, pos0, rot0, p);
  T e = mexp(-dist * t.softness);
  T infl = (e < T(1)) ? e : T(1);
#pragma unroll
  for (int k = 0; k < 3; ++k) vout[k] = vin[k];
  if (!((t.softness > T(0) && infl > T(0.1)) || dist <= T(0))) return false;
  T D[3], cv[3], iv[3], vt[3];
  shape_normal(t, pos0, rot0, p, D);
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
MPM_DI void collide_vjp(const Tool<T>& t, const T* pos0, const T* rot0, const T* pos1, const T* rot1, const T* p,
                        T dt, const T* vin, const T* gout, T* gvin, T* gpos0, T* grot0, T* gpos1, T* grot1) {
  T dist = shape_sdf(t, pos0, rot0, p);
  T e = mexp(-dist * t.softness);
  T infl = (e < T(1)) ? e : T(1);
  if (!((t.softness > T(0) && infl > T(0.1)) || dist <= T(0))) {
#pragma unroll
    for (int k = 0; k < 3; ++k) gvin[k] = gout[k];
    return;
  }
  T D[3], cv[3], iv[3], vt[3];
  shape_normal(t, pos0, rot0, p, D);
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
  shape_sdf_vjp(t, pos0, rot0, p, g_dist, (T*)nullptr, gpos0, grot0);
  shape_normal_vjp(t, pos0, rot0, p, g_D, gpos0, grot0);
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
template <typename T>
MPM_DI void tool_collide(const Tool<T>& t, const Pose<T>& P0, const Pose<T>& P1, const T* p, T dt, T* v) {
  T out[3];
  if (t.type == TOOL_GRIPPER) {
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      T flag = side == 0 ? T(-1) : T(1);
      T f0[3], f1[3];
      finger_pos(P0, flag, f0);
      finger_pos(P1, flag, f1);
      collide_fwd(t, f0, P0.rot, f1, P1.rot, p, dt, v, out);
#pragma unroll
      for (int k = 0; k < 3; ++k) v[k] = out[k];
    }
    return;
  }
  collide_fwd(t, P0.pos, P0.rot, P1.pos, P1.rot, p, dt, v, out);
#pragma unroll
  for (int k = 0; k < 3; ++k) v[k] = out[k];
}
// g: in = d/d vout, out = d/d vin
template <typename T>
MPM_DI void tool_collide_vjp(const Tool<T>& t, const Pose<T>& P0, const Pose<T>& P1, const T* p, T dt,
                             const T* vin, T* g, PoseGrad<T>& g0, PoseGrad<T>& g1) {
  T gin[3];
  if (t.type == TOOL_GRIPPER) {
    T fa0[3], fa1[3], fb0[3], fb1[3], mid[3];
    finger_pos(P0, T(-1), fa0);
    finger_pos(P1, T(-1), fa1);
    finger_pos(P0, T(1), fb0);
    finger_pos(P1, T(1), fb1);
    collide_fwd(t, fa0, P0.rot, fa1, P1.rot, p, dt, vin, mid);
    T gf0[3] = {T(0), T(0), T(0)}, gf1[3] = {T(0), T(0), T(0)};
    collide_vjp(t, fb0, P0.rot, fb1, P1.rot, p, dt, mid, g, gin, gf0, g0.rot, gf1, g1.rot);
    finger_pos_vjp(P0, T(1), gf0, g0);
    finger_pos_vjp(P1, T(1), gf1, g1);
    T gin2[3];
    T ga0[3] = {T(0), T(0), T(0)}, ga1[3] = {T(0), T(0), T(0)};
    collide_vjp(t, fa0, P0.rot, fa1, P1.rot, p, dt, vin, gin, gin2, ga0, g0.rot, ga1, g1.rot);
    finger_pos_vjp(P0, T(-1), ga0, g0);
    finger_pos_vjp(P1, T(-1), ga1, g1);
#pragma unroll
    for (int k = 0; k < 3; ++k) g[k] = gin2[k];
    return;
  }
  collide_vjp(t, P0.pos, P0.rot, P1.pos, P1.rot, p, dt, vin, g, gin, g0.pos, g0.rot, g1.pos, g1.rot);
#pragma unroll
  for (int k = 0; k < 3; ++k) g[k] = gin[k];
}

// world SDF (Gripper.sdf = min of fingers, primitives.py:486-487)
template <typename T>
MPM_DI T tool_sdf(const Tool<T>& t, const Pose<T>& P, const T* p) {
  if (t.type == TOOL_GRIPPER) {
    T fa[3], fb[3];
    finger_pos(P, T(-1), fa);
    finger_pos(P, T(1), fb);
    T a = shape_sdf(t, fa, P.rot, p), b = shape_sdf(t, fb, P.rot, p);
    return (a < b) ? a : b;
  }
  return shape_sdf(t, P.pos, P.rot, p);
}
template <typename T>
MPM_DI void tool_sdf_vjp(const Tool<T>& t, const Pose<T>& P, const T* p, T g, T* gp, PoseGrad<T>& gP) {
  if (t.type == TOOL_GRIPPER) {
    T fa[3], fb[3];
    finger_pos(P, T(-1), fa);
    finger_pos(P, T(1), fb);
    T a = shape_sdf(t, fa, P.rot, p), b = shape_sdf(t, fb, P.rot, p);
    T gf[3] = {T(0), T(0), T(0)};
    if (a < b) {
      shape_sdf_vjp(t, fa, P.rot, p, g, gp, gf, gP.rot);
      finger_pos_vjp(P, T(-1), gf, gP);
    } else {
      shape_sdf_vjp(t, fb, P.rot, p, g, gp, gf, gP.rot);
      finger_pos_vjp(P, T(1), gf, gP);
    }
    return;
  }
  shape_sdf_vjp(t, P.pos, P.rot, p, g, gp, gP.pos, gP.rot);
}

}  // namespace mpm
