// Tool kinematics of one action in FP64, with tool-tool collision projection,
// and their adjoint.
//
//   set_velocity          primive_base.py:260-268; Gripper primitives.py:463-469,
//                         Chopsticks 238-245, Gripper2 595-601
//   forward_kinematics    primive_base.py:153-156; RollingPin primitives.py:104-117,
//                         RollingPinExt 122-135, Chopsticks 231-235, Gripper 457-460,
//                         Gripper2 589-592
//   collision projection  mpm_simulator.py:287-305 (set_surface_points,
//                         set_collision_idx, apply_collision_projection) with
//                         Primitive.get_collision_idx / collision_projection
//                         (primive_base.py:135-150) and Box._project (primitives.py:370-372)
//
// One warp per scene: lane t runs the kinematics of the scene's tool t, then
// the warp evaluates each collision pair's 600 surface points together.  The
// adjoint follows the reference's autodiff: apply_collision_projection.grad and
// set_surface_points.grad run before forward_kinematics.grad of the substep,
// read the poses of frame f+1 as stored after the projection, and take the
// surface point stored by the forward pass.
#include "mpm_launch.h"
#include "mpm_math.cuh"
#include "mpm_tools.cuh"

namespace mpm {

namespace {

MPM_DI bool has_gap_vel(int type) {
  return type == TOOL_GRIPPER || type == TOOL_CHOPSTICKS || type == TOOL_GRIPPER2;
}
// rotation applied on the right: rotation[f] * w2quat(w)
MPM_DI bool right_rotation(int type) { return has_gap_vel(type); }
MPM_DI bool rolling_pin(int type) { return type == TOOL_ROLLINGPIN || type == TOOL_ROLLINGPINEXT; }

MPM_DI void clamp_pos(const MpmToolDesc& d, const double* p0, const double* dv, double* p1) {
  for (int k = 0; k < 3; ++k) {
    double a = p0[k] + dv[k];
    double mn = (a < d.upper[k]) ? a : d.upper[k];
    p1[k] = (d.lower[k] < mn) ? mn : d.lower[k];
  }
}
// adjoint of clamp_pos: g flows to p0 and dv where neither bound is active
MPM_DI void clamp_pos_vjp(const MpmToolDesc& d, const double* p0, const double* dv, const double* g1, double* g0,
                          double* gdv) {
  for (int k = 0; k < 3; ++k) {
    double a = p0[k] + dv[k];
    double mn = (a < d.upper[k]) ? a : d.upper[k];
    if ((a < d.upper[k]) && (d.lower[k] < mn)) {
      g0[k] += g1[k];
      gdv[k] += g1[k];
    }
  }
}

// set_velocity: the velocity of every substep of the action
MPM_DI void action_velocity(const MpmToolDesc& d, const double* a, int n_sub, double* vv) {
  for (int k = 0; k < 8; ++k) vv[k] = 0.0;
  if (d.action_dim <= 0) return;
  for (int k = 0; k < 3; ++k) vv[k] = a[k] * d.action_scale[k] / n_sub;
  if (d.action_dim > 3)
    for (int k = 0; k < 3; ++k) vv[3 + k] = a[3 + k] * d.action_scale[3 + k] / n_sub;
  if (has_gap_vel(d.type)) vv[6] = a[6] * d.action_scale[6] / n_sub;
}

// RollingPin / RollingPinExt: v = (dw, dth, dy); the pin rolls about its own
// axis by dw and travels dw*0.03 (+ w[0] for RollingPinExt) along
// (0,1,0) x qrot(rot, (0,-1,0)), turns about the world y axis by dth and
// moves dy in y
MPM_DI void rolling_fk(const MpmToolDesc& d, const double* p0, const double* vv, double* p1) {
  const double dw = vv[0], dth = vv[1], dy = vv[2];
  const double down[3] = {0.0, -1.0, 0.0};
  double yd[3];
  qrot(p0 + 3, down, yd);
  const double s = dw * 0.03 + (d.type == TOOL_ROLLINGPINEXT ? vv[3] : 0.0);
  const double xd[3] = {yd[2] * s, dy, -yd[0] * s};
  clamp_pos(d, p0, xd, p1);
  const double wa[3] = {0.0, -dth, 0.0}, wb[3] = {0.0, dw, 0.0};
  double qa[4], qb[4], t[4];
  w2quat(wa, qa);
  w2quat(wb, qb);
  qmul(p0 + 3, qb, t);
  qmul(qa, t, p1 + 3);
  p1[7] = p0[7];
}
MPM_DI void rolling_fk_vjp(const MpmToolDesc& d, const double* p0, const double* vv, const double* g1, double* g0,
                           double* gvv) {
  const double dw = vv[0], dth = vv[1];
  const double down[3] = {0.0, -1.0, 0.0};
  double yd[3];
  qrot(p0 + 3, down, yd);
  const double s = dw * 0.03 + (d.type == TOOL_ROLLINGPINEXT ? vv[3] : 0.0);
  const double xd[3] = {yd[2] * s, vv[2], -yd[0] * s};
  double gxd[3] = {0.0, 0.0, 0.0};
  clamp_pos_vjp(d, p0, xd, g1, g0, gxd);
  gvv[2] += gxd[1];
  const double gs = gxd[0] * yd[2] - gxd[2] * yd[0];
  const double gyd[3] = {-gxd[2] * s, 0.0, gxd[0] * s};
  qrot_vjp(p0 + 3, down, gyd, g0 + 3, (double*)nullptr);
  gvv[0] += gs * 0.03;
  if (d.type == TOOL_ROLLINGPINEXT) gvv[3] += gs;
  const double wa[3] = {0.0, -dth, 0.0}, wb[3] = {0.0, dw, 0.0};
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
}

// forward_kinematics of every other type; wq = w2quat(w), the same for the
// whole action
MPM_DI void fk_step(const MpmToolDesc& d, const double* p0, const double* vv, const double* wq, double* p1) {
  if (rolling_pin(d.type)) {
    rolling_fk(d, p0, vv, p1);
    return;
  }
  clamp_pos(d, p0, vv, p1);
  if (right_rotation(d.type)) {
    qmul(p0 + 3, wq, p1 + 3);
  } else {
    qmul(wq, p0 + 3, p1 + 3);
  }
  if (d.type == TOOL_GRIPPER || d.type == TOOL_GRIPPER2) {  // min(max(gap - gap_vel, min_gap), max_gap)
    double a = p0[7] - vv[6];
    double mx = (d.min_gap < a) ? a : d.min_gap;
    p1[7] = (mx < d.max_gap) ? mx : d.max_gap;
  } else if (d.type == TOOL_CHOPSTICKS) {  // max(gap - gap_vel, minimal_gap)
    double a = p0[7] - vv[6];
    p1[7] = (d.min_gap < a) ? a : d.min_gap;
  } else {
    p1[7] = p0[7];
  }
}
// adjoint of fk_step (not rolling pins); the w2quat part is left in gwq
MPM_DI void fk_step_vjp(const MpmToolDesc& d, const double* p0, const double* vv, const double* wq, const double* g1,
                        double* g0, double* gvv, double* gwq) {
  clamp_pos_vjp(d, p0, vv, g1, g0, gvv);
  if (right_rotation(d.type)) {
    qmul_vjp(p0 + 3, wq, g1 + 3, g0 + 3, gwq);
  } else {
    qmul_vjp(wq, p0 + 3, g1 + 3, gwq, g0 + 3);
  }
  if (d.type == TOOL_GRIPPER || d.type == TOOL_GRIPPER2) {
    double a = p0[7] - vv[6];
    double mx = (d.min_gap < a) ? a : d.min_gap;
    if ((d.min_gap < a) && (mx < d.max_gap)) {
      g0[7] += g1[7];
      gvv[6] -= g1[7];
    }
  } else if (d.type == TOOL_CHOPSTICKS) {
    double a = p0[7] - vv[6];
    if (d.min_gap < a) {
      g0[7] += g1[7];
      gvv[6] -= g1[7];
    }
  } else {
    g0[7] += g1[7];
  }
}

constexpr int N_SURFACE_POINTS = 600;  // num_particle_collision (mpm_simulator.py:59)

// Box._project of the scaled random point, rotated and moved to the box pose
MPM_DI void surface_point(const MpmToolDesc& box, const double* pose, const double* rn, double* local,
                          double* world) {
  for (int k = 0; k < 3; ++k) {
    const double s = box.size[k];
    const double a = rn[k] * s;
    const double mn = (a < s) ? a : s;
    local[k] = (-s < mn) ? mn : -s;
  }
  qrot(pose + 3, local, world);
  for (int k = 0; k < 3; ++k) world[k] += pose[k];
}

// pair c of a scene: tool i (projected) and tool j (the box), scene-local
MPM_DI bool scene_pair(const MpmToolDesc* __restrict__ tools, int t0, int nt, int c, int& i, int& j) {
  int n = 0;
  for (int a = 0; a < nt; ++a)
    for (int b = 0; b < nt; ++b)
      if ((tools[t0 + a].collision_mask >> b) & 1) {
        if (n == c) {
          i = a;
          j = b;
          return true;
        }
        ++n;
      }
  return false;
}

// collision projection of the poses of one frame (pose1 = that frame's poses)
MPM_DI void project_frame(const MpmToolDesc* __restrict__ tools, int t0, int nt, int np, const double* coll_pts,
                          double* pose1, double* coll) {
  const int lane = threadIdx.x & 31;
  // set_surface_points + set_collision_idx for every pair, before any projection
  for (int c = 0; c < np; ++c) {
    int i = 0, j = 0;
    scene_pair(tools, t0, nt, c, i, j);
    Tool<double> ti;
    Pose<double> Pi;
    to_tool(tools[t0 + i], ti);
    to_pose(pose1 + 8 * (t0 + i), Pi);
    double best = INFINITY;
    int bidx = N_SURFACE_POINTS;
    for (int k = lane; k < N_SURFACE_POINTS; k += 32) {
      double local[3], pt[3];
      surface_point(tools[t0 + j], pose1 + 8 * (t0 + j), coll_pts + 3 * ((int64_t)c * N_SURFACE_POINTS + k), local,
                    pt);
      const double sd = tool_sdf(ti, Pi, pt);
      if (sd < best) {
        best = sd;
        bidx = k;
      }
    }
    // the first index of the minimum, if the minimum is below the initial 0
    double m = best;
    for (int o = 16; o > 0; o >>= 1) m = fmin(m, __shfl_xor_sync(0xffffffffu, m, o));
    const int cand = (best == m) ? bidx : N_SURFACE_POINTS;
    const int idx = __reduce_min_sync(0xffffffffu, cand);
    if (lane == 0) {
      double* rec = coll + 4 * c;
      if (m < 0.0 && idx < N_SURFACE_POINTS) {
        double local[3], pt[3];
        surface_point(tools[t0 + j], pose1 + 8 * (t0 + j), coll_pts + 3 * ((int64_t)c * N_SURFACE_POINTS + idx),
                      local, pt);
        rec[0] = (double)idx;
        rec[1] = pt[0];
        rec[2] = pt[1];
        rec[3] = pt[2];
      } else {
        rec[0] = -1.0;
        rec[1] = rec[2] = rec[3] = 0.0;
      }
    }
  }
  __syncwarp();
  // apply_collision_projection in pair order: pos_i += normalized(normal) * sdf
  if (lane == 0) {
    for (int c = 0; c < np; ++c) {
      const double* rec = coll + 4 * c;
      if (rec[0] < 0.0) continue;
      int i = 0, j = 0;
      scene_pair(tools, t0, nt, c, i, j);
      Tool<double> ti;
      Pose<double> Pi;
      to_tool(tools[t0 + i], ti);
      to_pose(pose1 + 8 * (t0 + i), Pi);
      const double pt[3] = {rec[1], rec[2], rec[3]};
      const double d = tool_sdf(ti, Pi, pt);
      double n[3];
      tool_normal(ti, Pi, pt, n);
      const double inv = 1.0 / sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
      for (int k = 0; k < 3; ++k) pose1[8 * (t0 + i) + k] += n[k] * inv * d;
    }
  }
  __syncwarp();
}

// adjoint of project_frame at one frame, pairs in reverse order
MPM_DI void project_frame_vjp(const MpmToolDesc* __restrict__ tools, int t0, int nt, int np, const double* coll_pts,
                              const double* pose1, const double* coll, double* g1) {
  if ((threadIdx.x & 31) == 0) {
    for (int c = np - 1; c >= 0; --c) {
      const double* rec = coll + 4 * c;
      if (rec[0] < 0.0) continue;
      int i = 0, j = 0;
      scene_pair(tools, t0, nt, c, i, j);
      Tool<double> ti;
      Pose<double> Pi;
      to_tool(tools[t0 + i], ti);
      to_pose(pose1 + 8 * (t0 + i), Pi);
      const double pt[3] = {rec[1], rec[2], rec[3]};
      const double d = tool_sdf(ti, Pi, pt);
      double n[3];
      tool_normal(ti, Pi, pt, n);
      const double len = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
      const double nn[3] = {n[0] / len, n[1] / len, n[2] / len};
      double* gi = g1 + 8 * (t0 + i);
      const double gs[3] = {gi[0], gi[1], gi[2]};  // adjoint of the shift added to pos_i
      const double gd = gs[0] * nn[0] + gs[1] * nn[1] + gs[2] * nn[2];
      const double gnn[3] = {gs[0] * d, gs[1] * d, gs[2] * d};
      const double dn = nn[0] * gnn[0] + nn[1] * gnn[1] + nn[2] * gnn[2];
      const double gn[3] = {(gnn[0] - nn[0] * dn) / len, (gnn[1] - nn[1] * dn) / len, (gnn[2] - nn[2] * dn) / len};
      PoseGrad<double> gP;
      gP.zero();
      double gp[3] = {0.0, 0.0, 0.0};
      tool_sdf_vjp(ti, Pi, pt, gd, gp, gP);
      tool_normal_vjp(ti, Pi, pt, gn, gp, gP);
      for (int k = 0; k < 3; ++k) gi[k] += gP.pos[k];
      for (int k = 0; k < 4; ++k) gi[3 + k] += gP.rot[k];
      gi[7] += gP.gap;
      // set_surface_points.grad: point = qrot(rot_j, local) + pos_j
      double local[3], w[3];
      const double* pj = pose1 + 8 * (t0 + j);
      surface_point(tools[t0 + j], pj, coll_pts + 3 * ((int64_t)c * N_SURFACE_POINTS + (int)rec[0]), local, w);
      double* gj = g1 + 8 * (t0 + j);
      for (int k = 0; k < 3; ++k) gj[k] += gp[k];
      qrot_vjp(pj + 3, local, gp, gj + 3, (double*)nullptr);
    }
  }
  __syncwarp();
}

__global__ void k_tools_action(const MpmToolDesc* __restrict__ tools, const int* __restrict__ tool_off,
                               const int* __restrict__ pair_off, int n_scenes, int n_tools, int n_pairs,
                               const double* __restrict__ coll_pts, const double* __restrict__ action,
                               double* __restrict__ vel, double* pose, double* __restrict__ coll, int n_sub) {
  const int scene = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  if (scene >= n_scenes) return;  // whole warps
  const int lane = threadIdx.x & 31;
  const int t0 = tool_off[scene], nt = tool_off[scene + 1] - t0;
  const int np = pair_off[scene + 1] - pair_off[scene];
  const bool mine = lane < nt;
  MpmToolDesc d;
  double vv[8], wq[4] = {1, 0, 0, 0};
  if (mine) {
    d = tools[t0 + lane];
    action_velocity(d, action + 8 * (t0 + lane), n_sub, vv);
    w2quat(vv + 3, wq);
  }
  for (int s = 0; s < n_sub; ++s) {
    if (mine) {
      const int t = t0 + lane;
      for (int k = 0; k < 8; ++k) vel[((int64_t)s * n_tools + t) * 8 + k] = vv[k];
      fk_step(d, pose + ((int64_t)s * n_tools + t) * 8, vv, wq, pose + ((int64_t)(s + 1) * n_tools + t) * 8);
    }
    __syncwarp();
    if (np > 0)
      project_frame(tools, t0, nt, np, coll_pts, pose + (int64_t)(s + 1) * n_tools * 8,
                    coll + ((int64_t)s * n_pairs + pair_off[scene]) * 4);
  }
}

__global__ void k_tools_action_bwd(const MpmToolDesc* __restrict__ tools, const int* __restrict__ tool_off,
                                   const int* __restrict__ pair_off, int n_scenes, int n_tools, int n_pairs,
                                   const double* __restrict__ coll_pts, const double* __restrict__ vel,
                                   const double* __restrict__ pose, const double* __restrict__ coll, double* g_pose,
                                   double* __restrict__ g_action, int n_sub) {
  const int scene = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  if (scene >= n_scenes) return;  // whole warps
  const int lane = threadIdx.x & 31;
  const int t0 = tool_off[scene], nt = tool_off[scene + 1] - t0;
  const int np = pair_off[scene + 1] - pair_off[scene];
  const bool mine = lane < nt;
  const int t = t0 + lane;
  MpmToolDesc d;
  if (mine) d = tools[t];
  double gvv_sum[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  // w2quat and its adjoint are evaluated once per run of substeps with the
  // same angular velocity (set_velocity writes one per action): the
  // quaternion gradient is summed over the run first (w2quat_vjp is linear in it)
  double w_run[3] = {0, 0, 0}, wq[4] = {1, 0, 0, 0}, gwq_run[4] = {0, 0, 0, 0};
  bool have_run = false;
  for (int s = n_sub - 1; s >= 0; --s) {
    if (np > 0)
      project_frame_vjp(tools, t0, nt, np, coll_pts, pose + (int64_t)(s + 1) * n_tools * 8,
                        coll + ((int64_t)s * n_pairs + pair_off[scene]) * 4, g_pose + (int64_t)(s + 1) * n_tools * 8);
    if (mine) {
      const double* p0 = pose + ((int64_t)s * n_tools + t) * 8;
      const double* vv = vel + ((int64_t)s * n_tools + t) * 8;
      const double* g1 = g_pose + ((int64_t)(s + 1) * n_tools + t) * 8;
      // frame s gets this step's contribution by atomic adds: frame 0 of the
      // action is also the last frame of the action before, whose MPM adjoint
      // may be adding pose gradients to it at the same time
      double g0[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      double gvv[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      if (rolling_pin(d.type)) {
        rolling_fk_vjp(d, p0, vv, g1, g0, gvv);
      } else {
        if (!have_run || vv[3] != w_run[0] || vv[4] != w_run[1] || vv[5] != w_run[2]) {
          if (have_run) w2quat_vjp(w_run, gwq_run, gvv_sum + 3);
          for (int k = 0; k < 3; ++k) w_run[k] = vv[3 + k];
          for (int k = 0; k < 4; ++k) gwq_run[k] = 0.0;
          w2quat(w_run, wq);
          have_run = true;
        }
        fk_step_vjp(d, p0, vv, wq, g1, g0, gvv, gwq_run);
      }
      double* gd = g_pose + ((int64_t)s * n_tools + t) * 8;
      for (int k = 0; k < 8; ++k)
        if (g0[k] != 0.0) atomicAdd(gd + k, g0[k]);
      for (int k = 0; k < 8; ++k) gvv_sum[k] += gvv[k];
    }
    __syncwarp();
  }
  if (mine) {
    if (have_run) w2quat_vjp(w_run, gwq_run, gvv_sum + 3);
    // set_velocity.grad: v = a * scale / n_sub for every substep of the action
    if (d.action_dim > 0) {
      for (int k = 0; k < 3; ++k) g_action[8 * t + k] += gvv_sum[k] * d.action_scale[k] / n_sub;
      if (d.action_dim > 3)
        for (int k = 0; k < 3; ++k) g_action[8 * t + 3 + k] += gvv_sum[3 + k] * d.action_scale[3 + k] / n_sub;
      if (has_gap_vel(d.type)) g_action[8 * t + 6] += gvv_sum[6] * d.action_scale[6] / n_sub;
    }
  }
}

}  // namespace

cudaError_t launch_tools_action(const LaunchCtx& L, int n_tools, const int* pair_off, int n_pairs,
                                const double* coll_pts, const double* action, double* vel, double* pose, double* coll,
                                int n_sub) {
  const int S = L.p->n_scenes;
  MPM_LAUNCH(L, MPM_K_OTHER, k_tools_action, (unsigned)((S * 32 + 127) / 128), 128, L.tools, L.tool_off, pair_off, S,
             n_tools, n_pairs, coll_pts, action, vel, pose, coll, n_sub);
  return cudaGetLastError();
}
cudaError_t launch_tools_action_bwd(const LaunchCtx& L, int n_tools, const int* pair_off, int n_pairs,
                                    const double* coll_pts, const double* vel, const double* pose, const double* coll,
                                    double* g_pose, double* g_action, int n_sub) {
  const int S = L.p->n_scenes;
  MPM_LAUNCH(L, MPM_K_OTHER, k_tools_action_bwd, (unsigned)((S * 32 + 127) / 128), 128, L.tools, L.tool_off,
             pair_off, S, n_tools, n_pairs, coll_pts, vel, pose, coll, g_pose, g_action, n_sub);
  return cudaGetLastError();
}

}  // namespace mpm
