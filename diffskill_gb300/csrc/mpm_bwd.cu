// Adjoint launchers: one substep's adjoint (grid recompute, g2p.grad,
// grid_op.grad, p2g.grad) and the soft-contact adjoint.
#include "mpm_kernels.cuh"
#include "mpm_launch.h"

namespace mpm {

template <typename T>
Consts<T> make_consts(const LaunchCtx& L);  // mpm_fwd.cu
template <typename T>
cudaError_t prepare_blocks(const LaunchCtx& L, const Consts<T>& c, const T* st, Node<T>* a, Node<T>* a_out,
                           Node<T>* b, const MpmGridStore* restore, int restore_slot, const MpmGridStore* reserve,
                           int reserve_slot, const double* pose_f, const double* pose_f1, bool premarked);
unsigned grid_blocks_launch(const LaunchCtx& L, int64_t total_blocks);

static inline unsigned blocks_for(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

template <typename T, typename S>
cudaError_t launch_substep_bwd(const LaunchCtx& L, const T* st0, const T* st1, const T* g1, T* g0,
                               const double* pose_f, const double* pose_f1, double* g_pose_f, double* g_pose_f1,
                               const MpmGridStore* store, int slot, unsigned phases) {
  Consts<T> c = make_consts<T>(L);
  Node<T>* gin = (Node<T>*)L.grid_a;
  Node<T>* gout = (Node<T>*)L.grid_b;
  Node<T>* g_gin = (Node<T>*)L.grid_c;
  Node<T>* g_gout = (Node<T>*)L.grid_d;
  const int* counter = reinterpret_cast<const int*>(L.blockbuf);
  const unsigned pb = blocks_for(c.n_particles, 128);
  const unsigned gb = grid_blocks_launch(L, (int64_t)c.n_scenes * c.NB3);
  const Tool<T>* tools_t = (const Tool<T>*)L.tools_t;
  const T* poses_t = (const T*)L.poses_t;
  if (phases & BWD_PREPARE) {
    // recompute the grids of this substep (substep_grad, mpm_simulator.py:327-333)
    // unless the grid store holds them (then p2g and grid_op return at once)
    const int64_t* saved = store ? store->slot_start + slot : nullptr;
    cudaError_t e = prepare_blocks<T>(L, c, st0, gin, gout, g_gout, store, slot, nullptr, -1, pose_f, pose_f1, false);
    if (e != cudaSuccess) return e;
    if (c.n_particles > 0) {
      // with a grid store the recompute usually exits at once: a grid of one
      // wave of CTAs that stride over the particles
      const unsigned cap = (unsigned)(L.sm_count * 6);
      MPM_LAUNCH_PDL(L, MPM_K_P2G_RECOMP, (k_p2g<T, S, true>), store && pb > cap ? cap : pb, 128, c, st0,
                     (T*)nullptr, L.pscene, gin, saved);
    }
    MPM_LAUNCH_PDL(L, MPM_K_GRID_OP, k_grid_op<T>, gb, 64, c, L.active, counter, gin, gout, tools_t, poses_t,
                   L.tool_off, MpmGridStore{}, -1, saved);
  }
  if ((phases & BWD_GRID) && c.n_particles > 0) {
    // FP32: the CTAs-per-SM variant the tuning selects.  BWD_G2P_PLAIN: the
    // kernel before it in the stream may be the previous substep's p2g.grad,
    // which writes the rows of g1 that g2p.grad reads before its wait
    const int v = sizeof(T) == 4 ? L.tune.g2p_adj_ctas : 0;
    const bool plain = (phases & BWD_G2P_PLAIN) != 0;
#define MPM_G2P_ADJ(K)                                                                                 \
  do {                                                                                                 \
    if (plain)                                                                                         \
      MPM_LAUNCH(L, MPM_K_G2P_ADJ, K, pb, 128, c, st0, st1, g1, g0, L.pscene, gout, g_gout);           \
    else                                                                                               \
      MPM_LAUNCH_PDL(L, MPM_K_G2P_ADJ, K, pb, 128, c, st0, st1, g1, g0, L.pscene, gout, g_gout);       \
  } while (0)
    if constexpr (sizeof(T) == 4) {
      if (v == 5)
        MPM_G2P_ADJ((k_g2p_adj<T, 5>));
      else if (v == 7)
        MPM_G2P_ADJ((k_g2p_adj<T, 7>));
      else if (v == 8)
        MPM_G2P_ADJ((k_g2p_adj<T, 8>));
      else
        MPM_G2P_ADJ(k_g2p_adj<T>);
    } else {
      (void)v;
      MPM_G2P_ADJ(k_g2p_adj<T>);
    }
#undef MPM_G2P_ADJ
  }
  if (phases & BWD_GRID) {
    // FP32: the CTAs-per-SM variant the tuning selects
    const int v = L.tune.grid_op_adj_ctas;
    if constexpr (sizeof(T) == 4) {
      if (v == 12)
        MPM_LAUNCH_PDL(L, MPM_K_GRID_OP_ADJ, (k_grid_op_adj<T, 12>), gb, 64, c, L.active, counter, gin, g_gout, g_gin,
                       tools_t, poses_t, L.tool_off, g_pose_f, g_pose_f1);
      else if (v == 16)
        MPM_LAUNCH_PDL(L, MPM_K_GRID_OP_ADJ, (k_grid_op_adj<T, 16>), gb, 64, c, L.active, counter, gin, g_gout, g_gin,
                       tools_t, poses_t, L.tool_off, g_pose_f, g_pose_f1);
      else
        MPM_LAUNCH_PDL(L, MPM_K_GRID_OP_ADJ, k_grid_op_adj<T>, gb, 64, c, L.active, counter, gin, g_gout, g_gin,
                       tools_t, poses_t, L.tool_off, g_pose_f, g_pose_f1);
    } else {
      (void)v;
      MPM_LAUNCH_PDL(L, MPM_K_GRID_OP_ADJ, k_grid_op_adj<T>, gb, 64, c, L.active, counter, gin, g_gout, g_gin, tools_t,
                     poses_t, L.tool_off, g_pose_f, g_pose_f1);
    }
  }
  if ((phases & BWD_PARTICLES) && c.n_particles > 0) {
    const int v = L.tune.p2g_adj_ctas;
    if constexpr (sizeof(T) == 4 && sizeof(S) == 4) {
      if (v == 4)
        MPM_LAUNCH_PDL(L, MPM_K_P2G_ADJ, (k_p2g_adj<T, S, 4>), pb, 128, c, st0, g1, g0, L.pscene, g_gin);
      else if (v == 6)
        MPM_LAUNCH_PDL(L, MPM_K_P2G_ADJ, (k_p2g_adj<T, S, 6>), pb, 128, c, st0, g1, g0, L.pscene, g_gin);
      else
        MPM_LAUNCH_PDL(L, MPM_K_P2G_ADJ, (k_p2g_adj<T, S>), pb, 128, c, st0, g1, g0, L.pscene, g_gin);
    } else {
      (void)v;
      MPM_LAUNCH_PDL(L, MPM_K_P2G_ADJ, (k_p2g_adj<T, S>), pb, 128, c, st0, g1, g0, L.pscene, g_gin);
    }
  }
  return cudaGetLastError();
}

// soft contact adjoint (loss.py:143-162 differentiated)
template <typename T>
__global__ void __launch_bounds__(128) k_contact_adj(Consts<T> c, const T* __restrict__ st,
                                                     const int* __restrict__ pscene,
                                                     const MpmToolDesc* __restrict__ tools,
                                                     const int* __restrict__ tool_off,
                                                     const double* __restrict__ pose,
                                                     const double* __restrict__ sums,
                                                     const double* __restrict__ g_min, T* __restrict__ gst,
                                                     double* __restrict__ g_pose) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= c.n_particles) return;
  int sc = pscene[p];
  T x[3];
  load_row(st, c.ld, p, 0, 3, x);
  T gx[3] = {T(0), T(0), T(0)};
  for (int t = tool_off[sc]; t < tool_off[sc + 1]; ++t) {
    if (tools[t].action_dim <= 0 || g_min[t] == 0.0) continue;
    Tool<T> tl;
    Pose<T> P;
    to_tool(tools[t], tl);
    to_pose(pose + 8 * t, P);
    T sd = tool_sdf(tl, P, x);
    if (!(T(0) < sd)) continue;
    double norm = sums[2 * t], md = sums[2 * t + 1] / norm;
    double d = double(sd), w = 1.0 / (1.0 + d * d * 10000.0);
    double g_norm = -g_min[t] * md / norm;
    double g_w = g_min[t] * d / norm + g_norm;
    double g_d = g_min[t] * w / norm + g_w * (-2e4 * d * w * w);
    PoseGrad<T> gP;
    gP.zero();
    tool_sdf_vjp(tl, P, x, T(g_d), gx, gP);
    const T* gv = &gP.pos[0];
    for (int k = 0; k < 3; ++k) atomicAdd(g_pose + 8 * t + k, double(gv[k]));
    for (int k = 0; k < 4; ++k) atomicAdd(g_pose + 8 * t + 3 + k, double(gP.rot[k]));
    atomicAdd(g_pose + 8 * t + 7, double(gP.gap));
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) gst[(int64_t)d * c.ld + p] += gx[d];
}

template <typename T>
cudaError_t launch_soft_contact_bwd(const LaunchCtx& L, int n_tools, const T* st, const double* pose,
                                    const double* sums, const double* g_min, T* gst, double* g_pose) {
  (void)n_tools;
  Consts<T> c = make_consts<T>(L);
  if (c.n_particles > 0)
    MPM_LAUNCH(L, MPM_K_OTHER, k_contact_adj<T>, blocks_for(c.n_particles, 128), 128, c, st, L.pscene, L.tools,
               L.tool_off, pose, sums, g_min, gst, g_pose);
  return cudaGetLastError();
}

// tool distance adjoint (compute_min_dist.grad, function.py:154-159)
template <typename T>
__global__ void __launch_bounds__(128) k_tool_distance_adj(Consts<T> c, const T* __restrict__ st,
                                                           const int* __restrict__ pscene,
                                                           const MpmToolDesc* __restrict__ tools,
                                                           const int* __restrict__ tool_off,
                                                           const int* __restrict__ col_off,
                                                           const double* __restrict__ pose,
                                                           const T* __restrict__ g_out, T* __restrict__ gst,
                                                           double* __restrict__ g_pose) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= c.n_particles) return;
  int sc = pscene[p];
  T x[3];
  load_row(st, c.ld, p, 0, 3, x);
  T gx[3] = {T(0), T(0), T(0)};
  for (int t = tool_off[sc]; t < tool_off[sc + 1]; ++t) {
    Tool<T> tl;
    Pose<T> P;
    to_tool(tools[t], tl);
    to_pose(pose + 8 * t, P);
    const int col = col_off[t];
    PoseGrad<T> gP;
    gP.zero();
    bool any = false;
    if (fingered(tl.type)) {
#pragma unroll
      for (int side = 0; side < 2; ++side) {
        T g = g_out[(int64_t)(col + side) * c.ld + p];
        if (g == T(0)) continue;
        any = true;
        T flag = side == 0 ? T(-1) : T(1);
        T fp[3], gf[3] = {T(0), T(0), T(0)};
        finger_pos(P, flag, fp);
        shape_sdf_vjp(tl, fp, P.rot, T(0), x, g, gx, gf, gP.rot, (T*)nullptr);
        finger_pos_vjp(P, flag, gf, gP);
      }
    } else {
      T g = g_out[(int64_t)col * c.ld + p];
      if (g != T(0)) {
        any = true;
        tool_sdf_vjp(tl, P, x, g, gx, gP);
      }
    }
    if (any) {
      for (int k = 0; k < 3; ++k) atomicAdd(g_pose + 8 * t + k, double(gP.pos[k]));
      for (int k = 0; k < 4; ++k) atomicAdd(g_pose + 8 * t + 3 + k, double(gP.rot[k]));
      atomicAdd(g_pose + 8 * t + 7, double(gP.gap));
    }
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) gst[(int64_t)d * c.ld + p] += gx[d];
}

template <typename T>
cudaError_t launch_tool_distance_bwd(const LaunchCtx& L, const int* col_off, const T* st, const double* pose,
                                     const T* g_out, T* gst, double* g_pose) {
  Consts<T> c = make_consts<T>(L);
  if (c.n_particles > 0)
    MPM_LAUNCH(L, MPM_K_OTHER, k_tool_distance_adj<T>, blocks_for(c.n_particles, 128), 128, c, st, L.pscene,
               L.tools, L.tool_off, col_off, pose, g_out, gst, g_pose);
  return cudaGetLastError();
}
template cudaError_t launch_tool_distance_bwd<float>(const LaunchCtx&, const int*, const float*, const double*,
                                                     const float*, float*, double*);
template cudaError_t launch_tool_distance_bwd<double>(const LaunchCtx&, const int*, const double*, const double*,
                                                      const double*, double*, double*);

#define MPM_INST_BWD(T, S)                                                                                  \
  template cudaError_t launch_substep_bwd<T, S>(const LaunchCtx&, const T*, const T*, const T*, T*, const double*, \
                                                const double*, double*, double*, const MpmGridStore*, int, unsigned);
MPM_INST_BWD(float, float)
MPM_INST_BWD(float, double)
MPM_INST_BWD(double, double)
template cudaError_t launch_soft_contact_bwd<float>(const LaunchCtx&, int, const float*, const double*, const double*,
                                                    const double*, float*, double*);
template cudaError_t launch_soft_contact_bwd<double>(const LaunchCtx&, int, const double*, const double*,
                                                     const double*, const double*, double*, double*);

}  // namespace mpm
