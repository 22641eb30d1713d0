// Forward launchers: substep (p2g -> grid_op -> g2p), density grid, density
// L1 loss and the soft tool-contact distance, for the three precision modes.
#include "mpm_kernels.cuh"
#include "mpm_launch.h"

namespace mpm {

template <typename T>
Consts<T> make_consts(const LaunchCtx& L) {
  const MpmParams& p = *L.p;
  Consts<T> c;
  c.n_grid = p.n_grid;
  c.n_scenes = p.n_scenes;
  c.n_particles = p.n_particles;
  c.ld = p.ld;
  c.G = L.G;
  c.nb = p.n_grid / 4;
  c.NB3 = (int64_t)c.nb * c.nb * c.nb;
  c.dx = T(p.dx);
  c.inv_dx = T(p.inv_dx);
  c.dt = T(p.dt);
  c.p_mass = T(p.p_mass);
  c.p_vol = T(p.p_vol);
  c.mu = T(p.mu);
  c.lam = T(p.lam);
  c.yield_stress = T(p.yield_stress);
  c.ks = T(-p.dt * p.p_vol * 4 * p.inv_dx * p.inv_dx);
  for (int k = 0; k < 3; ++k) c.gdt[k] = T(p.dt * p.gravity[k] * 30);
  c.ground_friction = T(p.ground_friction);
  c.x_lo = T(p.lower_bound * p.dx);
  c.x_hi = T(1.0 - 3 * p.dx);
  c.status = L.status;
  return c;
}
template Consts<float> make_consts<float>(const LaunchCtx&);
template Consts<double> make_consts<double>(const LaunchCtx&);

static inline unsigned blocks_for(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// Active blocks of frame st: mark, then compact the list and zero the listed
// blocks of grid a (and b if given).  Leaves the list in L.active and its
// length at L.blockbuf[0..3] (a ticket counter at [4..7]); the block flags at
// L.blockbuf + 16 are clean before and after (cleared by the compaction).
// ``restore`` (may be null): the adjoint's grid store; when its slot holds
// this substep the list, grid a and grid a_out (the grid_op output) are
// restored from it and b is zeroed.
// ``reserve`` (may be null): the forward's grid store; room for the list is
// reserved in slot ``reserve_slot`` by the compaction's last CTA.
// The compaction also fills L.poses_t for the poses pose_f, pose_f1.
// premarked (forward only): the flags and the header were set by the previous
// substep's g2p, so the marking launch is skipped.
template <typename T>
cudaError_t prepare_blocks(const LaunchCtx& L, const Consts<T>& c, const T* st, Node<T>* a, Node<T>* a_out,
                           Node<T>* b, const MpmGridStore* restore, int restore_slot, const MpmGridStore* reserve,
                           int reserve_slot, const double* pose_f, const double* pose_f1, bool premarked) {
  const int64_t total = (int64_t)c.n_scenes * c.NB3;
  int* counter = reinterpret_cast<int*>(L.blockbuf);
  unsigned* ticket = reinterpret_cast<unsigned*>(L.blockbuf + 4);
  unsigned char* flags = L.blockbuf + 16;
  const int64_t* saved = restore ? restore->slot_start + restore_slot : nullptr;
  // one thread per particle for the marking; the restore strides over the stored nodes
  unsigned mb = blocks_for(c.n_particles, 256);
  const unsigned floor_ctas = (unsigned)(L.sm_count * 8);
  if (restore && mb < floor_ctas) mb = floor_ctas;
  if (mb == 0) mb = 1;
  MpmGridStore rst{};
  if (restore) rst = *restore;
  if (!premarked || restore)
    MPM_LAUNCH_PDL(L, MPM_K_CLEAR, k_mark_or_restore<T>, mb, 256, c, st, L.pscene, flags, counter, rst,
               restore ? restore_slot : -1, L.active, a, a_out, b);
  MpmGridStore rs{};
  if (reserve) rs = *reserve;
  const PoseTableArgs tt{L.n_tools, pose_f, pose_f1, L.poses_t};
  MPM_LAUNCH_PDL(L, MPM_K_CLEAR, k_compact_clear<T>, blocks_for(total, 256), 256, flags, total, L.active, counter, ticket,
             a, b, saved, rs, reserve ? reserve_slot : -1, tt);
  return cudaGetLastError();
}
template cudaError_t prepare_blocks<float>(const LaunchCtx&, const Consts<float>&, const float*, Node<float>*,
                                           Node<float>*, Node<float>*, const MpmGridStore*, int,
                                           const MpmGridStore*, int, const double*, const double*, bool);
template cudaError_t prepare_blocks<double>(const LaunchCtx&, const Consts<double>&, const double*, Node<double>*,
                                            Node<double>*, Node<double>*, const MpmGridStore*, int,
                                            const MpmGridStore*, int, const double*, const double*, bool);

size_t tools_t_bytes(int64_t n_tools) { return (size_t)(n_tools > 0 ? n_tools : 1) * sizeof(Tool<double>); }
size_t poses_t_bytes(int64_t n_tools) { return (size_t)(n_tools > 0 ? n_tools : 1) * 16 * sizeof(double); }
cudaError_t convert_tools(int precision, int n, const MpmToolDesc* tools, void* tools_t, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const unsigned g = blocks_for(n, 128);
  if (precision == MPM_PREC_FP64)
    k_tools_convert<double><<<g, 128, 0, s>>>(n, tools, (Tool<double>*)tools_t);
  else
    k_tools_convert<float><<<g, 128, 0, s>>>(n, tools, (Tool<float>*)tools_t);
  return cudaGetLastError();
}

unsigned grid_blocks_launch(const LaunchCtx& L, int64_t total_blocks) {
  const int per_sm = L.tune.grid_ctas_per_sm > 0 ? L.tune.grid_ctas_per_sm : 16;
  int64_t g = (int64_t)L.sm_count * per_sm;
  return (unsigned)(g < total_blocks ? g : (total_blocks > 0 ? total_blocks : 1));
}

template <typename T, typename S>
cudaError_t launch_substep_fwd(const LaunchCtx& L, const T* st0, T* st1, const double* pose_f,
                               const double* pose_f1, const MpmGridStore* store, int slot, bool premarked,
                               bool mark_next) {
  Consts<T> c = make_consts<T>(L);
  Node<T>* gin = (Node<T>*)L.grid_a;
  Node<T>* gout = (Node<T>*)L.grid_b;
  const int* counter = reinterpret_cast<const int*>(L.blockbuf);
  cudaError_t e = prepare_blocks<T>(L, c, st0, gin, (Node<T>*)nullptr, (Node<T>*)nullptr, nullptr, -1, store, slot,
                                    pose_f, pose_f1, premarked);
  if (e != cudaSuccess) return e;
  if (c.n_particles > 0) {
    const unsigned pb = blocks_for(c.n_particles, 128);
    const int64_t* none = nullptr;
    // FP32: the CTAs-per-SM variant the tuning selects
    const int v = L.tune.p2g_ctas;
    if constexpr (sizeof(T) == 4 && sizeof(S) == 4) {
      if (v == 6)
        MPM_LAUNCH_PDL(L, MPM_K_P2G, (k_p2g<T, S, false, 6>), pb, 128, c, st0, st1, L.pscene, gin, none);
      else if (v == 8)
        MPM_LAUNCH_PDL(L, MPM_K_P2G, (k_p2g<T, S, false, 8>), pb, 128, c, st0, st1, L.pscene, gin, none);
      else
        MPM_LAUNCH_PDL(L, MPM_K_P2G, (k_p2g<T, S>), pb, 128, c, st0, st1, L.pscene, gin, none);
    } else {
      (void)v;
      MPM_LAUNCH_PDL(L, MPM_K_P2G, (k_p2g<T, S>), pb, 128, c, st0, st1, L.pscene, gin, none);
    }
  }
  MPM_LAUNCH_PDL(L, MPM_K_GRID_OP, k_grid_op<T>, grid_blocks_launch(L, (int64_t)c.n_scenes * c.NB3), 64, c, L.active,
             counter, gin, gout, (const Tool<T>*)L.tools_t, (const T*)L.poses_t, L.tool_off,
             store ? *store : MpmGridStore{}, store ? slot : -1, (const int64_t*)nullptr);
  if (c.n_particles > 0) {
    const unsigned pb = blocks_for(c.n_particles, 128);
    unsigned char* mark = mark_next ? L.blockbuf + 16 : (unsigned char*)nullptr;
    int* header = reinterpret_cast<int*>(L.blockbuf);
    const int v = L.tune.g2p_ctas;
    if constexpr (sizeof(T) == 4) {
      if (v == 10)
        MPM_LAUNCH_PDL(L, MPM_K_G2P, (k_g2p<T, 10>), pb, 128, c, st0, st1, L.pscene, gout, mark, header);
      else if (v == 12)
        MPM_LAUNCH_PDL(L, MPM_K_G2P, (k_g2p<T, 12>), pb, 128, c, st0, st1, L.pscene, gout, mark, header);
      else
        MPM_LAUNCH_PDL(L, MPM_K_G2P, k_g2p<T>, pb, 128, c, st0, st1, L.pscene, gout, mark, header);
    } else {
      (void)v;
      MPM_LAUNCH_PDL(L, MPM_K_G2P, k_g2p<T>, pb, 128, c, st0, st1, L.pscene, gout, mark, header);
    }
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_grid_mass(const LaunchCtx& L, const T* st, T* gm) {
  Consts<T> c = make_consts<T>(L);
  MPM_MEMSET(L, gm, (int64_t)c.n_scenes * c.G * sizeof(T));
  if (c.n_particles > 0)
    MPM_LAUNCH(L, MPM_K_OTHER, k_grid_mass<T>, blocks_for(c.n_particles, 128), 128, c, st, L.pscene, gm);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_grid_mass_bwd(const LaunchCtx& L, const T* st, const T* ggm, T* gst) {
  Consts<T> c = make_consts<T>(L);
  if (c.n_particles > 0)
    MPM_LAUNCH(L, MPM_K_OTHER, k_grid_mass_adj<T>, blocks_for(c.n_particles, 128), 128, c, st, L.pscene, ggm, gst);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_density_l1(const LaunchCtx& L, const T* gm, const T* tgt, double weight, double* loss, T* ggm) {
  const int S = L.p->n_scenes;
  MPM_MEMSET(L, loss, S * sizeof(double));
  int bps = (int)((L.G + 256 * 8 - 1) / (256 * 8));
  if (bps < 1) bps = 1;
  MPM_LAUNCH(L, MPM_K_OTHER, k_density_l1<T>, (unsigned)(S * bps), 256, L.G, gm, tgt, weight, loss, ggm, bps);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// soft contact distance (loss.py:143-162)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(128) k_contact_sums(Consts<T> c, const T* __restrict__ st,
                                                      const int* __restrict__ pscene,
                                                      const MpmToolDesc* __restrict__ tools,
                                                      const int* __restrict__ tool_off,
                                                      const double* __restrict__ pose, double* __restrict__ sums) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= c.n_particles) return;
  int sc = pscene[p];
  T x[3];
  load_row(st, c.ld, p, 0, 3, x);
  for (int t = tool_off[sc]; t < tool_off[sc + 1]; ++t) {
    if (tools[t].action_dim <= 0) continue;
    Tool<T> tl;
    Pose<T> P;
    to_tool(tools[t], tl);
    to_pose(pose + 8 * t, P);
    T sd = tool_sdf(tl, P, x);
    double d = (T(0) < sd) ? double(sd) : 0.0;
    double w = 1.0 / (1.0 + d * d * 10000.0);
    atomicAdd(sums + 2 * t, w);
    atomicAdd(sums + 2 * t + 1, d * w);
  }
}
__global__ void k_contact_finish(int n_tools, const double* __restrict__ sums, double* __restrict__ min_dist) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n_tools) min_dist[t] = sums[2 * t] > 0 ? sums[2 * t + 1] / sums[2 * t] : 0.0;
}

template <typename T>
cudaError_t launch_soft_contact(const LaunchCtx& L, int n_tools, const T* st, const double* pose, double* sums,
                                double* min_dist) {
  Consts<T> c = make_consts<T>(L);
  MPM_MEMSET(L, sums, 2 * n_tools * sizeof(double));
  if (c.n_particles > 0)
    MPM_LAUNCH(L, MPM_K_OTHER, k_contact_sums<T>, blocks_for(c.n_particles, 128), 128, c, st, L.pscene, L.tools,
               L.tool_off, pose, sums);
  MPM_LAUNCH(L, MPM_K_OTHER, k_contact_finish, blocks_for(n_tools, 64), 64, n_tools, sums, min_dist);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// per-particle tool distances (function.py:79-89)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(128) k_tool_distance(Consts<T> c, const T* __restrict__ st,
                                                       const int* __restrict__ pscene,
                                                       const MpmToolDesc* __restrict__ tools,
                                                       const int* __restrict__ tool_off,
                                                       const int* __restrict__ col_off,
                                                       const double* __restrict__ pose, T* __restrict__ out) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= c.n_particles) return;
  int sc = pscene[p];
  T x[3];
  load_row(st, c.ld, p, 0, 3, x);
  for (int t = tool_off[sc]; t < tool_off[sc + 1]; ++t) {
    Tool<T> tl;
    Pose<T> P;
    to_tool(tools[t], tl);
    to_pose(pose + 8 * t, P);
    const int col = col_off[t];
    if (fingered(tl.type)) {
      T fa[3], fb[3];
      finger_pos(P, T(-1), fa);
      finger_pos(P, T(1), fb);
      out[(int64_t)col * c.ld + p] = shape_sdf(tl, fa, P.rot, T(0), x);
      out[(int64_t)(col + 1) * c.ld + p] = shape_sdf(tl, fb, P.rot, T(0), x);
    } else {
      out[(int64_t)col * c.ld + p] = tool_sdf(tl, P, x);
    }
  }
}

template <typename T>
cudaError_t launch_tool_distance(const LaunchCtx& L, const int* col_off, int n_cols, const T* st, const double* pose,
                                 T* out) {
  Consts<T> c = make_consts<T>(L);
  MPM_MEMSET(L, out, (int64_t)n_cols * c.ld * sizeof(T));
  if (c.n_particles > 0)
    MPM_LAUNCH(L, MPM_K_OTHER, k_tool_distance<T>, blocks_for(c.n_particles, 128), 128, c, st, L.pscene, L.tools,
               L.tool_off, col_off, pose, out);
  return cudaGetLastError();
}
template cudaError_t launch_tool_distance<float>(const LaunchCtx&, const int*, int, const float*, const double*,
                                                 float*);
template cudaError_t launch_tool_distance<double>(const LaunchCtx&, const int*, int, const double*, const double*,
                                                  double*);

#define MPM_INST_FWD(T, S)                                                                             \
  template cudaError_t launch_substep_fwd<T, S>(const LaunchCtx&, const T*, T*, const double*, const double*, \
                                                const MpmGridStore*, int, bool, bool);
MPM_INST_FWD(float, float)
MPM_INST_FWD(float, double)
MPM_INST_FWD(double, double)
#define MPM_INST_T(T)                                                                                  \
  template cudaError_t launch_grid_mass<T>(const LaunchCtx&, const T*, T*);                            \
  template cudaError_t launch_grid_mass_bwd<T>(const LaunchCtx&, const T*, const T*, T*);              \
  template cudaError_t launch_density_l1<T>(const LaunchCtx&, const T*, const T*, double, double*, T*); \
  template cudaError_t launch_soft_contact<T>(const LaunchCtx&, int, const T*, const double*, double*, double*);
MPM_INST_T(float)
MPM_INST_T(double)

}  // namespace mpm
