// Internal launch interface between the C ABI (mpm_capi.cu) and the kernel
// translation units (mpm_fwd.cu, mpm_bwd.cu, mpm_loss.cu, mpm_kinematics.cu, mpm_render.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/mpm_gb300.h"

namespace mpm {

// Stores the message returned by mpm_last_error(NULL, ...) (mpm_capi.cu).
void record_global_error(const std::string& msg);

// Optional per-kernel CUDA-event timing (mpm_profile_enable).
struct Profiler {
  struct Rec {
    int kind;
    cudaEvent_t a, b;
  };
  bool on = false;
  Rec* recs = nullptr;
  int n = 0, cap = 0;
  cudaEvent_t* pool = nullptr;
  int pool_n = 0, pool_cap = 0;
};
// bracket a launch: begin() before, end() after (no-ops when profiling is off)
int prof_begin(Profiler* P, cudaStream_t s);
void prof_end(Profiler* P, int slot, int kind, cudaStream_t s);

struct LaunchCtx {
  const MpmParams* p;
  int64_t G;                   // n_grid^3
  const int* pscene;           // [n_particles] scene of each particle
  const MpmToolDesc* tools;    // [n_tools] device
  const int* tool_off;         // [n_scenes + 1] device
  int n_tools;
  unsigned int* status;        // sticky status word
  void* grid_a;                // scratch grids, n_scenes*G nodes of 4 reals
  void* grid_b;                //   (block-contiguous layout, see mpm_kernels.cuh)
  void* grid_c;
  void* grid_d;
  unsigned char* blockbuf;     // [16-byte counter header][n_scenes * NB3 block flags]
  int* active;                 // [n_scenes * NB3] list of active blocks
  const void* tools_t;         // [n_tools] Tool<T>, converted when the tools are set (convert_tools)
  void* poses_t;               // [n_tools * 16] T: poses of frames f, f+1, converted every substep
  int sm_count;                // multiprocessors of the device (grid-stride launch sizes)
  cudaStream_t stream;
  int64_t* launches;           // launch counter
  Profiler* prof;              // may be null
  MpmTuning tune = {0, 0, 0, 0, 0, 0};  // launch shapes (mpm_set_tuning); 0 = default
};

// launch helper: counts and (optionally) times one kernel launch
#define MPM_LAUNCH(L, KIND, KERNEL, GRID, BLOCK, ...)                 \
  do {                                                                 \
    int _slot = prof_begin((L).prof, (L).stream);                      \
    KERNEL<<<(GRID), (BLOCK), 0, (L).stream>>>(__VA_ARGS__);           \
    prof_end((L).prof, _slot, (KIND), (L).stream);                     \
    ++*(L).launches;                                                   \
  } while (0)
// Launch with programmatic stream serialization: the kernel may start while
// the previous kernel in the stream runs, and calls pdl_wait() before it
// touches that kernel's data (mpm_kernels.cuh).  A plain launch while the
// profiler times kernels one by one.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(cudaStream_t s, void (*kernel)(KArgs...), unsigned grid, unsigned block,
                              Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}
#define MPM_LAUNCH_PDL(L, KIND, KERNEL, GRID, BLOCK, ...)                         \
  do {                                                                            \
    if ((L).prof && (L).prof->on) {                                               \
      MPM_LAUNCH(L, KIND, KERNEL, GRID, BLOCK, __VA_ARGS__);                      \
    } else {                                                                      \
      cudaError_t _e = launch_pdl((L).stream, KERNEL, (GRID), (BLOCK), __VA_ARGS__); \
      ++*(L).launches;                                                            \
      if (_e != cudaSuccess) return _e;                                           \
    }                                                                             \
  } while (0)
#define MPM_MEMSET(L, PTR, BYTES)                                      \
  do {                                                                 \
    int _slot = prof_begin((L).prof, (L).stream);                      \
    cudaError_t _e = cudaMemsetAsync((PTR), 0, (BYTES), (L).stream);   \
    prof_end((L).prof, _slot, MPM_K_CLEAR, (L).stream);                \
    if (_e != cudaSuccess) return _e;                                  \
  } while (0)

// Scratch of the particle re-sort (mpm_sort.cu), owned by the handle: two
// key buffers and one index buffer of n_particles words, and the digit
// table of sort_hist_words(n_particles) words.
struct SortScratch {
  uint32_t* keys_a = nullptr;
  uint32_t* keys_b = nullptr;
  int32_t* vals_b = nullptr;
  uint32_t* hist = nullptr;
};
size_t sort_hist_words(int64_t n_particles);
// bits of the largest sort key ((scene * blocks + block) * 64 + cell)
int sort_key_bits(int n_scenes, int n_grid);
template <typename T>
cudaError_t launch_sort_frame(const LaunchCtx& L, const T* src, T* dst, int32_t* perm, const SortScratch& s);
template <typename T>
cudaError_t launch_unsort_frame(const LaunchCtx& L, const T* src, T* dst, const int32_t* perm);

// bytes of the converted tools and of the per-substep pose table (the
// double-precision sizes cover both precisions)
size_t tools_t_bytes(int64_t n_tools);
size_t poses_t_bytes(int64_t n_tools);
// converts n tool descriptors into Tool<T> of the handle's precision
cudaError_t convert_tools(int precision, int n, const MpmToolDesc* tools, void* tools_t, cudaStream_t s);

// bytes of the block-flag buffer (counter header + one flag per block)
inline size_t blockbuf_bytes(int64_t n_scenes, int n_grid) {
  const int64_t nb = n_grid / 4;
  return 16 + (size_t)(n_scenes * nb * nb * nb);
}

// premarked: the block flags of st0 were set by the previous substep's g2p
// (chained substeps), so the marking pass is skipped; mark_next: this
// substep's g2p flags the blocks of st1 for the next substep
template <typename T, typename S>
cudaError_t launch_substep_fwd(const LaunchCtx& L, const T* st0, T* st1, const double* pose_f,
                               const double* pose_f1, const MpmGridStore* store = nullptr, int slot = -1,
                               bool premarked = false, bool mark_next = false);
// The adjoint substep in three phases, which a caller may issue on two
// streams: BWD_PREPARE (active blocks, pose table, the grids restored from the
// store or recomputed), BWD_GRID (g2p.grad, grid_op.grad) and BWD_PARTICLES
// (p2g.grad).  BWD_G2P_PLAIN launches g2p.grad without the programmatic
// dependency on the kernel before it.
constexpr unsigned BWD_PREPARE = 1u, BWD_GRID = 2u, BWD_PARTICLES = 4u, BWD_G2P_PLAIN = 8u;
constexpr unsigned BWD_ALL = BWD_PREPARE | BWD_GRID | BWD_PARTICLES;
template <typename T, typename S>
cudaError_t launch_substep_bwd(const LaunchCtx& L, const T* st0, const T* st1, const T* g1, T* g0, const double* pose_f,
                               const double* pose_f1, double* g_pose_f, double* g_pose_f1,
                               const MpmGridStore* store = nullptr, int slot = -1, unsigned phases = BWD_ALL);
template <typename T>
cudaError_t launch_grid_mass(const LaunchCtx& L, const T* st, T* gm);
template <typename T>
cudaError_t launch_grid_mass_bwd(const LaunchCtx& L, const T* st, const T* ggm, T* gst);
template <typename T>
cudaError_t launch_density_l1(const LaunchCtx& L, const T* gm, const T* tgt, double weight, double* loss, T* ggm);
template <typename T>
cudaError_t launch_soft_contact(const LaunchCtx& L, int n_tools, const T* st, const double* pose, double* sums,
                                double* min_dist);
template <typename T>
cudaError_t launch_tool_distance(const LaunchCtx& L, const int* col_off, int n_cols, const T* st, const double* pose,
                                 T* out);
template <typename T>
cudaError_t launch_tool_distance_bwd(const LaunchCtx& L, const int* col_off, const T* st, const double* pose,
                                     const T* g_out, T* gst, double* g_pose);
// particle-SDF renderer (mpm_render.cu)
template <typename T>
cudaError_t launch_render_bake(const LaunchCtx& L, const T* st, int64_t p0, int64_t n, const unsigned int* colors,
                               const MpmRenderVolume& v);
template <typename T>
cudaError_t launch_render_trace(const LaunchCtx& L, const MpmRenderVolume& v, const MpmRenderView& view, int t0,
                                int nt, const double* pose, const float* tool_color, float* depth, float* normal,
                                float* color, float* image);
// tool kinematics of one action with collision projection (mpm_kinematics.cu)
cudaError_t launch_tools_action(const LaunchCtx& L, int n_tools, const int* pair_off, int n_pairs,
                                const double* coll_pts, const double* action, double* vel, double* pose, double* coll,
                                int n_sub);
cudaError_t launch_tools_action_bwd(const LaunchCtx& L, int n_tools, const int* pair_off, int n_pairs,
                                    const double* coll_pts, const double* vel, const double* pose, const double* coll,
                                    double* g_pose, double* g_action, int n_sub);
template <typename T>
cudaError_t launch_target_sdf(const LaunchCtx& L, int* flags, const T* dens, T* sdf, T* near, T* work, int n_iters);
template <typename T>
cudaError_t launch_sdf_loss(const LaunchCtx& L, const T* gm, const T* sdf, double weight, double* loss, T* ggm);
template <typename T>
cudaError_t launch_iou(const LaunchCtx& L, const T* gm, const T* tgt, double* iou);
template <typename T>
cudaError_t launch_contact_min(const LaunchCtx& L, int n_tools, const T* st, const double* pose, double* min_dist,
                               int64_t* argmin);
template <typename T>
cudaError_t launch_contact_min_bwd(const LaunchCtx& L, int n_tools, const T* st, const double* pose,
                                   const int64_t* argmin, const double* g_min, T* gst, double* g_pose);
template <typename T>
cudaError_t launch_soft_contact_bwd(const LaunchCtx& L, int n_tools, const T* st, const double* pose,
                                    const double* sums, const double* g_min, T* gst, double* g_pose);

}  // namespace mpm
