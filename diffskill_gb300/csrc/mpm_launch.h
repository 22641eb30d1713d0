// Internal launch interface between the C ABI (mpm_capi.cu) and the kernel
// translation units (mpm_fwd.cu, mpm_bwd.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/mpm_gb300.h"

namespace mpm {

struct LaunchCtx {
  const MpmParams* p;
  int64_t G;                   // n_grid^3
  const int* pscene;           // [n_particles] scene of each particle
  const MpmToolDesc* tools;    // [n_tools] device
  const int* tool_off;         // [n_scenes + 1] device
  unsigned int* status;        // sticky status word
  void* grid_a;                // scratch grids, n_scenes*G nodes of 4 reals
  void* grid_b;
  void* grid_c;
  void* grid_d;
  cudaStream_t stream;
  int64_t* launches;           // launch counter
};

template <typename T, typename S>
cudaError_t launch_substep_fwd(const LaunchCtx& L, const T* st0, T* st1, const double* pose_f,
                               const double* pose_f1);
template <typename T, typename S>
cudaError_t launch_substep_bwd(const LaunchCtx& L, const T* st0, const T* g1, T* g0, const double* pose_f,
                               const double* pose_f1, double* g_pose_f, double* g_pose_f1);
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
cudaError_t launch_soft_contact_bwd(const LaunchCtx& L, int n_tools, const T* st, const double* pose,
                                    const double* sums, const double* g_min, T* gst, double* g_pose);

}  // namespace mpm
