// mpm_substep_fwd_static: one forward substep of a single scene with no
// device allocation at all.
//
// Who needs it: callers that cannot call cudaMalloc.  A simulator stepped
// from inside another framework's GPU memory pool (PyTorch's caching
// allocator, an FFI custom-call hook) must not allocate behind that pool's
// back -- the pool may already hold nearly all of HBM, and a foreign
// cudaMalloc can fail or break its accounting.  A latency-bound control loop
// that steps the scene every tick cannot afford cudaMalloc / cudaFree either:
// both synchronise the whole device.  mpm_create allocates its grid scratch,
// so those callers use this entry point instead; they still pass the state,
// tool poses and output buffers, which they own.
//
// The scratch is the file-scope array g_static_scratch below (20 MiB + 64 KiB).  Every GPU that
// loads this library holds it until the process exits.  All calls share it
// and it keeps the last call's contents: the tool table, the scratch status
// word, the active-block flags and the grid blocks the scatter accumulates
// into are rewritten or cleared on every call; the scene-index region is
// zeroed once per device and never written afterwards.  Calls whose
// kernels overlap on the GPU (different streams, or different host threads,
// on the same device) race on the array; serialise them.
//
// Per call the host issues kernel launches only: the scene's tool table
// travels by value as a kernel parameter (k_static_setup), so no pageable
// host-to-device copy orders the call against the host.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "mpm_launch.h"
#include "mpm_tools.cuh"

namespace {

// Layout of the scratch array:
//   [0, 4)                      status word (when the caller passes none)
//   [16, 24)                    tool offsets {0, n_tools} of the one scene
//   [256, 256 + 8*tool size)    tool table
//   [4096, 4096 + 16 + 8000)    active-block counter and flags (<= 20^3 blocks)
//   [16384, 16384 + 32000)      active-block list
//   [49152, +8 Tool<double>)    the tools in the compute precision
//   [kPosesT, +8*16 doubles)     their poses at frames f, f+1 in the compute precision
//   [kHeader, +kScene)          zero scene index of every particle
//   [kHeader+kScene, +kGrids)   forward grid (mv, m) then velocity grid
constexpr size_t kBlockBuf = 4096;
constexpr size_t kActive = 16384;
constexpr size_t kToolsT = 49152;
constexpr size_t kPosesT = kToolsT + 8 * sizeof(mpm::Tool<double>);
constexpr int64_t kMaxBlocks = 8000;  // (80/4)^3
constexpr size_t kHeader = 65536;
constexpr int64_t kMaxParticles = int64_t(1) << 20;             // 1,048,576 particles
constexpr size_t kScene = size_t(kMaxParticles) * sizeof(int);  // 4 MiB
constexpr size_t kGrids = size_t(16) << 20;                     // 16 MiB for the two grids
constexpr size_t kScratchBytes = kHeader + kScene + kGrids;     // 20 MiB + 64 KiB
static_assert(kBlockBuf + 16 + kMaxBlocks <= kActive, "block flags overlap the list");
static_assert(kActive + kMaxBlocks * sizeof(int) <= kToolsT, "block list overlaps the tool table");
static_assert(kPosesT + 8 * 16 * sizeof(double) <= kHeader, "pose table overlaps the scene index");

static __device__ __align__(256) unsigned char g_static_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_base[kMaxDevices] = {nullptr};

// failures are reported through mpm_last_error(NULL, ...), like mpm_create's
int set_err(int code, const std::string& msg) {
  mpm::record_global_error(msg);
  return code;
}

// Once per device, with that device current: resolve the device address of
// the array (the host-side name is only a stand-in) and zero the scene-index
// region.
int scratch_base(int dev, unsigned char** out) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (dev < 0 || dev >= kMaxDevices) return set_err(MPM_E_INVALID, "mpm_substep_fwd_static: device index out of range");
  if (!g_base[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess)
      return set_err(MPM_E_CUDA, std::string("mpm_substep_fwd_static: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    unsigned char* base = static_cast<unsigned char*>(p);
    e = cudaMemset(base + kHeader, 0, kScene);
    // block flags start clean; every compaction clears the flags it reads
    if (e == cudaSuccess) e = cudaMemset(base + kBlockBuf, 0, 16 + kMaxBlocks);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess)
      return set_err(MPM_E_CUDA, std::string("mpm_substep_fwd_static: clearing the scene index and block flags: ") +
                                     cudaGetErrorString(e));
    g_base[dev] = base;
  }
  *out = g_base[dev];
  return MPM_OK;
}

bool aligned16(const void* p) { return p && (reinterpret_cast<uintptr_t>(p) % 16 == 0); }

// The per-call set-up, passed by value (about 2.1 KB of kernel parameters).
struct StaticSetup {
  int32_t n_tools;
  int32_t clear_status;  // zero the scratch status word (the caller gave none)
  MpmToolDesc tools[mpm::MAX_TOOLS_PER_SCENE];
};

// One warp: the tool offsets {0, n_tools}, the descriptor table, the tools in
// the compute precision T, and the scratch status word.
template <typename T>
__global__ void __launch_bounds__(32) k_static_setup(StaticSetup a) {
  unsigned char* base = g_static_scratch;
  const int i = threadIdx.x;
  if (i == 0) {
    int* toff = reinterpret_cast<int*>(base + 16);
    toff[0] = 0;
    toff[1] = a.n_tools;
    if (a.clear_status) *reinterpret_cast<unsigned int*>(base) = 0u;
  }
  if (i < a.n_tools) {
    reinterpret_cast<MpmToolDesc*>(base + 256)[i] = a.tools[i];
    mpm::to_tool(a.tools[i], reinterpret_cast<mpm::Tool<T>*>(base + kToolsT)[i]);
  }
}

}  // namespace

extern "C" {

// No counterpart in the reference.  See include/mpm_gb300.h.
int mpm_substep_fwd_static(const MpmParams* params, const MpmToolDesc* tools, int32_t n_tools, const void* state_f,
                           void* state_f1, const double* pose_f, const double* pose_f1, uint32_t* status,
                           void* stream) {
  if (!params) return set_err(MPM_E_INVALID, "mpm_substep_fwd_static: params is NULL");
  const MpmParams& p = *params;
  if (p.abi_version != MPM_ABI_VERSION) return set_err(MPM_E_INVALID, "mpm_substep_fwd_static: ABI version mismatch");
  if (p.precision < MPM_PREC_FP32 || p.precision > MPM_PREC_FP64)
    return set_err(MPM_E_INVALID, "mpm_substep_fwd_static: unknown precision");
  if (p.n_scenes != 1) return set_err(MPM_E_INVALID, "mpm_substep_fwd_static: exactly one scene is supported");
  if (p.n_grid < 8 || p.n_grid % 8 != 0)
    return set_err(MPM_E_INVALID, "mpm_substep_fwd_static: n_grid must be a positive multiple of 8");
  const int64_t G = int64_t(p.n_grid) * p.n_grid * p.n_grid;
  const size_t real = p.precision == MPM_PREC_FP64 ? sizeof(double) : sizeof(float);
  const size_t grid_bytes = size_t(G) * 4 * real;
  if (2 * grid_bytes > kGrids)
    return set_err(MPM_E_INVALID, "mpm_substep_fwd_static: two grids of n_grid^3 nodes need " +
                                      std::to_string(2 * grid_bytes) + " bytes, above the static limit of " +
                                      std::to_string(kGrids) + " (n_grid <= 80 in FP32, <= 64 in FP64)");
  if ((int64_t)(p.n_grid / 4) * (p.n_grid / 4) * (p.n_grid / 4) > kMaxBlocks)
    return set_err(MPM_E_INVALID, "mpm_substep_fwd_static: n_grid above the static limit of 80");
  if (p.n_particles < 0 || p.n_particles > kMaxParticles)
    return set_err(MPM_E_INVALID, "mpm_substep_fwd_static: n_particles must be in [0, " +
                                      std::to_string(kMaxParticles) + "]");
  if (p.ld < p.n_particles) return set_err(MPM_E_INVALID, "mpm_substep_fwd_static: ld < n_particles");
  if (n_tools < 0 || n_tools > mpm::MAX_TOOLS_PER_SCENE || (n_tools > 0 && !tools))
    return set_err(MPM_E_INVALID, "mpm_substep_fwd_static: n_tools must be in [0, " +
                                      std::to_string(mpm::MAX_TOOLS_PER_SCENE) + "] with a tool array");
  for (int i = 0; i < n_tools; ++i)
    if (tools[i].type < MPM_TOOL_SPHERE || tools[i].type > MPM_TOOL_GRIPPER || tools[i].scene != 0)
      return set_err(MPM_E_INVALID, "mpm_substep_fwd_static: tool " + std::to_string(i) +
                                        " has an unknown type or a scene other than 0");
  if (!aligned16(state_f) || !aligned16(state_f1) || state_f == state_f1)
    return set_err(MPM_E_INVALID, "mpm_substep_fwd_static: state_f and state_f1 must be distinct 16-byte aligned "
                                  "device pointers");
  if (n_tools > 0 && (!aligned16(pose_f) || !aligned16(pose_f1)))
    return set_err(MPM_E_INVALID, "mpm_substep_fwd_static: pose_f and pose_f1 must be 16-byte aligned");
  if (status && reinterpret_cast<uintptr_t>(status) % 4 != 0)
    return set_err(MPM_E_INVALID, "mpm_substep_fwd_static: status must be a 4-byte aligned device pointer");

  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_err(MPM_E_CUDA, std::string("mpm_substep_fwd_static: ") + cudaGetErrorString(e));
  unsigned char* base = nullptr;
  int rc = scratch_base(dev, &base);
  if (rc != MPM_OK) return rc;

  cudaStream_t s = static_cast<cudaStream_t>(stream);
  StaticSetup su;
  std::memset(&su, 0, sizeof(su));
  su.n_tools = n_tools;
  su.clear_status = status ? 0 : 1;
  for (int i = 0; i < n_tools; ++i) su.tools[i] = tools[i];
  if (p.precision == MPM_PREC_FP64)
    k_static_setup<double><<<1, 32, 0, s>>>(su);
  else
    k_static_setup<float><<<1, 32, 0, s>>>(su);
  e = cudaGetLastError();
  if (e != cudaSuccess) return set_err(MPM_E_CUDA, std::string("mpm_substep_fwd_static: ") + cudaGetErrorString(e));

  int64_t launches = 0;
  mpm::LaunchCtx L;
  L.p = params;
  L.G = G;
  L.pscene = reinterpret_cast<const int*>(base + kHeader);
  L.tools = reinterpret_cast<const MpmToolDesc*>(base + 256);
  L.tool_off = reinterpret_cast<const int*>(base + 16);
  L.n_tools = n_tools;
  // the caller's status word when given (sticky: the caller clears it), else
  // the scratch word, which is cleared per call and not reported
  L.status = status ? reinterpret_cast<unsigned int*>(status) : reinterpret_cast<unsigned int*>(base);
  L.grid_a = base + kHeader + kScene;              // active blocks cleared by the launcher before the scatter
  L.grid_b = base + kHeader + kScene + grid_bytes;  // fully written by grid_op
  L.grid_c = nullptr;
  L.grid_d = nullptr;
  L.blockbuf = base + kBlockBuf;  // flags cleared once above, then by every compaction
  L.active = reinterpret_cast<int*>(base + kActive);
  L.tools_t = base + kToolsT;
  L.poses_t = base + kPosesT;
  int sm = 1;
  if (cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sm < 1) sm = 1;
  L.sm_count = sm;
  L.stream = s;
  L.launches = &launches;
  L.prof = nullptr;
  switch (p.precision) {
    case MPM_PREC_FP32:
      e = mpm::launch_substep_fwd<float, float>(L, (const float*)state_f, (float*)state_f1, pose_f, pose_f1);
      break;
    case MPM_PREC_FP32_SVD64:
      e = mpm::launch_substep_fwd<float, double>(L, (const float*)state_f, (float*)state_f1, pose_f, pose_f1);
      break;
    default:
      e = mpm::launch_substep_fwd<double, double>(L, (const double*)state_f, (double*)state_f1, pose_f, pose_f1);
  }
  if (e != cudaSuccess) return set_err(MPM_E_CUDA, std::string("mpm_substep_fwd_static: ") + cudaGetErrorString(e));
  return MPM_OK;
}

}  // extern "C"
