// C ABI of the GB300 MPM substep (include/mpm_gb300.h): handle lifetime,
// argument checks and precision dispatch.
#include <cuda_runtime.h>

#include <cstdio>
#include <initializer_list>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "mpm_launch.h"
#include "mpm_math.cuh"
#include "mpm_tools.cuh"

struct MpmHandle {
  MpmParams p;
  int device = -1;
  int64_t G = 0;
  std::vector<int64_t> offsets;
  int* d_pscene = nullptr;
  int* d_tool_off = nullptr;
  int* d_col_off = nullptr;  // first tool-distance column of each tool
  int n_cols = 0;
  MpmToolDesc* d_tools = nullptr;
  int n_tools = 0;
  bool chained = false;           // mpm_set_chained
  MpmTuning tune = {0, 0, 0, 0, 0, 0};  // mpm_set_tuning
  const void* premarked = nullptr;  // frame whose block flags the last forward g2p set
  std::vector<MpmToolDesc> h_tools;
  unsigned int* d_status = nullptr;
  int* d_flags = nullptr;  // convergence flags of mpm_target_sdf
  int* d_pair_off = nullptr;  // [n_scenes + 1] first collision pair of each scene
  int n_pairs = 0;            // tool-tool collision pairs over all scenes
  int max_scene_pairs = 0;    // most pairs of one scene
  double* d_coll_pts = nullptr;  // [n][600][3] random points of mpm_set_collision_points
  int n_coll_pts = 0;            // pairs of points uploaded
  void* grid[4] = {nullptr, nullptr, nullptr, nullptr};
  unsigned char* d_blockbuf = nullptr;
  int* d_active = nullptr;
  void* d_tools_t = nullptr;  // tools in the compute precision (converted by mpm_set_tools)
  void* d_poses_t = nullptr;  // poses of the current substep in the compute precision
  mpm::SortScratch sort;      // particle re-sort (mpm_sort_frame)
  // pipelined adjoint (mpm_set_pipelined_adjoint): the grid preparation of an
  // adjoint substep runs on pipe_side beside the previous substep's p2g.grad
  bool pipelined = false;
  bool pipe_pending = false;          // the last call was a pipelined adjoint substep on pipe_stream
  void* pipe_stream = nullptr;
  cudaStream_t pipe_side = nullptr;
  cudaEvent_t pipe_grid_done = nullptr;  // recorded after grid_op.grad of the last call
  cudaEvent_t pipe_prep_done = nullptr;  // recorded after the side stream's preparation
  int sm_count = 1;
  std::string err;
  int64_t launches = 0;
  mpm::Profiler prof;
  std::vector<cudaEvent_t> events;  // event pool of the profiler
  std::vector<mpm::Profiler::Rec> recs;
};

namespace mpm {
void record_global_error(const std::string& msg);
int prof_begin(Profiler* P, cudaStream_t s) {
  if (!P || !P->on) return -1;
  if (P->pool_n + 2 > P->pool_cap) return -1;  // pool exhausted: drop this sample
  cudaEvent_t a = P->pool[P->pool_n];
  if (cudaEventRecord(a, s) != cudaSuccess) return -1;
  return P->pool_n;
}
void prof_end(Profiler* P, int slot, int kind, cudaStream_t s) {
  if (slot < 0 || !P || P->n >= P->cap) return;
  cudaEvent_t b = P->pool[slot + 1];
  if (cudaEventRecord(b, s) != cudaSuccess) return;
  P->recs[P->n++] = Profiler::Rec{kind, P->pool[slot], b};
  P->pool_n = slot + 2;
}
}  // namespace mpm

namespace {

std::mutex g_err_mu;
std::string g_create_err;

int fail(MpmHandle* h, int code, const std::string& msg) {
  if (h) {
    h->err = msg;
  } else {
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_create_err = msg;
  }
  return code;
}
}  // namespace

void mpm::record_global_error(const std::string& msg) {
  std::lock_guard<std::mutex> lk(g_err_mu);
  g_create_err = msg;
}

namespace {

int cuda_fail(MpmHandle* h, cudaError_t e, const char* where) {
  return fail(h, MPM_E_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}
size_t real_size(int precision) { return precision == MPM_PREC_FP64 ? sizeof(double) : sizeof(float); }

mpm::LaunchCtx ctx(MpmHandle* h, void* stream) {
  mpm::LaunchCtx L;
  L.p = &h->p;
  L.G = h->G;
  L.pscene = h->d_pscene;
  L.tools = h->d_tools;
  L.tool_off = h->d_tool_off;
  L.n_tools = h->n_tools;
  L.status = h->d_status;
  L.grid_a = h->grid[0];
  L.grid_b = h->grid[1];
  L.grid_c = h->grid[2];
  L.grid_d = h->grid[3];
  L.blockbuf = h->d_blockbuf;
  L.active = h->d_active;
  L.tools_t = h->d_tools_t;
  L.poses_t = h->d_poses_t;
  L.sm_count = h->sm_count;
  L.stream = (cudaStream_t)stream;
  L.launches = &h->launches;
  L.prof = &h->prof;
  L.tune = h->tune;
  return L;
}
int check_device(MpmHandle* h) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaGetDevice");
  if (dev != h->device)
    return fail(h, MPM_E_INVALID, "handle was created on device " + std::to_string(h->device) +
                                      " but device " + std::to_string(dev) + " is current");
  return MPM_OK;
}
int check_aligned(MpmHandle* h, const void* ptr, const char* name, bool allow_null = false, unsigned align = 16) {
  if (!ptr) return allow_null ? MPM_OK : fail(h, MPM_E_INVALID, std::string(name) + " is NULL");
  if (((uintptr_t)ptr) % align != 0)
    return fail(h, MPM_E_INVALID, std::string(name) + " is not " + std::to_string(align) + "-byte aligned");
  return MPM_OK;
}
#define MPM_TRY(x)          \
  do {                      \
    int _rc = (x);          \
    if (_rc != MPM_OK) return _rc; \
  } while (0)

}  // namespace

extern "C" {

const char* mpm_version(void) { return "mpm_gb300 3 (sm_103a)"; }

int mpm_create(const MpmParams* params, const int64_t* scene_offsets, MpmHandle** out) {
  if (!params || !scene_offsets || !out) return fail(nullptr, MPM_E_INVALID, "mpm_create: NULL argument");
  *out = nullptr;
  const MpmParams& p = *params;
  if (p.abi_version != MPM_ABI_VERSION)
    return fail(nullptr, MPM_E_INVALID, "mpm_create: ABI version mismatch (got " + std::to_string(p.abi_version) +
                                            ", library " + std::to_string(MPM_ABI_VERSION) + ")");
  if (p.precision < MPM_PREC_FP32 || p.precision > MPM_PREC_FP64)
    return fail(nullptr, MPM_E_INVALID, "mpm_create: unknown precision " + std::to_string(p.precision));
  if (p.n_grid < 8 || p.n_grid > 1024 || p.n_grid % 8 != 0)
    return fail(nullptr, MPM_E_INVALID, "mpm_create: n_grid must be a multiple of 8 in [8, 1024], got " +
                                            std::to_string(p.n_grid));
  if (p.n_scenes < 1) return fail(nullptr, MPM_E_INVALID, "mpm_create: n_scenes must be >= 1");
  if (p.n_particles < 0 || p.ld < p.n_particles || p.n_particles > (int64_t)INT32_MAX * 2)
    return fail(nullptr, MPM_E_INVALID, "mpm_create: need 0 <= n_particles <= ld");
  if (!(p.dt > 0) || !(p.dx > 0) || !(p.p_mass > 0))
    return fail(nullptr, MPM_E_INVALID, "mpm_create: dt, dx and p_mass must be positive");
  if (scene_offsets[0] != 0 || scene_offsets[p.n_scenes] != p.n_particles)
    return fail(nullptr, MPM_E_INVALID, "mpm_create: scene_offsets must start at 0 and end at n_particles");
  for (int s = 0; s < p.n_scenes; ++s)
    if (scene_offsets[s + 1] < scene_offsets[s])
      return fail(nullptr, MPM_E_INVALID, "mpm_create: scene_offsets must be non-decreasing");

  MpmHandle* h = new MpmHandle();
  h->p = p;
  h->G = (int64_t)p.n_grid * p.n_grid * p.n_grid;
  h->offsets.assign(scene_offsets, scene_offsets + p.n_scenes + 1);
  cudaError_t e = cudaGetDevice(&h->device);
  if (e != cudaSuccess) {
    delete h;
    return cuda_fail(nullptr, e, "mpm_create: cudaGetDevice");
  }
  std::vector<int> ps(p.n_particles);
  for (int s = 0; s < p.n_scenes; ++s)
    for (int64_t i = scene_offsets[s]; i < scene_offsets[s + 1]; ++i) ps[i] = s;
  std::vector<int> toff(p.n_scenes + 1, 0);
  const size_t gbytes = (size_t)p.n_scenes * h->G * 4 * real_size(p.precision);
  bool ok = true;
  ok = ok && cudaMalloc(&h->d_pscene, std::max<size_t>(1, ps.size()) * sizeof(int)) == cudaSuccess;
  ok = ok && cudaMalloc(&h->d_tool_off, toff.size() * sizeof(int)) == cudaSuccess;
  ok = ok && cudaMalloc(&h->d_status, sizeof(unsigned int)) == cudaSuccess;
  ok = ok && cudaMalloc(&h->d_flags, 4 * sizeof(int)) == cudaSuccess;
  ok = ok && cudaMalloc(&h->d_pair_off, toff.size() * sizeof(int)) == cudaSuccess;
  for (int i = 0; i < 4 && ok; ++i) ok = cudaMalloc(&h->grid[i], gbytes) == cudaSuccess;
  const int64_t nb = p.n_grid / 4;
  const int64_t nblocks = (int64_t)p.n_scenes * nb * nb * nb;
  ok = ok && cudaMalloc(&h->d_blockbuf, mpm::blockbuf_bytes(p.n_scenes, p.n_grid)) == cudaSuccess;
  // block flags start clean; every compaction clears the flags it reads
  ok = ok && cudaMemset(h->d_blockbuf, 0, mpm::blockbuf_bytes(p.n_scenes, p.n_grid)) == cudaSuccess;
  ok = ok && cudaMalloc(&h->d_active, nblocks * sizeof(int)) == cudaSuccess;
  const size_t np = (size_t)std::max<int64_t>(p.n_particles, 1);
  ok = ok && cudaMalloc(&h->sort.keys_a, np * sizeof(uint32_t)) == cudaSuccess;
  ok = ok && cudaMalloc(&h->sort.keys_b, np * sizeof(uint32_t)) == cudaSuccess;
  ok = ok && cudaMalloc(&h->sort.vals_b, np * sizeof(int32_t)) == cudaSuccess;
  ok = ok && cudaMalloc(&h->sort.hist, mpm::sort_hist_words(p.n_particles) * sizeof(uint32_t)) == cudaSuccess;
  // the pipelined adjoint's internal stream and events (created here, outside any stream capture)
  ok = ok && cudaStreamCreateWithFlags(&h->pipe_side, cudaStreamNonBlocking) == cudaSuccess;
  ok = ok && cudaEventCreateWithFlags(&h->pipe_grid_done, cudaEventDisableTiming) == cudaSuccess;
  ok = ok && cudaEventCreateWithFlags(&h->pipe_prep_done, cudaEventDisableTiming) == cudaSuccess;
  if (ok) cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, h->device);
  if (h->sm_count < 1) h->sm_count = 1;
  if (!ok) {
    cudaGetLastError();
    mpm_destroy(h);
    return fail(nullptr, MPM_E_NOMEM, "mpm_create: device allocation of " + std::to_string(4 * gbytes) +
                                          " grid bytes failed");
  }
  if (!ps.empty()) e = cudaMemcpy(h->d_pscene, ps.data(), ps.size() * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(h->d_tool_off, toff.data(), toff.size() * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(h->d_pair_off, toff.data(), toff.size() * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(h->d_status, 0, sizeof(unsigned int));
  if (e != cudaSuccess) {
    mpm_destroy(h);
    return cuda_fail(nullptr, e, "mpm_create: upload");
  }
  *out = h;
  return MPM_OK;
}

int mpm_destroy(MpmHandle* h) {
  if (!h) return MPM_OK;
  cudaFree(h->d_pscene);
  cudaFree(h->d_tool_off);
  cudaFree(h->d_col_off);
  cudaFree(h->d_tools);
  cudaFree(h->d_status);
  cudaFree(h->d_flags);
  cudaFree(h->d_pair_off);
  cudaFree(h->d_coll_pts);
  for (int i = 0; i < 4; ++i) cudaFree(h->grid[i]);
  cudaFree(h->d_blockbuf);
  cudaFree(h->d_active);
  cudaFree(h->d_tools_t);
  cudaFree(h->d_poses_t);
  cudaFree(h->sort.keys_a);
  cudaFree(h->sort.keys_b);
  cudaFree(h->sort.vals_b);
  cudaFree(h->sort.hist);
  if (h->pipe_side) cudaStreamDestroy(h->pipe_side);
  if (h->pipe_grid_done) cudaEventDestroy(h->pipe_grid_done);
  if (h->pipe_prep_done) cudaEventDestroy(h->pipe_prep_done);
  for (cudaEvent_t e : h->events) cudaEventDestroy(e);
  delete h;
  return MPM_OK;
}

int mpm_set_tools(MpmHandle* h, const MpmToolDesc* tools, int32_t n_tools) {
  if (!h) return fail(nullptr, MPM_E_INVALID, "mpm_set_tools: NULL handle");
  if (n_tools < 0 || (n_tools > 0 && !tools)) return fail(h, MPM_E_INVALID, "mpm_set_tools: bad tool array");
  MPM_TRY(check_device(h));
  std::vector<int> toff(h->p.n_scenes + 1, 0);
  int prev = 0;
  for (int i = 0; i < n_tools; ++i) {
    const MpmToolDesc& d = tools[i];
    if (d.type < MPM_TOOL_SPHERE || d.type > MPM_TOOL_GRIPPER2)
      return fail(h, MPM_E_INVALID, "mpm_set_tools: tool " + std::to_string(i) + " has unknown type");
    if (d.scene < 0 || d.scene >= h->p.n_scenes || d.scene < prev)
      return fail(h, MPM_E_INVALID, "mpm_set_tools: tools must be sorted by a valid scene index");
    if (d.action_dim < 0 || d.action_dim > 7)
      return fail(h, MPM_E_INVALID, "mpm_set_tools: action_dim must be in [0, 7]");
    prev = d.scene;
    toff[d.scene + 1]++;
  }
  for (int s = 0; s < h->p.n_scenes; ++s) {
    if (toff[s + 1] > mpm::MAX_TOOLS_PER_SCENE)
      return fail(h, MPM_E_INVALID, "mpm_set_tools: more than " + std::to_string(mpm::MAX_TOOLS_PER_SCENE) +
                                        " tools in scene " + std::to_string(s));
    toff[s + 1] += toff[s];
  }
  // collision pairs (i, j) of each scene, scene-local indices, in the order
  // of MPMSimulator.set_num_collision (mpm_simulator.py:69-80)
  std::vector<int> poff(h->p.n_scenes + 1, 0);
  int max_pairs = 0;
  for (int s = 0; s < h->p.n_scenes; ++s) {
    const int nt = toff[s + 1] - toff[s];
    int np = 0;
    for (int i = toff[s]; i < toff[s + 1]; ++i) {
      const uint32_t m = (uint32_t)tools[i].collision_mask;
      if (nt < 32 && (m >> nt) != 0)
        return fail(h, MPM_E_INVALID, "mpm_set_tools: tool " + std::to_string(i) +
                                          " has a collision_mask bit beyond its scene's tools");
      for (int j = 0; j < nt; ++j)
        if ((m >> j) & 1u) {
          if (toff[s] + j == i) return fail(h, MPM_E_INVALID, "mpm_set_tools: a tool cannot collide with itself");
          ++np;
        }
    }
    poff[s + 1] = poff[s] + np;
    max_pairs = std::max(max_pairs, np);
  }
  std::vector<int> coff(std::max(n_tools, 1), 0);
  int ncols = 0;
  for (int i = 0; i < n_tools; ++i) {
    coff[i] = ncols;
    ncols += (tools[i].type == MPM_TOOL_GRIPPER || tools[i].type == MPM_TOOL_GRIPPER2) ? 2 : 1;
  }
  cudaError_t e = cudaSuccess;
  if (n_tools > h->n_tools || !h->d_tools_t) {
    cudaFree(h->d_tools);
    cudaFree(h->d_col_off);
    cudaFree(h->d_tools_t);
    cudaFree(h->d_poses_t);
    h->d_tools = nullptr;
    h->d_col_off = nullptr;
    h->d_tools_t = nullptr;
    h->d_poses_t = nullptr;
    e = cudaMalloc(&h->d_tools, std::max(n_tools, 1) * sizeof(MpmToolDesc));
    if (e == cudaSuccess) e = cudaMalloc(&h->d_col_off, std::max(n_tools, 1) * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&h->d_tools_t, mpm::tools_t_bytes(n_tools));
    if (e == cudaSuccess) e = cudaMalloc(&h->d_poses_t, mpm::poses_t_bytes(n_tools));
    if (e != cudaSuccess) return cuda_fail(h, e, "mpm_set_tools: cudaMalloc");
  }
  if (n_tools > 0) e = cudaMemcpy(h->d_tools, tools, n_tools * sizeof(MpmToolDesc), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = mpm::convert_tools(h->p.precision, n_tools, h->d_tools, h->d_tools_t, nullptr);
  if (e == cudaSuccess) e = cudaStreamSynchronize(nullptr);
  if (e == cudaSuccess && n_tools > 0)
    e = cudaMemcpy(h->d_col_off, coff.data(), n_tools * sizeof(int), cudaMemcpyHostToDevice);
  h->n_cols = ncols;
  if (e == cudaSuccess) e = cudaMemcpy(h->d_tool_off, toff.data(), toff.size() * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(h->d_pair_off, poff.data(), poff.size() * sizeof(int), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(h, e, "mpm_set_tools: upload");
  h->n_pairs = poff[h->p.n_scenes];
  h->max_scene_pairs = max_pairs;
  h->n_tools = n_tools;
  h->h_tools.assign(tools, tools + n_tools);
  return MPM_OK;
}

int mpm_set_collision_points(MpmHandle* h, const double* points, int32_t n_pairs) {
  if (!h) return fail(nullptr, MPM_E_INVALID, "mpm_set_collision_points: NULL handle");
  if (n_pairs < 0 || (n_pairs > 0 && !points)) return fail(h, MPM_E_INVALID, "mpm_set_collision_points: bad array");
  MPM_TRY(check_device(h));
  cudaFree(h->d_coll_pts);
  h->d_coll_pts = nullptr;
  h->n_coll_pts = 0;
  if (n_pairs == 0) return MPM_OK;
  const size_t bytes = (size_t)n_pairs * 600 * 3 * sizeof(double);
  cudaError_t e = cudaMalloc(&h->d_coll_pts, bytes);
  if (e == cudaSuccess) e = cudaMemcpy(h->d_coll_pts, points, bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(h, e, "mpm_set_collision_points");
  h->n_coll_pts = n_pairs;
  return MPM_OK;
}

int mpm_collision_pairs(MpmHandle* h) { return h ? h->n_pairs : 0; }

static int check_collision(MpmHandle* h, const double* coll, const char* what) {
  if (h->n_pairs == 0) return MPM_OK;
  if (h->n_coll_pts < h->max_scene_pairs)
    return fail(h, MPM_E_INVALID, std::string(what) + ": a scene has " + std::to_string(h->max_scene_pairs) +
                                      " collision pairs but mpm_set_collision_points gave points for " +
                                      std::to_string(h->n_coll_pts));
  return check_aligned(h, coll, "coll");
}

int mpm_tools_action(MpmHandle* h, const double* action, double* vel, double* pose, double* coll, int32_t n_sub,
                     void* stream) {
  if (!h) return fail(nullptr, MPM_E_INVALID, "mpm_tools_action: NULL handle");
  if (n_sub < 1) return fail(h, MPM_E_INVALID, "mpm_tools_action: n_sub must be >= 1");
  if (h->n_tools == 0) return MPM_OK;
  MPM_TRY(check_device(h));
  MPM_TRY(check_aligned(h, action, "action"));
  MPM_TRY(check_aligned(h, vel, "vel"));
  MPM_TRY(check_aligned(h, pose, "pose"));
  MPM_TRY(check_collision(h, coll, "mpm_tools_action"));
  mpm::LaunchCtx L = ctx(h, stream);
  cudaError_t e = mpm::launch_tools_action(L, h->n_tools, h->d_pair_off, h->n_pairs, h->d_coll_pts, action, vel,
                                           pose, coll, n_sub);
  return e == cudaSuccess ? MPM_OK : cuda_fail(h, e, "mpm_tools_action");
}

int mpm_tools_action_bwd(MpmHandle* h, const double* vel, const double* pose, const double* coll, double* g_pose,
                         double* g_action, int32_t n_sub, void* stream) {
  if (!h) return fail(nullptr, MPM_E_INVALID, "mpm_tools_action_bwd: NULL handle");
  if (n_sub < 1) return fail(h, MPM_E_INVALID, "mpm_tools_action_bwd: n_sub must be >= 1");
  if (h->n_tools == 0) return MPM_OK;
  MPM_TRY(check_device(h));
  MPM_TRY(check_aligned(h, vel, "vel"));
  MPM_TRY(check_aligned(h, pose, "pose"));
  MPM_TRY(check_aligned(h, g_pose, "g_pose"));
  MPM_TRY(check_aligned(h, g_action, "g_action"));
  MPM_TRY(check_collision(h, coll, "mpm_tools_action_bwd"));
  mpm::LaunchCtx L = ctx(h, stream);
  cudaError_t e = mpm::launch_tools_action_bwd(L, h->n_tools, h->d_pair_off, h->n_pairs, h->d_coll_pts, vel, pose,
                                               coll, g_pose, g_action, n_sub);
  return e == cudaSuccess ? MPM_OK : cuda_fail(h, e, "mpm_tools_action_bwd");
}

static int check_store(MpmHandle* h, const MpmGridStore* store, int32_t slot) {
  if (!store) return MPM_OK;
  if (slot < 0 || slot >= store->n_slots) return fail(h, MPM_E_INVALID, "grid store slot out of range");
  if (store->capacity < 0 || !store->slot_start || !store->slot_count || !store->bump ||
      (store->capacity > 0 && (!store->blocks || !store->block_ids)))
    return fail(h, MPM_E_INVALID, "grid store has NULL buffers");
  return check_aligned(h, store->blocks, "store->blocks", store->capacity == 0);
}

static int substep_fwd_impl(MpmHandle* h, const void* state_f, void* state_f1, const double* pose_f,
                            const double* pose_f1, const MpmGridStore* store, int32_t slot, void* stream) {
  if (!h) return fail(nullptr, MPM_E_INVALID, "mpm_substep_fwd: NULL handle");
  MPM_TRY(check_device(h));
  MPM_TRY(check_aligned(h, state_f, "state_f"));
  MPM_TRY(check_aligned(h, state_f1, "state_f1"));
  if (state_f == state_f1) return fail(h, MPM_E_INVALID, "mpm_substep_fwd: state_f and state_f1 must differ");
  MPM_TRY(check_aligned(h, pose_f, "pose_f", h->n_tools == 0));
  MPM_TRY(check_aligned(h, pose_f1, "pose_f1", h->n_tools == 0));
  MPM_TRY(check_store(h, store, slot));
  mpm::LaunchCtx L = ctx(h, stream);
  // chained substeps: the previous forward substep's g2p flagged the blocks of
  // this substep's input frame
  const bool pre = h->chained && h->premarked == state_f;
  const bool next = h->chained;
  h->premarked = nullptr;
  h->pipe_pending = false;  // a forward substep rewrites the grids: no adjoint overlaps it
  cudaError_t e;
  switch (h->p.precision) {
    case MPM_PREC_FP32:
      e = mpm::launch_substep_fwd<float, float>(L, (const float*)state_f, (float*)state_f1, pose_f, pose_f1, store,
                                                slot, pre, next);
      break;
    case MPM_PREC_FP32_SVD64:
      e = mpm::launch_substep_fwd<float, double>(L, (const float*)state_f, (float*)state_f1, pose_f, pose_f1, store,
                                                 slot, pre, next);
      break;
    default:
      e = mpm::launch_substep_fwd<double, double>(L, (const double*)state_f, (double*)state_f1, pose_f, pose_f1,
                                                  store, slot, pre, next);
  }
  if (e != cudaSuccess) return cuda_fail(h, e, "mpm_substep_fwd");
  if (next) h->premarked = state_f1;
  return MPM_OK;
}

static int substep_bwd_impl(MpmHandle* h, const void* state_f, const void* state_f1, const void* g_state_f1,
                            void* g_state_f,
                            const double* pose_f, const double* pose_f1, double* g_pose_f, double* g_pose_f1,
                            const MpmGridStore* store, int32_t slot, void* stream) {
  if (!h) return fail(nullptr, MPM_E_INVALID, "mpm_substep_bwd: NULL handle");
  MPM_TRY(check_device(h));
  MPM_TRY(check_aligned(h, state_f, "state_f"));
  MPM_TRY(check_aligned(h, state_f1, "state_f1", true));
  MPM_TRY(check_aligned(h, g_state_f1, "g_state_f1"));
  MPM_TRY(check_aligned(h, g_state_f, "g_state_f"));
  if (g_state_f == g_state_f1) return fail(h, MPM_E_INVALID, "mpm_substep_bwd: g_state_f and g_state_f1 must differ");
  bool nt = h->n_tools == 0;
  MPM_TRY(check_aligned(h, pose_f, "pose_f", nt));
  MPM_TRY(check_aligned(h, pose_f1, "pose_f1", nt));
  MPM_TRY(check_aligned(h, g_pose_f, "g_pose_f", nt));
  MPM_TRY(check_aligned(h, g_pose_f1, "g_pose_f1", nt));
  MPM_TRY(check_store(h, store, slot));
  mpm::LaunchCtx L = ctx(h, stream);
  h->premarked = nullptr;  // the adjoint's compaction may consume the flags
  auto run = [&](const mpm::LaunchCtx& C, unsigned phases) -> cudaError_t {
    switch (h->p.precision) {
      case MPM_PREC_FP32:
        return mpm::launch_substep_bwd<float, float>(C, (const float*)state_f, (const float*)state_f1,
                                                     (const float*)g_state_f1, (float*)g_state_f, pose_f, pose_f1,
                                                     g_pose_f, g_pose_f1, store, slot, phases);
      case MPM_PREC_FP32_SVD64:
        return mpm::launch_substep_bwd<float, double>(C, (const float*)state_f, (const float*)state_f1,
                                                      (const float*)g_state_f1, (float*)g_state_f, pose_f, pose_f1,
                                                      g_pose_f, g_pose_f1, store, slot, phases);
      default:
        return mpm::launch_substep_bwd<double, double>(C, (const double*)state_f, (const double*)state_f1,
                                                       (const double*)g_state_f1, (double*)g_state_f, pose_f,
                                                       pose_f1, g_pose_f, g_pose_f1, store, slot, phases);
    }
  };
  cudaError_t e = cudaSuccess;
  if (!h->pipelined || h->prof.on) {  // the profiler times the kernels one at a time
    e = run(L, mpm::BWD_ALL);
    h->pipe_pending = false;
  } else {
    // The previous call left its p2g.grad queued on this stream after an
    // event that follows its grid_op.grad.  This substep's preparation (block
    // list, pose table, grids restored or recomputed) touches neither that
    // kernel's inputs nor its outputs, so it runs on the side stream as soon
    // as grid_op.grad is done, beside that p2g.grad; g2p.grad then waits for
    // both.
    const cudaStream_t main = (cudaStream_t)stream;
    unsigned grid_phases = mpm::BWD_GRID;
    if (h->pipe_pending && h->pipe_stream == stream) {
      mpm::LaunchCtx S = L;
      S.stream = h->pipe_side;
      e = cudaStreamWaitEvent(h->pipe_side, h->pipe_grid_done, 0);
      if (e == cudaSuccess) e = run(S, mpm::BWD_PREPARE);
      if (e == cudaSuccess) e = cudaEventRecord(h->pipe_prep_done, h->pipe_side);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(main, h->pipe_prep_done, 0);
      grid_phases |= mpm::BWD_G2P_PLAIN;  // the kernel before it on this stream is the previous p2g.grad
    } else {
      e = run(L, mpm::BWD_PREPARE);
    }
    if (e == cudaSuccess) e = run(L, grid_phases);
    if (e == cudaSuccess) e = cudaEventRecord(h->pipe_grid_done, main);
    if (e == cudaSuccess) e = run(L, mpm::BWD_PARTICLES);
    h->pipe_pending = e == cudaSuccess;
    h->pipe_stream = stream;
  }
  return e == cudaSuccess ? MPM_OK : cuda_fail(h, e, "mpm_substep_bwd");
}

int mpm_set_pipelined_adjoint(MpmHandle* h, int32_t on) {
  if (!h) return fail(nullptr, MPM_E_INVALID, "mpm_set_pipelined_adjoint: NULL handle");
  h->pipelined = on != 0;
  h->pipe_pending = false;
  return MPM_OK;
}

int mpm_set_chained(MpmHandle* h, int32_t on) {
  if (!h) return fail(nullptr, MPM_E_INVALID, "mpm_set_chained: NULL handle");
  h->chained = on != 0;
  h->premarked = nullptr;
  return MPM_OK;
}

int mpm_set_tuning(MpmHandle* h, const MpmTuning* t) {
  if (!h) return fail(nullptr, MPM_E_INVALID, "mpm_set_tuning: NULL handle");
  if (!t) return fail(h, MPM_E_INVALID, "mpm_set_tuning: NULL tuning");
  auto in = [](int v, std::initializer_list<int> ok) {
    for (int o : ok)
      if (v == o) return true;
    return false;
  };
  if (!in(t->p2g_ctas, {0, 6, 7, 8})) return fail(h, MPM_E_INVALID, "mpm_set_tuning: p2g_ctas must be 0, 6, 7 or 8");
  if (!in(t->g2p_adj_ctas, {0, 5, 6, 7, 8}))
    return fail(h, MPM_E_INVALID, "mpm_set_tuning: g2p_adj_ctas must be 0, 5, 6, 7 or 8");
  if (!in(t->p2g_adj_ctas, {0, 4, 5, 6}))
    return fail(h, MPM_E_INVALID, "mpm_set_tuning: p2g_adj_ctas must be 0, 4, 5 or 6");
  if (t->grid_ctas_per_sm != 0 && (t->grid_ctas_per_sm < 2 || t->grid_ctas_per_sm > 64))
    return fail(h, MPM_E_INVALID, "mpm_set_tuning: grid_ctas_per_sm must be 0 or in [2, 64]");
  if (!in(t->g2p_ctas, {0, 8, 10, 12})) return fail(h, MPM_E_INVALID, "mpm_set_tuning: g2p_ctas must be 0, 8, 10 or 12");
  if (!in(t->grid_op_adj_ctas, {0, 6, 12, 16}))
    return fail(h, MPM_E_INVALID, "mpm_set_tuning: grid_op_adj_ctas must be 0, 6, 12 or 16");
  h->tune = *t;
  return MPM_OK;
}

int mpm_get_tuning(MpmHandle* h, MpmTuning* t) {
  if (!h || !t) return fail(h, MPM_E_INVALID, "mpm_get_tuning: NULL argument");
  *t = h->tune;
  if (!t->p2g_ctas) t->p2g_ctas = 7;
  if (!t->g2p_adj_ctas) t->g2p_adj_ctas = 6;
  if (!t->p2g_adj_ctas) t->p2g_adj_ctas = 5;
  if (!t->grid_ctas_per_sm) t->grid_ctas_per_sm = 16;
  if (!t->g2p_ctas) t->g2p_ctas = 8;
  if (!t->grid_op_adj_ctas) t->grid_op_adj_ctas = 6;
  return MPM_OK;
}

int mpm_substep_fwd(MpmHandle* h, const void* state_f, void* state_f1, const double* pose_f, const double* pose_f1,
                    void* stream) {
  return substep_fwd_impl(h, state_f, state_f1, pose_f, pose_f1, nullptr, -1, stream);
}
int mpm_substep_fwd_store(MpmHandle* h, const void* state_f, void* state_f1, const double* pose_f,
                          const double* pose_f1, const MpmGridStore* store, int32_t slot, void* stream) {
  if (!store) return fail(h, MPM_E_INVALID, "mpm_substep_fwd_store: NULL store");
  return substep_fwd_impl(h, state_f, state_f1, pose_f, pose_f1, store, slot, stream);
}
int mpm_substep_bwd(MpmHandle* h, const void* state_f, const void* state_f1, const void* g_state_f1,
                    void* g_state_f, const double* pose_f, const double* pose_f1, double* g_pose_f,
                    double* g_pose_f1, void* stream) {
  return substep_bwd_impl(h, state_f, state_f1, g_state_f1, g_state_f, pose_f, pose_f1, g_pose_f, g_pose_f1,
                          nullptr, -1, stream);
}
int mpm_substep_bwd_store(MpmHandle* h, const void* state_f, const void* state_f1, const void* g_state_f1,
                          void* g_state_f, const double* pose_f, const double* pose_f1, double* g_pose_f,
                          double* g_pose_f1, const MpmGridStore* store, int32_t slot, void* stream) {
  if (!store) return fail(h, MPM_E_INVALID, "mpm_substep_bwd_store: NULL store");
  return substep_bwd_impl(h, state_f, state_f1, g_state_f1, g_state_f, pose_f, pose_f1, g_pose_f, g_pose_f1, store,
                          slot, stream);
}

int mpm_grid_mass(MpmHandle* h, const void* state, void* grid_m, void* stream) {
  if (!h) return fail(nullptr, MPM_E_INVALID, "mpm_grid_mass: NULL handle");
  MPM_TRY(check_device(h));
  MPM_TRY(check_aligned(h, state, "state"));
  MPM_TRY(check_aligned(h, grid_m, "grid_m"));
  mpm::LaunchCtx L = ctx(h, stream);
  cudaError_t e = h->p.precision == MPM_PREC_FP64
                      ? mpm::launch_grid_mass<double>(L, (const double*)state, (double*)grid_m)
                      : mpm::launch_grid_mass<float>(L, (const float*)state, (float*)grid_m);
  return e == cudaSuccess ? MPM_OK : cuda_fail(h, e, "mpm_grid_mass");
}

namespace {
// the frames [a, a + 24 ld) and [b, b + 24 ld) share no byte
bool frames_disjoint(const MpmHandle* h, const void* a, const void* b) {
  const uintptr_t n = (uintptr_t)(24 * h->p.ld) * real_size(h->p.precision);
  const uintptr_t x = (uintptr_t)a, y = (uintptr_t)b;
  return x + n <= y || y + n <= x;
}
int check_sortable(MpmHandle* h, const char* fn) {
  if (h->p.n_particles > (int64_t)INT32_MAX)
    return fail(h, MPM_E_INVALID, std::string(fn) + ": more than 2^31 - 1 particles");
  if (mpm::sort_key_bits(h->p.n_scenes, h->p.n_grid) > 32)
    return fail(h, MPM_E_INVALID, std::string(fn) + ": n_scenes * n_grid^3 must be below 2^32");
  return MPM_OK;
}
}  // namespace

int mpm_sort_frame(MpmHandle* h, const void* src, void* dst, int32_t* perm, void* stream) {
  if (!h) return fail(nullptr, MPM_E_INVALID, "mpm_sort_frame: NULL handle");
  MPM_TRY(check_device(h));
  MPM_TRY(check_aligned(h, src, "src"));
  MPM_TRY(check_aligned(h, dst, "dst"));
  MPM_TRY(check_aligned(h, perm, "perm", false, 4));  // int32, read one word at a time
  MPM_TRY(check_sortable(h, "mpm_sort_frame"));
  if (!frames_disjoint(h, src, dst)) return fail(h, MPM_E_INVALID, "mpm_sort_frame: src and dst overlap");
  mpm::LaunchCtx L = ctx(h, stream);
  cudaError_t e = h->p.precision == MPM_PREC_FP64
                      ? mpm::launch_sort_frame<double>(L, (const double*)src, (double*)dst, perm, h->sort)
                      : mpm::launch_sort_frame<float>(L, (const float*)src, (float*)dst, perm, h->sort);
  if (e != cudaSuccess) return cuda_fail(h, e, "mpm_sort_frame");
  // same particle set: the block flags a chained forward set for src hold for dst
  if (h->premarked == src) h->premarked = dst;
  return MPM_OK;
}

int mpm_unsort_frame(MpmHandle* h, const void* g_src, void* g_dst, const int32_t* perm, void* stream) {
  if (!h) return fail(nullptr, MPM_E_INVALID, "mpm_unsort_frame: NULL handle");
  MPM_TRY(check_device(h));
  MPM_TRY(check_aligned(h, g_src, "g_src"));
  MPM_TRY(check_aligned(h, g_dst, "g_dst"));
  MPM_TRY(check_aligned(h, perm, "perm", false, 4));  // int32, read one word at a time
  MPM_TRY(check_sortable(h, "mpm_unsort_frame"));
  if (!frames_disjoint(h, g_src, g_dst)) return fail(h, MPM_E_INVALID, "mpm_unsort_frame: g_src and g_dst overlap");
  mpm::LaunchCtx L = ctx(h, stream);
  cudaError_t e = h->p.precision == MPM_PREC_FP64
                      ? mpm::launch_unsort_frame<double>(L, (const double*)g_src, (double*)g_dst, perm)
                      : mpm::launch_unsort_frame<float>(L, (const float*)g_src, (float*)g_dst, perm);
  return e == cudaSuccess ? MPM_OK : cuda_fail(h, e, "mpm_unsort_frame");
}

int mpm_grid_mass_bwd(MpmHandle* h, const void* state, const void* g_grid_m, void* g_state, void* stream) {
  if (!h) return fail(nullptr, MPM_E_INVALID, "mpm_grid_mass_bwd: NULL handle");
  MPM_TRY(check_device(h));
  MPM_TRY(check_aligned(h, state, "state"));
  MPM_TRY(check_aligned(h, g_grid_m, "g_grid_m"));
  MPM_TRY(check_aligned(h, g_state, "g_state"));
  mpm::LaunchCtx L = ctx(h, stream);
  cudaError_t e =
      h->p.precision == MPM_PREC_FP64
          ? mpm::launch_grid_mass_bwd<double>(L, (const double*)state, (const double*)g_grid_m, (double*)g_state)
          : mpm::launch_grid_mass_bwd<float>(L, (const float*)state, (const float*)g_grid_m, (float*)g_state);
  return e == cudaSuccess ? MPM_OK : cuda_fail(h, e, "mpm_grid_mass_bwd");
}

int mpm_density_l1(MpmHandle* h, const void* grid_m, const void* target, double weight, double* loss,
                   void* g_grid_m, void* stream) {
  if (!h) return fail(nullptr, MPM_E_INVALID, "mpm_density_l1: NULL handle");
  MPM_TRY(check_device(h));
  MPM_TRY(check_aligned(h, grid_m, "grid_m"));
  MPM_TRY(check_aligned(h, target, "target"));
  MPM_TRY(check_aligned(h, loss, "loss"));
  MPM_TRY(check_aligned(h, g_grid_m, "g_grid_m", true));
  mpm::LaunchCtx L = ctx(h, stream);
  cudaError_t e = h->p.precision == MPM_PREC_FP64
                      ? mpm::launch_density_l1<double>(L, (const double*)grid_m, (const double*)target, weight, loss,
                                                       (double*)g_grid_m)
                      : mpm::launch_density_l1<float>(L, (const float*)grid_m, (const float*)target, weight, loss,
                                                      (float*)g_grid_m);
  return e == cudaSuccess ? MPM_OK : cuda_fail(h, e, "mpm_density_l1");
}

int mpm_soft_contact(MpmHandle* h, const void* state, const double* pose, double* sums, double* min_dist,
                     void* stream) {
  if (!h) return fail(nullptr, MPM_E_INVALID, "mpm_soft_contact: NULL handle");
  if (h->n_tools == 0) return MPM_OK;
  MPM_TRY(check_device(h));
  MPM_TRY(check_aligned(h, state, "state"));
  MPM_TRY(check_aligned(h, pose, "pose"));
  MPM_TRY(check_aligned(h, sums, "sums"));
  MPM_TRY(check_aligned(h, min_dist, "min_dist"));
  mpm::LaunchCtx L = ctx(h, stream);
  cudaError_t e =
      h->p.precision == MPM_PREC_FP64
          ? mpm::launch_soft_contact<double>(L, h->n_tools, (const double*)state, pose, sums, min_dist)
          : mpm::launch_soft_contact<float>(L, h->n_tools, (const float*)state, pose, sums, min_dist);
  return e == cudaSuccess ? MPM_OK : cuda_fail(h, e, "mpm_soft_contact");
}

int mpm_soft_contact_bwd(MpmHandle* h, const void* state, const double* pose, const double* sums,
                         const double* g_min_dist, void* g_state, double* g_pose, void* stream) {
  if (!h) return fail(nullptr, MPM_E_INVALID, "mpm_soft_contact_bwd: NULL handle");
  if (h->n_tools == 0) return MPM_OK;
  MPM_TRY(check_device(h));
  MPM_TRY(check_aligned(h, state, "state"));
  MPM_TRY(check_aligned(h, pose, "pose"));
  MPM_TRY(check_aligned(h, sums, "sums"));
  MPM_TRY(check_aligned(h, g_min_dist, "g_min_dist"));
  MPM_TRY(check_aligned(h, g_state, "g_state"));
  MPM_TRY(check_aligned(h, g_pose, "g_pose"));
  mpm::LaunchCtx L = ctx(h, stream);
  cudaError_t e = h->p.precision == MPM_PREC_FP64
                      ? mpm::launch_soft_contact_bwd<double>(L, h->n_tools, (const double*)state, pose, sums,
                                                             g_min_dist, (double*)g_state, g_pose)
                      : mpm::launch_soft_contact_bwd<float>(L, h->n_tools, (const float*)state, pose, sums,
                                                            g_min_dist, (float*)g_state, g_pose);
  return e == cudaSuccess ? MPM_OK : cuda_fail(h, e, "mpm_soft_contact_bwd");
}

int mpm_target_sdf(MpmHandle* h, const void* target_density, void* target_sdf, void* nearest, void* work,
                   int32_t n_iters, void* stream) {
  if (!h) return fail(nullptr, MPM_E_INVALID, "mpm_target_sdf: NULL handle");
  if (n_iters < 0) return fail(h, MPM_E_INVALID, "mpm_target_sdf: n_iters < 0");
  MPM_TRY(check_device(h));
  MPM_TRY(check_aligned(h, target_density, "target_density"));
  MPM_TRY(check_aligned(h, target_sdf, "target_sdf"));
  MPM_TRY(check_aligned(h, nearest, "nearest"));
  MPM_TRY(check_aligned(h, work, "work"));
  mpm::LaunchCtx L = ctx(h, stream);
  cudaError_t e = h->p.precision == MPM_PREC_FP64
                      ? mpm::launch_target_sdf<double>(L, h->d_flags, (const double*)target_density,
                                                       (double*)target_sdf, (double*)nearest, (double*)work, n_iters)
                      : mpm::launch_target_sdf<float>(L, h->d_flags, (const float*)target_density,
                                                      (float*)target_sdf, (float*)nearest, (float*)work, n_iters);
  return e == cudaSuccess ? MPM_OK : cuda_fail(h, e, "mpm_target_sdf");
}

int mpm_sdf_loss(MpmHandle* h, const void* grid_m, const void* target_sdf, double weight, double* loss,
                 void* g_grid_m, void* stream) {
  if (!h) return fail(nullptr, MPM_E_INVALID, "mpm_sdf_loss: NULL handle");
  MPM_TRY(check_device(h));
  MPM_TRY(check_aligned(h, grid_m, "grid_m"));
  MPM_TRY(check_aligned(h, target_sdf, "target_sdf"));
  MPM_TRY(check_aligned(h, loss, "loss"));
  MPM_TRY(check_aligned(h, g_grid_m, "g_grid_m", true));
  mpm::LaunchCtx L = ctx(h, stream);
  cudaError_t e = h->p.precision == MPM_PREC_FP64
                      ? mpm::launch_sdf_loss<double>(L, (const double*)grid_m, (const double*)target_sdf, weight,
                                                     loss, (double*)g_grid_m)
                      : mpm::launch_sdf_loss<float>(L, (const float*)grid_m, (const float*)target_sdf, weight, loss,
                                                    (float*)g_grid_m);
  return e == cudaSuccess ? MPM_OK : cuda_fail(h, e, "mpm_sdf_loss");
}

int mpm_iou(MpmHandle* h, const void* grid_m, const void* target, double* iou, void* stream) {
  if (!h) return fail(nullptr, MPM_E_INVALID, "mpm_iou: NULL handle");
  MPM_TRY(check_device(h));
  MPM_TRY(check_aligned(h, grid_m, "grid_m"));
  MPM_TRY(check_aligned(h, target, "target"));
  MPM_TRY(check_aligned(h, iou, "iou"));
  mpm::LaunchCtx L = ctx(h, stream);
  cudaError_t e = h->p.precision == MPM_PREC_FP64
                      ? mpm::launch_iou<double>(L, (const double*)grid_m, (const double*)target, iou)
                      : mpm::launch_iou<float>(L, (const float*)grid_m, (const float*)target, iou);
  return e == cudaSuccess ? MPM_OK : cuda_fail(h, e, "mpm_iou");
}

int mpm_contact_min_dist(MpmHandle* h, const void* state, const double* pose, double* min_dist, int64_t* argmin,
                         void* stream) {
  if (!h) return fail(nullptr, MPM_E_INVALID, "mpm_contact_min_dist: NULL handle");
  if (h->n_tools == 0) return MPM_OK;
  MPM_TRY(check_device(h));
  MPM_TRY(check_aligned(h, state, "state"));
  MPM_TRY(check_aligned(h, pose, "pose"));
  MPM_TRY(check_aligned(h, min_dist, "min_dist"));
  MPM_TRY(check_aligned(h, argmin, "argmin"));
  mpm::LaunchCtx L = ctx(h, stream);
  cudaError_t e =
      h->p.precision == MPM_PREC_FP64
          ? mpm::launch_contact_min<double>(L, h->n_tools, (const double*)state, pose, min_dist, argmin)
          : mpm::launch_contact_min<float>(L, h->n_tools, (const float*)state, pose, min_dist, argmin);
  return e == cudaSuccess ? MPM_OK : cuda_fail(h, e, "mpm_contact_min_dist");
}

int mpm_contact_min_dist_bwd(MpmHandle* h, const void* state, const double* pose, const int64_t* argmin,
                             const double* g_min_dist, void* g_state, double* g_pose, void* stream) {
  if (!h) return fail(nullptr, MPM_E_INVALID, "mpm_contact_min_dist_bwd: NULL handle");
  if (h->n_tools == 0) return MPM_OK;
  MPM_TRY(check_device(h));
  MPM_TRY(check_aligned(h, state, "state"));
  MPM_TRY(check_aligned(h, pose, "pose"));
  MPM_TRY(check_aligned(h, argmin, "argmin"));
  MPM_TRY(check_aligned(h, g_min_dist, "g_min_dist"));
  MPM_TRY(check_aligned(h, g_state, "g_state"));
  MPM_TRY(check_aligned(h, g_pose, "g_pose"));
  mpm::LaunchCtx L = ctx(h, stream);
  cudaError_t e = h->p.precision == MPM_PREC_FP64
                      ? mpm::launch_contact_min_bwd<double>(L, h->n_tools, (const double*)state, pose, argmin,
                                                            g_min_dist, (double*)g_state, g_pose)
                      : mpm::launch_contact_min_bwd<float>(L, h->n_tools, (const float*)state, pose, argmin,
                                                           g_min_dist, (float*)g_state, g_pose);
  return e == cudaSuccess ? MPM_OK : cuda_fail(h, e, "mpm_contact_min_dist_bwd");
}

static int check_volume(MpmHandle* h, const MpmRenderVolume* v, const char* what) {
  if (!v) return fail(h, MPM_E_INVALID, std::string(what) + ": NULL volume");
  for (int c = 0; c < 3; ++c)
    if (v->res[c] < 2 || v->res[c] > 4096)
      return fail(h, MPM_E_INVALID, std::string(what) + ": volume resolution must be in [2, 4096]");
  if (v->bake_size < 0 || v->bake_size > 64 || !(v->dx > 0))
    return fail(h, MPM_E_INVALID, std::string(what) + ": bad bake_size or dx");
  MPM_TRY(check_aligned(h, v->packed, "vol->packed"));
  MPM_TRY(check_aligned(h, v->sdf, "vol->sdf"));
  MPM_TRY(check_aligned(h, v->sdf_copy, "vol->sdf_copy"));
  MPM_TRY(check_aligned(h, v->color, "vol->color"));
  MPM_TRY(check_aligned(h, v->bbox, "vol->bbox"));
  return check_aligned(h, v->kbox, "vol->kbox");
}

int mpm_render_bake(MpmHandle* h, const void* state, int32_t scene, const uint32_t* colors,
                    const MpmRenderVolume* vol, void* stream) {
  if (!h) return fail(nullptr, MPM_E_INVALID, "mpm_render_bake: NULL handle");
  if (scene < 0 || scene >= h->p.n_scenes) return fail(h, MPM_E_INVALID, "mpm_render_bake: scene out of range");
  MPM_TRY(check_device(h));
  MPM_TRY(check_aligned(h, state, "state"));
  MPM_TRY(check_volume(h, vol, "mpm_render_bake"));
  const int64_t p0 = h->offsets[scene], n = h->offsets[scene + 1] - p0;
  mpm::LaunchCtx L = ctx(h, stream);
  cudaError_t e = h->p.precision == MPM_PREC_FP64
                      ? mpm::launch_render_bake<double>(L, (const double*)state, p0, n, colors, *vol)
                      : mpm::launch_render_bake<float>(L, (const float*)state, p0, n, colors, *vol);
  return e == cudaSuccess ? MPM_OK : cuda_fail(h, e, "mpm_render_bake");
}

int mpm_render_trace(MpmHandle* h, const MpmRenderVolume* vol, const MpmRenderView* view, int32_t scene,
                     const double* pose, const float* tool_color, float* depth, float* normal, float* color,
                     float* image, void* stream) {
  if (!h) return fail(nullptr, MPM_E_INVALID, "mpm_render_trace: NULL handle");
  if (scene < 0 || scene >= h->p.n_scenes) return fail(h, MPM_E_INVALID, "mpm_render_trace: scene out of range");
  if (!view || view->res[0] < 1 || view->res[1] < 1 || view->res[0] > 16384 || view->res[1] > 16384)
    return fail(h, MPM_E_INVALID, "mpm_render_trace: bad view");
  MPM_TRY(check_device(h));
  MPM_TRY(check_volume(h, vol, "mpm_render_trace"));
  int t0 = 0, nt = 0;
  for (int i = 0; i < h->n_tools; ++i)
    if (h->h_tools[i].scene == scene) {
      if (nt == 0) t0 = i;
      ++nt;
    }
  if (nt > 0) {
    MPM_TRY(check_aligned(h, pose, "pose"));
    MPM_TRY(check_aligned(h, tool_color, "tool_color"));
  }
  MPM_TRY(check_aligned(h, depth, "depth"));
  MPM_TRY(check_aligned(h, normal, "normal"));
  MPM_TRY(check_aligned(h, color, "color"));
  MPM_TRY(check_aligned(h, image, "image", true));
  mpm::LaunchCtx L = ctx(h, stream);
  cudaError_t e = h->p.precision == MPM_PREC_FP64
                      ? mpm::launch_render_trace<double>(L, *vol, *view, t0, nt, pose, tool_color, depth, normal,
                                                         color, image)
                      : mpm::launch_render_trace<float>(L, *vol, *view, t0, nt, pose, tool_color, depth, normal,
                                                        color, image);
  return e == cudaSuccess ? MPM_OK : cuda_fail(h, e, "mpm_render_trace");
}

int mpm_tool_distance_cols(MpmHandle* h) { return h ? h->n_cols : 0; }

int mpm_tool_distance(MpmHandle* h, const void* state, const double* pose, void* out, void* stream) {
  if (!h) return fail(nullptr, MPM_E_INVALID, "mpm_tool_distance: NULL handle");
  if (h->n_tools == 0) return MPM_OK;
  MPM_TRY(check_device(h));
  MPM_TRY(check_aligned(h, state, "state"));
  MPM_TRY(check_aligned(h, pose, "pose"));
  MPM_TRY(check_aligned(h, out, "out"));
  mpm::LaunchCtx L = ctx(h, stream);
  cudaError_t e = h->p.precision == MPM_PREC_FP64
                      ? mpm::launch_tool_distance<double>(L, h->d_col_off, h->n_cols, (const double*)state, pose,
                                                          (double*)out)
                      : mpm::launch_tool_distance<float>(L, h->d_col_off, h->n_cols, (const float*)state, pose,
                                                         (float*)out);
  return e == cudaSuccess ? MPM_OK : cuda_fail(h, e, "mpm_tool_distance");
}

int mpm_tool_distance_bwd(MpmHandle* h, const void* state, const double* pose, const void* g_out, void* g_state,
                          double* g_pose, void* stream) {
  if (!h) return fail(nullptr, MPM_E_INVALID, "mpm_tool_distance_bwd: NULL handle");
  if (h->n_tools == 0) return MPM_OK;
  MPM_TRY(check_device(h));
  MPM_TRY(check_aligned(h, state, "state"));
  MPM_TRY(check_aligned(h, pose, "pose"));
  MPM_TRY(check_aligned(h, g_out, "g_out"));
  MPM_TRY(check_aligned(h, g_state, "g_state"));
  MPM_TRY(check_aligned(h, g_pose, "g_pose"));
  mpm::LaunchCtx L = ctx(h, stream);
  cudaError_t e = h->p.precision == MPM_PREC_FP64
                      ? mpm::launch_tool_distance_bwd<double>(L, h->d_col_off, (const double*)state, pose,
                                                              (const double*)g_out, (double*)g_state, g_pose)
                      : mpm::launch_tool_distance_bwd<float>(L, h->d_col_off, (const float*)state, pose,
                                                             (const float*)g_out, (float*)g_state, g_pose);
  return e == cudaSuccess ? MPM_OK : cuda_fail(h, e, "mpm_tool_distance_bwd");
}

int mpm_status(MpmHandle* h, uint32_t* status, int32_t clear, void* stream) {
  if (!h || !status) return fail(h, MPM_E_INVALID, "mpm_status: NULL argument");
  MPM_TRY(check_device(h));
  unsigned int v = 0;
  cudaError_t e = cudaMemcpyAsync(&v, h->d_status, sizeof(v), cudaMemcpyDeviceToHost, (cudaStream_t)stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e == cudaSuccess && clear) e = cudaMemsetAsync(h->d_status, 0, sizeof(unsigned int), (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(h, e, "mpm_status");
  *status = v;
  return MPM_OK;
}

int mpm_last_error(MpmHandle* h, char* buf, size_t len) {
  if (!buf || len == 0) return MPM_E_INVALID;
  std::string msg;
  if (h) {
    msg = h->err;
  } else {
    std::lock_guard<std::mutex> lk(g_err_mu);
    msg = g_create_err;
  }
  std::snprintf(buf, len, "%s", msg.c_str());
  return MPM_OK;
}

int64_t mpm_launch_count(MpmHandle* h) { return h ? h->launches : 0; }

int mpm_profile_enable(MpmHandle* h, int32_t enable) {
  if (!h) return fail(nullptr, MPM_E_INVALID, "mpm_profile_enable: NULL handle");
  MPM_TRY(check_device(h));
  const int kPairs = 1 << 16;
  if (enable && h->events.empty()) {
    h->events.resize(2 * kPairs);
    for (auto& e : h->events) {
      cudaError_t err = cudaEventCreate(&e);
      if (err != cudaSuccess) return cuda_fail(h, err, "mpm_profile_enable: cudaEventCreate");
    }
    h->recs.resize(kPairs);
  }
  h->prof.on = enable != 0;
  h->prof.pool = h->events.data();
  h->prof.pool_cap = (int)h->events.size();
  h->prof.recs = h->recs.data();
  h->prof.cap = (int)h->recs.size();
  return MPM_OK;
}

int mpm_profile_read(MpmHandle* h, double* ms, int64_t* count) {
  if (!h || !ms || !count) return fail(h, MPM_E_INVALID, "mpm_profile_read: NULL argument");
  MPM_TRY(check_device(h));
  for (int k = 0; k < MPM_K_COUNT; ++k) {
    ms[k] = 0.0;
    count[k] = 0;
  }
  for (int i = 0; i < h->prof.n; ++i) {
    const mpm::Profiler::Rec& r = h->prof.recs[i];
    cudaError_t e = cudaEventSynchronize(r.b);
    float t = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, r.a, r.b);
    if (e != cudaSuccess) return cuda_fail(h, e, "mpm_profile_read");
    if (r.kind >= 0 && r.kind < MPM_K_COUNT) {
      ms[r.kind] += t;
      count[r.kind] += 1;
    }
  }
  h->prof.n = 0;
  h->prof.pool_n = 0;
  return MPM_OK;
}

}  // extern "C"
