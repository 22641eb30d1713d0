// Loss kernels of plb/engine/losses/loss.py beyond the density L1 term:
//   - target-SDF propagation: update_target_sdf / update_target (loss.py:105-134);
//   - SDF loss: compute_sdf_loss_kernel (loss.py:178-180);
//   - IoU: iou_kernel (loss.py:294-308);
//   - hard contact distance: compute_contact_distance_kernel (loss.py:151-155),
//     started from 100000 as compute_loss_kernel does (loss.py:243-244), with an adjoint.
// Dense grids here are real[n_scenes][n_grid^3], node (i,j,k) at (i*n+j)*n+k,
// the C order of the reference's (n,n,n) fields.
#include <climits>

#include "mpm_kernels.cuh"
#include "mpm_launch.h"

namespace mpm {

template <typename T>
Consts<T> make_consts(const LaunchCtx& L);  // mpm_fwd.cu

static inline unsigned blocks_for(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// products and sums without FMA contraction, so the device rounds every
// operation as the oracle does
MPM_DI float mul_rn(float a, float b) { return __fmul_rn(a, b); }
MPM_DI double mul_rn(double a, double b) { return __dmul_rn(a, b); }
MPM_DI float add_rn(float a, float b) { return __fadd_rn(a, b); }
MPM_DI double add_rn(double a, double b) { return __dadd_rn(a, b); }

// ---------------------------------------------------------------------------
// target SDF: one Jacobi iteration of update_target_sdf per launch
// ---------------------------------------------------------------------------
// A node whose target density exceeds 1e-4 gets sdf 0 and itself as nearest
// point.  Any other node takes, over the offsets (-3..2)^3 \ {0} in the
// reference's ndrange order, the first strict minimum of
// sqrt(|grid_pos - nearest_copy[v]|^2 + 1e-8) among in-grid neighbours with
// sdf_copy[v] < 1000, else sdf 1000.  One CTA computes an 8^3 tile of one
// scene from a 13^3 shared-memory copy of (sdf, nearest) around it.
//
// The square root is taken only for candidates whose squared distance is
// below the best one so far: sqrt(dd + 1e-8) is monotone in dd, so a
// candidate with dd >= best_dd cannot have a strictly smaller distance and
// skipping it leaves the reference's result unchanged.
//
// flags[3] detect convergence: launch t reads flags[(t-1)%3] (set by launch
// t-1 when any node changed), sets flags[t%3] on change and clears
// flags[(t+1)%3] for launch t+1.  Once an iteration changes nothing, every
// later one would reproduce the same values, so those launches return at once.
constexpr int TS_TILE = 8;
constexpr int TS_SPAN = TS_TILE + 5;  // halo of 3 below and 2 above
constexpr int TS_N = TS_SPAN * TS_SPAN * TS_SPAN;
constexpr double TS_INF = 1000.0;

template <typename T>
__global__ void __launch_bounds__(512) k_target_sdf(int n, int64_t G, int tiles, const T* __restrict__ dens,
                                                    const T* sdf_c, const T* near_c, T* __restrict__ sdf_o,
                                                    T* __restrict__ near_o, T* sdf_o2, T* near_o2, double dx,
                                                    int* __restrict__ flags, int iter) {
  extern __shared__ __align__(16) unsigned char ts_smem[];
  T* s_sdf = reinterpret_cast<T*>(ts_smem);
  T* s_near = s_sdf + TS_N;  // [TS_N][3]
  if (iter > 0 && flags[(iter - 1) % 3] == 0) {
    if (blockIdx.x == 0 && threadIdx.x == 0) flags[(iter + 1) % 3] = 0;
    return;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) flags[(iter + 1) % 3] = 0;
  const int t3 = tiles * tiles * tiles;
  const int scene = blockIdx.x / t3;
  const int tb = blockIdx.x % t3;
  const int o0 = (tb / (tiles * tiles)) * TS_TILE, o1 = ((tb / tiles) % tiles) * TS_TILE, o2 = (tb % tiles) * TS_TILE;
  const int64_t base = (int64_t)scene * G;
  const T inf = T(TS_INF);
  if (iter > 0) {
    for (int s = threadIdx.x; s < TS_N; s += blockDim.x) {
      const int a = o0 - 3 + s / (TS_SPAN * TS_SPAN), b = o1 - 3 + (s / TS_SPAN) % TS_SPAN, c = o2 - 3 + s % TS_SPAN;
      T v = inf, q0 = T(0), q1 = T(0), q2 = T(0);
      if (a >= 0 && a < n && b >= 0 && b < n && c >= 0 && c < n) {
        const int64_t id = base + ((int64_t)a * n + b) * n + c;
        v = sdf_c[id];
        q0 = near_c[3 * id];
        q1 = near_c[3 * id + 1];
        q2 = near_c[3 * id + 2];
      }
      s_sdf[s] = v;
      s_near[3 * s] = q0;
      s_near[3 * s + 1] = q1;
      s_near[3 * s + 2] = q2;
    }
    __syncthreads();
  }
  const int l0 = threadIdx.x / 64, l1 = (threadIdx.x / 8) % 8, l2 = threadIdx.x % 8;
  const int i0 = o0 + l0, i1 = o1 + l1, i2 = o2 + l2;
  if (i0 >= n || i1 >= n || i2 >= n) return;
  const int64_t id = base + ((int64_t)i0 * n + i1) * n + i2;
  const T gp[3] = {T(double(i0) * dx), T(double(i1) * dx), T(double(i2) * dx)};
  T best = inf, bn[3] = {T(0), T(0), T(0)};
  if (double(dens[id]) > 1e-4) {
    best = T(0);
    bn[0] = gp[0];
    bn[1] = gp[1];
    bn[2] = gp[2];
  } else if (iter > 0) {
    T bdd = T(1e30);
    for (int a = 0; a < 6; ++a)
      for (int b = 0; b < 6; ++b)
#pragma unroll 6
        for (int c = 0; c < 6; ++c) {
          if (a == 3 && b == 3 && c == 3) continue;
          const int s = ((l0 + a) * TS_SPAN + (l1 + b)) * TS_SPAN + (l2 + c);
          if (!(s_sdf[s] < inf)) continue;
          const T d0 = gp[0] - s_near[3 * s], d1 = gp[1] - s_near[3 * s + 1], d2 = gp[2] - s_near[3 * s + 2];
          const T dd = add_rn(add_rn(mul_rn(d0, d0), mul_rn(d1, d1)), mul_rn(d2, d2));
          if (dd < bdd) {
            const T dist = sqrt(add_rn(dd, T(1e-8)));
            if (dist < best) {
              best = dist;
              bdd = dd;
              bn[0] = s_near[3 * s];
              bn[1] = s_near[3 * s + 1];
              bn[2] = s_near[3 * s + 2];
            }
          }
        }
  }
  sdf_o[id] = best;
  near_o[3 * id] = bn[0];
  near_o[3 * id + 1] = bn[1];
  near_o[3 * id + 2] = bn[2];
  if (iter == 0) {  // both buffers hold iteration 0, so an early exit at launch 1 leaves no stale buffer
    sdf_o2[id] = best;
    near_o2[3 * id] = bn[0];
    near_o2[3 * id + 1] = bn[1];
    near_o2[3 * id + 2] = bn[2];
  }
  bool changed;
  if (iter == 0) {
    changed = best < inf;
  } else {
    const int s = ((l0 + 3) * TS_SPAN + (l1 + 3)) * TS_SPAN + (l2 + 3);
    changed = !(best == s_sdf[s]) || !(bn[0] == s_near[3 * s] && bn[1] == s_near[3 * s + 1] &&
                                      bn[2] == s_near[3 * s + 2]);
  }
  if (changed) flags[iter % 3] = 1;
}

template <typename T>
cudaError_t launch_target_sdf(const LaunchCtx& L, int* flags, const T* dens, T* sdf, T* near, T* work,
                              int n_iters) {
  const int n = L.p->n_grid, S = L.p->n_scenes;
  if (n_iters <= 0 || S <= 0) return cudaSuccess;
  const int tiles = (n + TS_TILE - 1) / TS_TILE;
  const size_t smem = (size_t)TS_N * 4 * sizeof(T);
  cudaError_t e = cudaFuncSetAttribute(k_target_sdf<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  MPM_MEMSET(L, flags, 3 * sizeof(int));
  T* w_sdf = work;
  T* w_near = work + (int64_t)S * L.G;
  for (int t = 0; t < n_iters; ++t) {
    // the last iteration writes the caller's arrays
    const bool to_out = ((n_iters - 1 - t) % 2) == 0;
    T* rs = to_out ? w_sdf : sdf;
    T* rn = to_out ? w_near : near;
    T* ws = to_out ? sdf : w_sdf;
    T* wn = to_out ? near : w_near;
    int _slot = prof_begin(L.prof, L.stream);
    k_target_sdf<T><<<(unsigned)(S * tiles * tiles * tiles), 512, smem, L.stream>>>(
        n, L.G, tiles, dens, rs, rn, ws, wn, rs, rn, (double)L.p->dx, flags, t);
    prof_end(L.prof, _slot, MPM_K_OTHER, L.stream);
    ++*L.launches;
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// SDF loss and IoU: one CTA per scene, fixed-order FP64 reductions
// ---------------------------------------------------------------------------
constexpr int RED_THREADS = 512;

MPM_DI double block_sum(double v, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
  return s;  // valid in thread 0
}
MPM_DI double block_max(double v, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = red[0];
  if (threadIdx.x == 0)
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) s = fmax(s, red[w]);
  return s;  // valid in thread 0
}

// loss[s] = weight * sum_I sdf*m; g_grid_m += weight * sdf
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_sdf_loss(int64_t G, const T* __restrict__ gm,
                                                          const T* __restrict__ sdf, double weight,
                                                          double* __restrict__ loss, T* __restrict__ ggm) {
  __shared__ double red[32];
  const int64_t base = (int64_t)blockIdx.x * G;
  double acc = 0.0;
  for (int64_t i = threadIdx.x; i < G; i += blockDim.x) {
    const T sd = sdf[base + i];
    acc += double(sd * gm[base + i]);
    if (ggm) ggm[base + i] += T(weight) * sd;
  }
  const double s = block_sum(acc, red);
  if (threadIdx.x == 0) loss[blockIdx.x] = weight * s;
}

template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_iou(int64_t G, const T* __restrict__ gm, const T* __restrict__ tgt,
                                                     double* __restrict__ iou) {
  __shared__ double red[32];
  const int64_t base = (int64_t)blockIdx.x * G;
  // the maxima start at 0 as the reference's atomic_max accumulators do
  double ma = 0.0, mb = 0.0, I = 0.0, Ua = 0.0, Ub = 0.0;
  for (int64_t i = threadIdx.x; i < G; i += blockDim.x) {
    const double a = double(gm[base + i]), b = double(tgt[base + i]);
    ma = fmax(ma, a);
    mb = fmax(mb, b);
    I += a * b;
    Ua += a;
    Ub += b;
  }
  ma = block_max(ma, red);
  mb = block_max(mb, red);
  I = block_sum(I, red);
  Ua = block_sum(Ua, red);
  Ub = block_sum(Ub, red);
  if (threadIdx.x == 0) {
    const double In = I / ma / mb;
    const double U = Ua / ma + Ub / mb;
    iou[blockIdx.x] = In / (U - In);
  }
}

template <typename T>
cudaError_t launch_sdf_loss(const LaunchCtx& L, const T* gm, const T* sdf, double weight, double* loss, T* ggm) {
  if (L.p->n_scenes > 0)
    MPM_LAUNCH(L, MPM_K_OTHER, k_sdf_loss<T>, (unsigned)L.p->n_scenes, RED_THREADS, L.G, gm, sdf, weight, loss,
               ggm);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_iou(const LaunchCtx& L, const T* gm, const T* tgt, double* iou) {
  if (L.p->n_scenes > 0)
    MPM_LAUNCH(L, MPM_K_OTHER, k_iou<T>, (unsigned)L.p->n_scenes, RED_THREADS, L.G, gm, tgt, iou);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// hard contact distance: min over particles of max(sdf, 0) per movable tool
// ---------------------------------------------------------------------------
// The minimum is an atomicMin on the bit pattern of the non-negative FP64
// distance (which orders like the value), kept in min_dist itself; a second
// pass takes the lowest particle index attaining it.
template <typename T>
MPM_DI double contact_d(const MpmToolDesc& d, const double* pose, const T* x) {
  Tool<T> tl;
  Pose<T> P;
  to_tool(d, tl);
  to_pose(pose, P);
  const T sd = tool_sdf(tl, P, x);
  return (T(0) < sd) ? double(sd) : 0.0;
}

__global__ void k_contact_min_init(int n_tools, double* __restrict__ min_dist, int64_t* __restrict__ argmin) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tools) return;
  min_dist[t] = 100000.0;
  argmin[t] = -1;  // all bits set: the largest value for the unsigned atomicMin
}

template <typename T>
__global__ void __launch_bounds__(128) k_contact_min(Consts<T> c, const T* __restrict__ st,
                                                     const int* __restrict__ pscene,
                                                     const MpmToolDesc* __restrict__ tools,
                                                     const int* __restrict__ tool_off,
                                                     const double* __restrict__ pose, double* __restrict__ min_dist) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= c.n_particles) return;
  const int sc = pscene[p];
  T x[3];
  load_row(st, c.ld, p, 0, 3, x);
  for (int t = tool_off[sc]; t < tool_off[sc + 1]; ++t) {
    if (tools[t].action_dim <= 0) continue;
    const double d = contact_d<T>(tools[t], pose + 8 * t, x);
    atomicMin(reinterpret_cast<unsigned long long*>(min_dist + t), (unsigned long long)__double_as_longlong(d));
  }
}

template <typename T>
__global__ void __launch_bounds__(128) k_contact_argmin(Consts<T> c, const T* __restrict__ st,
                                                        const int* __restrict__ pscene,
                                                        const MpmToolDesc* __restrict__ tools,
                                                        const int* __restrict__ tool_off,
                                                        const double* __restrict__ pose,
                                                        const double* __restrict__ min_dist,
                                                        int64_t* __restrict__ argmin) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= c.n_particles) return;
  const int sc = pscene[p];
  T x[3];
  load_row(st, c.ld, p, 0, 3, x);
  for (int t = tool_off[sc]; t < tool_off[sc + 1]; ++t) {
    if (tools[t].action_dim <= 0) continue;
    const double d = contact_d<T>(tools[t], pose + 8 * t, x);
    if (d == min_dist[t]) atomicMin(reinterpret_cast<unsigned long long*>(argmin + t), (unsigned long long)p);
  }
}

__global__ void k_contact_min_finish(const MpmToolDesc* __restrict__ tools, int n_tools,
                                     double* __restrict__ min_dist) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n_tools && tools[t].action_dim <= 0) min_dist[t] = 0.0;
}

template <typename T>
cudaError_t launch_contact_min(const LaunchCtx& L, int n_tools, const T* st, const double* pose, double* min_dist,
                               int64_t* argmin) {
  Consts<T> c = make_consts<T>(L);
  MPM_LAUNCH(L, MPM_K_OTHER, k_contact_min_init, blocks_for(n_tools, 64), 64, n_tools, min_dist, argmin);
  if (c.n_particles > 0) {
    MPM_LAUNCH(L, MPM_K_OTHER, k_contact_min<T>, blocks_for(c.n_particles, 128), 128, c, st, L.pscene, L.tools,
               L.tool_off, pose, min_dist);
    MPM_LAUNCH(L, MPM_K_OTHER, k_contact_argmin<T>, blocks_for(c.n_particles, 128), 128, c, st, L.pscene, L.tools,
               L.tool_off, pose, min_dist, argmin);
  }
  MPM_LAUNCH(L, MPM_K_OTHER, k_contact_min_finish, blocks_for(n_tools, 64), 64, L.tools, n_tools, min_dist);
  return cudaGetLastError();
}

// adjoint: d min / d x_argmin = d max(sdf,0) / dx, zero when sdf <= 0
template <typename T>
__global__ void k_contact_min_adj(Consts<T> c, const T* __restrict__ st, const MpmToolDesc* __restrict__ tools,
                                  int n_tools, const double* __restrict__ pose, const int64_t* __restrict__ argmin,
                                  const double* __restrict__ g_min, T* __restrict__ gst,
                                  double* __restrict__ g_pose) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tools) return;
  const int64_t p = argmin[t];
  if (tools[t].action_dim <= 0 || p < 0 || p >= c.n_particles || g_min[t] == 0.0) return;
  T x[3];
  load_row(st, c.ld, p, 0, 3, x);
  Tool<T> tl;
  Pose<T> P;
  to_tool(tools[t], tl);
  to_pose(pose + 8 * t, P);
  if (!(T(0) < tool_sdf(tl, P, x))) return;
  T gx[3] = {T(0), T(0), T(0)};
  PoseGrad<T> gP;
  gP.zero();
  tool_sdf_vjp(tl, P, x, T(g_min[t]), gx, gP);
  for (int k = 0; k < 3; ++k) atomicAdd(gst + (int64_t)k * c.ld + p, gx[k]);
  for (int k = 0; k < 3; ++k) g_pose[8 * t + k] += double(gP.pos[k]);
  for (int k = 0; k < 4; ++k) g_pose[8 * t + 3 + k] += double(gP.rot[k]);
  g_pose[8 * t + 7] += double(gP.gap);
}

template <typename T>
cudaError_t launch_contact_min_bwd(const LaunchCtx& L, int n_tools, const T* st, const double* pose,
                                   const int64_t* argmin, const double* g_min, T* gst, double* g_pose) {
  Consts<T> c = make_consts<T>(L);
  MPM_LAUNCH(L, MPM_K_OTHER, k_contact_min_adj<T>, blocks_for(n_tools, 64), 64, c, st, L.tools, n_tools, pose,
             argmin, g_min, gst, g_pose);
  return cudaGetLastError();
}

#define MPM_INST_LOSS(T)                                                                                       \
  template cudaError_t launch_target_sdf<T>(const LaunchCtx&, int*, const T*, T*, T*, T*, int);                \
  template cudaError_t launch_sdf_loss<T>(const LaunchCtx&, const T*, const T*, double, double*, T*);          \
  template cudaError_t launch_iou<T>(const LaunchCtx&, const T*, const T*, double*);                          \
  template cudaError_t launch_contact_min<T>(const LaunchCtx&, int, const T*, const double*, double*, int64_t*); \
  template cudaError_t launch_contact_min_bwd<T>(const LaunchCtx&, int, const T*, const double*, const int64_t*, \
                                                 const double*, T*, double*);
MPM_INST_LOSS(float)
MPM_INST_LOSS(double)

}  // namespace mpm
