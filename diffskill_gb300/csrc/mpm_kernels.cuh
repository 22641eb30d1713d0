// Kernels of the differentiable MLS-MPM substep, templated on
//   T  : particle state and grid precision (float or double)
//   TS : precision of F_tmp, the SVD, the von Mises return map, the stress
//        and their adjoints (float, or double for the FP32_SVD64 mode).
//
// Forward  (MPMSimulator.substep, plb/engine/mpm_simulator.py:307-323):
//   k_p2g      compute_F_tmp + svd + p2g      (122-129, 166-225)
//   k_grid_op  grid_op + Primitive.collide    (231-262, primive_base.py:96-120)
//   k_g2p      g2p                            (265-284)
// Adjoint  (MPMSimulator.substep_grad, 325-345), after recomputing the grid:
//   k_g2p_adj      g2p.grad            scatter into the grid-velocity adjoint
//   k_grid_op_adj  grid_op.grad        per node, tool-pose gradients warp-summed, FP64 atomics
//   k_p2g_adj      p2g.grad + svd_grad + compute_F_tmp.grad (gather)
//
// Particle state is component-major: row k of a frame is st[k*ld + p].
//
// Sparse grid: the scratch grids of a substep are stored block-contiguous
// (blocks of 4x4x4 nodes, 64 nodes = 1 KiB in FP32 per block).  Each substep
// marks the blocks that particle stencils touch (k_mark_or_restore), compacts
// them into a device-side list and clears only those (k_compact_clear), and
// runs grid_op / grid_op.grad over that list with
// grid-stride loops (no host round trip; capturable in a CUDA graph).  Nodes
// outside the list hold no mass, so grid_op leaves them at zero exactly as the
// dense reference does; g2p and p2g.grad only read nodes inside the list.
#pragma once
#include "../../include/mpm_gb300.h"
#include "mpm_math.cuh"
#include "mpm_svd.cuh"
#include "mpm_tools.cuh"

namespace mpm {

// grid node: (mv or v).xyz, m
template <typename T>
struct alignas(4 * sizeof(T)) Node {
  T x, y, z, w;
};

template <typename T>
struct Consts {
  int n_grid;
  int n_scenes;
  int64_t n_particles;
  int64_t ld;
  int64_t G;    // n_grid^3
  int nb;       // blocks per axis (n_grid / 4)
  int64_t NB3;  // blocks per scene
  T dx, inv_dx, dt, p_mass, p_vol;
  T mu, lam, yield_stress;
  T ks;      // -dt * p_vol * 4 * inv_dx^2 (mpm_simulator.py:214)
  T gdt[3];  // dt * gravity * 30 (mpm_simulator.py:235)
  T ground_friction;
  T x_lo, x_hi;  // g2p clamp bounds (mpm_simulator.py:283)
  unsigned int* status;
};

MPM_DI void atomic_add_node(Node<float>* n, float a, float b, float c, float d) {
  atomicAdd(reinterpret_cast<float4*>(n), make_float4(a, b, c, d));
}
MPM_DI void atomic_add_node(Node<double>* n, double a, double b, double c, double d) {
  atomicAdd(&n->x, a);
  atomicAdd(&n->y, b);
  atomicAdd(&n->z, c);
  atomicAdd(&n->w, d);
}
MPM_DI void atomic_add_node3(Node<float>* n, float a, float b, float c) {
  atomicAdd(reinterpret_cast<float4*>(n), make_float4(a, b, c, 0.f));
}
MPM_DI void atomic_add_node3(Node<double>* n, double a, double b, double c) {
  atomicAdd(&n->x, a);
  atomicAdd(&n->y, b);
  atomicAdd(&n->z, c);
}

// L2 prefetch of the line holding p (no register, no wait)
MPM_DI void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// Programmatic dependent launch (griddepcontrol).  A kernel launched with
// programmatic stream serialization may start while the kernel before it in
// the stream is still running: pdl_wait() returns once that kernel has
// completed and its writes are visible (at once after a plain launch), so a
// thread reads nothing that kernel writes, and writes nothing it reads,
// before its pdl_wait().  pdl_trigger() lets the CTAs of the dependent kernel
// launch from then on (they take SMs this kernel's tail leaves idle).
MPM_DI void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
MPM_DI void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// quadratic B-spline stencil (mpm_simulator.py:201-204); base truncates like
// ti.cast(int)
template <typename T>
struct Stencil {
  int base[3];
  T fx[3];
  T w[3][3];  // w[k][d]
};
template <typename T>
MPM_DI bool make_stencil(const Consts<T>& c, const T* x, Stencil<T>& s) {
  bool ok = true;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    T t = x[d] * c.inv_dx - T(0.5);
    s.base[d] = (int)t;
    T f = x[d] * c.inv_dx - T(s.base[d]);
    s.fx[d] = f;
    s.w[0][d] = T(0.5) * (T(1.5) - f) * (T(1.5) - f);
    s.w[1][d] = T(0.75) - (f - T(1)) * (f - T(1));
    s.w[2][d] = T(0.5) * (f - T(0.5)) * (f - T(0.5));
    ok = ok && (t > T(-1)) && s.base[d] >= 0 && s.base[d] + 2 < c.n_grid;
  }
  return ok;
}
template <typename T>
MPM_DI T dweight(const Stencil<T>& s, int k, int d) {
  T f = s.fx[d];
  return k == 0 ? -(T(1.5) - f) : (k == 1 ? T(-2) * (f - T(1)) : (f - T(0.5)));
}
template <typename T>
MPM_DI int64_t node_of(const Consts<T>& c, const Stencil<T>& s, int ox, int oy, int oz) {
  return ((int64_t)(s.base[0] + ox) * c.n_grid + (s.base[1] + oy)) * c.n_grid + (s.base[2] + oz);
}

// Offsets, within one scene's block-contiguous grid, of the stencil nodes
// base+o per axis: node (i,j,k) -> ((bi*nb + bj)*nb + bk)*64 + (li*16 + lj*4 + lk)
struct StencilAddr {
  int ax[3], ay[3], az[3];
  MPM_DI int at(int ox, int oy, int oz) const { return ax[ox] + ay[oy] + az[oz]; }
};
template <typename T>
MPM_DI StencilAddr stencil_addr(const Consts<T>& c, const Stencil<T>& s) {
  StencilAddr a;
  const int nb = c.nb;
#pragma unroll
  for (int o = 0; o < 3; ++o) {
    const int i = s.base[0] + o, j = s.base[1] + o, k = s.base[2] + o;
    a.ax[o] = ((i >> 2) * nb * nb << 6) + ((i & 3) << 4);
    a.ay[o] = ((j >> 2) * nb << 6) + ((j & 3) << 2);
    a.az[o] = ((k >> 2) << 6) + (k & 3);
  }
  return a;
}
// grid coordinates of node l (0..63) of global block gb (= scene*NB3 + local block)
template <typename T>
MPM_DI int block_node(const Consts<T>& c, int64_t gb, int l, int* I) {
  const int scene = (int)(gb / c.NB3);
  const int64_t lb = gb - (int64_t)scene * c.NB3;
  const int nb = c.nb;
  I[0] = (int)(lb / ((int64_t)nb * nb)) * 4 + (l >> 4);
  I[1] = (int)((lb / nb) % nb) * 4 + ((l >> 2) & 3);
  I[2] = (int)(lb % nb) * 4 + (l & 3);
  return scene;
}

// Warp-level segmented reduction of the scatter.  Particles are sorted by
// base cell, so lanes with equal key (scene, base cell) are contiguous and
// scatter into the same 27 nodes: an inclusive segmented scan leaves each
// segment's sum in its last lane, which alone issues the atomic.  Lanes with a
// unique key (out of range, out of grid) form single-lane segments.
struct WarpSeg {
  int start;  // first lane of this lane's segment
  bool tail;  // this lane ends its segment
  int steps;  // doubling steps that cover the longest segment (warp-uniform)
};
MPM_DI WarpSeg warp_segments(long long key) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const long long prev = __shfl_up_sync(full, key, 1);
  const bool head = lane == 0 || prev != key;
  const unsigned heads = __ballot_sync(full, head);
  WarpSeg g;
  g.start = 31 - __clz(heads & (full >> (31 - lane)));
  g.tail = lane == 31 || ((heads >> (lane + 1)) & 1u);
  const unsigned run = __reduce_max_sync(full, (unsigned)(lane - g.start + 1));
  g.steps = run <= 1 ? 0 : 32 - __clz(run - 1);
  return g;
}
template <typename T>
MPM_DI T seg_scan(T v, const WarpSeg& g) {
  const int lane = threadIdx.x & 31;
  for (int i = 0, d = 1; i < g.steps; ++i, d <<= 1) {
    const T t = __shfl_up_sync(0xffffffffu, v, d);
    if (lane - d >= g.start) v += t;
  }
  return v;
}
// Segment ends of a warp for the slab scatter: bit r of `tails` is set when
// lane r ends its run of equal keys, bit r of `emit` when that run is in the
// grid (out-of-grid lanes carry unique keys, so they are runs of one).
MPM_DI void warp_tails(long long key, bool ok, unsigned& tails, unsigned& emit) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const long long next = __shfl_down_sync(full, key, 1);
  const bool tail = lane == 31 || next != key;
  tails = __ballot_sync(full, tail);
  emit = __ballot_sync(full, tail && ok);
}

// FP32 slab scatter.  The 27-node stencil is scattered one ox slab (9 nodes)
// at a time: every lane writes its 9 node values into row `lane` of v, then
// lanes 0..26 read the table by columns, lane = g + 3 j summing column j over
// rows [11 g, 11 g + 11).  Each run of equal keys closed inside a row group
// issues one red.global.add.v4.f32 per node; the run still open at the end of
// a group is carried into the next group by two shuffles.  This replaces a
// shuffle scan of 4 values x 27 nodes x up to 5 steps per lane with 27
// shared-memory stores, 11 loads per slab and 8 shuffles per slab, and keeps
// one atomic per (run, node).  Row stride 9 x 16 B: the stores (lane l, slot
// 9 l + n) and the loads (slot 99 g + 9 i + j, i.e. 3 g + i + j mod 8 with
// lane = g + 3 j) fall in distinct 16-byte bank groups within each quarter
// warp.
struct SlabStage {
  float4 v[33][9];  // row 32: read, never used (the open run of group 2 after row 31)
  Node<float>* base[32];  // grid of the row's scene + ax[ox] of the row's base cell
  int ay[32][3], az[32][3];
};
// Packed FP32 pairs (add/mul/fma .f32x2): one instruction for two lanes of
// arithmetic, each rounded as the scalar operation would be
MPM_DI unsigned long long f2_bits(float2 a) { return *reinterpret_cast<unsigned long long*>(&a); }
MPM_DI float2 f2_of(unsigned long long b) { return *reinterpret_cast<float2*>(&b); }
MPM_DI float2 add2(float2 a, float2 b) {
  unsigned long long d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_bits(a)), "l"(f2_bits(b)));
  return f2_of(d);
}
MPM_DI float2 mul2(float2 a, float2 b) {
  unsigned long long d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_bits(a)), "l"(f2_bits(b)));
  return f2_of(d);
}
// a += b, in two packed pair additions or four scalar ones (measured: the
// packed form helps p2g and slows g2p.grad, whose fourth lane is zero)
template <bool Packed = false>
MPM_DI void f4_add(float4& a, const float4& b) {
  if constexpr (Packed) {
    const float2 lo = add2(make_float2(a.x, a.y), make_float2(b.x, b.y));
    const float2 hi = add2(make_float2(a.z, a.w), make_float2(b.z, b.w));
    a = make_float4(lo.x, lo.y, hi.x, hi.y);
  } else {
    a.x += b.x;
    a.y += b.y;
    a.z += b.z;
    a.w += b.w;
  }
}
MPM_DI float4 f4_shfl_up(const float4& a, int d) {
  return make_float4(__shfl_up_sync(0xffffffffu, a.x, d), __shfl_up_sync(0xffffffffu, a.y, d),
                     __shfl_up_sync(0xffffffffu, a.z, d), __shfl_up_sync(0xffffffffu, a.w, d));
}
MPM_DI void slab_emit(const SlabStage& sb, int r, int oy, int oz, const float4& a) {
  atomicAdd(reinterpret_cast<float4*>(sb.base[r] + sb.ay[r][oy] + sb.az[r][oz]), a);
}
// call between two __syncwarp()s, after all lanes wrote their row of sb.v
template <bool Packed = false>
MPM_DI void slab_reduce(const SlabStage& sb, unsigned tails, unsigned emit) {
  const int lane = threadIdx.x & 31;
  // lanes 27..31 (g = 3) read lane 24's cells (a broadcast) and emit nothing
  const int g = lane < 27 ? lane % 3 : 3;
  const int j = lane < 27 ? lane / 3 : 8;
  const int oy = j / 3, oz = j - 3 * (j / 3);
  const int r0 = 11 * (g < 3 ? g : 0);
  const unsigned mine = g < 3 ? tails >> r0 : 0u;  // group 2: bit 10 (row 32) is 0
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f), head = acc;
  int head_row = -1;
#pragma unroll
  for (int i = 0; i < 11; ++i) {
    f4_add<Packed>(acc, sb.v[r0 + i][j]);
    if ((mine >> i) & 1u) {
      if (g > 0 && head_row < 0) {
        head = acc;  // closes a run that may have started in the group before
        head_row = r0 + i;
      } else if ((emit >> (r0 + i)) & 1u) {
        slab_emit(sb, r0 + i, oy, oz, acc);
      }
      acc = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
  // acc = the open run at the group's end; group 2 always closes (row 31)
  const float4 c1 = f4_shfl_up(acc, 1);  // group 1: open run of group 0
  float4 fwd = acc;
  if (g == 1 && head_row < 0) f4_add(fwd, c1);  // group 1 without a tail passes the run on
  const float4 c2 = f4_shfl_up(fwd, 1);          // group 2: open run of groups 0..1
  if (g >= 1 && g < 3 && head_row >= 0) {
    f4_add(head, g == 1 ? c1 : c2);
    if ((emit >> head_row) & 1u) slab_emit(sb, head_row, oy, oz, head);
  }
}

template <typename T>
MPM_DI void zero_stencil(Stencil<T>& s) {
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    s.base[d] = 0;
    s.fx[d] = T(1);
#pragma unroll
    for (int k = 0; k < 3; ++k) s.w[k][d] = T(0);
  }
}
// a[i] for a runtime i in 0..2 without local memory
template <typename T>
MPM_DI T sel3(T a0, T a1, T a2, int i) {
  return i == 0 ? a0 : (i == 1 ? a1 : a2);
}
template <typename T>
MPM_DI void add3(T& a0, T& a1, T& a2, int i, T v) {
  a0 += i == 0 ? v : T(0);
  a1 += i == 1 ? v : T(0);
  a2 += i == 2 ? v : T(0);
}

template <typename T>
MPM_DI long long cell_key(const Consts<T>& c, int scene, const Stencil<T>& s) {
  return (long long)scene * c.G + ((long long)s.base[0] * c.n_grid + s.base[1]) * c.n_grid + s.base[2];
}

// Loads issued before a kernel's pdl_wait() go to L2 (ld.global.cg): a
// dependent launch may start on an SM whose L1 still holds lines of an older
// content of the same buffer, and only the wait makes the earlier kernels'
// writes visible through L1.  L2 is coherent, and everything these loads read
// was written by kernels that completed before this one started.
template <typename T>
MPM_DI void load_row_cg(const T* __restrict__ st, int64_t ld, int64_t p, int r0, int n, T* out) {
#pragma unroll
  for (int k = 0; k < n; ++k) out[k] = __ldcg(st + (int64_t)(r0 + k) * ld + p);
}
template <typename T>
MPM_DI void load_row(const T* __restrict__ st, int64_t ld, int64_t p, int r0, int n, T* out) {
#pragma unroll
  for (int k = 0; k < n; ++k) out[k] = st[(int64_t)(r0 + k) * ld + p];
}
template <typename T>
MPM_DI void store_row(T* __restrict__ st, int64_t ld, int64_t p, int r0, int n, const T* in) {
#pragma unroll
  for (int k = 0; k < n; ++k) st[(int64_t)(r0 + k) * ld + p] = in[k];
}

// ---------------------------------------------------------------------------
// per-particle p2g math: F_tmp, SVD, von Mises, stress (mpm_simulator.py:
// 122-124, 127-129, 166-182, 205-215) in the precision S
// ---------------------------------------------------------------------------
template <typename S>
struct P2G {
  S U[9], s[3], V[9];
  S sm1[3];  // s - 1 (FP32: from the shifted SVD, exact as s -> 1)
  S sigc[3], ehat[3], nrm, dg, k, e[3];
  bool yield;
  S newF[9], J, R[9];
  S em1[3];  // singular values of newF minus 1 (e - 1 when yielding, else s - 1)
  S A[9];    // newF - R (FP32: U diag(e - 1) V^T, no cancellation)
};
template <typename S>
struct MatConsts {
  S dt, mu, lam, ys, ks, p_mass;
};
// affine = ks (2 mu A newF^T + lam J (J - 1) I) + p_mass C (mpm_simulator.py:213-215)
template <typename S>
MPM_DI void p2g_affine(const MatConsts<S>& m, const P2G<S>& P, S Jm1, const S* C, S* affine) {
  S st[9];
  mmT(P.A, P.newF, st);
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    S v = S(2) * m.mu * st[i];
    if (i % 4 == 0) v += m.lam * P.J * Jm1;
    affine[i] = m.ks * v + m.p_mass * C[i];
  }
}
// FP32 p2g math in terms of the displacement D = F_tmp - I.  The stress
// 2 mu (newF - R) newF^T + lam J (J - 1) I is a difference of numbers near 1
// (newF, R, J) when it is evaluated as written; in FP32 that cancellation
// leaves about 1e-7 / |strain| of relative error in every particle's stress
// (1e-4 at a strain of 1e-3), which then drives the trajectory apart from the
// FP64 one.  Here every small quantity is formed directly: D = G + dt C (I + G)
// with G = F - I (exact for F_ii in [0.5, 2]); the SVD of I + D from the
// shifted matrix (svd3_shifted) with s - 1; log(s) = log1p(s - 1); the
// projected singular values e - 1 = expm1(eps'); newF - R = U diag(e - 1) V^T;
// J - 1 = det(I + D) - 1 = tr D + (tr(D)^2 - tr(D^2)) / 2 + det D (elastic) or
// expm1(sum eps) (yield: the von Mises map keeps the volume).  The stored F
// of a yielding particle is formed as I + (D + U diag(e - s) V^T), its
// plastic correction e - s = s expm1(-k eps_hat) taken without cancellation,
// so it carries one FP32 rounding, as an elastic particle's I + D does.
// Mathematically the same function as the reference's (mpm_simulator.py:
// 122-129, 166-225).  The stress takes the SVD basis,
// (newF - R) newF^T = U diag((e - 1) e) U^T; new_F (may be null: the
// adjoint's recompute) receives the updated F.
MPM_DI void p2g_particle_f32(const MatConsts<float>& m, const float* C, const float* F, P2G<float>& P,
                             float* affine, float* new_F) {
  float G[9], CG[9], D[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) G[i] = F[i] - ((i % 4 == 0) ? 1.f : 0.f);
  mm(C, G, CG);
#pragma unroll
  for (int i = 0; i < 9; ++i) D[i] = G[i] + m.dt * (C[i] + CG[i]);
  svd3_shifted(D, P.U, P.s, P.sm1, P.V);
  float eps[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const bool above = 0.05f < P.s[i];
    P.sigc[i] = above ? P.s[i] : 0.05f;
    eps[i] = above ? log1p_strain(P.sm1[i]) : logf(0.05f);
  }
  const float esum = eps[0] + eps[1] + eps[2];
  const float mean = fast_div(esum, 3.f);
#pragma unroll
  for (int i = 0; i < 3; ++i) P.ehat[i] = eps[i] - mean;
  P.nrm = sqrtf(dot3(P.ehat, P.ehat) + 1e-8f);
  P.dg = P.nrm - fast_div(m.ys, 2.f * m.mu);
  P.yield = P.dg > 0.f;
  float* em1 = P.em1;
  float pc[3];  // e - s, the return map's change of the singular values
  if (P.yield) {
    P.k = fast_div(P.dg, P.nrm);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      em1[i] = expm1_strain(eps[i] - P.k * P.ehat[i]);
      P.e[i] = 1.f + em1[i];
      // both small and accurate to ~1e-7 of themselves: the difference keeps that accuracy
      pc[i] = 0.05f < P.s[i] ? em1[i] - P.sm1[i] : P.e[i] - P.s[i];
    }
  } else {
    P.k = 0.f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      P.e[i] = 1.f;
      em1[i] = P.sm1[i];
      pc[i] = 0.f;
    }
  }
  // J - 1: det(I + D) - 1 by its invariants; the return map keeps the volume,
  // unless a singular value sits at the 0.05 floor (then J = prod sigc)
  float Jm1;
  if (P.yield && !(0.05f < P.s[0] && 0.05f < P.s[1] && 0.05f < P.s[2])) {
    Jm1 = expm1f(esum);
  } else {
    const float tr = D[0] + D[4] + D[8];
    float D2 = 0.f;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) D2 += D[i * 3 + j] * D[j * 3 + i];
    Jm1 = tr + 0.5f * (tr * tr - D2) + det3(D);
  }
  P.J = 1.f + Jm1;
  // (newF - R) newF^T = U diag(e - 1) V^T V diag(e) U^T = U diag((e - 1) e) U^T
  float h[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) h[i] = em1[i] * (1.f + em1[i]);
  const float lj = m.lam * P.J * Jm1;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = i; j < 3; ++j) {
      float st = P.U[i * 3] * P.U[j * 3] * h[0] + P.U[i * 3 + 1] * P.U[j * 3 + 1] * h[1] +
                 P.U[i * 3 + 2] * P.U[j * 3 + 2] * h[2];
      st = 2.f * m.mu * st + (i == j ? lj : 0.f);
      affine[i * 3 + j] = m.ks * st + m.p_mass * C[i * 3 + j];
      if (j != i) affine[j * 3 + i] = m.ks * st + m.p_mass * C[j * 3 + i];
    }
  if (new_F) {
    if (P.yield) {
      float UP[9], corr[9];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int cc = 0; cc < 3; ++cc) UP[r * 3 + cc] = P.U[r * 3 + cc] * pc[cc];
      mmT(UP, P.V, corr);
#pragma unroll
      for (int i = 0; i < 9; ++i) new_F[i] = (D[i] + corr[i]) + ((i % 4 == 0) ? 1.f : 0.f);
    } else {
#pragma unroll
      for (int i = 0; i < 9; ++i) new_F[i] = D[i] + ((i % 4 == 0) ? 1.f : 0.f);  // F_tmp
    }
  }
}
// affine (the APIC matrix with the stress) and, when new_F is given, the
// updated F; P keeps what the adjoint needs
template <typename S>
MPM_DI void p2g_particle(const MatConsts<S>& m, const S* C, const S* F, P2G<S>& P, S* affine, S* new_F) {
  if constexpr (sizeof(S) == 4) {
    p2g_particle_f32(m, C, F, P, affine, new_F);
  } else {
    // FP64: the reference's order of operations
    S IC[9], Ftmp[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) IC[i] = m.dt * C[i] + ((i % 4 == 0) ? S(1) : S(0));
    mm(IC, F, Ftmp);
    svd3(Ftmp, P.U, P.s, P.V);
    S eps[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      P.sm1[i] = P.s[i] - S(1);
      P.sigc[i] = (S(0.05) < P.s[i]) ? P.s[i] : S(0.05);
      eps[i] = mlog(P.sigc[i]);
    }
    S mean = fast_div(eps[0] + eps[1] + eps[2], S(3));
#pragma unroll
    for (int i = 0; i < 3; ++i) P.ehat[i] = eps[i] - mean;
    P.nrm = msqrt(dot3(P.ehat, P.ehat) + S(1e-8));
    P.dg = P.nrm - fast_div(m.ys, S(2) * m.mu);
    P.yield = P.dg > S(0);
    if (P.yield) {
      P.k = fast_div(P.dg, P.nrm);
#pragma unroll
      for (int i = 0; i < 3; ++i) P.e[i] = mexp(eps[i] - P.k * P.ehat[i]);
      S UD[9];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int cc = 0; cc < 3; ++cc) UD[r * 3 + cc] = P.U[r * 3 + cc] * P.e[cc];
      mmT(UD, P.V, P.newF);
    } else {
      P.k = S(0);
#pragma unroll
      for (int i = 0; i < 3; ++i) P.e[i] = S(1);
#pragma unroll
      for (int i = 0; i < 9; ++i) P.newF[i] = Ftmp[i];
    }
    P.J = det3(P.newF);
    mmT(P.U, P.V, P.R);
#pragma unroll
    for (int i = 0; i < 9; ++i) P.A[i] = P.newF[i] - P.R[i];
#pragma unroll
    for (int i = 0; i < 3; ++i) P.em1[i] = (P.yield ? P.e[i] : P.s[i]) - S(1);
    p2g_affine(m, P, P.J - S(1), C, affine);
    if (new_F) {
#pragma unroll
      for (int i = 0; i < 9; ++i) new_F[i] = P.newF[i];
    }
  }
}
// gradient of the singular values through the return map (yield branch of
// compute_von_mises, mpm_simulator.py:166-180), from the diagonal of
// M_N = U^T g_newF V (d loss / d e_i = M_N,ii)
template <typename S>
MPM_DI void return_map_sigma_grad(const P2G<S>& P, const S* MN, S* gs) {
  S g_eps2[3], g_eps[3], g_ehat[3], g_k = S(0);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    g_eps2[i] = MN[i * 4] * P.e[i];
    g_eps[i] = g_eps2[i];
    g_k -= g_eps2[i] * P.ehat[i];
    g_ehat[i] = -P.k * g_eps2[i];
  }
  S g_nrm = -fast_div(g_k * P.dg, P.nrm * P.nrm) + fast_div(g_k, P.nrm);
#pragma unroll
  for (int i = 0; i < 3; ++i) g_ehat[i] += fast_div(g_nrm * P.ehat[i], P.nrm);
  S sh = fast_div(g_ehat[0] + g_ehat[1] + g_ehat[2], S(3));
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    g_eps[i] += g_ehat[i] - sh;
    gs[i] = (S(0.05) < P.s[i]) ? fast_div(g_eps[i], P.sigc[i]) : S(0);
  }
}

// FP32 adjoint of p2g_particle_f32 in the SVD basis.  With G = U^T g_raw U
// (g_raw = ks g_affine), e' = 1 + em1 the singular values of newF, and the
// stress's matrices written in the bases U, V:
//   U^T (g_raw newF) V   = G diag(e')        (the adjoint of A = newF - R)
//   U^T (g_raw^T A) V    = G^T diag(e' - 1)  (through the right factor newF^T)
//   U^T cof(newF) V      = J diag(1 / e')    (d det / d newF)
// M_R = U^T g_R V = -2 mu G diag(e') and M_N = U^T g_newF V need no newF, A
// or cofactor matrix.  The SVD part is svd3_bwd_factored_basis; the elastic
// branch's direct newF = F_tmp term joins it in the same basis, so one
// transform U Y V^T gives the gradient of F_tmp.
MPM_DI void p2g_particle_vjp_f32(const MatConsts<float>& m, const float* C, const float* F, const P2G<float>& P,
                                 const float* g_affine, const float* g_newF_in, float* g_C, float* g_F) {
  float G[9], t9[9], MR[9], MN[9];
  {
    float g_raw[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) g_raw[i] = m.ks * g_affine[i];
    mTm(P.U, g_raw, t9);
    mm(t9, P.U, G);
  }
  const float g_J = m.lam * (2.f * P.J - 1.f) * (G[0] + G[4] + G[8]);  // tr g_raw = tr G
  mTm(P.U, g_newF_in, t9);
  mm(t9, P.V, MN);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const float ej = 1.f + P.em1[j];
      const float a = 2.f * m.mu * G[i * 3 + j] * ej;
      MR[i * 3 + j] = -a;
      MN[i * 3 + j] += a + 2.f * m.mu * G[j * 3 + i] * P.em1[j] + (i == j ? fast_div(g_J * P.J, ej) : 0.f);
    }
  float gs[3] = {0.f, 0.f, 0.f}, Y[9];
  if (P.yield) return_map_sigma_grad(P, MN, gs);
  svd3_bwd_factored_basis(P.s, P.sm1, MR, MN, P.e, P.em1, 1.f - P.k, P.yield, gs, Y);
  if (!P.yield) {
#pragma unroll
    for (int i = 0; i < 9; ++i) Y[i] += MN[i];  // newF = F_tmp
  }
  float g_Ftmp[9];
  mm(P.U, Y, t9);
  mmT(t9, P.V, g_Ftmp);
  mmT(g_Ftmp, F, t9);  // Ftmp = (I + dt C) F
#pragma unroll
  for (int i = 0; i < 9; ++i) g_C[i] = m.p_mass * g_affine[i] + m.dt * t9[i];
  float IC[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) IC[i] = m.dt * C[i] + ((i % 4 == 0) ? 1.f : 0.f);
  mTm(IC, g_Ftmp, g_F);
}

// FP64 adjoint of p2g_particle: the reference's order of operations, with
// backward_svd as the reference writes it; g_C, g_F are written
MPM_DI void p2g_particle_vjp_f64(const MatConsts<double>& m, const double* C, const double* F, const P2G<double>& P,
                                 const double* g_affine, const double* g_newF_in, double* g_C, double* g_F) {
  using S = double;
  S g_raw[9], tmp[9], g_newF[9], g_R[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    g_raw[i] = m.ks * g_affine[i];
    g_C[i] = m.p_mass * g_affine[i];
  }
  mm(g_raw, P.newF, tmp);  // d/dA of tr(g^T A newF^T)
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    g_R[i] = S(-2) * m.mu * tmp[i];
    g_newF[i] = S(2) * m.mu * tmp[i] + g_newF_in[i];
  }
  mTm(g_raw, P.A, tmp);  // d/dnewF of the right factor
  S g_J = m.lam * (S(2) * P.J - S(1)) * (g_raw[0] + g_raw[4] + g_raw[8]);
  S cf[9];
  cof3(P.newF, cf);
#pragma unroll
  for (int i = 0; i < 9; ++i) g_newF[i] += S(2) * m.mu * tmp[i] + g_J * cf[i];
  S gs[3] = {S(0), S(0), S(0)}, g_Ftmp[9], gA[9];
  S gU[9], gV[9];
  mm(g_R, P.V, gU);  // R = U V^T
  mTm(g_R, P.U, gV);
  if (P.yield) {
    S GV[9], GtU[9], UtGV[9];
    mm(g_newF, P.V, GV);
    mTm(g_newF, P.U, GtU);
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int cc = 0; cc < 3; ++cc) {
        gU[r * 3 + cc] += GV[r * 3 + cc] * P.e[cc];
        gV[r * 3 + cc] += GtU[r * 3 + cc] * P.e[cc];
      }
    mTm(P.U, GV, UtGV);
    return_map_sigma_grad(P, UtGV, gs);
#pragma unroll
    for (int i = 0; i < 9; ++i) g_Ftmp[i] = S(0);
  } else {
#pragma unroll
    for (int i = 0; i < 9; ++i) g_Ftmp[i] = g_newF[i];
  }
  svd3_bwd(P.U, P.s, P.V, gU, gs, gV, gA);
#pragma unroll
  for (int i = 0; i < 9; ++i) g_Ftmp[i] += gA[i];
  mmT(g_Ftmp, F, tmp);  // Ftmp = (I + dt C) F
#pragma unroll
  for (int i = 0; i < 9; ++i) g_C[i] += m.dt * tmp[i];
  S IC[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) IC[i] = m.dt * C[i] + ((i % 4 == 0) ? S(1) : S(0));
  mTm(IC, g_Ftmp, g_F);
}
MPM_DI void p2g_particle_vjp(const MatConsts<float>& m, const float* C, const float* F, const P2G<float>& P,
                             const float* g_affine, const float* g_newF_in, float* g_C, float* g_F) {
  p2g_particle_vjp_f32(m, C, F, P, g_affine, g_newF_in, g_C, g_F);
}
MPM_DI void p2g_particle_vjp(const MatConsts<double>& m, const double* C, const double* F, const P2G<double>& P,
                             const double* g_affine, const double* g_newF_in, double* g_C, double* g_F) {
  p2g_particle_vjp_f64(m, C, F, P, g_affine, g_newF_in, g_C, g_F);
}

template <typename T, typename S>
MPM_DI MatConsts<S> mat_consts(const Consts<T>& c) {
  MatConsts<S> m;
  m.dt = S(c.dt);
  m.mu = S(c.mu);
  m.lam = S(c.lam);
  m.ys = S(c.yield_stress);
  m.ks = S(c.ks);
  m.p_mass = S(c.p_mass);
  return m;
}

// flags[scene*NB3 + block] = 1 for the blocks of the stencil at `base` (a lane
// with ok), called by all 32 lanes of a warp.  In cell order neighbouring
// particles touch the same blocks, so a lane whose (scene, block range)
// equals the previous lane's writes nothing: about one flag store per block
// per warp instead of one per particle.
template <typename T>
MPM_DI void mark_stencil_blocks(const Consts<T>& c, bool ok, const int* base, int scene,
                                unsigned char* __restrict__ flags) {
  const int lane = threadIdx.x & 31;
  int lo[3] = {0, 0, 0}, ext[3] = {0, 0, 0};
  unsigned long long key = ~0ull;
  if (ok) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      lo[d] = base[d] >> 2;
      ext[d] = ((base[d] + 2) >> 2) - lo[d];  // 0 or 1
    }
    // n_grid <= 1024: block coordinates fit 9 bits
    key = ((unsigned long long)scene << 30) | ((unsigned long long)lo[0] << 21) |
          ((unsigned long long)lo[1] << 12) | ((unsigned long long)lo[2] << 3) |
          (unsigned long long)(ext[0] << 2 | ext[1] << 1 | ext[2]);
  }
  const unsigned long long prev = __shfl_up_sync(0xffffffffu, key, 1);
  if (ok && (lane == 0 || prev != key)) {
    // the 1, 2, 4 or 8 blocks (lo + {0, ext}) as predicated stores; the
    // offset within a scene fits 32 bits (nb <= 256)
    unsigned char* f = flags + (int64_t)scene * c.NB3;
    const int nb = c.nb;
    const int i0 = (lo[0] * nb + lo[1]) * nb + lo[2];
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      const int di = m >> 2, dj = (m >> 1) & 1, dk = m & 1;
      if (di <= ext[0] && dj <= ext[1] && dk <= ext[2]) f[i0 + (di * nb + dj) * nb + dk] = 1;
    }
  }
}

// ---------------------------------------------------------------------------
// forward kernels
// ---------------------------------------------------------------------------
// one 128-particle chunk of p2g (all 128 threads of the block take part)
template <typename T, typename S>
MPM_DI void p2g_chunk(const Consts<T>& c, const T* __restrict__ st, T* __restrict__ st_out,
                      const int* __restrict__ pscene, Node<T>* __restrict__ grid, int64_t p) {
  const bool valid = p < c.n_particles;  // every lane stays for the warp scan
  Stencil<T> s;
  zero_stencil(s);
  bool ok = false;
  int scene = 0;
  // node value of stencil offset o: wgt(o) * (pm + affine o), where
  // affine = dx A and pm = m v - affine fx (= m v + A dp at o = 0, dp = (o - fx) dx);
  // stepped across the stencil by additions of affine's columns
  T affine[9], pm[3] = {T(0), T(0), T(0)};
#pragma unroll
  for (int k = 0; k < 9; ++k) affine[k] = T(0);
  if (valid) {
    T x[3], v[3];
    S C[9], F[9];
    load_row_cg(st, c.ld, p, 0, 3, x);
    load_row_cg(st, c.ld, p, 3, 3, v);
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      C[k] = S(__ldcg(st + (int64_t)(6 + k) * c.ld + p));
      F[k] = S(__ldcg(st + (int64_t)(15 + k) * c.ld + p));
    }
    const int sc = __ldcg(pscene + p);  // issued with the state rows
    ok = make_stencil(c, x, s);
    MatConsts<S> m = mat_consts<T, S>(c);
    P2G<S> P;
    S aff[9];
    S nF[9];
    p2g_particle(m, C, F, P, aff, st_out ? nF : (S*)nullptr);
    if (st_out) {
#pragma unroll
      for (int k = 0; k < 9; ++k) st_out[(int64_t)(15 + k) * c.ld + p] = T(nF[k]);
    }
    if (!ok) atomicOr(c.status, MPM_STATUS_OUT_OF_GRID);
    if (!finite(P.J)) atomicOr(c.status, MPM_STATUS_NONFINITE);
    if (ok) {
      scene = sc;
#pragma unroll
      for (int k = 0; k < 9; ++k) affine[k] = T(aff[k]) * c.dx;
#pragma unroll
      for (int k = 0; k < 3; ++k)
        pm[k] = c.p_mass * v[k] - (affine[3 * k] * s.fx[0] + affine[3 * k + 1] * s.fx[1] + affine[3 * k + 2] * s.fx[2]);
    } else {
      zero_stencil(s);
    }
  }
  const long long key = ok ? cell_key(c, scene, s) : -1 - (long long)(threadIdx.x & 31);
  Node<T>* g = grid + (int64_t)scene * c.G;
  const StencilAddr A = stencil_addr(c, s);
  constexpr bool slab = sizeof(T) == 4;
  const int lane = threadIdx.x & 31;
  WarpSeg seg{};
  unsigned tails = 0, emit = 0;
  SlabStage* sb = nullptr;
  if constexpr (slab) {
    __shared__ SlabStage stage[4];  // one per warp of the 128-thread block
    sb = &stage[threadIdx.x >> 5];
    warp_tails(key, ok, tails, emit);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      sb->ay[lane][k] = A.ay[k];
      sb->az[lane][k] = A.az[k];
    }
  } else {
    seg = warp_segments(key);
  }
  pdl_wait();  // the grid blocks are zeroed by the compaction before
  pdl_trigger();
  if constexpr (slab) {
    // FP32: the node value wgt (m v + A dp, m) in packed pairs: (x, y) and
    // (z, m), stepped across the stencil by the columns of A (and 0 for m)
    float2 cxA = make_float2(pm[0], pm[1]), cxB = make_float2(pm[2], c.p_mass);
    const float2 a0A = make_float2(affine[0], affine[3]), a0B = make_float2(affine[6], 0.f);
    const float2 a1A = make_float2(affine[1], affine[4]), a1B = make_float2(affine[7], 0.f);
    const float2 a2A = make_float2(affine[2], affine[5]), a2B = make_float2(affine[8], 0.f);
#pragma unroll 1
    for (int ox = 0; ox < 3; ++ox) {
      const float wx = sel3(s.w[0][0], s.w[1][0], s.w[2][0], ox);
      const int ax = sel3(A.ax[0], A.ax[1], A.ax[2], ox);
      float2 cyA = cxA, cyB = cxB;
#pragma unroll
      for (int oy = 0; oy < 3; ++oy) {
        float2 czA = cyA, czB = cyB;
#pragma unroll
        for (int oz = 0; oz < 3; ++oz) {
          const float wgt = wx * s.w[oy][1] * s.w[oz][2];
          const float2 w2 = make_float2(wgt, wgt);
          const float2 lo = mul2(w2, czA), hi = mul2(w2, czB);
          sb->v[lane][oy * 3 + oz] = make_float4(lo.x, lo.y, hi.x, hi.y);
          czA = add2(czA, a2A);
          czB = add2(czB, a2B);
        }
        cyA = add2(cyA, a1A);
        cyB = add2(cyB, a1B);
      }
      cxA = add2(cxA, a0A);
      cxB = add2(cxB, a0B);
      sb->base[lane] = g + ax;
      __syncwarp();
      slab_reduce<true>(*sb, tails, emit);
      __syncwarp();
    }
  } else {
    T cx[3] = {pm[0], pm[1], pm[2]};
#pragma unroll 1
    for (int ox = 0; ox < 3; ++ox) {
      const T wx = sel3(s.w[0][0], s.w[1][0], s.w[2][0], ox);
      const int ax = sel3(A.ax[0], A.ax[1], A.ax[2], ox);
      T cy[3] = {cx[0], cx[1], cx[2]};
#pragma unroll
      for (int oy = 0; oy < 3; ++oy) {
        T cz[3] = {cy[0], cy[1], cy[2]};
#pragma unroll
        for (int oz = 0; oz < 3; ++oz) {
          const T wgt = wx * s.w[oy][1] * s.w[oz][2];
          T mv[4];
#pragma unroll
          for (int k = 0; k < 3; ++k) mv[k] = wgt * cz[k];
          mv[3] = wgt * c.p_mass;
          if (seg.steps) {
#pragma unroll
            for (int k = 0; k < 4; ++k) mv[k] = seg_scan(mv[k], seg);
          }
          if (ok && seg.tail) atomic_add_node(g + ax + A.ay[oy] + A.az[oz], mv[0], mv[1], mv[2], mv[3]);
#pragma unroll
          for (int k = 0; k < 3; ++k) cz[k] += affine[3 * k + 2];
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) cy[k] += affine[3 * k + 1];
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) cx[k] += affine[3 * k];
    }
  }
}
// FP32: 7 CTAs of 128 threads per SM by default (at most 73 registers, no
// spill; measured 6 % faster than 6 CTAs); MB > 0 compiles the kernel for MB
// CTAs per SM instead (the autotuner's candidates, MpmTuning.p2g_ctas).
// Strided: the CTAs stride over the particle chunks (the adjoint's recompute,
// which exits at once when the grid store holds the substep)
template <typename T, typename S, bool Strided = false, int MB = 0>
__global__ void __launch_bounds__(128, MB > 0 ? MB : ((sizeof(T) == 4 && sizeof(S) == 4) ? 7 : 4)) k_p2g(Consts<T> c, const T* __restrict__ st, T* __restrict__ st_out,
                                             const int* __restrict__ pscene, Node<T>* __restrict__ grid,
                                             const int64_t* __restrict__ saved) {
  if (saved && __ldcg(saved) >= 0) {  // the grid of this substep was restored from the grid store
    pdl_wait();  // completes only after the kernel before it (dependent launches chain through it)
    return;
  }
  if constexpr (Strided) {
    for (int64_t p0 = (int64_t)blockIdx.x * blockDim.x; p0 < c.n_particles; p0 += (int64_t)gridDim.x * blockDim.x)
      p2g_chunk<T, S>(c, st, st_out, pscene, grid, p0 + threadIdx.x);
  } else {
    p2g_chunk<T, S>(c, st, st_out, pscene, grid, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
  }
}

// Tools in the compute precision, for grid_op and grid_op.grad.  The tool
// fields (primive_base.py:313-329) are converted once when the tools are set
// (k_tools_convert: tools_t[i] = Tool<T> of descriptor i).  The poses of
// frames f and f+1 are converted every substep by the block compaction
// (poses_t[16 i + k]: k < 8 frame f, else frame f+1, one value per thread).
// Both kernels read them straight from global memory: the lanes of a warp
// load the same words (a broadcast), with no per-block staging, barrier or
// FP64 conversion.
template <typename T>
__global__ void __launch_bounds__(128) k_tools_convert(int n, const MpmToolDesc* __restrict__ tools,
                                                       Tool<T>* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) to_tool(tools[i], out[i]);
}
struct PoseTableArgs {
  int n_tools;
  const double *pose_f, *pose_f1;
  void* poses;  // T[n_tools * 16]
};
template <typename T>
MPM_DI void pose_table_fill(const PoseTableArgs& a, int64_t i, int64_t stride) {
  for (int64_t j = i; j < (int64_t)a.n_tools * 16; j += stride) {
    const int64_t t = j >> 4;
    const int k = (int)(j & 15);
    static_cast<T*>(a.poses)[j] = T(k < 8 ? a.pose_f[8 * t + k] : a.pose_f1[8 * t + k - 8]);
  }
}
// the tools of one scene: tool[t], pose p0(t) at frame f, p1(t) at frame f+1
template <typename T>
struct SceneToolView {
  int n;
  const Tool<T>* tool;
  const Pose<T>* pose;
  MPM_DI SceneToolView(const Tool<T>* tools_t, const T* poses_t, const int* tool_off, int scene) {
    const int t0 = tool_off[scene];
    n = tool_off[scene + 1] - t0;
    tool = tools_t + t0;
    pose = reinterpret_cast<const Pose<T>*>(poses_t + 16 * (int64_t)t0);
  }
  MPM_DI const Pose<T>& p0(int t) const { return pose[2 * t]; }
  MPM_DI const Pose<T>& p1(int t) const { return pose[2 * t + 1]; }
};

// wall conditions of grid_op (mpm_simulator.py:241-260) with optional tape
template <typename T>
struct WallTape {
  T v_pre[3][3];
  bool low[3], up[3];
};
template <typename T>
MPM_DI void walls(const Consts<T>& c, const int* I, T* v, WallTape<T>* tp) {
  const int bound = 3;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (tp) {
#pragma unroll
      for (int k = 0; k < 3; ++k) tp->v_pre[d][k] = v[k];
    }
    bool low = I[d] < bound && v[d] < T(0);
    if (tp) tp->low[d] = low;
    if (low) {
      if (d != 1 || c.ground_friction == T(0)) {
        v[d] = T(0);
      } else if (c.ground_friction < T(10)) {
        T lin = v[1] + T(1e-30);
        T vit[3] = {v[0] - T(I[0]) * T(1e-30), v[1] - lin - T(I[1]) * T(1e-30), v[2] - T(I[2]) * T(1e-30)};
        T lit = msqrt(dot3(vit, vit) + T(1e-8));
        T a = T(1) + c.ground_friction * lin / lit;
        T fac = (T(0) < a) ? a : T(0);
#pragma unroll
        for (int k = 0; k < 3; ++k) v[k] = fac * (vit[k] + T(I[k]) * T(1e-30));
        v[1] = T(0);
      } else {
        v[0] = v[1] = v[2] = T(0);
      }
    }
    bool up = I[d] > c.n_grid - bound && v[d] > T(0);
    if (tp) tp->up[d] = up;
    if (up) v[d] = T(0);
  }
}
template <typename T>
MPM_DI void walls_vjp(const Consts<T>& c, const int* I, const WallTape<T>& tp, T* g) {
#pragma unroll
  for (int d = 2; d >= 0; --d) {
    if (tp.up[d]) g[d] = T(0);
    if (!tp.low[d]) continue;
    if (d != 1 || c.ground_friction == T(0)) {
      g[d] = T(0);
    } else if (c.ground_friction < T(10)) {
      const T* v = tp.v_pre[d];
      T lin = v[1] + T(1e-30);
      T vit[3] = {v[0] - T(I[0]) * T(1e-30), v[1] - lin - T(I[1]) * T(1e-30), v[2] - T(I[2]) * T(1e-30)};
      T lit = msqrt(dot3(vit, vit) + T(1e-8));
      T a = T(1) + c.ground_friction * lin / lit;
      T fac = (T(0) < a) ? a : T(0);
      const T go[3] = {g[0], T(0), g[2]};
      const T w[3] = {vit[0] + T(I[0]) * T(1e-30), vit[1] + T(I[1]) * T(1e-30), vit[2] + T(I[2]) * T(1e-30)};
      T g_fac = dot3(go, w);
      T g_vit[3] = {fac * go[0], fac * go[1], fac * go[2]};
      T g_lin = T(0), g_lit = T(0);
      if (T(0) < a) {
        g_lin = g_fac * c.ground_friction / lit;
        g_lit = -g_fac * c.ground_friction * lin / (lit * lit);
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) g_vit[k] += g_lit * vit[k] / lit;
      g_lin -= g_vit[1];
      g[0] = g_vit[0];
      g[1] = g_vit[1] + g_lin;
      g[2] = g_vit[2];
    } else {
      g[0] = g[1] = g[2] = T(0);
    }
  }
}

// grid_op over the active blocks: one 64-thread CTA per block, grid-stride.
// store_slot >= 0: list block b of grid_in and of grid_out are also copied to
// the grid store at slot_start + b (reserved by the compaction; -1 when the
// store is full).  saved (may be null; the adjoint's recompute): when it
// points at a slot start >= 0 both grids were restored from the store and the
// kernel returns at once.  FP32: at least 16 CTAs per SM (64 registers, a small
// spill): with the grid-stride width of 16 CTAs per SM all of them are
// resident at once (measured 9.8 -> 9.2 us on 32 scenes against 80 registers).
template <typename T>
__global__ void __launch_bounds__(64, sizeof(T) == 4 ? 16 : 1) k_grid_op(Consts<T> c, const int* __restrict__ active,
                                                const int* __restrict__ n_active,
                                                const Node<T>* __restrict__ grid_in, Node<T>* __restrict__ grid_out,
                                                const Tool<T>* __restrict__ tools_t, const T* __restrict__ poses_t,
                                                const int* __restrict__ tool_off, MpmGridStore store,
                                                int store_slot, const int64_t* __restrict__ saved) {
  pdl_wait();     // the grid is p2g's output
  pdl_trigger();  // g2p reads its particle rows while the grid is updated
  if (saved && *saved >= 0) return;
  const int na = *n_active;
  const int64_t start = store_slot >= 0 ? store.slot_start[store_slot] : -1;
  for (int b = blockIdx.x; b < na; b += gridDim.x) {
    const int64_t gb = active[b];
    int I[3];
    const int scene = block_node(c, gb, threadIdx.x, I);
    const SceneToolView<T> sh(tools_t, poses_t, tool_off, scene);
    const int64_t idx = gb * 64 + threadIdx.x;
    Node<T> in = grid_in[idx];
    Node<T>* stored = start >= 0 ? reinterpret_cast<Node<T>*>(store.blocks) + ((start + b) << 7) : nullptr;
    if (stored) {
      stored[threadIdx.x] = in;
      if (threadIdx.x == 0) store.block_ids[start + b] = (int)gb;
    }
    Node<T> out = {T(0), T(0), T(0), in.w};
    if (in.w > T(1e-12)) {
      T inv = T(1) / in.w;
      T v[3] = {inv * in.x + c.gdt[0], inv * in.y + c.gdt[1], inv * in.z + c.gdt[2]};
      const T p[3] = {T(I[0]) * c.dx, T(I[1]) * c.dx, T(I[2]) * c.dx};
      for (int t = 0; t < sh.n; ++t) tool_collide(sh.tool[t], sh.p0(t), sh.p1(t), p, c.dt, v);
      walls(c, I, v, (WallTape<T>*)nullptr);
      if (!(finite(v[0]) && finite(v[1]) && finite(v[2]))) atomicOr(c.status, MPM_STATUS_NONFINITE);
      out.x = v[0];
      out.y = v[1];
      out.z = v[2];
    }
    grid_out[idx] = out;
    if (stored) stored[64 + threadIdx.x] = out;
  }
}

// g2p of particle p (mpm_simulator.py:265-284): writes rows 0..14 of st_out
// and xn; returns false (the state copied unchanged) for a particle whose
// stencil left the grid
template <typename T>
MPM_DI bool g2p_particle(const Consts<T>& c, const T* __restrict__ st, T* __restrict__ st_out, int64_t p, int scene,
                         const Node<T>* __restrict__ grid, T* xn) {
  T x[3];
  load_row_cg(st, c.ld, p, 0, 3, x);
  Stencil<T> s;
  if (!make_stencil(c, x, s)) {  // flagged by k_p2g; the particle keeps its state
#pragma unroll
    for (int k = 0; k < 15; ++k) st_out[(int64_t)k * c.ld + p] = __ldcg(st + (int64_t)k * c.ld + p);
    return false;
  }
  const Node<T>* g = grid + (int64_t)scene * c.G;
  const StencilAddr A = stencil_addr(c, s);
  pdl_wait();  // the grid is grid_op's output
  // C = k4 sum_o wgt v(o) (o - fx)^T = k4 (m1 - nv fx^T) with m1 = sum_o wgt v(o) o^T:
  // the offsets o are 0, 1, 2, so m1 takes only additions
  T nv[3] = {T(0), T(0), T(0)}, m1[9], nC[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) m1[k] = T(0);
  const T k4 = T(4) * c.inv_dx;
#pragma unroll
  for (int ox = 0; ox < 3; ++ox)
#pragma unroll
    for (int oy = 0; oy < 3; ++oy)
#pragma unroll
      for (int oz = 0; oz < 3; ++oz) {
        T wgt = s.w[ox][0] * s.w[oy][1] * s.w[oz][2];
        Node<T> gv = g[A.at(ox, oy, oz)];
        const T q[3] = {wgt * gv.x, wgt * gv.y, wgt * gv.z};
        const int o[3] = {ox, oy, oz};
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          nv[i] += q[i];
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            if (o[j] == 1) m1[i * 3 + j] += q[i];
            if (o[j] == 2) m1[i * 3 + j] += T(2) * q[i];
          }
        }
      }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) nC[i * 3 + j] = k4 * (m1[i * 3 + j] - s.fx[j] * nv[i]);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    T t = x[i] + c.dt * nv[i];
    T mn = (t < c.x_hi) ? t : c.x_hi;
    xn[i] = (c.x_lo < mn) ? mn : c.x_lo;
  }
  store_row(st_out, c.ld, p, 0, 3, xn);
  store_row(st_out, c.ld, p, 3, 3, nv);
  store_row(st_out, c.ld, p, 6, 9, nC);
  return true;
}
// mark (may be null; chained forward substeps): also flags the blocks the
// stencils of the new positions touch, for the next substep, whose
// compaction reads them instead of a marking pass; header[0..1] (list length,
// reservation ticket) are reset for that substep.
// At least MB CTAs of 128 threads per SM (MpmTuning.g2p_ctas; 0 = 8 in FP32:
// at most 64 registers)
template <typename T, int MB = 0>
__global__ void __launch_bounds__(128, MB > 0 ? MB : (sizeof(T) == 4 ? 8 : 1)) k_g2p(Consts<T> c, const T* __restrict__ st, T* __restrict__ st_out,
                                             const int* __restrict__ pscene, const Node<T>* __restrict__ grid,
                                             unsigned char* __restrict__ mark, int* __restrict__ header) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = p < c.n_particles;
  const int scene = valid ? __ldcg(pscene + p) : 0;  // issued with x
  T xn[3] = {T(0), T(0), T(0)};
  const bool moved = valid && g2p_particle(c, st, st_out, p, scene, grid, xn);
  pdl_wait();  // grid_op reads the header reset below (and lanes without a stencil have not waited)
  pdl_trigger();
  if (mark) {  // uniform; all lanes take part in the warp's writer election
    Stencil<T> sn;
    zero_stencil(sn);
    const bool ok = moved && make_stencil(c, xn, sn);
    mark_stencil_blocks(c, ok, sn.base, scene, mark);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      header[0] = 0;
      header[1] = 0;
    }
  }
}

// ---------------------------------------------------------------------------
// adjoint kernels
// ---------------------------------------------------------------------------
// g2p.grad: writes the x rows of g0 (partial) and scatters into g_grid
// st1 (frame f+1, may be null): its v rows are the g2p output, so the clamp
// mask needs no second gather of the grid.
// FP32: 6 CTAs of 128 threads per SM by default (at most 80 registers, a
// small spill; measured 20 % faster than the unconstrained 108 registers);
// MB > 0: MB CTAs per SM (MpmTuning.g2p_adj_ctas)
template <typename T, int MB = 0>
__global__ void __launch_bounds__(128, MB > 0 ? MB : (sizeof(T) == 4 ? 6 : 2)) k_g2p_adj(Consts<T> c, const T* __restrict__ st, const T* __restrict__ st1,
                                                 const T* __restrict__ g1, T* __restrict__ g0,
                                                 const int* __restrict__ pscene, const Node<T>* __restrict__ grid,
                                                 Node<T>* __restrict__ g_grid) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = p < c.n_particles;  // every lane stays for the warp scan
  Stencil<T> s;
  zero_stencil(s);
  bool ok = false;
  int scene = 0;
  T x[3] = {T(0), T(0), T(0)};
  T nv[3] = {T(0), T(0), T(0)};
  T gnv[3] = {T(0), T(0), T(0)}, gC[9], gx[3] = {T(0), T(0), T(0)}, gx1[3] = {T(0), T(0), T(0)};
#pragma unroll
  for (int k = 0; k < 9; ++k) gC[k] = T(0);
  if (valid) {
    // every row this particle needs is requested together with x
    load_row_cg(st, c.ld, p, 0, 3, x);
    if (st1) load_row_cg(st1, c.ld, p, 3, 3, nv);
    load_row_cg(g1, c.ld, p, 0, 3, gx1);
    load_row_cg(g1, c.ld, p, 3, 3, gnv);
    load_row_cg(g1, c.ld, p, 6, 9, gC);
    scene = __ldcg(pscene + p);
    ok = make_stencil(c, x, s);
    if (!ok) {
      zero_stencil(s);
      scene = 0;
      const T z[3] = {T(0), T(0), T(0)};
      store_row(g0, c.ld, p, 0, 3, z);
    }
  }
  if (!ok) {  // no contribution (and no 0 * inf) from particles outside the grid
#pragma unroll
    for (int k = 0; k < 3; ++k) nv[k] = gnv[k] = gx1[k] = T(0);
#pragma unroll
    for (int k = 0; k < 9; ++k) gC[k] = T(0);
  }
  const int64_t off = (int64_t)scene * c.G;
  const Node<T>* g = grid + off;
  Node<T>* gg = g_grid + off;
  const StencilAddr A = stencil_addr(c, s);
  pdl_wait();  // the restored (or recomputed) grid and the zeroed g_grid
  pdl_trigger();
  if (ok) {
    if (!st1) {
#pragma unroll
      for (int ox = 0; ox < 3; ++ox)
#pragma unroll
        for (int oy = 0; oy < 3; ++oy)
#pragma unroll
          for (int oz = 0; oz < 3; ++oz) {
            T wgt = s.w[ox][0] * s.w[oy][1] * s.w[oz][2];
            Node<T> n = g[A.at(ox, oy, oz)];
            nv[0] += wgt * n.x;
            nv[1] += wgt * n.y;
            nv[2] += wgt * n.z;
          }
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      T t = x[i] + c.dt * nv[i];
      T mn = (t < c.x_hi) ? t : c.x_hi;
      bool pass = (t < c.x_hi) && (c.x_lo < mn);
      T gt = pass ? gx1[i] : T(0);
      gx[i] = gt;
      gnv[i] += c.dt * gt;
    }
  }
  const long long key = ok ? cell_key(c, scene, s) : -1 - (long long)(threadIdx.x & 31);
  constexpr bool slab = sizeof(T) == 4;
  const int lane = threadIdx.x & 31;
  WarpSeg seg{};
  unsigned tails = 0, emit = 0;
  SlabStage* sb = nullptr;
  if constexpr (slab) {
    __shared__ SlabStage stage[4];  // one per warp of the 128-thread block
    sb = &stage[threadIdx.x >> 5];
    warp_tails(key, ok, tails, emit);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      sb->ay[lane][k] = A.ay[k];
      sb->az[lane][k] = A.az[k];
    }
  } else {
    seg = warp_segments(key);
  }
  const T k4 = T(4) * c.inv_dx;
  T gw[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) gw[a][b] = T(0);
  // the x-derivative through dp = o - fx of sum_o wgt gv(o) . (k4 gC dp) is
  // -k4 gC^T sum_o wgt gv(o) = -k4 gC^T new_v
  T gfx[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) gfx[j] = -k4 * (gC[j] * nv[0] + gC[3 + j] * nv[1] + gC[6 + j] * nv[2]);
  // u(o) = gnv + k4 gC (o - fx): the node value is wgt(o) u(o) and the weight
  // adjoint gv(o) . u(o); u is stepped across the stencil by the columns of k4 gC
  T ux[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int j = 0; j < 3; ++j) gC[3 * i + j] *= k4;
    ux[i] = gnv[i] - (gC[3 * i] * s.fx[0] + gC[3 * i + 1] * s.fx[1] + gC[3 * i + 2] * s.fx[2]);
  }
  // weight adjoints g_wgt(o) = gv(o) . u(o): the 27 gathers of the grid
  // velocity in one unrolled loop (their loads issue together), before the
  // scatter, which then touches no global memory but its atomics
  if (ok) {
    T vx[3] = {ux[0], ux[1], ux[2]};
#pragma unroll
    for (int ox = 0; ox < 3; ++ox) {
      T vy[3] = {vx[0], vx[1], vx[2]};
#pragma unroll
      for (int oy = 0; oy < 3; ++oy) {
        T vz[3] = {vy[0], vy[1], vy[2]};
#pragma unroll
        for (int oz = 0; oz < 3; ++oz) {
          const Node<T> n = g[A.at(ox, oy, oz)];
          const T gv[3] = {n.x, n.y, n.z};
          const T g_wgt = dot3(gv, vz);
          gw[ox][0] += g_wgt * s.w[oy][1] * s.w[oz][2];
          gw[oy][1] += g_wgt * s.w[ox][0] * s.w[oz][2];
          gw[oz][2] += g_wgt * s.w[ox][0] * s.w[oy][1];
#pragma unroll
          for (int i = 0; i < 3; ++i) vz[i] += gC[3 * i + 2];
        }
#pragma unroll
        for (int i = 0; i < 3; ++i) vy[i] += gC[3 * i + 1];
      }
#pragma unroll
      for (int i = 0; i < 3; ++i) vx[i] += gC[3 * i];
    }
  }
#pragma unroll 1
  for (int ox = 0; ox < 3; ++ox) {
    const T wx = sel3(s.w[0][0], s.w[1][0], s.w[2][0], ox);
    const int ax = sel3(A.ax[0], A.ax[1], A.ax[2], ox);
    T uy[3] = {ux[0], ux[1], ux[2]};
#pragma unroll
    for (int oy = 0; oy < 3; ++oy) {
      T uz[3] = {uy[0], uy[1], uy[2]};
#pragma unroll
      for (int oz = 0; oz < 3; ++oz) {
        const T wgt = wx * s.w[oy][1] * s.w[oz][2];
        T sc3[3] = {wgt * uz[0], wgt * uz[1], wgt * uz[2]};
        if constexpr (slab) {
          sb->v[lane][oy * 3 + oz] = make_float4(sc3[0], sc3[1], sc3[2], 0.f);
        } else {
          if (seg.steps) {
#pragma unroll
            for (int k = 0; k < 3; ++k) sc3[k] = seg_scan(sc3[k], seg);
          }
          if (ok && seg.tail) atomic_add_node3(gg + ax + A.ay[oy] + A.az[oz], sc3[0], sc3[1], sc3[2]);
        }
#pragma unroll
        for (int i = 0; i < 3; ++i) uz[i] += gC[3 * i + 2];
      }
#pragma unroll
      for (int i = 0; i < 3; ++i) uy[i] += gC[3 * i + 1];
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) ux[i] += gC[3 * i];
    if constexpr (slab) {
      sb->base[lane] = gg + ax;
      __syncwarp();
      slab_reduce(*sb, tails, emit);
      __syncwarp();
    }
  }
  if (ok) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
#pragma unroll
      for (int k = 0; k < 3; ++k) gfx[d] += gw[k][d] * dweight(s, k, d);
      gx[d] += c.inv_dx * gfx[d];
    }
    store_row(g0, c.ld, p, 0, 3, gx);
  }
}

// grid_op.grad over the active blocks: g_grid (velocity adjoint) -> g_in
// (mv.xyz, m); tool-pose gradients of frames f and f+1 reduced per warp in
// FP64 and added with one atomic per warp and component.
// Sums 16 values over the 32 lanes of a warp by recursive halving
// (reduce-scatter): each level sends half of the values still held to the
// partner lane and keeps the other half, 16 shuffles in all instead of 80
// for 16 butterfly all-reduces.  Returns the full sum of value k (set on
// return, from lane bits 4..1); lanes 2j and 2j+1 hold the same k.
template <typename T>
MPM_DI T warp_reduce_scatter16(T (&v)[16], int& k) {
  const int lane = threadIdx.x & 31;
  const bool h4 = lane & 16, h3 = lane & 8, h2 = lane & 4, h1 = lane & 2;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const T send = h4 ? v[i] : v[i + 8];
    const T keep = h4 ? v[i + 8] : v[i];
    v[i] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const T send = h3 ? v[i] : v[i + 4];
    const T keep = h3 ? v[i + 4] : v[i];
    v[i] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
  }
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const T send = h2 ? v[i] : v[i + 2];
    const T keep = h2 ? v[i + 2] : v[i];
    v[i] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
  }
  {
    const T send = h1 ? v[0] : v[1];
    const T keep = h1 ? v[1] : v[0];
    v[0] = keep + __shfl_xor_sync(0xffffffffu, send, 2);
  }
  k = (h4 ? 8 : 0) + (h3 ? 4 : 0) + (h2 ? 2 : 0) + (h1 ? 1 : 0);
  return v[0] + __shfl_xor_sync(0xffffffffu, v[0], 1);
}

// At least MB CTAs of 64 threads per SM (MpmTuning.grid_op_adj_ctas; 0 = 6:
// at most 168 registers)
template <typename T, int MB = 0>
__global__ void __launch_bounds__(64, MB > 0 ? MB : (sizeof(T) == 4 ? 6 : 1)) k_grid_op_adj(Consts<T> c, const int* __restrict__ active,
                                                    const int* __restrict__ n_active,
                                                    const Node<T>* __restrict__ grid_in,
                                                    const Node<T>* __restrict__ g_grid, Node<T>* __restrict__ g_in,
                                                    const Tool<T>* __restrict__ tools_t,
                                                    const T* __restrict__ poses_t, const int* __restrict__ tool_off,
                                                    double* __restrict__ g_pose_f, double* __restrict__ g_pose_f1) {
  pdl_wait();     // g_grid is g2p.grad's output
  pdl_trigger();  // p2g.grad recomputes its particles' stress meanwhile
  const int na = *n_active;
  for (int b = blockIdx.x; b < na; b += gridDim.x) {
    const int64_t gb = active[b];
    int I[3];
    const int scene = block_node(c, gb, threadIdx.x, I);
    const SceneToolView<T> sh(tools_t, poses_t, tool_off, scene);
    const int64_t idx = gb * 64 + threadIdx.x;
    Node<T> in = grid_in[idx];
    Node<T> go = g_grid[idx];
    const bool active_node = in.w > T(1e-12) && (go.x != T(0) || go.y != T(0) || go.z != T(0));
    const T p[3] = {T(I[0]) * c.dx, T(I[1]) * c.dx, T(I[2]) * c.dx};
    T vt[MAX_TOOLS_PER_SCENE + 1][3];
    WallTape<T> wt;
    T g[3] = {go.x, go.y, go.z};
    const T inv = active_node ? T(1) / in.w : T(0);
    if (active_node) {
      T v[3] = {inv * in.x + c.gdt[0], inv * in.y + c.gdt[1], inv * in.z + c.gdt[2]};
      for (int t = 0; t < sh.n; ++t) {
#pragma unroll
        for (int k = 0; k < 3; ++k) vt[t][k] = v[k];
        tool_collide(sh.tool[t], sh.p0(t), sh.p1(t), p, c.dt, v);
      }
      walls(c, I, v, &wt);
      walls_vjp(c, I, wt, g);
    }
    const int t0 = tool_off[scene];
    for (int t = sh.n - 1; t >= 0; --t) {
      PoseGrad<T> g0, g1;
      g0.zero();
      g1.zero();
      if (active_node) tool_collide_vjp(sh.tool[t], sh.p0(t), sh.p1(t), p, c.dt, vt[t], g, g0, g1);
      if (__any_sync(0xffffffffu, active_node)) {
        double* d0 = g_pose_f + 8 * (t0 + t);
        double* d1 = g_pose_f1 + 8 * (t0 + t);
        T v16[16] = {g0.pos[0], g0.pos[1], g0.pos[2], g0.rot[0], g0.rot[1], g0.rot[2], g0.rot[3], g0.gap,
                     g1.pos[0], g1.pos[1], g1.pos[2], g1.rot[0], g1.rot[1], g1.rot[2], g1.rot[3], g1.gap};
        int k;
        const T v = warp_reduce_scatter16(v16, k);
        if ((threadIdx.x & 1) == 0 && v != T(0)) atomicAdd((k < 8 ? d0 + k : d1 + (k - 8)), double(v));
      }
    }
    Node<T> res = {T(0), T(0), T(0), T(0)};
    if (active_node) {
      res.x = g[0] * inv;
      res.y = g[1] * inv;
      res.z = g[2] * inv;
      res.w = -(g[0] * in.x + g[1] * in.y + g[2] * in.z) * inv * inv;
    }
    g_in[idx] = res;
  }
}

// p2g.grad + svd_grad + compute_F_tmp.grad: gathers g_in; reads the partial
// x gradient left in g0 by k_g2p_adj and writes all 24 rows of g0.
// FP32: at most 102 registers by default (5 CTAs of 128 threads per SM; a
// small spill), measured 3 % faster than 4 CTAs at 128 registers; MB > 0: MB
// CTAs per SM (MpmTuning.p2g_adj_ctas)
template <typename T, typename S, int MB = 0>
__global__ void __launch_bounds__(128, MB > 0 ? MB : ((sizeof(T) == 4 && sizeof(S) == 4) ? 5 : 2)) k_p2g_adj(Consts<T> c, const T* __restrict__ st, const T* __restrict__ g1,
                                                 T* __restrict__ g0, const int* __restrict__ pscene,
                                                 const Node<T>* __restrict__ g_in) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= c.n_particles) return;
  // the adjoint rows read after the forward recompute and the gather are
  // fetched into L2 now, so those later loads do not wait on DRAM
#pragma unroll
  for (int k = 0; k < 3; ++k) prefetch_l2(g0 + (int64_t)k * c.ld + p);
#pragma unroll
  for (int k = 15; k < 24; ++k) prefetch_l2(g1 + (int64_t)k * c.ld + p);
  T x[3], v[3];
  S C[9], F[9];
  load_row_cg(st, c.ld, p, 0, 3, x);
  load_row_cg(st, c.ld, p, 3, 3, v);
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    C[k] = S(__ldcg(st + (int64_t)(6 + k) * c.ld + p));
    F[k] = S(__ldcg(st + (int64_t)(15 + k) * c.ld + p));
  }
  const int scene = __ldcg(pscene + p);  // issued with the state rows
  Stencil<T> s;
  bool ok = make_stencil(c, x, s);
  MatConsts<S> m = mat_consts<T, S>(c);
  P2G<S> P;
  S aff[9];
  p2g_particle(m, C, F, P, aff, (S*)nullptr);
  T affine[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) affine[k] = T(aff[k]);
  T gx[3], gv[3] = {T(0), T(0), T(0)};
  load_row_cg(g0, c.ld, p, 0, 3, gx);
  S g_aff[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) g_aff[k] = S(0);
  pdl_wait();  // g_in is grid_op.grad's output
  pdl_trigger();
  if (ok) {
    const Node<T>* gg = g_in + (int64_t)scene * c.G;
    const StencilAddr A = stencil_addr(c, s);
    T ga[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) ga[k] = T(0);
    T gw[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) gw[a][b] = T(0);
    // q(o) = wgt(o) gn(o) and sq = sum_o q(o): the adjoints of m v (gv = m sq) and of
    // dp = (o - fx) dx through A dp (gfx = -dx A^T sq) need only the sum; the adjoint
    // of A (ga = sum_o q dp^T) takes sum_o q o^T, additions only as o is 0, 1, 2; the
    // node value m v + A dp is stepped across the stencil by the columns of dx A
    T sq[3] = {T(0), T(0), T(0)};
    T ad[9], cx[3];
#pragma unroll
    for (int k = 0; k < 9; ++k) ad[k] = affine[k] * c.dx;
#pragma unroll
    for (int k = 0; k < 3; ++k) cx[k] = c.p_mass * v[k] - (ad[3 * k] * s.fx[0] + ad[3 * k + 1] * s.fx[1] + ad[3 * k + 2] * s.fx[2]);
#pragma unroll
    for (int ox = 0; ox < 3; ++ox) {
      T cy[3] = {cx[0], cx[1], cx[2]};
#pragma unroll
      for (int oy = 0; oy < 3; ++oy) {
        T cz[3] = {cy[0], cy[1], cy[2]};
#pragma unroll
        for (int oz = 0; oz < 3; ++oz) {
          T wgt = s.w[ox][0] * s.w[oy][1] * s.w[oz][2];
          const int o[3] = {ox, oy, oz};
          Node<T> n = gg[A.at(ox, oy, oz)];
          const T gn[3] = {n.x, n.y, n.z};
          T g_wgt = dot3(gn, cz) + n.w * c.p_mass;
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            const T q = wgt * gn[k];
            sq[k] += q;
#pragma unroll
            for (int j = 0; j < 3; ++j) {
              if (o[j] == 1) ga[3 * k + j] += q;
              if (o[j] == 2) ga[3 * k + j] += T(2) * q;
            }
          }
          gw[ox][0] += g_wgt * s.w[oy][1] * s.w[oz][2];
          gw[oy][1] += g_wgt * s.w[ox][0] * s.w[oz][2];
          gw[oz][2] += g_wgt * s.w[ox][0] * s.w[oy][1];
#pragma unroll
          for (int k = 0; k < 3; ++k) cz[k] += ad[3 * k + 2];
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) cy[k] += ad[3 * k + 1];
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) cx[k] += ad[3 * k];
    }
    // ga = sum_o q (o - fx)^T dx from its accumulated sum_o q o^T
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int j = 0; j < 3; ++j) ga[3 * k + j] = c.dx * (ga[3 * k + j] - s.fx[j] * sq[k]);
    T gfx[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) gfx[j] = -(ad[j] * sq[0] + ad[3 + j] * sq[1] + ad[6 + j] * sq[2]);
#pragma unroll
    for (int k = 0; k < 3; ++k) gv[k] = c.p_mass * sq[k];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
#pragma unroll
      for (int k = 0; k < 3; ++k) gfx[d] += gw[k][d] * dweight(s, k, d);
      gx[d] += c.inv_dx * gfx[d];
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) g_aff[k] = S(ga[k]);
  }
  S gF1[9], gC[9], gF[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) gF1[k] = S(g1[(int64_t)(15 + k) * c.ld + p]);
  p2g_particle_vjp(m, C, F, P, g_aff, gF1, gC, gF);
  store_row(g0, c.ld, p, 0, 3, gx);
  store_row(g0, c.ld, p, 3, 3, gv);
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    g0[(int64_t)(6 + k) * c.ld + p] = T(gC[k]);
    g0[(int64_t)(15 + k) * c.ld + p] = T(gF[k]);
  }
}

// ---------------------------------------------------------------------------
// active-block bookkeeping
// ---------------------------------------------------------------------------
// Start of a substep's block bookkeeping, one launch:
// - restore (when the grid store's slot holds this substep): the active list,
//   its length, grid a (p2g) and grid a_out (grid_op output) come back from
//   the store, and the same blocks of grid b (may be null) are zeroed;
// - otherwise: the list length and the reservation ticket are reset, and
//   flags[scene*NB3 + block] = 1 for every block a particle stencil touches
//   (mark_stencil_blocks).  The flags are clean on entry (the compaction
//   clears every flag it reads).
// Grid-stride over warp-aligned ranges.
template <typename T>
__global__ void __launch_bounds__(256) k_mark_or_restore(Consts<T> c, const T* __restrict__ st,
                                                         const int* __restrict__ pscene,
                                                         unsigned char* __restrict__ flags, int* __restrict__ header,
                                                         MpmGridStore store, int slot, int* __restrict__ active,
                                                         Node<T>* __restrict__ a, Node<T>* __restrict__ a_out,
                                                         Node<T>* __restrict__ b) {
  pdl_wait();
  pdl_trigger();
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t start = slot >= 0 ? store.slot_start[slot] : -1;
  if (start >= 0) {
    const int cnt = store.slot_count[slot];
    if (blockIdx.x == 0 && threadIdx.x == 0) header[0] = cnt;
    const Node<T>* src = reinterpret_cast<const Node<T>*>(store.blocks);
    const Node<T> z = {T(0), T(0), T(0), T(0)};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (int64_t)cnt * 64; i += stride) {
      const int blk = store.block_ids[start + (i >> 6)];
      if ((i & 63) == 0) active[i >> 6] = blk;
      const Node<T>* sb = src + ((start + (i >> 6)) << 7) + (i & 63);
      a[(int64_t)blk * 64 + (i & 63)] = sb[0];
      if (a_out) a_out[(int64_t)blk * 64 + (i & 63)] = sb[64];
      if (b) b[(int64_t)blk * 64 + (i & 63)] = z;
    }
    return;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    header[0] = 0;  // list length (the compaction's append counter)
    header[1] = 0;  // reservation ticket
  }
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p - (threadIdx.x & 31) < c.n_particles;
       p += stride) {
    bool ok = false;
    int scene = 0;
    Stencil<T> s;
    zero_stencil(s);
    if (p < c.n_particles) {
      T x[3];
      load_row(st, c.ld, p, 0, 3, x);
      scene = pscene[p];  // issued with the x loads
      ok = make_stencil(c, x, s);  // out-of-grid particles are skipped (and flagged) by the scatter
    }
    mark_stencil_blocks(c, ok, s.base, scene, flags);
  }
}

// Grid store: the forward grids of a substep (the active blocks of the p2g
// grid and of the grid_op output) are kept so the adjoint substep restores
// them instead of recomputing p2g and grid_op (copy in k_grid_op, restore in
// k_mark_or_restore).  One thread reserves room for n active blocks
// of substep `slot` (bump allocator); slot_start = -1 when the store is full
// (the adjoint then recomputes)
MPM_DI void store_reserve(const MpmGridStore& st, int slot, int n) {
  const unsigned long long start = atomicAdd(st.bump, (unsigned long long)n);
  const bool fits = start + (unsigned long long)n <= (unsigned long long)st.capacity;
  st.slot_start[slot] = fits ? (int64_t)start : -1;
  st.slot_count[slot] = fits ? n : 0;
}

// List of flagged blocks (warp-aggregated append; order is not significant).
// Every flag read is cleared, so the flags are clean for the next substep.
// The appending warp zeroes its blocks in grids a and b (either may be null).
// With reserve_slot >= 0 the last CTA to finish (threadfence + ticket, no
// waiting) reserves room for the list in the grid store.  The threads also
// convert the substep's tool poses (pose_table_fill).
template <typename T>
__global__ void __launch_bounds__(256) k_compact_clear(unsigned char* __restrict__ flags, int64_t total,
                                                       int* __restrict__ active, int* __restrict__ counter,
                                                       unsigned* __restrict__ ticket, Node<T>* __restrict__ a,
                                                       Node<T>* __restrict__ b, const int64_t* __restrict__ saved,
                                                       MpmGridStore store, int reserve_slot, PoseTableArgs pt) {
  pdl_wait();
  pdl_trigger();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  pose_table_fill<T>(pt, i, (int64_t)gridDim.x * blockDim.x);
  if (saved && *saved >= 0) return;  // list and grid a restored; b zeroed by the restore
  const bool f = i < total && flags[i] != 0;
  if (f) flags[i] = 0;
  unsigned m = __ballot_sync(0xffffffffu, f);
  const int lane = threadIdx.x & 31;
  if (m) {
    const int leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (f) active[base + __popc(m & ((1u << lane) - 1u))] = (int)i;
    const int64_t w0 = i - lane;
    const Node<T> z = {T(0), T(0), T(0), T(0)};
    while (m) {
      const int k = __ffs(m) - 1;
      m &= m - 1;
      const int64_t node0 = (w0 + k) * 64;
#pragma unroll
      for (int l = 0; l < 64; l += 32) {
        if (a) a[node0 + l + lane] = z;
        if (b) b[node0 + l + lane] = z;
      }
    }
  }
  if (reserve_slot >= 0) {
    __shared__ bool last;
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
      __threadfence();
      store_reserve(store, reserve_slot, atomicAdd(counter, 0));
    }
  }
}

// ---------------------------------------------------------------------------
// density grid and losses
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(128) k_grid_mass(Consts<T> c, const T* __restrict__ st,
                                                   const int* __restrict__ pscene, T* __restrict__ gm) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= c.n_particles) return;
  T x[3];
  load_row(st, c.ld, p, 0, 3, x);
  Stencil<T> s;
  if (!make_stencil(c, x, s)) {
    atomicOr(c.status, MPM_STATUS_OUT_OF_GRID);
    return;
  }
  T* g = gm + (int64_t)pscene[p] * c.G;
#pragma unroll
  for (int ox = 0; ox < 3; ++ox)
#pragma unroll
    for (int oy = 0; oy < 3; ++oy)
#pragma unroll
      for (int oz = 0; oz < 3; ++oz)
        atomicAdd(g + node_of(c, s, ox, oy, oz), s.w[ox][0] * s.w[oy][1] * s.w[oz][2] * c.p_mass);
}
template <typename T>
__global__ void __launch_bounds__(128) k_grid_mass_adj(Consts<T> c, const T* __restrict__ st,
                                                       const int* __restrict__ pscene, const T* __restrict__ ggm,
                                                       T* __restrict__ gst) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= c.n_particles) return;
  T x[3];
  load_row(st, c.ld, p, 0, 3, x);
  Stencil<T> s;
  if (!make_stencil(c, x, s)) return;
  const T* g = ggm + (int64_t)pscene[p] * c.G;
  T gw[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) gw[a][b] = T(0);
#pragma unroll
  for (int ox = 0; ox < 3; ++ox)
#pragma unroll
    for (int oy = 0; oy < 3; ++oy)
#pragma unroll
      for (int oz = 0; oz < 3; ++oz) {
        T gg = g[node_of(c, s, ox, oy, oz)] * c.p_mass;
        gw[ox][0] += gg * s.w[oy][1] * s.w[oz][2];
        gw[oy][1] += gg * s.w[ox][0] * s.w[oz][2];
        gw[oz][2] += gg * s.w[ox][0] * s.w[oy][1];
      }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    T gfx = T(0);
#pragma unroll
    for (int k = 0; k < 3; ++k) gfx += gw[k][d] * dweight(s, k, d);
    gst[(int64_t)d * c.ld + p] += c.inv_dx * gfx;
  }
}
// per-scene sum |m - target| in FP64; blocks never straddle scenes
template <typename T>
__global__ void __launch_bounds__(256) k_density_l1(int64_t G, const T* __restrict__ gm, const T* __restrict__ tgt,
                                                    double weight, double* __restrict__ loss, T* __restrict__ ggm,
                                                    int blocks_per_scene) {
  int scene = blockIdx.x / blocks_per_scene;
  int b = blockIdx.x % blocks_per_scene;
  const T* a = gm + (int64_t)scene * G;
  const T* t = tgt + (int64_t)scene * G;
  double acc = 0.0;
  for (int64_t i = (int64_t)b * blockDim.x + threadIdx.x; i < G; i += (int64_t)blocks_per_scene * blockDim.x) {
    T d = a[i] - t[i];
    acc += fabs(double(d));
    if (ggm) ggm[(int64_t)scene * G + i] = T(weight) * sgn(d);
  }
  __shared__ double red[8];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    atomicAdd(loss + scene, weight * s);
  }
}

}  // namespace mpm
