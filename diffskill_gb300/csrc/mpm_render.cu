// Particle-SDF renderer as compute kernels (taichi_three/tina/core/particle_sdf.py,
// ParticleSDFRaster, used by plb/env_modeling/tina_renderer.py):
//
//   bake   initialize_particles_kernel + plb_set_particles + build_sdf_from_particles
//          (particle_sdf.py:548-568, 237-265): the particles' bounding box, a
//          splat of (quantised distance << 24 | rgb) by 64-bit atomicMin into a
//          voxel volume, the decode into SDF and colour, two 27-point smoothings.
//   trace  render_color + next_hit (particle_sdf.py:185-217, 353-440): one ray
//          per pixel from the view matrices, the ground, sphere tracing of the
//          tools' SDFs, the particle SDF marched with back-step refinement;
//          depth (view-space z), normal and colour per pixel, and the Lambert
//          shading of tina's Lighting.shade_color with the default lights.
//
// All arithmetic is FP32 as in the reference's f32 fields.  This file is
// compiled with -fmad=false so every operation rounds on its own, like the
// oracle's restatement.
#include <climits>

#include "mpm_launch.h"
#include "mpm_math.cuh"
#include "mpm_tools.cuh"

namespace mpm {

namespace {

constexpr float R_INF = 1e10f;          // inf of plb/engine/renderer/renderer_utils.py
constexpr float R_DIST_LIMIT = 100.0f;  // dist_limit
constexpr unsigned long long R_EMPTY = 0xFFFFFFFFull;  // ((1 << 31) - 1 + 1) * 2 - 1

__global__ void k_rb_init(int* kbox) {
  if (threadIdx.x < 3) kbox[threadIdx.x] = INT_MAX;
  else if (threadIdx.x < 6) kbox[threadIdx.x] = INT_MIN;
}

// floor(x * inv_dx) per axis, min and max over the scene's particles
template <typename T>
__global__ void k_rb_box(const T* __restrict__ st, int64_t ld, int64_t p0, int64_t n, float inv_dx,
                         int* __restrict__ kbox) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int c = 0; c < 3; ++c) {
    const float x = (float)st[(int64_t)c * ld + p0 + i];
    const int k = (int)floorf(x * inv_dx);
    atomicMin(kbox + c, k);
    atomicMax(kbox + 3 + c, k);
  }
}

// bbox[0] = (floor(x/dx) - 6) dx (min), bbox[1] = bbox[0] + res * dx; the
// reference asserts that the particles' box fits the volume
__global__ void k_rb_box_finish(const int* __restrict__ kbox, float dx_f, double dx_d, int r0, int r1, int r2,
                                float* __restrict__ bbox, unsigned int* __restrict__ status) {
  if (threadIdx.x != 0) return;
  const int res[3] = {r0, r1, r2};
  bool fits = kbox[0] != INT_MAX;
  for (int c = 0; c < 3; ++c) {
    const float lo = ((float)kbox[c] - 6.0f) * dx_f;
    const float hi = ((float)kbox[3 + c] - 6.0f) * dx_f;
    if (!(((double)hi - (double)lo) / dx_d < (double)res[c])) fits = false;
    bbox[c] = lo;
    bbox[3 + c] = (float)((double)lo + (double)res[c] * dx_d);
  }
  if (!fits) atomicOr(status, MPM_STATUS_RENDER_BOX);
}

__global__ void k_rb_fill(unsigned long long* __restrict__ packed, int64_t nvox) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nvox) packed[i] = R_EMPTY;
}

// one thread per (particle, x offset); offsets (-size-1 .. size]^3
template <typename T>
__global__ void k_rb_splat(const T* __restrict__ st, int64_t ld, int64_t p0, int64_t n,
                           const unsigned int* __restrict__ colors, const float* __restrict__ bbox, float inv_dx,
                           int size, int r0, int r1, int r2, unsigned long long* __restrict__ packed) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int oi = (int)blockIdx.y - size - 1;
  float p[3];
  int coord[3];
  for (int c = 0; c < 3; ++c) {
    p[c] = ((float)st[(int64_t)c * ld + p0 + i] - bbox[c]) * inv_dx;
    coord[c] = (int)p[c];
  }
  const unsigned long long col = colors ? (unsigned long long)colors[i] : 0xFFFFFFull;
  const int ix = coord[0] + oi;
  if (ix < 0 || ix >= r0) return;
  const float d0 = (float)ix - p[0];
  for (int oj = -size - 1; oj < size + 1; ++oj) {
    const int iy = coord[1] + oj;
    if (iy < 0 || iy >= r1) continue;
    const float d1 = (float)iy - p[1];
    for (int ok = -size - 1; ok < size + 1; ++ok) {
      const int iz = coord[2] + ok;
      if (iz < 0 || iz >= r2) continue;
      const float d2 = (float)iz - p[2];
      const float dist = sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
      float q = 51.0f * dist;  // 255 * 0.2 * dist
      q = (0.0f < q) ? q : 0.0f;
      q = (q < 255.0f) ? q : 255.0f;
      const unsigned long long v = ((unsigned long long)(long long)q << 24) + col;
      atomicMin(packed + ((int64_t)ix * r1 + iy) * r2 + iz, v);
    }
  }
}

// decode: colour bytes 0..2 (blue, green, red), SDF byte 3, each / 255
__global__ void k_rb_decode(const unsigned long long* __restrict__ packed, int64_t nvox, float* __restrict__ sdf,
                            float* __restrict__ color) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nvox) return;
  unsigned long long c = packed[i];
  for (int j = 2; j >= 0; --j) {
    color[3 * i + j] = (float)(long long)(c & 255ull) / 255.0f;
    c >>= 8;
  }
  sdf[i] = (float)(long long)(c & 255ull) / 255.0f;
}

// smooth (particle_sdf.py:223-233): 27-point mean inside, 1 on the boundary
__global__ void k_rb_smooth(const float* __restrict__ in, float* __restrict__ out, int r0, int r1, int r2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nvox = (int64_t)r0 * r1 * r2;
  if (i >= nvox) return;
  const int x = (int)(i / ((int64_t)r1 * r2)), y = (int)((i / r2) % r1), z = (int)(i % r2);
  if (x >= 1 && y >= 1 && z >= 1 && x < r0 - 1 && y < r1 - 1 && z < r2 - 1) {
    float sum = 0.0f;
    for (int a = -1; a < 2; ++a)
      for (int b = -1; b < 2; ++b)
        for (int c = -1; c < 2; ++c) sum += in[((int64_t)(x + a) * r1 + (y + b)) * r2 + (z + c)];
    out[i] = sum / 27.0f;
  } else {
    out[i] = 1.0f;
  }
}

// ------------------------------------------------------------------ trace
struct V3 {
  float x, y, z;
};
MPM_DI V3 v3(float a, float b, float c) { return V3{a, b, c}; }
MPM_DI V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
MPM_DI V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
MPM_DI V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
MPM_DI float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
MPM_DI float comp(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
MPM_DI V3 normalized(V3 a) {  // taichi's normalized(): (1 / norm) * v
  const float inv = 1.0f / sqrtf(dot(a, a));
  return a * inv;
}
// mapply_pos (tina/common.py:169-183): (M [p, 1])_xyz / (M [p, 1])_w, M row-major
MPM_DI V3 mapply_pos(const float* M, V3 p) {
  float r[3];
  for (int i = 0; i < 3; ++i) r[i] = M[4 * i + 3] + M[4 * i] * p.x + M[4 * i + 1] * p.y + M[4 * i + 2] * p.z;
  const float w = M[15] + M[12] * p.x + M[13] * p.y + M[14] * p.z;
  return v3(r[0] / w, r[1] / w, r[2] / w);
}

struct Volume {
  const float* sdf;
  const float* color;
  float b0[3], b1[3];
  int res[3];
  float threshold;
};
// sample_tex (particle_sdf.py:271-290), nc channels at stride nc
MPM_DI void sample_tex(const float* tex, int nc, const int* res, const float* q, float* out) {
  float pos[3], fx[3];
  int b[3], b1[3];
  for (int c = 0; c < 3; ++c) {
    pos[c] = q[c] * (float)res[c];
    const int t = (int)pos[c];
    b[c] = (t < res[c] - 1) ? t : res[c] - 1;
    fx[c] = pos[c] - (float)b[c];
    b1[c] = (b[c] + 1 < res[c] - 1) ? b[c] + 1 : res[c] - 1;
  }
  auto at = [&](int x, int y, int z, int ch) {
    return tex[(((int64_t)x * res[1] + y) * res[2] + z) * nc + ch];
  };
  for (int ch = 0; ch < nc; ++ch) {
    const float c00 = at(b[0], b[1], b[2], ch) * (1 - fx[0]) + at(b1[0], b[1], b[2], ch) * fx[0];
    const float c01 = at(b[0], b[1], b1[2], ch) * (1 - fx[0]) + at(b1[0], b[1], b1[2], ch) * fx[0];
    const float c10 = at(b[0], b1[1], b[2], ch) * (1 - fx[0]) + at(b1[0], b1[1], b[2], ch) * fx[0];
    const float c11 = at(b[0], b1[1], b1[2], ch) * (1 - fx[0]) + at(b1[0], b1[1], b1[2], ch) * fx[0];
    const float c0 = c00 * (1 - fx[1]) + c10 * fx[1];
    const float c1 = c01 * (1 - fx[1]) + c11 * fx[1];
    out[ch] = c0 * (1 - fx[2]) + c1 * fx[2];
  }
}
// pos normalised to the volume box; inside iff every coordinate is in [0, 1]
MPM_DI bool vol_coord(const Volume& V, V3 pos, float* q) {
  for (int c = 0; c < 3; ++c) q[c] = (comp(pos, c) - V.b0[c]) / (V.b1[c] - V.b0[c]);
  const float mn = fminf(fminf(q[0], q[1]), q[2]), mx = fmaxf(fmaxf(q[0], q[1]), q[2]);
  return mn >= 0.0f && mx <= 1.0f;
}
MPM_DI float sample_sdf(const Volume& V, V3 pos) {
  float q[3], s = 0.0f;
  if (vol_coord(V, pos, q)) {
    sample_tex(V.sdf, 1, V.res, q, &s);
    s = s - V.threshold;
  }
  return s;
}
MPM_DI V3 sample_color(const Volume& V, V3 pos) {
  float q[3], c[3] = {0.0f, 0.0f, 0.0f};
  if (vol_coord(V, pos, q)) sample_tex(V.color, 3, V.res, q, c);
  return v3(c[0], c[1], c[2]);
}
// central differences with d = 1e-3, normalised (particle_sdf.py:306-315)
MPM_DI V3 sample_normal(const Volume& V, V3 p) {
  const float d = 1e-3f;
  float n[3];
  for (int i = 0; i < 3; ++i) {
    V3 inc = p, dec = p;
    if (i == 0) { inc.x += d; dec.x -= d; }
    if (i == 1) { inc.y += d; dec.y -= d; }
    if (i == 2) { inc.z += d; dec.z -= d; }
    n[i] = (0.5f / d) * (sample_sdf(V, inc) - sample_sdf(V, dec));
  }
  return normalized(v3(n[0], n[1], n[2]));
}
// ray_aabb_intersection (plb/engine/renderer/renderer_utils.py:53-73)
MPM_DI bool ray_aabb(const float* bmin, const float* bmax, V3 o, V3 d, float& tnear, float& tfar) {
  bool hit = true;
  float near_i = -R_INF, far_i = R_INF;
  for (int i = 0; i < 3; ++i) {
    const float oi = comp(o, i), di = comp(d, i);
    if (di == 0.0f) {
      if (oi < bmin[i] || oi > bmax[i]) hit = false;
    } else {
      const float i1 = (bmin[i] - oi) / di, i2 = (bmax[i] - oi) / di;
      const float nf = (i2 < i1) ? i1 : i2;  // max(i1, i2)
      const float nn = (i1 < i2) ? i1 : i2;  // min(i1, i2)
      far_i = (nf < far_i) ? nf : far_i;
      near_i = (near_i < nn) ? nn : near_i;
    }
  }
  if (near_i > far_i) hit = false;
  tnear = near_i;
  tfar = far_i;
  return hit;
}

struct Camera {
  float m[32];  // V2W then W2V, row-major 4x4
};

template <typename TT>
__global__ void __launch_bounds__(128)
    k_rb_trace(const float* __restrict__ vsdf, const float* __restrict__ vcolor, const float* __restrict__ bbox,
               int r0, int r1, int r2, float threshold, Camera cam, int resx, int resy, float biasx, float biasy,
               const MpmToolDesc* __restrict__ tools, int t0, int nt, const double* __restrict__ pose,
               const float* __restrict__ tool_color, int show_particles, float* __restrict__ depth,
               float* __restrict__ normal, float* __restrict__ color, float* __restrict__ image) {
  const int64_t pix = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= (int64_t)resx * resy) return;
  const int px = (int)(pix / resy), py = (int)(pix % resy);
  const float* V2W = cam.m;
  const float* W2V = cam.m + 16;
  Volume V;
  V.sdf = vsdf;
  V.color = vcolor;
  V.res[0] = r0;
  V.res[1] = r1;
  V.res[2] = r2;
  for (int c = 0; c < 3; ++c) {
    V.b0[c] = bbox[c];
    V.b1[c] = bbox[3 + c];
  }
  V.threshold = threshold;
  // render_color: camera-plane point and ray direction of the pixel
  const float u = ((float)px + biasx) / (float)resx * 2.0f - 1.0f;
  const float w = ((float)py + biasy) / (float)resy * 2.0f - 1.0f;
  const V3 Pl = mapply_pos(V2W, v3(u, w, 1.0f));
  const V3 o = mapply_pos(V2W, v3(u, w, 0.0f));
  const V3 d = normalized(Pl - o);
  // next_hit: the ground first
  float closest = 0.99f;
  V3 nrm = v3(0.0f, 1.0f, 0.0f);
  V3 col = v3(0.3f * 0.3f, 0.5f * 0.3f, 0.7f * 0.3f);
  // the tools, sphere traced with their SDFs at the given pose
  if (nt > 0) {
    int j = 0, sid = 0;
    float dist = 0.0f, sval = R_INF;
    V3 pp = o;
    while (j < 200 && dist < R_DIST_LIMIT && sval > 1e-8f) {
      pp = o + d * dist;
      sval = R_INF;
      for (int i = 0; i < nt; ++i) {
        Tool<TT> tl;
        Pose<TT> P;
        to_tool(tools[t0 + i], tl);
        to_pose(pose + 8 * (t0 + i), P);
        const TT q[3] = {TT(pp.x), TT(pp.y), TT(pp.z)};
        const float dd = (float)tool_sdf(tl, P, q);
        if (dd < sval) {
          sval = dd;
          sid = i;
        }
      }
      dist += sval;
      ++j;
    }
    const float dz = mapply_pos(W2V, pp).z;
    if (dz < closest && dz < R_DIST_LIMIT) {
      closest = dz;
      Tool<TT> tl;
      Pose<TT> P;
      to_tool(tools[t0 + sid], tl);
      to_pose(pose + 8 * (t0 + sid), P);
      const V3 h = o + d * dist;
      const TT q[3] = {TT(h.x), TT(h.y), TT(h.z)};
      TT n[3];
      tool_normal(tl, P, q, n);
      nrm = v3((float)n[0], (float)n[1], (float)n[2]);
      col = v3(tool_color[3 * (t0 + sid)], tool_color[3 * (t0 + sid) + 1], tool_color[3 * (t0 + sid) + 2]);
    }
  }
  // the particles' SDF
  float tnear, tfar;
  if (show_particles && ray_aabb(V.b0, V.b1, o, d, tnear, tfar)) {
    tnear = (0.0f < tnear) ? tnear : 0.0f;
    V3 pos = o + d * (tnear + 1e-4f);
    V3 step = v3(0.0f, 0.0f, 0.0f);
    for (int j = 0; j < 500; ++j) {
      const float s = sample_sdf(V, pos);
      if (s < 0.0f) {
        V3 back = step;
        for (int k = 0; k < 20; ++k) {
          back = back * 0.5f;
          if (sample_sdf(V, pos - back) < 0.0f) pos = pos - back;
        }
        const float dz = mapply_pos(W2V, pos).z;
        if (dz < closest) {
          closest = dz;
          nrm = sample_normal(V, pos);
          col = sample_color(V, pos);
        }
        break;
      }
      const float a = s * 0.005f;
      step = d * ((a < 0.002f) ? 0.002f : a);
      pos = pos + step;
    }
  }
  col = col * 3.0f;
  depth[pix] = closest;
  normal[3 * pix] = nrm.x;
  normal[3 * pix + 1] = nrm.y;
  normal[3 * pix + 2] = nrm.z;
  color[3 * pix] = col.x;
  color[3 * pix + 1] = col.y;
  color[3 * pix + 2] = col.z;
  if (image) {
    // Lighting.shade_color with Diffuse = Lambert * colour: ambient 0.1 * colour
    // plus the default light (direction (1,2,3) normalised, colour 0.9) times colour / pi
    const float il = 1.0f / sqrtf(14.0f);
    const float cos_i = nrm.x * il + nrm.y * (2.0f * il) + nrm.z * (3.0f * il);
    const float lam = cos_i > 0.0f ? cos_i * 0.9f * (1.0f / 3.14159265358979f) : 0.0f;
    image[3 * pix] = 0.1f * col.x + lam * col.x;
    image[3 * pix + 1] = 0.1f * col.y + lam * col.y;
    image[3 * pix + 2] = 0.1f * col.z + lam * col.z;
  }
}

inline unsigned nblk(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

}  // namespace

template <typename T>
cudaError_t launch_render_bake(const LaunchCtx& L, const T* st, int64_t p0, int64_t n, const unsigned int* colors,
                               const MpmRenderVolume& v) {
  const int64_t nvox = (int64_t)v.res[0] * v.res[1] * v.res[2];
  const float dx_f = (float)v.dx, inv_dx = (float)(1.0 / v.dx);
  MPM_LAUNCH(L, MPM_K_OTHER, k_rb_init, 1, 32, v.kbox);
  if (n > 0) MPM_LAUNCH(L, MPM_K_OTHER, k_rb_box<T>, nblk(n, 256), 256, st, L.p->ld, p0, n, inv_dx, v.kbox);
  MPM_LAUNCH(L, MPM_K_OTHER, k_rb_box_finish, 1, 32, v.kbox, dx_f, v.dx, v.res[0], v.res[1], v.res[2], v.bbox,
             L.status);
  MPM_LAUNCH(L, MPM_K_OTHER, k_rb_fill, nblk(nvox, 256), 256, v.packed, nvox);
  if (n > 0) {
    dim3 grid(nblk(n, 128), 2 * v.bake_size + 2);
    MPM_LAUNCH(L, MPM_K_OTHER, k_rb_splat<T>, grid, 128, st, L.p->ld, p0, n, colors, v.bbox, inv_dx, v.bake_size,
               v.res[0], v.res[1], v.res[2], v.packed);
  }
  MPM_LAUNCH(L, MPM_K_OTHER, k_rb_decode, nblk(nvox, 256), 256, v.packed, nvox, v.sdf, v.color);
  MPM_LAUNCH(L, MPM_K_OTHER, k_rb_smooth, nblk(nvox, 256), 256, v.sdf, v.sdf_copy, v.res[0], v.res[1], v.res[2]);
  MPM_LAUNCH(L, MPM_K_OTHER, k_rb_smooth, nblk(nvox, 256), 256, v.sdf_copy, v.sdf, v.res[0], v.res[1], v.res[2]);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_render_trace(const LaunchCtx& L, const MpmRenderVolume& v, const MpmRenderView& view, int t0,
                                int nt, const double* pose, const float* tool_color, float* depth, float* normal,
                                float* color, float* image) {
  Camera cam;
  for (int k = 0; k < 16; ++k) {
    cam.m[k] = view.v2w[k];
    cam.m[16 + k] = view.w2v[k];
  }
  const int64_t npix = (int64_t)view.res[0] * view.res[1];
  MPM_LAUNCH(L, MPM_K_OTHER, k_rb_trace<T>, nblk(npix, 128), 128, v.sdf, v.color, v.bbox, v.res[0], v.res[1],
             v.res[2], view.sdf_threshold, cam, view.res[0], view.res[1], view.bias[0], view.bias[1], L.tools, t0,
             nt, pose, tool_color, view.show_particles, depth, normal, color, image);
  return cudaGetLastError();
}

#define MPM_INST_RENDER(T)                                                                                         \
  template cudaError_t launch_render_bake<T>(const LaunchCtx&, const T*, int64_t, int64_t, const unsigned int*,    \
                                             const MpmRenderVolume&);                                              \
  template cudaError_t launch_render_trace<T>(const LaunchCtx&, const MpmRenderVolume&, const MpmRenderView&, int, \
                                              int, const double*, const float*, float*, float*, float*, float*);
MPM_INST_RENDER(float)
MPM_INST_RENDER(double)

}  // namespace mpm
