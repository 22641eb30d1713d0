// Particle re-sort by (scene, 4^3 grid block, cell) and its adjoint.
//
// The scatter (p2g, g2p.grad) and gather (g2p, p2g.grad) kernels want the
// particles of one cell next to each other and the cells of one block next
// to each other: their warp runs then cover one cell, and a CTA's stencils
// stay inside a few grid blocks.  Particles drift between cells as the
// simulation runs, so the frames are re-sorted every few substeps.  The
// reference has no such step (Taichi's dense fields are scattered into in
// launch order, plb/engine/mpm_simulator.py:199-225); a re-sort only
// permutes particles inside their scene, so losses and action gradients do
// not depend on it.
//
// The sort is a stable least-significant-digit radix sort over 32-bit keys
// ((scene * blocks_per_scene + block) * 64 + cell), 8 bits per pass and only
// as many passes as the largest key needs (three for 64 scenes of a 64^3
// grid).  Each pass: a digit histogram per tile of 1024 keys, an exclusive
// scan of each digit's row of tile counts (one CTA per digit), and a scatter
// that adds the counts of the smaller digits and ranks the keys of its tile
// stably (a warp takes 4 rounds of 32 consecutive keys; peers of one digit
// are found with __match_any_sync).  Tiles of 1024 keys rather than 4096 put
// four times as many CTAs on the SMs (re-sort of 1.2M particles 116.8 ->
// 108.9 us).  Ties keep their original order, so the permutation is
// deterministic.  The 24 rows of the frame are then gathered once through
// the permutation into the destination frame; the adjoint scatters a frame
// gradient back through the same permutation.
#include "mpm_kernels.cuh"
#include "mpm_launch.h"

namespace mpm {

namespace {
constexpr int kSortThreads = 256;  // 8 warps
constexpr int kSortRounds = 4;     // keys per lane in the scatter
constexpr int kSortTile = kSortThreads * kSortRounds;
constexpr int kRadix = 256;
constexpr int kFrameRows = 24;

unsigned blocks_of(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }
}  // namespace

MPM_DI float mul_rn(float a, float b) { return __fmul_rn(a, b); }
MPM_DI double mul_rn(double a, double b) { return __dmul_rn(a, b); }
MPM_DI float sub_rn(float a, float b) { return __fsub_rn(a, b); }
MPM_DI double sub_rn(double a, double b) { return __dsub_rn(a, b); }

// key and index of particle p; the base cell truncates (x n - 1/2) toward
// zero and clamps it to the grid, as the stencil's base does (a product and
// a difference each rounded, no fused multiply-add)
template <typename T>
__global__ void __launch_bounds__(256) k_sort_keys(const T* __restrict__ st, int64_t ld, int64_t n, int n_grid,
                                                   const int* __restrict__ pscene, uint32_t* __restrict__ keys,
                                                   int32_t* __restrict__ vals) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  int b[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int i = (int)sub_rn(mul_rn(st[(int64_t)d * ld + p], T(n_grid)), T(0.5));
    b[d] = i < 0 ? 0 : (i > n_grid - 1 ? n_grid - 1 : i);
  }
  const uint32_t nb = (uint32_t)(n_grid >> 2);
  const uint32_t blk = (((uint32_t)b[0] >> 2) * nb + ((uint32_t)b[1] >> 2)) * nb + ((uint32_t)b[2] >> 2);
  const uint32_t cell = (((uint32_t)b[0] & 3u) << 4) | (((uint32_t)b[1] & 3u) << 2) | ((uint32_t)b[2] & 3u);
  keys[p] = ((uint32_t)pscene[p] * (nb * nb * nb) + blk) * 64u + cell;
  vals[p] = (int32_t)p;
}

// digit counts of one tile: hist[digit * n_tiles + tile]
__global__ void __launch_bounds__(kSortThreads) k_radix_hist(const uint32_t* __restrict__ keys, int64_t n, int shift,
                                                             uint32_t* __restrict__ hist, int n_tiles) {
  __shared__ unsigned cnt[kRadix];
  cnt[threadIdx.x] = 0u;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kSortTile;
#pragma unroll 4
  for (int i = 0; i < kSortRounds; ++i) {
    const int64_t q = base + (int64_t)i * kSortThreads + threadIdx.x;
    if (q < n) atomicAdd(&cnt[(keys[q] >> shift) & (kRadix - 1)], 1u);
  }
  __syncthreads();
  hist[(int64_t)threadIdx.x * n_tiles + blockIdx.x] = cnt[threadIdx.x];
}

// exclusive scan over 256 values, one per thread of a 256-thread CTA; also
// returns the total (ws: 8 words of shared memory)
MPM_DI unsigned block_scan256(unsigned v, unsigned* ws, unsigned& total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned inc = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const unsigned y = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= d) inc += y;
  }
  if (lane == 31) ws[w] = inc;
  __syncthreads();
  unsigned before = 0u, all = 0u;
#pragma unroll
  for (int k = 0; k < kSortThreads / 32; ++k) {
    const unsigned t = ws[k];
    before += k < w ? t : 0u;
    all += t;
  }
  __syncthreads();  // ws may be reused
  total = all;
  return before + inc - v;
}

// per digit (one CTA each): exclusive scan of its row hist[d][0 .. n_tiles)
// in place, and the digit's total count in digit_total[d]
__global__ void __launch_bounds__(kSortThreads) k_radix_scan(uint32_t* __restrict__ hist, int n_tiles,
                                                             uint32_t* __restrict__ digit_total) {
  __shared__ unsigned ws[kSortThreads / 32];
  uint32_t* row = hist + (int64_t)blockIdx.x * n_tiles;
  unsigned carry = 0u;
  for (int c = 0; c < n_tiles; c += kSortThreads) {
    const int t = c + threadIdx.x;
    const unsigned v = t < n_tiles ? row[t] : 0u;
    unsigned sum;
    const unsigned ex = block_scan256(v, ws, sum);
    if (t < n_tiles) row[t] = carry + ex;
    carry += sum;
  }
  if (threadIdx.x == 0) digit_total[blockIdx.x] = carry;
}

// stable scatter of one pass: a key's place is the scanned count of its
// digit in earlier tiles, plus the keys of that digit before it in this tile
__global__ void __launch_bounds__(kSortThreads) k_radix_scatter(const uint32_t* __restrict__ kin,
                                                                const int32_t* __restrict__ vin,
                                                                uint32_t* __restrict__ kout,
                                                                int32_t* __restrict__ vout, int64_t n, int shift,
                                                                const uint32_t* __restrict__ hist, int n_tiles,
                                                                const uint32_t* __restrict__ digit_total) {
  __shared__ unsigned warp_cnt[kSortThreads / 32][kRadix];
  __shared__ unsigned tile_off[kRadix];
  __shared__ unsigned ws[kSortThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int d = lane; d < kRadix; d += 32) warp_cnt[w][d] = 0u;
  {  // keys of smaller digits, then keys of this digit in earlier tiles
    unsigned all;
    const unsigned below_digit = block_scan256(digit_total[threadIdx.x], ws, all);
    tile_off[threadIdx.x] = below_digit + hist[(int64_t)threadIdx.x * n_tiles + blockIdx.x];
  }
  __syncwarp();
  const int64_t base = (int64_t)blockIdx.x * kSortTile + (int64_t)w * (32 * kSortRounds);
  const unsigned below = (1u << lane) - 1u;
  uint32_t key[kSortRounds];
  int32_t val[kSortRounds];
  unsigned rank[kSortRounds];
#pragma unroll
  for (int i = 0; i < kSortRounds; ++i) {
    const int64_t q = base + (int64_t)i * 32 + lane;
    const bool ok = q < n;
    key[i] = ok ? kin[q] : 0u;
    val[i] = ok ? vin[q] : 0;
    const unsigned d = (key[i] >> shift) & (kRadix - 1);
    // lanes past the end match nobody (a value no digit takes)
    const unsigned peers = __match_any_sync(0xffffffffu, ok ? d : (unsigned)kRadix + lane);
    const unsigned seen = warp_cnt[w][d];
    const unsigned before = ok ? seen : 0u;
    __syncwarp();
    if (ok && lane == __ffs(peers) - 1) warp_cnt[w][d] = before + __popc(peers);
    __syncwarp();
    rank[i] = before + __popc(peers & below);
  }
  __syncthreads();
  {  // per digit: the counts of the warps before each warp
    const int d = threadIdx.x;
    unsigned run = 0u;
#pragma unroll
    for (int v = 0; v < kSortThreads / 32; ++v) {
      const unsigned c = warp_cnt[v][d];
      warp_cnt[v][d] = run;
      run += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < kSortRounds; ++i) {
    const int64_t q = base + (int64_t)i * 32 + lane;
    if (q < n) {
      const unsigned d = (key[i] >> shift) & (kRadix - 1);
      const unsigned pos = tile_off[d] + warp_cnt[w][d] + rank[i];
      kout[pos] = key[i];
      vout[pos] = val[i];
    }
  }
}

// dst[:, i] = src[:, perm[i]] over the 24 rows of a frame
template <typename T>
__global__ void __launch_bounds__(256) k_sort_gather(const T* __restrict__ src, T* __restrict__ dst, int64_t ld,
                                                     int64_t n, const int32_t* __restrict__ perm) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int64_t q = perm[p];
#pragma unroll
  for (int r = 0; r < kFrameRows; ++r) dst[(int64_t)r * ld + p] = src[(int64_t)r * ld + q];
}

// dst[:, perm[i]] = src[:, i]: the adjoint of k_sort_gather
template <typename T>
__global__ void __launch_bounds__(256) k_unsort_scatter(const T* __restrict__ src, T* __restrict__ dst, int64_t ld,
                                                        int64_t n, const int32_t* __restrict__ perm) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int64_t q = perm[p];
#pragma unroll
  for (int r = 0; r < kFrameRows; ++r) dst[(int64_t)r * ld + q] = src[(int64_t)r * ld + p];
}

int sort_tiles(int64_t n) { return (int)((n + kSortTile - 1) / kSortTile); }
// the (digit, tile) table and the 256 digit totals behind it
size_t sort_hist_words(int64_t n) { return (size_t)kRadix * (size_t)((sort_tiles(n) > 0 ? sort_tiles(n) : 1) + 1); }

int sort_key_bits(int n_scenes, int n_grid) {
  const uint64_t nb = (uint64_t)(n_grid / 4);
  const uint64_t max_key = (uint64_t)n_scenes * nb * nb * nb * 64u - 1u;
  int bits = 0;
  while (bits < 64 && (max_key >> bits) != 0u) ++bits;
  return bits;
}

template <typename T>
cudaError_t launch_sort_frame(const LaunchCtx& L, const T* src, T* dst, int32_t* perm, const SortScratch& s) {
  const MpmParams& p = *L.p;
  const int64_t n = p.n_particles;
  if (n == 0) return cudaSuccess;
  const int bits = sort_key_bits(p.n_scenes, p.n_grid);
  const int passes = bits <= 0 ? 0 : (bits + 7) / 8;
  const int tiles = sort_tiles(n);
  // ping-pong so that the last pass writes its indices into perm
  uint32_t* k[2] = {s.keys_a, s.keys_b};
  int32_t* v[2] = {passes % 2 == 0 ? perm : s.vals_b, passes % 2 == 0 ? s.vals_b : perm};
  MPM_LAUNCH(L, MPM_K_SORT, k_sort_keys<T>, blocks_of(n, 256), 256, src, p.ld, n, p.n_grid, L.pscene, k[0], v[0]);
  uint32_t* totals = s.hist + (size_t)kRadix * tiles;
  for (int i = 0; i < passes; ++i) {
    const int a = i & 1, b = a ^ 1;
    MPM_LAUNCH(L, MPM_K_SORT, k_radix_hist, (unsigned)tiles, kSortThreads, k[a], n, 8 * i, s.hist, tiles);
    MPM_LAUNCH(L, MPM_K_SORT, k_radix_scan, (unsigned)kRadix, kSortThreads, s.hist, tiles, totals);
    MPM_LAUNCH(L, MPM_K_SORT, k_radix_scatter, (unsigned)tiles, kSortThreads, k[a], v[a], k[b], v[b], n, 8 * i,
               (const uint32_t*)s.hist, tiles, (const uint32_t*)totals);
  }
  MPM_LAUNCH(L, MPM_K_SORT, k_sort_gather<T>, blocks_of(n, 256), 256, src, dst, p.ld, n, (const int32_t*)perm);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_unsort_frame(const LaunchCtx& L, const T* src, T* dst, const int32_t* perm) {
  const MpmParams& p = *L.p;
  const int64_t n = p.n_particles;
  if (n == 0) return cudaSuccess;
  MPM_LAUNCH(L, MPM_K_SORT, k_unsort_scatter<T>, blocks_of(n, 256), 256, src, dst, p.ld, n, perm);
  return cudaGetLastError();
}

template cudaError_t launch_sort_frame<float>(const LaunchCtx&, const float*, float*, int32_t*, const SortScratch&);
template cudaError_t launch_sort_frame<double>(const LaunchCtx&, const double*, double*, int32_t*,
                                               const SortScratch&);
template cudaError_t launch_unsort_frame<float>(const LaunchCtx&, const float*, float*, const int32_t*);
template cudaError_t launch_unsort_frame<double>(const LaunchCtx&, const double*, double*, const int32_t*);

}  // namespace mpm
