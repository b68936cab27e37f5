// Mapping (K1), tile binning (K2), gridder (K3) and degridder (K4).
//
// Reference behaviour: processing_components/griddata/gridding.py
//   convolution_mapping            :24-96
//   grid_visibility_to_griddata    :99-133
//   degrid_visibility_from_griddata:233-267
//
// Data flow on the device
//   k_map      uvw, frequency -> RowMap + bin key per row, histogram of keys
//   k_scan     exclusive scan of the histogram -> bin offsets
//   k_scatter  rows -> bin order (sidx = original row id, smap = RowMap)
//   k_grid     one CTA per chunk of sorted rows; each run of rows of one
//              (chan, w-plane, uv-tile) bin accumulates into a shared-memory
//              subgrid (tile + kernel halo) that is flushed to the grid with
//              one vector atomic per touched cell
//   k_degrid   same chunking; the bin's subgrid is staged in shared memory and
//              each row is a warp-wide dot product reduced with shuffles
#include <cuda.h>  // CUtensorMap and its enums; the encoder is looked up in the driver at run time

#include <cstdarg>
#include <cstring>
#include <atomic>
#include <mutex>
#include <string>

#include "common.cuh"
#include "mapping.cuh"

namespace arlgpu {

static thread_local std::string g_last_error;

int fail(int code, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char *what, const char *file, int line) {
  return fail(ARLGPU_ERR_CUDA, "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
}

const char *last_error() { return g_last_error.c_str(); }

static std::atomic<unsigned long long> g_launches{0};

// Kernel-variant choices (set by the autotuner through arlgpu_set_tuning).
static std::atomic<int> g_tune_grid_kernel{4};    // 0: atomics + TwoSum, 1: band owner, 2: lean, 3: uncompensated,
                                                  // 4: fixed point + residual, 5: fixed point
static std::atomic<int> g_tune_degrid_kernel{3};  // 0: warp per row, 1: batched rows, 2: lean, 3: lean packed FMA
static std::atomic<int> g_tune_subgrid{0};        // subgrid edge SG (0: automatic)
static std::atomic<int> g_tune_chunk{512};        // sorted rows per gridder / degridder CTA
static std::atomic<int> g_tune_persistent{2};     // lean / fixed-point kernels: 0 = one CTA per chunk, 1 = resident grid taking every gridDim-th chunk, 2 = resident grid fed by a device work queue
static std::atomic<int> g_tune_dsfft{1};          // FP32C inverse transforms: 1 = double-single FFT, 0 = cuFFT FP64
static std::atomic<int> g_tune_small_rows{2};     // rows per warp in the FP32C gridder when S <= 8
static std::atomic<int> g_tune_small_rows_dg{4};  // rows per warp in the packed degridder when S <= 8
static std::atomic<int> g_tune_lanes{0};          // lanes per row for every segment (0: by support)
static std::atomic<int> g_tune_gather{1};         // FP32C gridder, one polarisation: rows copied into bin order first
static std::atomic<int> g_tune_stash{1};          // packed degridder, one polarisation: row set-up from the footprint pass
void count_launch(unsigned n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
bool tune_dsfft() { return g_tune_dsfft.load() != 0; }

// K1: mapping + bin key + histogram.
__global__ void k_map(const double *__restrict__ uvw, const double *__restrict__ freq, int64_t nvis,
                      Geom g, uint32_t *__restrict__ keys, RowMap *__restrict__ maps,
                      uint32_t *__restrict__ hist) {
  const int lane = threadIdx.x & 31;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < nvis;
       base += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = base + threadIdx.x;
    uint32_t key = 0xffffffffu;
    if (r < nvis) {
      Mapped m = map_row(uvw[3 * r], uvw[3 * r + 1], uvw[3 * r + 2], freq[r], g);
      RowMap rm;
      rm.pu = m.pu;
      rm.pv = m.pv;
      rm.sub = (uint32_t)m.uf | ((uint32_t)m.vf << 8) | ((uint32_t)m.zc << 16);
      rm.cz = (uint32_t)m.ch | ((uint32_t)m.zg << 16);
      key = m.ok ? bin_of(m.ch, m.zg, m.pu, m.pv, g) : g.nbins;
      st_map16(maps + r, rm);
      keys[r] = key;
    }
    // Warp-aggregated histogram increment.
    unsigned same = __match_any_sync(0xffffffffu, key);
    if (key != 0xffffffffu && lane == __ffs(same) - 1) atomicAdd(&hist[key], (uint32_t)__popc(same));
  }
}

// Mapping export for arlgpu_convolution_mapping: the same indices the plan
// uses (map_raw), clamped only to fit int32.
__global__ void k_map_export(const double *__restrict__ uvw, const double *__restrict__ freq, int64_t nvis,
                             Geom g, int32_t *pu, int32_t *puo, int32_t *pv, int32_t *pvo, int32_t *pwg,
                             int32_t *pwc, int32_t *pf, unsigned long long *nbad) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nvis;
       r += (int64_t)gridDim.x * blockDim.x) {
    const double u = uvw[3 * r], v = uvw[3 * r + 1], w = uvw[3 * r + 2], f = freq[r];
    const RawMap m = map_raw(u, v, w, f, g);
    auto c = [](double x) { return (int32_t)fmax(fmin(x, 2e9), -2e9); };
    pu[r] = c(m.pu);
    pv[r] = c(m.pv);
    puo[r] = c(m.uf);
    pvo[r] = c(m.vf);
    pwg[r] = c(m.zg);
    pwc[r] = c(m.zc);
    pf[r] = c(m.ch);
    if (!map_row(u, v, w, f, g).ok) atomicAdd(nbad, 1ull);
  }
}

// K2a: exclusive scan of hist[0..n) into off[0..n]; one CTA of 1024 threads.
__global__ void k_scan(const uint32_t *__restrict__ hist, uint32_t n, uint32_t *__restrict__ off,
                       int64_t *n_bad_dev, uint32_t nbins) {
  __shared__ uint32_t part[1024];
  const uint32_t per = (n + blockDim.x - 1) / blockDim.x;
  const uint32_t b = threadIdx.x * per;
  const uint32_t e = min(b + per, n);
  uint32_t s = 0;
  for (uint32_t i = b; i < e; ++i) s += hist[i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (uint32_t d = 1; d < blockDim.x; d <<= 1) {
    uint32_t t = threadIdx.x >= d ? part[threadIdx.x - d] : 0;
    __syncthreads();
    part[threadIdx.x] += t;
    __syncthreads();
  }
  uint32_t run = threadIdx.x ? part[threadIdx.x - 1] : 0;
  for (uint32_t i = b; i < e; ++i) {
    off[i] = run;
    run += hist[i];
  }
  if (threadIdx.x == blockDim.x - 1) off[n] = part[blockDim.x - 1];
  if (threadIdx.x == 0 && n_bad_dev) *n_bad_dev = (int64_t)hist[nbins];
}

// Large histograms (more than kScanTile bins): a three-pass scan.  Pass 1:
// block b scans bins [b kScanTile, (b + 1) kScanTile) into off (exclusive,
// block-local) and writes its total; pass 2: one CTA scans the totals;
// pass 3: each block adds its offset.  Integer sums, so the result equals
// the single-CTA scan's.
constexpr uint32_t kScanTile = 8192;  // 1024 threads x 8 bins

__device__ __forceinline__ uint32_t block_excl_scan_1024(uint32_t v, uint32_t *s_warp, uint32_t *total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = s_warp[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    s_warp[lane] = w;  // inclusive over warps
  }
  __syncthreads();
  const uint32_t before = warp ? s_warp[warp - 1] : 0u;
  *total = s_warp[31];
  return before + x - v;
}

__global__ void __launch_bounds__(1024) k_scan_tiles(const uint32_t *__restrict__ hist, uint32_t n,
                                                     uint32_t *__restrict__ off, uint32_t *__restrict__ tile_sum) {
  __shared__ uint32_t s_warp[32];
  const uint32_t b0 = blockIdx.x * kScanTile + threadIdx.x * 8;
  uint32_t v[8], t = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    v[k] = b0 + k < n ? hist[b0 + k] : 0u;
    t += v[k];
  }
  uint32_t total;
  uint32_t run = block_excl_scan_1024(t, s_warp, &total);
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    if (b0 + k < n) off[b0 + k] = run;
    run += v[k];
  }
  if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) k_scan_totals(uint32_t *__restrict__ tile_sum, uint32_t ntiles,
                                                      uint32_t *__restrict__ off, uint32_t n,
                                                      int64_t *n_bad_dev, const uint32_t *__restrict__ hist,
                                                      uint32_t nbins) {
  __shared__ uint32_t s_warp[32];
  // ntiles <= 8192: eight totals per thread
  const uint32_t b0 = threadIdx.x * 8;
  uint32_t v[8], t = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    v[k] = b0 + k < ntiles ? tile_sum[b0 + k] : 0u;
    t += v[k];
  }
  uint32_t total;
  uint32_t run = block_excl_scan_1024(t, s_warp, &total);
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    if (b0 + k < ntiles) tile_sum[b0 + k] = run;
    run += v[k];
  }
  if (threadIdx.x == 0) {
    off[n] = total;
    if (n_bad_dev) *n_bad_dev = (int64_t)hist[nbins];
  }
}

__global__ void k_scan_add(uint32_t *__restrict__ off, uint32_t n, const uint32_t *__restrict__ tile_sum) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) off[i] += tile_sum[i / kScanTile];
}

// K2b: scatter rows into bin order (hist reused as zeroed per-bin cursors).
__global__ void k_scatter(const uint32_t *__restrict__ keys, const RowMap *__restrict__ maps, int64_t nvis,
                          const uint32_t *__restrict__ off, uint32_t *__restrict__ cursor,
                          uint32_t *__restrict__ sidx, RowMap *__restrict__ smap) {
  const int lane = threadIdx.x & 31;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < nvis;
       base += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = base + threadIdx.x;
    uint32_t key = r < nvis ? keys[r] : 0xffffffffu;
    unsigned same = __match_any_sync(0xffffffffu, key);
    int leader = __ffs(same) - 1;
    uint32_t start = 0;
    if (key != 0xffffffffu && lane == leader) start = atomicAdd(&cursor[key], (uint32_t)__popc(same));
    start = __shfl_sync(0xffffffffu, start, leader);
    if (key != 0xffffffffu) {
      uint32_t pos = off[key] + start + __popc(same & ((1u << lane) - 1u));
      sidx[pos] = (uint32_t)r;
      st_map16(smap + pos, ld_map16(maps + r));
    }
  }
}

// Mean w of the rows of each grid w-plane (over all channels), from a built
// plan, in two deterministic steps.  The sorted rows of bin run (c, z) (all
// uv-tiles of channel c, plane z) are split into P equal shares; block
// (c, z, p) sums w over its share (fixed per-thread order, fixed tree), then
// one thread per plane adds its shares in (c, p) order and divides by the
// row count.  Planes without rows get 0.
__global__ void k_plane_wsum(const double *__restrict__ uvw, const uint32_t *__restrict__ sidx,
                             const uint32_t *__restrict__ off, Geom g, uint32_t P, double *__restrict__ part) {
  __shared__ double ssum[256];
  const uint32_t item = blockIdx.x, p = item % P, cz = item / P;
  const uint32_t tiles = (uint32_t)g.ntv * g.ntu;
  const uint32_t r0 = off[cz * tiles], len = off[(cz + 1) * tiles] - r0;
  const uint32_t a = r0 + (uint32_t)(((uint64_t)len * p) / P), b = r0 + (uint32_t)(((uint64_t)len * (p + 1)) / P);
  double sum = 0.0;
  for (uint32_t r = a + threadIdx.x; r < b; r += blockDim.x) sum += uvw[3 * (size_t)sidx[r] + 2];
  ssum[threadIdx.x] = sum;
  __syncthreads();
  for (int d = blockDim.x / 2; d > 0; d >>= 1) {
    if (threadIdx.x < d) ssum[threadIdx.x] += ssum[threadIdx.x + d];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[item] = ssum[0];
}

__global__ void k_plane_wmean(const double *__restrict__ part, const uint32_t *__restrict__ off, Geom g, uint32_t P,
                              double *__restrict__ wmean) {
  const int z = blockIdx.x * blockDim.x + threadIdx.x;
  if (z >= g.nw) return;
  const uint32_t tiles = (uint32_t)g.ntv * g.ntu;
  double sum = 0.0;
  uint64_t cnt = 0;
  for (int c = 0; c < g.nchan; ++c) {
    const uint32_t cz = (uint32_t)c * g.nw + z;
    for (uint32_t p = 0; p < P; ++p) sum += part[cz * P + p];
    cnt += off[(cz + 1) * tiles] - off[cz * tiles];
  }
  wmean[z] = cnt ? sum / (double)cnt : 0.0;
}

// ---------------------------------------------------------------------------
// Complex helpers
// ---------------------------------------------------------------------------
template <typename CT> __device__ __forceinline__ CT czero();
template <> __device__ __forceinline__ float2 czero<float2>() { return make_float2(0.f, 0.f); }
template <> __device__ __forceinline__ double2 czero<double2>() { return make_double2(0.0, 0.0); }

template <typename CT> __device__ __forceinline__ void red_global(CT *p, CT v);
template <> __device__ __forceinline__ void red_global<float2>(float2 *p, float2 v) { atomicAdd(p, v); }
template <> __device__ __forceinline__ void red_global<double2>(double2 *p, double2 v) {
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
}

// Shared-memory accumulation of one complex value.  The FP32 variant keeps a
// compensation term per cell: the atomic returns the value it replaced, so the
// exact rounding error of that addition (Knuth TwoSum) can be added to a second
// accumulator; the cell's value is sum + compensation.
template <typename R> struct SmemAcc;
template <> struct SmemAcc<float> {
  static constexpr int kWords = 2;  // float2 sum + float2 compensation per cell
  __device__ static __forceinline__ void add(float2 *sum, float2 *comp, float2 v) {
    float o = atomicAdd(&sum->x, v.x);
    float s = o + v.x, bp = s - o;
    float e = (o - (s - bp)) + (v.x - bp);
    atomicAdd(&comp->x, e);
    o = atomicAdd(&sum->y, v.y);
    s = o + v.y;
    bp = s - o;
    e = (o - (s - bp)) + (v.y - bp);
    atomicAdd(&comp->y, e);
  }
};
template <> struct SmemAcc<double> {
  static constexpr int kWords = 1;
  __device__ static __forceinline__ void add(double2 *sum, double2 *, double2 v) {
    atomicAdd(&sum->x, v.x);
    atomicAdd(&sum->y, v.y);
  }
};

// Uncompensated shared-memory accumulation (grid_kernel 3, kept only to
// measure what the compensation costs; not part of the FP32C contract).
template <typename R> struct PlainAcc {
  static constexpr int kWords = 1;
  __device__ static __forceinline__ void add(typename Cplx<R>::T *sum, typename Cplx<R>::T *,
                                             typename Cplx<R>::T v) {
    atomicAdd(&sum->x, v.x);
    atomicAdd(&sum->y, v.y);
  }
  // Planar layout: one real value into its own plane.
  __device__ static __forceinline__ void add1(R *sum, R *, R v) { atomicAdd(sum, v); }
};

// Planar (re / im in separate planes) compensated accumulation of one real
// value: FP32 adds the atomic's rounding error (TwoSum on the value the atomic
// replaced) to a compensation plane; FP64 adds directly.
template <typename R> struct PlanarAcc;
template <> struct PlanarAcc<float> {
  static constexpr int kWords = 2;
  __device__ static __forceinline__ void add1(float *sum, float *comp, float v) {
    const float o = atomicAdd(sum, v);
    const float s = o + v, bp = s - o;
    atomicAdd(comp, (o - (s - bp)) + (v - bp));
  }
};
template <> struct PlanarAcc<double> {
  static constexpr int kWords = 1;
  __device__ static __forceinline__ void add1(double *sum, double *, double v) { atomicAdd(sum, v); }
};

template <typename R> struct VisT;
template <> struct VisT<float> { using C = float2; using W = float; };
template <> struct VisT<double> { using C = double2; using W = double; };

struct SegInfo {
  uint32_t end;
  int ch, zg, u0, v0;
  bool direct;
};

// Resolve the bin run that starts at sorted position pos inside [.., c1).
__device__ __forceinline__ SegInfo seg_at(uint32_t pos, uint32_t c1, const RowMap *smap,
                                          const uint32_t *off, const Geom &g) {
  SegInfo s;
  RowMap m = smap[pos];
  s.ch = m.cz & 0xffff;
  s.zg = m.cz >> 16;
  uint32_t key = bin_of(s.ch, s.zg, m.pu, m.pv, g);
  s.end = min(off[key + 1], c1);
  s.u0 = (m.pu / g.T) * g.T - (g.S >> 1);
  s.v0 = (m.pv / g.T) * g.T - (g.S >> 1);
  // Few rows for a whole subgrid: go straight to global memory.
  s.direct = (uint64_t)(s.end - pos) * g.S * g.S * 2ull < (uint64_t)g.SG * g.SG;
  return s;
}

// Footprint of one segment in subgrid coordinates: the bounding box
// [x0, x1) x [y0, y1) of its rows' windows, the largest window edge (rows of
// one segment share a grid plane, but under w-projection their cf planes, and
// so their supports, differ) and, for the gridder, the largest |Re| / |Im| of
// vis * weight.  One block-wide pass over the segment's rows;
// contains a __syncthreads.  s_red holds NW * 6 words; callers alternate two
// such buffers between consecutive segments, so a segment's writes never meet
// the previous segment's reads when no other barrier lies between them.
struct SegBox {
  int x0, x1, y0, y1, sz;
  float vmax;
};

// STASH: the pass also leaves each row's set-up in shared memory for the row
// loop (RowStash, indexed by sorted position - pos), computed here one row per
// lane instead of once per row by a whole warp.
constexpr int kStashRows = 512;  // rows a stash holds: chunks of at most this many rows
struct RowStash {
  int *koff;      // offset of the row's sub-kernel window in the cf table (its (toff, toff) tap)
  int *geo;       // window origin in the subgrid (x | y << 8) and support (<< 16)
  uint32_t *idx;  // the row's index in the caller's arrays
};

template <int NW, int NPOL, bool VMAX, bool SORTED = false, bool STASH = false>
__device__ __forceinline__ SegBox seg_box(const SegInfo &sg, uint32_t pos, const RowMap *__restrict__ smap,
                                          const uint32_t *__restrict__ sidx, const float2 *__restrict__ vis,
                                          const float *__restrict__ wt, const Geom &g, int *s_red,
                                          RowStash rs = RowStash{nullptr, nullptr, nullptr}) {
  int x0 = 0x7fffffff, y0 = 0x7fffffff, x1 = -0x7fffffff, y1 = -0x7fffffff, sz = 0;
  float vm = 0.f;
  for (uint32_t r = pos + threadIdx.x; r < sg.end; r += blockDim.x) {
    const RowMap m = smap[r];
    sz = plane_sz(g, m.sub >> 16);
    const int lx = m.pu - (sz >> 1) - sg.u0, ly = m.pv - (sz >> 1) - sg.v0;
    if (STASH) {
      const int uf = m.sub & 0xff, vf = (m.sub >> 8) & 0xff, zc = m.sub >> 16, toff = (g.S - sz) >> 1;
      rs.koff[r - pos] = (int)(sg.ch * g.cf_chan_stride + zc * g.cf_z_stride) + ((vf * g.O + uf) * g.S + toff) * g.S +
                         toff;
      rs.geo[r - pos] = lx | (ly << 8) | (sz << 16);
      if (!SORTED) rs.idx[r - pos] = sidx[r];
    }
    x0 = min(x0, lx);
    x1 = max(x1, lx + sz);
    y0 = min(y0, ly);
    y1 = max(y1, ly + sz);
    if (VMAX) {
      const uint32_t idx = SORTED ? r : sidx[r];  // SORTED: vis / wt already in bin order
#pragma unroll
      for (int p = 0; p < NPOL; ++p) {
        const float2 v = vis[(size_t)idx * NPOL + p];
        const float w = wt[(size_t)idx * NPOL + p];
        vm = fmaxf(vm, fmaxf(fabsf(v.x * w), fabsf(v.y * w)));
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    x0 = min(x0, __shfl_xor_sync(0xffffffffu, x0, o));
    y0 = min(y0, __shfl_xor_sync(0xffffffffu, y0, o));
    x1 = max(x1, __shfl_xor_sync(0xffffffffu, x1, o));
    y1 = max(y1, __shfl_xor_sync(0xffffffffu, y1, o));
    sz = max(sz, __shfl_xor_sync(0xffffffffu, sz, o));
    if (VMAX) vm = fmaxf(vm, __shfl_xor_sync(0xffffffffu, vm, o));
  }
  const int warp = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    s_red[warp * 6 + 0] = x0;
    s_red[warp * 6 + 1] = x1;
    s_red[warp * 6 + 2] = y0;
    s_red[warp * 6 + 3] = y1;
    s_red[warp * 6 + 4] = sz;
    s_red[warp * 6 + 5] = __float_as_int(vm);
  }
  __syncthreads();
  SegBox b;
  b.x0 = s_red[0];
  b.x1 = s_red[1];
  b.y0 = s_red[2];
  b.y1 = s_red[3];
  b.sz = s_red[4];
  b.vmax = __int_as_float(s_red[5]);
#pragma unroll
  for (int k = 1; k < NW; ++k) {
    b.x0 = min(b.x0, s_red[k * 6 + 0]);
    b.x1 = max(b.x1, s_red[k * 6 + 1]);
    b.y0 = min(b.y0, s_red[k * 6 + 2]);
    b.y1 = max(b.y1, s_red[k * 6 + 3]);
    b.sz = max(b.sz, s_red[k * 6 + 4]);
    if (VMAX) b.vmax = fmaxf(b.vmax, __int_as_float(s_red[k * 6 + 5]));
  }
  return b;
}

// A segment goes straight to global memory when its rows' windows do not
// overlap enough to repay staging: rows * sz^2 taps (sz the largest support)
// against the footprint.
__device__ __forceinline__ bool seg_direct(const SegBox &b, uint32_t rows) {
  return (uint64_t)rows * (uint64_t)(b.sz * b.sz) <= (uint64_t)(b.x1 - b.x0) * (uint64_t)(b.y1 - b.y0);
}

template <typename R, int NW>
__global__ void __launch_bounds__(NW * 32)
k_grid(Geom g, const RowMap *__restrict__ smap, const uint32_t *__restrict__ sidx,
       const uint32_t *__restrict__ off, uint32_t chunk,
       const typename VisT<R>::C *__restrict__ vis, const typename VisT<R>::W *__restrict__ wt,
       const typename Cplx<R>::T *__restrict__ cf, typename Cplx<R>::T *__restrict__ grid,
       double *__restrict__ sumwt, uint32_t *) {  // one CTA per chunk: no work queue
  using CT = typename Cplx<R>::T;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int SG = g.SG, SG2 = SG * SG, npol = g.npol;
  CT *sub = reinterpret_cast<CT *>(smraw);
  CT *comp = sub + (size_t)npol * SG2;  // used by the FP32 variant only
  const uint32_t nvalid = off[g.nbins];
  const uint32_t c0 = blockIdx.x * chunk;
  if (c0 >= nvalid) return;
  const uint32_t c1 = min(c0 + chunk, nvalid);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int S = g.S, O = g.O;
  const int64_t plane_elems = (int64_t)g.ny * g.nx;

  uint32_t pos = c0;
  while (pos < c1) {
    const SegInfo sg = seg_at(pos, c1, smap, off, g);
    if (!sg.direct) {
      for (int k = threadIdx.x; k < npol * SG2 * SmemAcc<R>::kWords; k += blockDim.x) sub[k] = czero<CT>();
      __syncthreads();
    }
    double wsum[4] = {0.0, 0.0, 0.0, 0.0};
    for (uint32_t r = pos + warp; r < sg.end; r += NW) {
      const RowMap m = smap[r];
      const uint32_t idx = sidx[r];
      const int uf = m.sub & 0xff, vf = (m.sub >> 8) & 0xff, zc = m.sub >> 16;
      const int sz = plane_sz(g, zc);
      const int toff = (S - sz) >> 1;
      const int wu = m.pu - (sz >> 1), wv = m.pv - (sz >> 1);  // window origin, grid pixels
      CT vw[4];
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        if (p < npol) {
          CT v = vis[(size_t)idx * npol + p];
          R w = wt[(size_t)idx * npol + p];
          vw[p].x = v.x * w;
          vw[p].y = v.y * w;
          if (lane == 0) wsum[p] += (double)w;
        }
      }
      const CT *cfr = cf + sg.ch * g.cf_chan_stride + zc * g.cf_z_stride +
                      ((int64_t)(vf * O + uf) * S + toff) * S + toff;
      const int n = sz * sz, q = 32 / sz, rr = 32 - q * sz;
      int j = lane / sz, i = lane - j * sz;
      for (int t = lane; t < n; t += 32) {
#pragma unroll
        for (int p = 0; p < 4; ++p) {
          if (p < npol) {
            CT tp = cfr[p * g.cf_pol_stride + j * S + i];
            CT c;  // conj(tap) * vw
            c.x = tp.x * vw[p].x + tp.y * vw[p].y;
            c.y = tp.x * vw[p].y - tp.y * vw[p].x;
            if (sg.direct) {
              red_global<CT>(grid + ((int64_t)(sg.ch * npol + p) * g.nw + sg.zg) * plane_elems +
                                 (int64_t)(wv + j) * g.nx + (wu + i),
                             c);
            } else {
              const int cell = p * SG2 + (wv - sg.v0 + j) * SG + (wu - sg.u0 + i);
              SmemAcc<R>::add(sub + cell, comp + cell, c);
            }
          }
        }
        i += rr;
        j += q;
        if (i >= sz) {
          i -= sz;
          ++j;
        }
      }
    }
    // Per-segment weight sums: all rows of a segment share one channel.
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      if (p < npol) {
        double s = wsum[p];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0 && s != 0.0) atomicAdd(&sumwt[sg.ch * npol + p], s);
      }
    }
    if (!sg.direct) {
      __syncthreads();
      for (int k = threadIdx.x; k < npol * SG2; k += blockDim.x) {
        CT val = sub[k];
        if (SmemAcc<R>::kWords == 2) {
          CT e = comp[k];
          val.x += e.x;
          val.y += e.y;
        }
        if (val.x == (R)0 && val.y == (R)0) continue;
        const int p = k / SG2, rem = k - p * SG2, y = rem / SG, x = rem - y * SG;
        const int gy = sg.v0 + y, gx = sg.u0 + x;
        if (gy < 0 || gy >= g.ny || gx < 0 || gx >= g.nx) continue;
        red_global<CT>(grid + ((int64_t)(sg.ch * npol + p) * g.nw + sg.zg) * plane_elems +
                           (int64_t)gy * g.nx + gx,
                       val);
      }
      __syncthreads();
    }
    pos = sg.end;
  }
}

// Per-cell compensated accumulation by the cell's single owner thread (no
// atomics): Kahan for FP32, a plain add for FP64.
template <typename R> struct OwnerAcc;
template <> struct OwnerAcc<float> {
  __device__ static __forceinline__ void add(float2 *sum, float2 *comp, float2 v) {
    float2 s = *sum, c = *comp;
    float y = v.x - c.x, t = s.x + y;
    c.x = (t - s.x) - y;
    s.x = t;
    y = v.y - c.y;
    t = s.y + y;
    c.y = (t - s.y) - y;
    s.y = t;
    *sum = s;
    *comp = c;
  }
};
template <> struct OwnerAcc<double> {
  __device__ static __forceinline__ void add(double2 *sum, double2 *, double2 v) {
    double2 s = *sum;
    s.x += v.x;
    s.y += v.y;
    *sum = s;
  }
};

// Row data staged in shared memory for a batch of rows.
template <typename CT> struct StagedRow {
  RowMap m;
  CT vw[4];
};

// K3 (band-owner variant): one CTA per chunk of sorted rows.  For each bin run
// the (T + S)^2 subgrid lives in shared memory and warp w owns subgrid rows
// [w B, w B + B), B = SG / NW.  Every warp walks every row of the run (their
// metadata staged once per batch in shared memory) and adds only the window
// taps that fall in its band, so each cell has exactly one writer: a plain
// read-modify-write with a per-cell Kahan term, in a fixed row order.  Bin
// runs with few rows skip the subgrid and add their taps to the grid directly.
template <typename R, int NW>
__global__ void __launch_bounds__(NW * 32)
k_grid_band(Geom g, const RowMap *__restrict__ smap, const uint32_t *__restrict__ sidx,
            const uint32_t *__restrict__ off, uint32_t chunk,
            const typename VisT<R>::C *__restrict__ vis, const typename VisT<R>::W *__restrict__ wt,
            const typename Cplx<R>::T *__restrict__ cf, typename Cplx<R>::T *__restrict__ grid,
            double *__restrict__ sumwt, uint32_t *) {  // one CTA per chunk: no work queue
  using CT = typename Cplx<R>::T;
  constexpr int BATCH = NW * 32;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int SG = g.SG, SG2 = SG * SG, npol = g.npol;
  StagedRow<CT> *rows = reinterpret_cast<StagedRow<CT> *>(smraw);
  CT *sub = reinterpret_cast<CT *>(smraw + sizeof(StagedRow<CT>) * BATCH);
  CT *comp = sub + (size_t)npol * SG2;
  const uint32_t nvalid = off[g.nbins];
  const uint32_t c0 = blockIdx.x * chunk;
  if (c0 >= nvalid) return;
  const uint32_t c1 = min(c0 + chunk, nvalid);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int S = g.S, O = g.O;
  const int B = SG / NW, band0 = warp * B;
  const int64_t plane_elems = (int64_t)g.ny * g.nx;

  uint32_t pos = c0;
  while (pos < c1) {
    const SegInfo sg = seg_at(pos, c1, smap, off, g);
    if (!sg.direct) {
      for (int k = threadIdx.x; k < npol * SG2 * SmemAcc<R>::kWords; k += blockDim.x) sub[k] = czero<CT>();
    }
    double wsum[4] = {0.0, 0.0, 0.0, 0.0};
    for (uint32_t rb = pos; rb < sg.end; rb += BATCH) {
      const int nb = (int)min((uint32_t)BATCH, sg.end - rb);
      __syncthreads();  // previous batch fully consumed (and subgrid zeroed)
      if ((int)threadIdx.x < nb) {
        StagedRow<CT> st;
        st.m = smap[rb + threadIdx.x];
        const uint32_t idx = sidx[rb + threadIdx.x];
#pragma unroll
        for (int p = 0; p < 4; ++p) {
          if (p < npol) {
            const CT v = vis[(size_t)idx * npol + p];
            const R w = wt[(size_t)idx * npol + p];
            st.vw[p].x = v.x * w;
            st.vw[p].y = v.y * w;
            wsum[p] += (double)w;
          }
        }
        rows[threadIdx.x] = st;
      }
      __syncthreads();
      for (int k = 0; k < nb; ++k) {
        const RowMap m = rows[k].m;
        const int uf = m.sub & 0xff, vf = (m.sub >> 8) & 0xff, zc = m.sub >> 16;
        const int sz = plane_sz(g, zc);
        const int toff = (S - sz) >> 1;
        const int wu = m.pu - (sz >> 1), wv = m.pv - (sz >> 1);
        const CT *cfr = cf + sg.ch * g.cf_chan_stride + zc * g.cf_z_stride +
                        ((int64_t)(vf * O + uf) * S + toff) * S + toff;
        if (sg.direct) {
          if ((k % NW) != warp) continue;
          const int n = sz * sz, q = 32 / sz, rr = 32 - q * sz;
          int j = lane / sz, i = lane - j * sz;
          for (int t = lane; t < n; t += 32) {
#pragma unroll
            for (int p = 0; p < 4; ++p) {
              if (p < npol) {
                const CT vw = rows[k].vw[p];
                const CT tp = cfr[p * g.cf_pol_stride + j * S + i];
                CT c;
                c.x = tp.x * vw.x + tp.y * vw.y;
                c.y = tp.x * vw.y - tp.y * vw.x;
                red_global<CT>(grid + ((int64_t)(sg.ch * npol + p) * g.nw + sg.zg) * plane_elems +
                                   (int64_t)(wv + j) * g.nx + (wu + i),
                               c);
              }
            }
            i += rr;
            j += q;
            if (i >= sz) {
              i -= sz;
              ++j;
            }
          }
          continue;
        }
        const int lv = wv - sg.v0, lu = wu - sg.u0;
        const int j0 = max(lv, band0) - lv, j1 = min(lv + sz, band0 + B) - lv;
        if (j0 >= j1) continue;
        const int n = (j1 - j0) * sz, q = 32 / sz, rr = 32 - q * sz;
        int j = j0 + lane / sz, i = lane - (lane / sz) * sz;
        for (int t = lane; t < n; t += 32) {
#pragma unroll
          for (int p = 0; p < 4; ++p) {
            if (p < npol) {
              const CT vw = rows[k].vw[p];
              const CT tp = cfr[p * g.cf_pol_stride + j * S + i];
              CT c;  // conj(tap) * vw
              c.x = tp.x * vw.x + tp.y * vw.y;
              c.y = tp.x * vw.y - tp.y * vw.x;
              const int cell = p * SG2 + (lv + j) * SG + (lu + i);
              OwnerAcc<R>::add(sub + cell, comp + cell, c);
            }
          }
          i += rr;
          j += q;
          if (i >= sz) {
            i -= sz;
            ++j;
          }
        }
        __syncwarp();
      }
    }
    // Weight sums: each row was staged by exactly one thread.
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      if (p < npol) {
        double s = wsum[p];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0 && s != 0.0) atomicAdd(&sumwt[sg.ch * npol + p], s);
      }
    }
    __syncthreads();
    if (!sg.direct) {
      for (int k = threadIdx.x; k < npol * SG2; k += blockDim.x) {
        CT val = sub[k];
        if (SmemAcc<R>::kWords == 2) {
          CT e = comp[k];
          val.x -= e.x;
          val.y -= e.y;
        }
        if (val.x == (R)0 && val.y == (R)0) continue;
        const int p = k / SG2, rem = k - p * SG2, y = rem / SG, x = rem - y * SG;
        const int gy = sg.v0 + y, gx = sg.u0 + x;
        if (gy < 0 || gy >= g.ny || gx < 0 || gx >= g.nx) continue;
        red_global<CT>(grid + ((int64_t)(sg.ch * npol + p) * g.nw + sg.zg) * plane_elems +
                           (int64_t)gy * g.nx + gx,
                       val);
      }
      __syncthreads();
    }
    pos = sg.end;
  }
}

template <typename R, int NW>
__global__ void __launch_bounds__(NW * 32)
k_degrid(Geom g, const RowMap *__restrict__ smap, const uint32_t *__restrict__ sidx,
         const uint32_t *__restrict__ off, uint32_t chunk, int64_t nvis,
         const typename Cplx<R>::T *__restrict__ cf, const typename Cplx<R>::T *__restrict__ grid,
         typename VisT<R>::C *__restrict__ vis_out, uint32_t *) {  // one CTA per chunk: no work queue
  using CT = typename Cplx<R>::T;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int SG = g.SG, SG2 = SG * SG, npol = g.npol;
  CT *sub = reinterpret_cast<CT *>(smraw);
  const uint32_t nvalid = off[g.nbins];
  const uint32_t c0 = blockIdx.x * chunk;
  if (c0 >= (uint32_t)nvis) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (c0 + chunk > nvalid) {
    // Rejected rows (sorted after every valid row) are predicted as zero.
    const uint32_t b = max(c0, nvalid), e = min(c0 + chunk, (uint32_t)nvis);
    for (uint32_t r = b + threadIdx.x; r < e; r += blockDim.x)
      for (int p = 0; p < npol; ++p) vis_out[(size_t)sidx[r] * npol + p] = czero<CT>();
    if (c0 >= nvalid) return;
  }
  const uint32_t c1 = min(c0 + chunk, nvalid);
  const int S = g.S, O = g.O;
  const int64_t plane_elems = (int64_t)g.ny * g.nx;

  uint32_t pos = c0;
  while (pos < c1) {
    const SegInfo sg = seg_at(pos, c1, smap, off, g);
    const CT *gplane = grid + (int64_t)(sg.ch * npol) * g.nw * plane_elems + (int64_t)sg.zg * plane_elems;
    if (!sg.direct) {
      for (int k = threadIdx.x; k < npol * SG2; k += blockDim.x) {
        const int p = k / SG2, rem = k - p * SG2, y = rem / SG, x = rem - y * SG;
        const int gy = sg.v0 + y, gx = sg.u0 + x;
        CT val = czero<CT>();
        if (gy >= 0 && gy < g.ny && gx >= 0 && gx < g.nx)
          val = gplane[(int64_t)p * g.nw * plane_elems + (int64_t)gy * g.nx + gx];
        sub[k] = val;
      }
      __syncthreads();
    }
    for (uint32_t r = pos + warp; r < sg.end; r += NW) {
      const RowMap m = smap[r];
      const uint32_t idx = sidx[r];
      const int uf = m.sub & 0xff, vf = (m.sub >> 8) & 0xff, zc = m.sub >> 16;
      const int sz = plane_sz(g, zc);
      const int toff = (S - sz) >> 1;
      const int wu = m.pu - (sz >> 1), wv = m.pv - (sz >> 1);
      const CT *cfr = cf + sg.ch * g.cf_chan_stride + zc * g.cf_z_stride +
                      ((int64_t)(vf * O + uf) * S + toff) * S + toff;
      CT acc[4];
#pragma unroll
      for (int p = 0; p < 4; ++p) acc[p] = czero<CT>();
      const int n = sz * sz, q = 32 / sz, rr = 32 - q * sz;
      int j = lane / sz, i = lane - j * sz;
      for (int t = lane; t < n; t += 32) {
#pragma unroll
        for (int p = 0; p < 4; ++p) {
          if (p < npol) {
            CT tp = cfr[p * g.cf_pol_stride + j * S + i];
            CT gv;
            if (sg.direct)
              gv = gplane[(int64_t)p * g.nw * plane_elems + (int64_t)(wv + j) * g.nx + (wu + i)];
            else
              gv = sub[p * SG2 + (wv - sg.v0 + j) * SG + (wu - sg.u0 + i)];
            acc[p].x += gv.x * tp.x - gv.y * tp.y;
            acc[p].y += gv.x * tp.y + gv.y * tp.x;
          }
        }
        i += rr;
        j += q;
        if (i >= sz) {
          i -= sz;
          ++j;
        }
      }
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        if (p < npol) {
          R ax = acc[p].x, ay = acc[p].y;
          for (int o = 16; o > 0; o >>= 1) {
            ax += __shfl_xor_sync(0xffffffffu, ax, o);
            ay += __shfl_xor_sync(0xffffffffu, ay, o);
          }
          if (lane == p) {
            CT out;
            out.x = ax;
            out.y = ay;
            vis_out[(size_t)idx * npol + p] = out;
          }
        }
      }
    }
    if (!sg.direct) __syncthreads();
    pos = sg.end;
  }
}

// K4 (batched variant): as k_degrid, but each warp loads the metadata of 32
// rows at once (one row per lane, so 32 independent loads are in flight),
// broadcasts them with shuffles, and runs the tap loop two taps at a time with
// independent accumulators.
template <typename R, int NW>
__global__ void __launch_bounds__(NW * 32)
k_degrid_batch(Geom g, const RowMap *__restrict__ smap, const uint32_t *__restrict__ sidx,
               const uint32_t *__restrict__ off, uint32_t chunk, int64_t nvis,
               const typename Cplx<R>::T *__restrict__ cf, const typename Cplx<R>::T *__restrict__ grid,
               typename VisT<R>::C *__restrict__ vis_out, uint32_t *) {  // one CTA per chunk: no work queue
  using CT = typename Cplx<R>::T;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int SG = g.SG, SG2 = SG * SG, npol = g.npol;
  CT *sub = reinterpret_cast<CT *>(smraw);
  const uint32_t nvalid = off[g.nbins];
  const uint32_t c0 = blockIdx.x * chunk;
  if (c0 >= (uint32_t)nvis) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (c0 + chunk > nvalid) {
    const uint32_t b = max(c0, nvalid), e = min(c0 + chunk, (uint32_t)nvis);
    for (uint32_t r = b + threadIdx.x; r < e; r += blockDim.x)
      for (int p = 0; p < npol; ++p) vis_out[(size_t)sidx[r] * npol + p] = czero<CT>();
    if (c0 >= nvalid) return;
  }
  const uint32_t c1 = min(c0 + chunk, nvalid);
  const int S = g.S, O = g.O;
  const int64_t plane_elems = (int64_t)g.ny * g.nx;

  uint32_t pos = c0;
  while (pos < c1) {
    const SegInfo sg = seg_at(pos, c1, smap, off, g);
    const CT *gplane = grid + (int64_t)(sg.ch * npol) * g.nw * plane_elems + (int64_t)sg.zg * plane_elems;
    if (!sg.direct) {
      for (int k = threadIdx.x; k < npol * SG2; k += blockDim.x) {
        const int p = k / SG2, rem = k - p * SG2, y = rem / SG, x = rem - y * SG;
        const int gy = sg.v0 + y, gx = sg.u0 + x;
        CT val = czero<CT>();
        if (gy >= 0 && gy < g.ny && gx >= 0 && gx < g.nx)
          val = gplane[(int64_t)p * g.nw * plane_elems + (int64_t)gy * g.nx + gx];
        sub[k] = val;
      }
      __syncthreads();
    }
    for (uint32_t rb = pos + 32 * warp; rb < sg.end; rb += 32 * NW) {
      const int nb = (int)min(32u, sg.end - rb);
      RowMap mine;
      uint32_t myidx = 0;
      if (lane < nb) {
        mine = smap[rb + lane];
        myidx = sidx[rb + lane];
      }
      for (int k = 0; k < nb; ++k) {
        const int pu = __shfl_sync(0xffffffffu, mine.pu, k);
        const int pv = __shfl_sync(0xffffffffu, mine.pv, k);
        const uint32_t subf = __shfl_sync(0xffffffffu, mine.sub, k);
        const uint32_t idx = __shfl_sync(0xffffffffu, myidx, k);
        const int uf = subf & 0xff, vf = (subf >> 8) & 0xff, zc = subf >> 16;
        const int sz = plane_sz(g, zc);
        const int toff = (S - sz) >> 1;
        const int wu = pu - (sz >> 1), wv = pv - (sz >> 1);
        const CT *cfr = cf + sg.ch * g.cf_chan_stride + zc * g.cf_z_stride +
                        ((int64_t)(vf * O + uf) * S + toff) * S + toff;
        const int n = sz * sz, q = 32 / sz, rr = 32 - q * sz;
        const int lv = wv - sg.v0, lu = wu - sg.u0;
#pragma unroll
        for (int p = 0; p < 4; ++p) {
          if (p >= npol) break;
          const CT *cp = cfr + p * g.cf_pol_stride;
          R ax = 0, ay = 0, bx = 0, by = 0;
          int j = lane / sz, i = lane - j * sz;
          int t = lane;
          for (; t + 32 < n; t += 64) {
            int j2 = j + q, i2 = i + rr;
            if (i2 >= sz) {
              i2 -= sz;
              ++j2;
            }
            const CT t1 = cp[j * S + i], t2 = cp[j2 * S + i2];
            CT g1, g2;
            if (sg.direct) {
              const CT *gp = gplane + (int64_t)p * g.nw * plane_elems;
              g1 = gp[(int64_t)(wv + j) * g.nx + (wu + i)];
              g2 = gp[(int64_t)(wv + j2) * g.nx + (wu + i2)];
            } else {
              g1 = sub[p * SG2 + (lv + j) * SG + (lu + i)];
              g2 = sub[p * SG2 + (lv + j2) * SG + (lu + i2)];
            }
            ax += g1.x * t1.x - g1.y * t1.y;
            ay += g1.x * t1.y + g1.y * t1.x;
            bx += g2.x * t2.x - g2.y * t2.y;
            by += g2.x * t2.y + g2.y * t2.x;
            j = j2 + q;
            i = i2 + rr;
            if (i >= sz) {
              i -= sz;
              ++j;
            }
          }
          if (t < n) {
            const CT t1 = cp[j * S + i];
            CT g1;
            if (sg.direct)
              g1 = gplane[(int64_t)p * g.nw * plane_elems + (int64_t)(wv + j) * g.nx + (wu + i)];
            else
              g1 = sub[p * SG2 + (lv + j) * SG + (lu + i)];
            ax += g1.x * t1.x - g1.y * t1.y;
            ay += g1.x * t1.y + g1.y * t1.x;
          }
          ax += bx;
          ay += by;
          for (int o = 16; o > 0; o >>= 1) {
            ax += __shfl_xor_sync(0xffffffffu, ax, o);
            ay += __shfl_xor_sync(0xffffffffu, ay, o);
          }
          if (lane == 0) {
            CT out;
            out.x = ax;
            out.y = ay;
            vis_out[(size_t)idx * npol + p] = out;
          }
        }
      }
    }
    if (!sg.direct) __syncthreads();
    pos = sg.end;
  }
}

// Next chunk of sorted rows for a chunk-looping kernel: every gridDim.x-th
// chunk after this one (static), or, with a device work queue, the next
// unclaimed chunk: thread 0 takes it with one atomic on the queue word (zeroed
// before the launch; chunks 0 .. gridDim.x - 1 are the CTAs' first) and the
// barriers broadcast it.  Block-uniform.
__device__ __forceinline__ uint64_t next_chunk(uint64_t cb, uint32_t *queue, uint32_t *s_slot) {
  if (!queue) return cb + gridDim.x;
  __syncthreads();  // every thread has read the previous value
  if (threadIdx.x == 0) *s_slot = gridDim.x + atomicAdd(queue, 1u);
  __syncthreads();
  return *s_slot;
}

// Per-row set-up shared by the lean kernels: the sub-kernel base pointer and
// the 32-bit tap / subgrid offsets of this lane's first tap, plus the offset
// steps for "32 taps further" (q rows and rr columns, with a row wrap).
struct RowWalk {
  int n, sz;     // taps in the window, window edge
  int i, ko, so; // column of the current tap, its tap-table and subgrid offsets
  int q, rr;     // 32 = q * sz + rr
  int dko, dso;  // offset steps without a wrap
  int wko, wso;  // extra step when the column wraps
};

__device__ __forceinline__ RowWalk row_walk(int sz, int S, int SG, int lv, int lu, int lane) {
  RowWalk w;
  w.sz = sz;
  w.n = sz * sz;
  w.q = 32 / sz;
  w.rr = 32 - w.q * sz;
  const int j = lane / sz;
  w.i = lane - j * sz;
  w.ko = j * S + w.i;
  w.so = (lv + j) * SG + lu + w.i;
  w.dko = w.q * S + w.rr;
  w.dso = w.q * SG + w.rr;
  w.wko = S - sz;
  w.wso = SG - sz;
  return w;
}

__device__ __forceinline__ void row_step(RowWalk &w) {
  w.i += w.rr;
  w.ko += w.dko;
  w.so += w.dso;
  if (w.i >= w.sz) {
    w.i -= w.sz;
    w.ko += w.wko;
    w.so += w.wso;
  }
}

// Compile-time integer / boolean arguments for the generic tap-group lambdas.
template <int V> struct IntC { static constexpr int value = V; };
template <bool V> struct BoolC { static constexpr bool value = V; };

// Tap walk through a per-CTA byte table.  For an even support sz the taps of
// a window are numbered t = 0 .. sz^2 - 1 in row-major order and lane l of a
// warp takes taps l, l + 32, l + 64, ...; tab[tap_base(sz) + t] = t / sz is the
// window row of tap t.  Tap t then sits at  t + j (S - sz)  in the cf
// sub-kernel (row stride S) and at  t + j (W - sz)  in a target of row stride
// W (the shared subgrid, or the grid itself), so a tap costs one byte load
// and two integer multiply-adds, with no per-tap division or wrap test.
__host__ __device__ constexpr int tap_base(int sz) {
  return 4 * (sz / 2 - 1) * (sz / 2) * (sz - 1) / 6;  // sum of s^2 over even s < sz
}
__host__ __device__ constexpr int tap_table_bytes(int S) { return (tap_base(S + 2) + 15) & ~15; }

__device__ __forceinline__ void build_tap_table(unsigned char *tab, int S) {
  for (int sz = 2; sz <= S; sz += 2) {
    const int b = tap_base(sz), n = sz * sz;
    for (int t = threadIdx.x; t < n; t += blockDim.x) tab[b + t] = (unsigned char)(t / sz);
  }
}

// K3 (lean variant): warp per row, compensated shared-memory atomics as in
// k_grid, specialised on the polarisation count, with 32-bit incremental
// offsets into the tap table and the subgrid.
template <typename R, int NPOL, int NW, typename ACC = PlanarAcc<R>>
__global__ void __launch_bounds__(NW * 32)
k_grid_lean(Geom g, const RowMap *__restrict__ smap, const uint32_t *__restrict__ sidx,
            const uint32_t *__restrict__ off, uint32_t chunk,
            const typename VisT<R>::C *__restrict__ vis, const typename VisT<R>::W *__restrict__ wt,
            const typename Cplx<R>::T *__restrict__ cf, typename Cplx<R>::T *__restrict__ grid,
            double *__restrict__ sumwt, uint32_t *__restrict__ queue) {
  using CT = typename Cplx<R>::T;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int SG = g.SG, SG2 = SG * SG;
  // Planar subgrid: plane (p, c) at sub + (2 p + c) SG2, c = 0 real, 1 imaginary;
  // FP32 keeps the compensation planes after all value planes.
  R *sub = reinterpret_cast<R *>(smraw);
  R *comp = sub + (size_t)2 * NPOL * SG2;
  unsigned char *tab = smraw + (size_t)2 * NPOL * SG2 * ACC::kWords * sizeof(R);
  const uint32_t nvalid = off[g.nbins];
  // Chunks of sorted rows: chunk blockIdx.x, then every gridDim.x-th after it
  // (one chunk per CTA, or a persistent grid of resident CTAs).
  if ((uint64_t)blockIdx.x * chunk >= nvalid) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int S = g.S, O = g.O;
  const int ps = (int)g.cf_pol_stride;
  const int64_t plane_elems = (int64_t)g.ny * g.nx;

  // The planes are zero between segments: the flush clears what it reads.
  for (int k = threadIdx.x; k < 2 * NPOL * SG2 * ACC::kWords; k += blockDim.x) sub[k] = (R)0;
  build_tap_table(tab, S);
  __shared__ int s_red[2][NW * 6];
  __shared__ uint32_t s_next[2], s_chunk;
  int parity = 0;
  for (uint64_t cb = blockIdx.x; cb * chunk < nvalid; cb = next_chunk(cb, queue, &s_chunk)) {
  const uint32_t c0 = (uint32_t)(cb * chunk), c1 = min(c0 + chunk, nvalid);
  uint32_t pos = c0;
  while (pos < c1) {
    const SegInfo sg = seg_at(pos, c1, smap, off, g);
    if (threadIdx.x == 0) s_next[parity] = pos + NW;  // published by the barrier in seg_box
    uint32_t *next_row = &s_next[parity];
    const SegBox box = seg_box<NW, 1, false>(sg, pos, smap, sidx, nullptr, nullptr, g, s_red[parity]);
    parity ^= 1;
    const bool direct = seg_direct(box, sg.end - pos);
    double wsum[NPOL];
#pragma unroll
    for (int p = 0; p < NPOL; ++p) wsum[p] = 0.0;
    // Rows after each warp's first come from a shared counter, one at a
    // time, which balances rows of different support across the warps; each
    // warp holds the next row's index and metadata while it computes the
    // current one.
    uint32_t r = pos + warp;
    RowMap mnext;
    uint32_t inext = 0;
    if (r < sg.end) {
      mnext = smap[r];
      inext = sidx[r];
    }
    while (r < sg.end) {
      const RowMap m = mnext;
      const uint32_t idx = inext;
      uint32_t rn = 0;
      if (lane == 0) rn = atomicAdd(next_row, 1u);
      rn = __shfl_sync(0xffffffffu, rn, 0);
      if (rn < sg.end) {
        mnext = smap[rn];
        inext = sidx[rn];
      }
      r = rn;
      const int uf = m.sub & 0xff, vf = (m.sub >> 8) & 0xff, zc = m.sub >> 16;
      const int sz = plane_sz(g, zc);
      const int toff = (S - sz) >> 1;
      const int wu = m.pu - (sz >> 1), wv = m.pv - (sz >> 1);
      CT vw[NPOL];
#pragma unroll
      for (int p = 0; p < NPOL; ++p) {
        const CT v = vis[(size_t)idx * NPOL + p];
        const R w = wt[(size_t)idx * NPOL + p];
        vw[p].x = v.x * w;
        vw[p].y = v.y * w;
        if (lane == 0) wsum[p] += (double)w;
      }
      const CT *kb = cf + sg.ch * g.cf_chan_stride + zc * g.cf_z_stride +
                     ((int64_t)(vf * O + uf) * S + toff) * S + toff;
      const int n = sz * sz, dk = S - sz;
      const unsigned char *tj = tab + tap_base(sz) + lane;
      const CT *kl = kb + lane;
      if (direct) {
        CT *gl = grid + (int64_t)(sg.ch * NPOL) * g.nw * plane_elems + (int64_t)sg.zg * plane_elems +
                 (int64_t)wv * g.nx + wu + lane;
        const int dg = (int)g.nx - sz;
        for (int t = 0; t + lane < n; t += 32) {
          const int j = tj[t];
#pragma unroll
          for (int p = 0; p < NPOL; ++p) {
            const CT tp = kl[p * ps + t + j * dk];
            CT c;
            c.x = tp.x * vw[p].x + tp.y * vw[p].y;
            c.y = tp.x * vw[p].y - tp.y * vw[p].x;
            red_global<CT>(gl + (int64_t)p * g.nw * plane_elems + t + j * dg, c);
          }
        }
        continue;
      }
      const int wofs = (wv - sg.v0) * SG + (wu - sg.u0) + lane, dg = SG - sz;
      for (int t = 0; t + lane < n; t += 32) {
        const int j = tj[t];
        const int so = wofs + t + j * dg;
#pragma unroll
        for (int p = 0; p < NPOL; ++p) {
          const CT tp = kl[p * ps + t + j * dk];
          CT c;  // conj(tap) * vw
          c.x = tp.x * vw[p].x + tp.y * vw[p].y;
          c.y = tp.x * vw[p].y - tp.y * vw[p].x;
          ACC::add1(sub + 2 * p * SG2 + so, comp + 2 * p * SG2 + so, c.x);
          ACC::add1(sub + (2 * p + 1) * SG2 + so, comp + (2 * p + 1) * SG2 + so, c.y);
        }
      }
    }
#pragma unroll
    for (int p = 0; p < NPOL; ++p) {
      double s = wsum[p];
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0 && s != 0.0) atomicAdd(&sumwt[sg.ch * NPOL + p], s);
    }
    if (!direct) {
      __syncthreads();
      // Flush the footprint and clear it: warps over its rows, lanes over its columns.
      for (int y = box.y0 + warp; y < box.y1; y += NW) {
        const int gy = sg.v0 + y;
        for (int x = box.x0 + lane; x < box.x1; x += 32) {
          const int gx = sg.u0 + x, cell = y * SG + x;
#pragma unroll
          for (int p = 0; p < NPOL; ++p) {
            CT val;
            val.x = sub[2 * p * SG2 + cell];
            val.y = sub[(2 * p + 1) * SG2 + cell];
            sub[2 * p * SG2 + cell] = (R)0;
            sub[(2 * p + 1) * SG2 + cell] = (R)0;
            if (ACC::kWords == 2) {
              val.x += comp[2 * p * SG2 + cell];
              val.y += comp[(2 * p + 1) * SG2 + cell];
              comp[2 * p * SG2 + cell] = (R)0;
              comp[(2 * p + 1) * SG2 + cell] = (R)0;
            }
            if (val.x == (R)0 && val.y == (R)0) continue;
            if (gy < 0 || gy >= g.ny || gx < 0 || gx >= g.nx) continue;
            red_global<CT>(grid + ((int64_t)(sg.ch * NPOL + p) * g.nw + sg.zg) * plane_elems +
                               (int64_t)gy * g.nx + gx,
                           val);
          }
        }
      }
    }
    pos = sg.end;
  }
  }
}

// Bin-order copies of one-polarisation rows' vis and weight for the FP32C
// gridder.  They go into the plan's mapping scratch (the per-row keys and
// RowMaps k_map writes for k_scatter), which is dead once the plan is built,
// so the gridder reads vis and weight contiguously by sorted position instead
// of gathering them through the sort index inside its row loop.  Copies, not
// products: the gridder forms vis * weight exactly as before.
__global__ void k_gather_rows(const uint32_t *__restrict__ sidx, const uint32_t *__restrict__ off, uint32_t nbins,
                              const float2 *__restrict__ vis, const float *__restrict__ wt,
                              float2 *__restrict__ vis_s, float *__restrict__ wt_s) {
  const uint32_t nvalid = off[nbins];
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < nvalid; r += gridDim.x * blockDim.x) {
    const uint32_t i = sidx[r];
    vis_s[r] = vis[i];
    wt_s[r] = wt[i];
  }
}

// K3 (fixed-point variant, FP32C only; grid_kernel 4 and 5).
//
// Each staged segment (the rows of one bin inside one chunk) is accumulated in
// 32-bit integers.  The footprint pass over the segment's rows also finds the
// largest |Re| / |Im| of vis * weight, vmax; with tap_absmax bounding every tap
// component, each contribution conj(tap) * vis * weight has components of at
// most B = 2 * tap_absmax * vmax.  Contributions are scaled by 2^e, the
// largest power of two <= L / B with L = min(2^21, 2^30 / rows), rounded to
// integers by one FMA with the 1.5 * 2^23 shift (exact round-to-nearest for
// magnitudes below 2^22), and added with integer shared-memory atomics whose
// result is unused: the tile sums are exact and independent of the order of
// the atomics, and no warp waits on an atomic's returned value.  A cell sums
// at most `rows` contributions, so it stays below 2^30.
//
// RESID (grid_kernel 4, the FP32C gridder when tap_absmax is given): the
// rounding residual of each scaled contribution (one FMA, |residual| <= 1/2)
// is rounded to units of 2^-f, f = min(20, 30 - ceil(log2 rows)), and summed
// in a second integer plane.  A flushed cell is (sum + residual sum 2^-f) 2^-e,
// formed with one FMA: the sum of the FP32 contributions to within 2^-f-1 of a
// unit per contribution (about 2^-42 of the segment's largest contribution for
// segments of up to 512 rows) plus the final FP32 rounding.  With biased raw
// sums (fx_add, the default instantiations) f = min(20, 21 - ceil(log2 rows)):
// 2^-34 of the largest contribution for 512 rows, still 2^-10 of the FP32
// rounding of that contribution itself.  Without RESID
// (grid_kernel 5, measurement only) each contribution carries a quantisation
// error of up to half a unit, 2^-e-1.
// int32 -> FP32 with round-to-nearest, without the conversion instruction
// (GB300 issues conversions to its narrow FP64/conversion pipe): the two
// 16-bit halves of q are exact FP32 values through the 1.5 * 2^23 shift, and
// one FMA rounds hi * 2^16 + lo once, as the conversion would.
__device__ __forceinline__ float i2f_rn(int q) {
  const float fh = __int_as_float((q >> 16) + 0x4B400000) - 12582912.0f;
  const float fl = __int_as_float((q & 0xffff) + 0x4B400000) - 12582912.0f;
  return fmaf(fh, 65536.0f, fl);
}

// BIASED (with RESID, segments of at most 512 rows): each atomic adds the
// rounded value's float bit pattern itself, kFxBias + q, instead of q, which
// saves one integer subtraction per atomic (four per tap).  Every tap adds to
// all the planes of its cell, so each raw cell sum is n kFxBias + (its sum),
// modulo 2^32, with n the number of taps the cell took, the same for every
// plane of the cell.  The flush recovers n from the real residual plane:
// kFxBias = 301 * 2^22, so n kFxBias only touches bits 22-31, where it is
// 2^22 (301 n mod 1024); with the residual unit chosen so that the plane's
// true sum stays below 2^20 in magnitude, the low 22 bits of the raw sum are
// that true sum (sign-extended), the high 10 bits are 301 n mod 1024, and
// n = 677 * (those bits) mod 1024 (677 = 301^-1 mod 1024; n <= 512).  A raw
// residual sum of zero means n = 0: the cell took no tap.
constexpr uint32_t kFxBias = 0x4B400000u;  // bit pattern of 1.5 * 2^23
constexpr uint32_t kFxBiasInv = 677u;      // inverse of 301 modulo 2^10

template <bool RESID, bool BIASED = false>
__device__ __forceinline__ void fx_add(int *q, int *r, float x, float scale, float rscale) {
  const float t = fmaf(x, scale, 12582912.0f);
  atomicAdd(q, BIASED ? __float_as_int(t) : __float_as_int(t) - 0x4B400000);
  if (RESID) {
    // residual x * scale - round(x * scale), |.| <= 1/2, as a second limb in
    // units of 1 / rscale: |limb| <= rscale / 2 <= 2^19, and a cell's sum of
    // limbs stays below 2^29 (rscale <= 2^30 / rows; 2^20 when BIASED)
    const float rs = fmaf(x, scale, 12582912.0f - t);
    const float t2 = fmaf(rs, rscale, 12582912.0f);
    atomicAdd(r, BIASED ? __float_as_int(t2) : __float_as_int(t2) - 0x4B400000);
  }
}

// Tap count n of a cell from its raw real-residual sum (BIASED sums).
__device__ __forceinline__ uint32_t fx_taps(uint32_t raw_r) {
  const int low = (int)(raw_r << 10) >> 10;  // the plane's true sum
  return (((raw_r - (uint32_t)low) >> 22) * kFxBiasInv) & 1023u;
}

template <int NPOL, int NW, bool RESID, int LPR = 0, int SGC = 0, bool SORTED = false, bool STASH = false>
__global__ void __launch_bounds__(NW * 32)
k_grid_fx(Geom g, const RowMap *__restrict__ smap, const uint32_t *__restrict__ sidx,
          const uint32_t *__restrict__ off, uint32_t chunk, const float2 *__restrict__ vis,
          const float *__restrict__ wt, const float2 *__restrict__ cf, float2 *__restrict__ grid,
          double *__restrict__ sumwt, uint32_t *__restrict__ queue) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ int s_red[2][NW * 6];
  // SGC != 0: the subgrid edge as a compile-time constant, so that plane
  // offsets in shared memory fold into the instructions' immediates.
  // Planes of SG rows of SP words (fx_pitch).
  constexpr int SPC = SGC ? fx_pitch(SGC) : 0;
  const int SG = SGC ? SGC : g.SG, SP = SPC ? SPC : fx_pitch(SG), SG2 = SG * SP;
  // Planar subgrid: integer plane (p, c) at subq + (2 p + c) SG2 (c = 0 real,
  // 1 imaginary); with RESID the residual-limb planes follow all of them.
  // The planes are zero between segments: the flush clears what it reads.
  int *subq = reinterpret_cast<int *>(smraw);
  int *subr = subq + (size_t)2 * NPOL * SG2;
  constexpr int kPlanes = RESID ? 4 * NPOL : 2 * NPOL;
  // Biased raw sums (fx_add): segments of at most kStashRows rows.
  constexpr bool BIASED = RESID && STASH;
  unsigned char *tab = smraw + (size_t)kPlanes * SG2 * 4;
  const uint32_t nvalid = off[g.nbins];
  // Chunks of sorted rows: chunk blockIdx.x, then every gridDim.x-th after it
  // (one chunk per CTA, or a persistent grid of resident CTAs).
  if ((uint64_t)blockIdx.x * chunk >= nvalid) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int S = g.S, O = g.O;
  const int ps = (int)g.cf_pol_stride;
  const int64_t plane_elems = (int64_t)g.ny * g.nx;
  for (int k = threadIdx.x; k < kPlanes * SG2; k += blockDim.x) subq[k] = 0;
  build_tap_table(tab, S);

  __shared__ uint32_t s_next[2], s_chunk;
  // Row set-up records (STASH), double-buffered like s_red; without SORTED
  // rows they carry each row's index in the caller's arrays too.
  constexpr int kSR = STASH ? kStashRows : 1;
  __shared__ int s_koff[2][kSR], s_geo[2][kSR];
  __shared__ uint32_t s_idx[2][STASH && !SORTED ? kStashRows : 1];
  int parity = 0;
  for (uint64_t cb = blockIdx.x; cb * chunk < nvalid; cb = next_chunk(cb, queue, &s_chunk)) {
  const uint32_t c0 = (uint32_t)(cb * chunk), c1 = min(c0 + chunk, nvalid);
  uint32_t pos = c0;
  while (pos < c1) {
    const SegInfo sg = seg_at(pos, c1, smap, off, g);
    if (threadIdx.x == 0) s_next[parity] = pos;  // published by the barrier in seg_box
    uint32_t *next_row = &s_next[parity];
    const RowStash rs{s_koff[parity], s_geo[parity], s_idx[parity]};
    const SegBox box = seg_box<NW, NPOL, true, SORTED, STASH>(sg, pos, smap, sidx, vis, wt, g, s_red[parity], rs);
    parity ^= 1;
    const uint32_t rows = sg.end - pos;
    const bool direct = seg_direct(box, rows);
    // Power-of-two units, so that unscaling at the flush is exact:
    // scale = 2^e <= L / B, rscale = 2^f <= min(2^20, 2^30 / rows).
    float scale = 0.f, inv = 0.f, rscale = 0.f, rinv = 0.f;
    if (!direct) {
      const float lim = rows <= 512u ? 2097152.f : 1073741824.f / (float)rows;
      const float bound = 2.f * g.tap_absmax * box.vmax;
      if (bound > 0.f) {
        const float q = fminf(lim / bound, 1e30f);  // tiny segments: coarser units, never inf
        int e;
        frexpf(q, &e);  // q = m 2^e, m in [1/2, 1)
        scale = ldexpf(1.f, e - 1);
        inv = ldexpf(1.f, 1 - e);
      }
      const int lr = 32 - __clz((int)rows - 1);  // ceil(log2(rows))
      // a cell's residual sum: at most rows * rscale / 2 = 2^(lr + f - 1)
      const int f = min(20, (BIASED ? 21 : 30) - lr);
      rscale = ldexpf(1.f, f);
      rinv = ldexpf(1.f, -f);
    }
    // Weight sums per row slot (lane 0, and lane 16 with two rows per warp),
    // kept as an FP32 value plus its TwoSum error (FP64 issue is scarce on
    // GB300; the pair is exact to ~1e-14).
    float wsum[NPOL], wcomp[NPOL];
#pragma unroll
    for (int p = 0; p < NPOL; ++p) wsum[p] = wcomp[p] = 0.f;
    // Rows per warp: LP lanes per row; the default one-row-per-warp
    // variant runs a segment two rows per warp when its largest support is
    // at most 16 (256 taps), sharing the per-row set-up between two rows.
    auto row_loop = [&](auto lpr_c) {
      constexpr int LP = decltype(lpr_c)::value;
      constexpr int RP = 32 / LP;
      const int hl = lane & (LP - 1), half = lane / LP;
      // Rows come from a shared counter, RP at a time (one per row slot of
      // the warp), which balances rows of different support across the warps;
      // each warp holds its next rows' indices and metadata while it computes
      // the current ones.  rbase is warp-uniform; this lane's row is
      // rbase + half.
      uint32_t rbase = 0;
      if (lane == 0) rbase = atomicAdd(next_row, (uint32_t)RP);
      rbase = __shfl_sync(0xffffffffu, rbase, 0);
      RowMap mnext;
      uint32_t inext = 0;
      // With STASH the sorted position goes into inext (the record's index);
      // the caller's row index comes from the record.
      if (rbase + half < sg.end) {
        if constexpr (!STASH) mnext = smap[rbase + half];
        inext = SORTED || STASH ? rbase + half : sidx[rbase + half];
      }
      while (rbase < sg.end) {
        const RowMap m = mnext;
        const uint32_t idx = inext;
        const bool act = rbase + half < sg.end;
        uint32_t rn = 0;
        if (lane == 0) rn = atomicAdd(next_row, (uint32_t)RP);
        rn = __shfl_sync(0xffffffffu, rn, 0);
        if (rn + half < sg.end) {
          if constexpr (!STASH) mnext = smap[rn + half];
          inext = SORTED || STASH ? rn + half : sidx[rn + half];
        }
        rbase = rn;
        if (!act) continue;
        int sz, wu, wv;
        const float2 *kb;
        uint32_t ridx = idx;  // the row's index into vis / wt
        if constexpr (STASH) {
          const int geo = rs.geo[idx - pos];  // idx is the sorted position here
          sz = geo >> 16;
          wu = sg.u0 + (geo & 0xff);
          wv = sg.v0 + ((geo >> 8) & 0xff);
          kb = cf + rs.koff[idx - pos];
          if constexpr (!SORTED) ridx = rs.idx[idx - pos];
        } else {
          const int uf = m.sub & 0xff, vf = (m.sub >> 8) & 0xff, zc = m.sub >> 16;
          sz = plane_sz(g, zc);
          const int toff = (S - sz) >> 1;
          wu = m.pu - (sz >> 1);
          wv = m.pv - (sz >> 1);
          kb = cf + sg.ch * g.cf_chan_stride + zc * g.cf_z_stride + ((int64_t)(vf * O + uf) * S + toff) * S + toff;
        }
        float2 vw[NPOL];
  #pragma unroll
        for (int p = 0; p < NPOL; ++p) {
          const float2 v = vis[(size_t)ridx * NPOL + p];
          const float w = wt[(size_t)ridx * NPOL + p];
          vw[p].x = v.x * w;
          vw[p].y = v.y * w;
          if (hl == 0) {
            const float s2 = wsum[p] + w, bp = s2 - wsum[p];
            wcomp[p] += (wsum[p] - (s2 - bp)) + (w - bp);
            wsum[p] = s2;
          }
        }
        const int n = sz * sz, dk = S - sz;
        const unsigned char *tj = tab + tap_base(sz) + hl;
        const float2 *kl = kb + hl;
        if (direct) {
          float2 *gl = grid + (int64_t)(sg.ch * NPOL) * g.nw * plane_elems + (int64_t)sg.zg * plane_elems +
                       (int64_t)wv * g.nx + wu + hl;
          const int dg = (int)g.nx - sz;
          for (int t = 0; t + hl < n; t += LP) {
            const int j = tj[t];
  #pragma unroll
            for (int p = 0; p < NPOL; ++p) {
              const float2 tp = kl[p * ps + t + j * dk];
              float2 c;
              c.x = tp.x * vw[p].x + tp.y * vw[p].y;
              c.y = tp.x * vw[p].y - tp.y * vw[p].x;
              red_global<float2>(gl + (int64_t)p * g.nw * plane_elems + t + j * dg, c);
            }
          }
          continue;
        }
        const int wofs = (wv - sg.v0) * SP + (wu - sg.u0) + hl, dg = SP - sz;
        // Groups of K warp steps: all tap loads of a group are in flight before
        // its first atomic.  Full groups of four run unmasked; the last 1 to 4
        // steps run as one group of exactly that many, masked per lane only in
        // its partial last step.  With one kernel for every polarisation
        // (pol stride 0, as ARL's PSWF and w-kernels are) a tap is loaded once.
        auto taps = [&](auto same) {
          auto group = [&](int t, auto kk, auto masked) {
            constexpr int K = decltype(kk)::value;
            int j[K];
            bool on[K];
            float2 tp[NPOL][K];
  #pragma unroll
            for (int u = 0; u < K; ++u) {
              on[u] = !decltype(masked)::value || t + LP * u + hl < n;
              j[u] = on[u] ? tj[t + LP * u] : 0;
  #pragma unroll
              for (int p = 0; p < NPOL; ++p)
                tp[p][u] = decltype(same)::value && p > 0 ? tp[0][u]
                           : on[u] ? kl[p * ps + t + LP * u + j[u] * dk] : make_float2(0.f, 0.f);
            }
  #pragma unroll
            for (int u = 0; u < K; ++u) {
              if (!on[u]) break;
              const int so = wofs + t + LP * u + j[u] * dg;
  #pragma unroll
              for (int p = 0; p < NPOL; ++p) {
                const float cx = tp[p][u].x * vw[p].x + tp[p][u].y * vw[p].y;  // conj(tap) * vw
                const float cy = tp[p][u].x * vw[p].y - tp[p][u].y * vw[p].x;
                fx_add<RESID, BIASED>(subq + 2 * p * SG2 + so, subr + 2 * p * SG2 + so, cx, scale, rscale);
                fx_add<RESID, BIASED>(subq + (2 * p + 1) * SG2 + so, subr + (2 * p + 1) * SG2 + so, cy, scale,
                                      rscale);
              }
            }
          };
          int t = 0;
          for (; t + 4 * LP <= n; t += 4 * LP) group(t, IntC<4>(), BoolC<false>());
          switch ((n - t + LP - 1) / LP) {
            case 1: group(t, IntC<1>(), BoolC<true>()); break;
            case 2: group(t, IntC<2>(), BoolC<true>()); break;
            case 3: group(t, IntC<3>(), BoolC<true>()); break;
            case 4: group(t, IntC<4>(), BoolC<true>()); break;
            default: break;
          }
        };
        if constexpr (NPOL == 4) {  // two polarisations: the second path spills
          if (ps == 0)
            taps(BoolC<true>());
          else
            taps(BoolC<false>());
        } else {
          taps(BoolC<false>());
        }
      }
    };
    if constexpr (LPR == 0) {  // lanes per row chosen per segment
      if (box.sz <= 16)
        row_loop(IntC<16>());
      else
        row_loop(IntC<32>());
    } else {
      row_loop(IntC<LPR>());
    }
    {  // the lanes that hold a row slot's weight sums
#pragma unroll
      for (int p = 0; p < NPOL; ++p) {
        const double s = (double)wsum[p] + (double)wcomp[p];
        if (s != 0.0) atomicAdd(&sumwt[sg.ch * NPOL + p], s);
      }
    }
    if (!direct) {
      __syncthreads();
      // Flush the footprint (and clear it for the next segment): warps over
      // its rows, lanes over its columns.
      for (int y = box.y0 + warp; y < box.y1; y += NW) {
        const int gy = sg.v0 + y;
        for (int x = box.x0 + lane; x < box.x1; x += 32) {
          const int gx = sg.u0 + x, cell = y * SP + x;
          uint32_t bias = 0;  // BIASED: n kFxBias, carried by every raw sum of the cell
          if constexpr (BIASED) {
            const uint32_t raw = (uint32_t)subr[cell];
            if (raw == 0u) continue;  // no tap: every plane of the cell is zero
            bias = fx_taps(raw) * kFxBias;
          }
#pragma unroll
          for (int p = 0; p < NPOL; ++p) {
            const int qx = (int)((uint32_t)subq[2 * p * SG2 + cell] - bias);
            const int qy = (int)((uint32_t)subq[(2 * p + 1) * SG2 + cell] - bias);
            const int rx = RESID ? (int)((uint32_t)subr[2 * p * SG2 + cell] - bias) : 0;
            const int ry = RESID ? (int)((uint32_t)subr[(2 * p + 1) * SG2 + cell] - bias) : 0;
            // an untouched cell's planes are already zero; a touched cell's
            // raw sums (BIASED) are cleared even where its true sums are zero
            const bool zero = qx == 0 && qy == 0 && rx == 0 && ry == 0;
            if (zero && !BIASED) continue;
            subq[2 * p * SG2 + cell] = 0;
            subq[(2 * p + 1) * SG2 + cell] = 0;
            if (RESID) {
              subr[2 * p * SG2 + cell] = 0;
              subr[(2 * p + 1) * SG2 + cell] = 0;
            }
            if (zero || gy < 0 || gy >= g.ny || gx < 0 || gx >= g.nx) continue;
            // inv and rinv * inv are powers of two: one rounding in the FMA
            // (and in the int -> float conversions of sums beyond 2^24)
            float2 val;
            val.x = fmaf(i2f_rn(rx), rinv * inv, i2f_rn(qx) * inv);
            val.y = fmaf(i2f_rn(ry), rinv * inv, i2f_rn(qy) * inv);
            red_global<float2>(grid + ((int64_t)(sg.ch * NPOL + p) * g.nw + sg.zg) * plane_elems +
                                   (int64_t)gy * g.nx + gx,
                               val);
          }
        }
      }
    }
    pos = sg.end;
  }
  }
}

// Packed FP32 multiply-add: d = a * b + c on both halves of a float pair.
__device__ __forceinline__ unsigned long long ffma2(unsigned long long a, unsigned long long b,
                                                   unsigned long long c) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

// K4 (lean variant): warp per row, specialised on the polarisation count, tap
// walk through the row table, groups of up to four steps in flight.
// DUP (FP32 only, degrid_kernel 3): the staged subgrid holds each cell as
// (re, re, im, im), so a tap is two packed multiply-adds,
// (sum re t.re, sum re t.im) and (sum im t.re, sum im t.im), instead of four.
// STASH (with a chunk of at most kStashRows rows and a cf table of fewer than
// 2^31 taps): the footprint pass leaves each row's set-up in shared memory.
template <typename R, int NPOL, int NW, bool DUP = false, int LPR = 0, int SGC = 0, bool STASH = false>
__global__ void __launch_bounds__(NW * 32)
k_degrid_lean(Geom g, const RowMap *__restrict__ smap, const uint32_t *__restrict__ sidx,
              const uint32_t *__restrict__ off, uint32_t chunk, int64_t nvis,
              const typename Cplx<R>::T *__restrict__ cf, const typename Cplx<R>::T *__restrict__ grid,
              typename VisT<R>::C *__restrict__ vis_out, uint32_t *__restrict__ queue) {
  using CT = typename Cplx<R>::T;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int SG = SGC ? SGC : g.SG, SG2 = SG * SG;  // SGC != 0: compile-time edge
  static_assert(!DUP || sizeof(R) == 4, "the packed variant is FP32 only");
  CT *sub = reinterpret_cast<CT *>(smraw);
  float4 *sub4 = reinterpret_cast<float4 *>(smraw);  // DUP layout
  unsigned char *tab = smraw + (size_t)NPOL * SG2 * (DUP ? sizeof(float4) : sizeof(CT));
  const uint32_t nvalid = off[g.nbins];
  // Chunks of sorted rows: chunk blockIdx.x, then every gridDim.x-th after it
  // (one chunk per CTA, or a persistent grid of resident CTAs).
  const uint64_t nchunks = ((uint64_t)nvis + chunk - 1) / chunk;
  if (blockIdx.x >= nchunks) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int S = g.S, O = g.O;
  const int ps = (int)g.cf_pol_stride;
  const int64_t plane_elems = (int64_t)g.ny * g.nx;

  __shared__ int s_red[2][NW * 6];
  __shared__ uint32_t s_next[2], s_chunk;
  // Row set-up records, double-buffered like s_red (segment s + 2 rewrites a
  // buffer only after every warp has passed segment s + 1's barrier).
  constexpr int kSR = STASH ? kStashRows : 1;
  __shared__ int s_koff[2][kSR], s_geo[2][kSR];
  __shared__ uint32_t s_idx[2][kSR];
  build_tap_table(tab, S);  // ordered before first use by the barrier in seg_box
  int parity = 0;
  for (uint64_t cb = blockIdx.x; cb < nchunks; cb = next_chunk(cb, queue, &s_chunk)) {
  const uint32_t c0 = (uint32_t)(cb * chunk);
  if (c0 + chunk > nvalid) {  // rows the plan rejected: zero output
    const uint32_t b = max(c0, nvalid), e = (uint32_t)min((uint64_t)c0 + chunk, (uint64_t)nvis);
    for (uint32_t r = b + threadIdx.x; r < e; r += blockDim.x)
      for (int p = 0; p < NPOL; ++p) vis_out[(size_t)sidx[r] * NPOL + p] = czero<CT>();
    if (c0 >= nvalid) continue;
  }
  const uint32_t c1 = min(c0 + chunk, nvalid);
  uint32_t pos = c0;
  while (pos < c1) {
    const SegInfo sg = seg_at(pos, c1, smap, off, g);
    if (threadIdx.x == 0) s_next[parity] = pos;  // published by the barrier in seg_box
    uint32_t *next_row = &s_next[parity];
    const RowStash rs{s_koff[parity], s_geo[parity], s_idx[parity]};
    // The footprint pass ends in a barrier, which also orders the previous
    // segment's reads of the subgrid before this segment's staging.
    const SegBox box = seg_box<NW, 1, false, false, STASH>(sg, pos, smap, sidx, nullptr, nullptr, g, s_red[parity], rs);
    parity ^= 1;
    const bool direct = seg_direct(box, sg.end - pos);
    const CT *gplane = grid + (int64_t)(sg.ch * NPOL) * g.nw * plane_elems + (int64_t)sg.zg * plane_elems;
    if (!direct) {
      // Stage the footprint only: warps over its rows, lanes over its columns.
      for (int y = box.y0 + warp; y < box.y1; y += NW) {
        const int gy = sg.v0 + y;
        for (int x = box.x0 + lane; x < box.x1; x += 32) {
          const int gx = sg.u0 + x;
          const bool in = gy >= 0 && gy < g.ny && gx >= 0 && gx < g.nx;
#pragma unroll
          for (int p = 0; p < NPOL; ++p) {
            const CT v = in ? gplane[(int64_t)p * g.nw * plane_elems + (int64_t)gy * g.nx + gx] : czero<CT>();
            if (DUP)
              sub4[p * SG2 + y * SG + x] = make_float4((float)v.x, (float)v.x, (float)v.y, (float)v.y);
            else
              sub[p * SG2 + y * SG + x] = v;
          }
        }
      }
      __syncthreads();
    }
    // Rows per warp: LP lanes per row; the default one-row-per-warp
    // variant runs a segment four rows per warp when its largest support is
    // at most 8 and two when at most 16 (256 taps), sharing the per-row
    // set-up between the rows.
    auto row_loop = [&](auto lpr_c) {
      constexpr int LP = decltype(lpr_c)::value;
      constexpr int RP = 32 / LP;
      const int hl = lane & (LP - 1), half = lane / LP;
      // Rows come from a shared counter, RP at a time (one per row slot of
      // the warp), which balances rows of different support across the warps;
      // each warp holds its next rows' indices and metadata while it computes
      // the current ones.  rbase is warp-uniform; this lane's row is
      // rbase + half.
      uint32_t rbase = 0;
      if (lane == 0) rbase = atomicAdd(next_row, (uint32_t)RP);
      rbase = __shfl_sync(0xffffffffu, rbase, 0);
      RowMap mnext;
      uint32_t inext = 0;
      if constexpr (!STASH) {
        if (rbase + half < sg.end) {
          mnext = smap[rbase + half];
          inext = sidx[rbase + half];
        }
      }
      while (rbase < sg.end) {
        const RowMap m = mnext;
        uint32_t idx = inext;
        const bool act = rbase + half < sg.end;
        const uint32_t rk = rbase + half - pos;  // this lane's row in the stash (STASH)
        uint32_t rn = 0;
        if (lane == 0) rn = atomicAdd(next_row, (uint32_t)RP);
        rn = __shfl_sync(0xffffffffu, rn, 0);
        if constexpr (!STASH) {
          if (rn + half < sg.end) {
            mnext = smap[rn + half];
            inext = sidx[rn + half];
          }
        }
        rbase = rn;
        R ax[NPOL], ay[NPOL];
  #pragma unroll
        for (int p = 0; p < NPOL; ++p) ax[p] = ay[p] = 0;
        if (act) {
        int sz, wu, wv;
        const CT *kb;
        if constexpr (STASH) {
          const int geo = rs.geo[rk];
          idx = rs.idx[rk];
          sz = geo >> 16;
          wu = sg.u0 + (geo & 0xff);
          wv = sg.v0 + ((geo >> 8) & 0xff);
          kb = cf + rs.koff[rk];
        } else {
          const int uf = m.sub & 0xff, vf = (m.sub >> 8) & 0xff, zc = m.sub >> 16;
          sz = plane_sz(g, zc);
          const int toff = (S - sz) >> 1;
          wu = m.pu - (sz >> 1);
          wv = m.pv - (sz >> 1);
          kb = cf + sg.ch * g.cf_chan_stride + zc * g.cf_z_stride + ((int64_t)(vf * O + uf) * S + toff) * S + toff;
        }
        const CT *gl;
        int64_t pstride;
        int dg;
        if (direct) {
          gl = gplane + (int64_t)wv * g.nx + wu + hl;
          pstride = (int64_t)g.nw * plane_elems;
          dg = (int)g.nx - sz;
        } else {
          gl = sub + (wv - sg.v0) * SG + (wu - sg.u0) + hl;
          pstride = SG2;
          dg = SG - sz;
        }
        const int n = sz * sz, dk = S - sz;
        const unsigned char *tj = tab + tap_base(sz) + hl;
        const CT *kl = kb + hl;
        // Groups of K warp steps: every load of a group is in flight before the
        // multiply-adds that use it.  Full groups of four run unmasked; the
        // last 1 to 4 steps run as one group of exactly that many steps, masked
        // per lane only in its partial last step.
        auto group = [&](int t, auto kk, auto masked) {
          constexpr int K = decltype(kk)::value;
          int j[K];
          bool on[K];
  #pragma unroll
          for (int u = 0; u < K; ++u) {
            on[u] = !decltype(masked)::value || t + LP * u + hl < n;
            j[u] = on[u] ? tj[t + LP * u] : 0;
          }
  #pragma unroll
          for (int p = 0; p < NPOL; ++p) {
            CT tp[K], gv[K];
  #pragma unroll
            for (int u = 0; u < K; ++u) {
              tp[u] = on[u] ? kl[p * ps + t + LP * u + j[u] * dk] : czero<CT>();
              gv[u] = on[u] ? gl[p * pstride + t + LP * u + j[u] * dg] : czero<CT>();
            }
  #pragma unroll
            for (int u = 0; u < K; ++u) {
              ax[p] += gv[u].x * tp[u].x - gv[u].y * tp[u].y;
              ay[p] += gv[u].x * tp[u].y + gv[u].y * tp[u].x;
            }
          }
        };
        // The packed variant: accumulators (sum re t.re, sum re t.im) and
        // (sum im t.re, sum im t.im) per polarisation.
        unsigned long long pa[NPOL], pb[NPOL];
  #pragma unroll
        for (int p = 0; p < NPOL; ++p) pa[p] = pb[p] = 0ull;
        const int wofs4 = (wv - sg.v0) * SG + (wu - sg.u0) + hl;
        // With one kernel for every polarisation (pol stride 0) a tap is
        // loaded once for all of them.
        auto group2 = [&](int t, auto kk, auto masked, auto same) {
          constexpr int K = decltype(kk)::value;
          int j[K];
          bool on[K];
          unsigned long long tp0[K];
  #pragma unroll
          for (int u = 0; u < K; ++u) {
            on[u] = !decltype(masked)::value || t + LP * u + hl < n;
            j[u] = on[u] ? tj[t + LP * u] : 0;
            if (decltype(same)::value)
              tp0[u] = on[u] ? *reinterpret_cast<const unsigned long long *>(kl + t + LP * u + j[u] * dk) : 0ull;
          }
  #pragma unroll
          for (int p = 0; p < NPOL; ++p) {
            unsigned long long tp[K];
            ulonglong2 gv[K];
  #pragma unroll
            for (int u = 0; u < K; ++u) {
              tp[u] = decltype(same)::value ? tp0[u]
                      : on[u] ? *reinterpret_cast<const unsigned long long *>(kl + p * ps + t + LP * u + j[u] * dk)
                              : 0ull;
              gv[u] = on[u] ? *reinterpret_cast<const ulonglong2 *>(sub4 + p * SG2 + wofs4 + t + LP * u + j[u] * dg)
                            : make_ulonglong2(0ull, 0ull);
            }
  #pragma unroll
            for (int u = 0; u < K; ++u) {
              pa[p] = ffma2(gv[u].x, tp[u], pa[p]);
              pb[p] = ffma2(gv[u].y, tp[u], pb[p]);
            }
          }
        };
        auto taps2 = [&](auto same) {
          int t = 0;
          for (; t + 4 * LP <= n; t += 4 * LP) group2(t, IntC<4>(), BoolC<false>(), same);
          switch ((n - t + LP - 1) / LP) {
            case 1: group2(t, IntC<1>(), BoolC<true>(), same); break;
            case 2: group2(t, IntC<2>(), BoolC<true>(), same); break;
            case 3: group2(t, IntC<3>(), BoolC<true>(), same); break;
            case 4: group2(t, IntC<4>(), BoolC<true>(), same); break;
            default: break;
          }
        };
        int t = 0;
        if (DUP && !direct) {
          if constexpr (NPOL > 1) {
            if (ps == 0)
              taps2(BoolC<true>());
            else
              taps2(BoolC<false>());
          } else {
            taps2(BoolC<false>());
          }
  #pragma unroll
          for (int p = 0; p < NPOL; ++p) {
            const float2 a2 = *reinterpret_cast<const float2 *>(&pa[p]);
            const float2 b2 = *reinterpret_cast<const float2 *>(&pb[p]);
            ax[p] = (R)(a2.x - b2.y);
            ay[p] = (R)(a2.y + b2.x);
          }
        } else {
          for (; t + 4 * LP <= n; t += 4 * LP) group(t, IntC<4>(), BoolC<false>());
          switch ((n - t + LP - 1) / LP) {
            case 1: group(t, IntC<1>(), BoolC<true>()); break;
            case 2: group(t, IntC<2>(), BoolC<true>()); break;
            case 3: group(t, IntC<3>(), BoolC<true>()); break;
            case 4: group(t, IntC<4>(), BoolC<true>()); break;
            default: break;
          }
        }
        }  // act
        // Reduce over each row's LP lanes (all lanes take part).
  #pragma unroll
        for (int p = 0; p < NPOL; ++p) {
          R sx = ax[p], sy = ay[p];
          for (int o = LP / 2; o > 0; o >>= 1) {
            sx += __shfl_xor_sync(0xffffffffu, sx, o);
            sy += __shfl_xor_sync(0xffffffffu, sy, o);
          }
          if (act && hl == p) {
            CT out;
            out.x = sx;
            out.y = sy;
            vis_out[(size_t)idx * NPOL + p] = out;
          }
        }
      }
    };
    if constexpr (LPR == 0) {  // lanes per row chosen per segment
      if (box.sz <= 8)
        row_loop(IntC<8>());
      else if (box.sz <= 16)
        row_loop(IntC<16>());
      else
        row_loop(IntC<32>());
    } else {
      row_loop(IntC<LPR>());
    }
    pos = sg.end;
  }
  }
}

// ---------------------------------------------------------------------------
// K4 (TMA variant, degrid_kernel 4): the packed FP32 degridder with the grid
// footprint and the kernel taps staged in shared memory by the tensor-memory
// accelerator.  FP32C, one polarisation, supports up to 32, subgrid edge 48.
//
// Grid: after the footprint pass, thread 0 loads the segment's whole
// (SG + 2) x SG subgrid tile of its grid plane with one 3-D tensor copy
// (cells outside the grid arrive as zeros), into the tap-ring area, which is
// idle between segments; the footprint cells are then expanded to the
// (re, re, im, im) layout of the packed multiply-adds.
//
// Taps: each warp streams its rows' sub-kernels through a private ring in
// shared memory.  A row's window of sz x sz taps is cut into pieces of up to
// eight kernel rows; piece k of a row is one 2-D tensor copy of a box
// bw x 8 taps (bw = sz, or sz + 2 when the window's first column is odd, so
// that the copy starts on a 16-byte boundary) from the cf table viewed as
// [rows][S].  Lane 0 issues pieces in order into the ring (a byte FIFO with
// kQ mbarriers, piece q completing on barrier q mod kQ in phase (q / kQ) & 1);
// the warp consumes them in the same order.  While it computes the current
// step of rows (one, two or four rows per warp, as the lean kernel), the
// pieces of its next step (already taken from the segment's row counter) are
// in flight.  Every wait is bounded: a wait that gives up sets bit 0 of *err
// and the kernel carries on, draining its copies (also bounded) before it
// exits, so a fault shows as a flag, never as a hang.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_done(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Wait for the phase of the given parity to complete; gives up after about a
// second (2^24 polls, backing off with nanosleep) and returns false.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  for (uint32_t it = 0; it < (1u << 24); ++it) {
    if (mbar_done(bar, parity)) return true;
    if (it >= 32) __nanosleep(64);
  }
  return false;
}
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

struct TmaDesc {
  CUtensorMap tap[16];  // cf table as [rows][S] 8-byte taps; map m has a box of (2 m + 2) x 8 taps
  CUtensorMap grid;     // grid as [planes][ny][nx] 8-byte cells; box (SG + 2) x SG x 1
};

constexpr int kTmaRing = 6144;  // tap-ring bytes per warp
constexpr int kTmaQ = 8;        // tap pieces in flight per warp (mbarriers per warp)
constexpr int kTmaSG = 48;      // subgrid edge of the TMA degridder
constexpr int kTmaMaxS = 32;    // largest support it takes

// Tap pieces of one step of rows (one to four rows), identical in every lane
// of the warp.  Pieces are numbered column-major: piece (h, k) -- kernel rows
// 8k .. 8k + 7 of row h -- comes after every piece of a smaller k.
struct TmaStep {
  int n;                 // rows in the step
  int np[4], bw[4];      // pieces and box width of each row
  int x[4], y[4];        // copy coordinates of each row's piece 0
  int total, maxk;       // pieces in the step, largest piece count
};

__device__ __forceinline__ int tma_piece_index(const TmaStep &s, int h, int k) {
  int i = 0;
  for (int kk = 0; kk < k; ++kk)
    for (int r = 0; r < s.n; ++r) i += kk < s.np[r];
  for (int r = 0; r < h; ++r) i += k < s.np[r];
  return i;
}

template <int NW>
__global__ void __launch_bounds__(NW * 32, 2)
k_degrid_tma(const __grid_constant__ TmaDesc tmd, Geom g, const RowMap *__restrict__ smap,
             const uint32_t *__restrict__ sidx, const uint32_t *__restrict__ off, uint32_t chunk, int64_t nvis,
             const float2 *__restrict__ cf, const float2 *__restrict__ grid, float2 *__restrict__ vis_out,
             uint32_t *__restrict__ queue, uint32_t *__restrict__ err) {
  constexpr int SG = kTmaSG, SG2 = SG * SG, RW = SG + 2;  // RW: row pitch of the copied grid tile
  extern __shared__ __align__(16) unsigned char smraw[];
  // Tensor copies land on 128-byte boundaries: the dynamic area starts after
  // the static one, so round its base up (the launch adds 128 bytes).
  unsigned char *base = smraw + ((128u - (smem_u32(smraw) & 127u)) & 127u);
  float4 *sub4 = reinterpret_cast<float4 *>(base);                        // [SG][SG] (re, re, im, im)
  unsigned char *ring_all = base + (size_t)SG2 * sizeof(float4);          // [NW][kTmaRing], 128-byte aligned
  unsigned char *tab = ring_all + (size_t)NW * kTmaRing;
  __shared__ __align__(8) uint64_t s_bar[NW][kTmaQ];
  __shared__ __align__(8) uint64_t s_gbar;
  __shared__ uint32_t s_poff[NW][kTmaQ], s_pend[NW][kTmaQ];
  __shared__ int s_red[2][NW * 6];
  __shared__ uint32_t s_next[2], s_chunk;
  const uint32_t nvalid = off[g.nbins];
  const uint64_t nchunks = ((uint64_t)nvis + chunk - 1) / chunk;
  if (blockIdx.x >= nchunks) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int S = g.S, O = g.O;
  const int64_t plane_elems = (int64_t)g.ny * g.nx;
  unsigned char *ring = ring_all + (size_t)warp * kTmaRing;
  if (threadIdx.x == 0) {
    for (int w = 0; w < NW; ++w)
      for (int q = 0; q < kTmaQ; ++q) mbar_init(&s_bar[w][q], 1);
    mbar_init(&s_gbar, 1);
    fence_mbar_init();
  }
  build_tap_table(tab, S);
  __syncthreads();
  // Warp-uniform FIFO state: bytes allocated / released (monotone), pieces
  // issued / consumed.
  uint32_t tail = 0, head = 0, qi = 0, qc = 0;
  uint32_t gphase = 0;  // phase parity of the grid-tile barrier
  bool ok = true;

  // Issue piece i of step st if the ring and the barrier window have room.
  auto try_issue = [&](const TmaStep &st, int i) -> bool {
    int h = 0, k = 0;
    {
      int c = i;
      bool found = false;
      for (int kk = 0; kk < 4 && !found; ++kk)
        for (int r = 0; r < st.n && !found; ++r)
          if (kk < st.np[r]) {
            if (c == 0) {
              h = r;
              k = kk;
              found = true;
            } else {
              --c;
            }
          }
    }
    const uint32_t bytes = (uint32_t)st.bw[h] * 64u;
    uint32_t o = tail % kTmaRing;
    const uint32_t skip = o + bytes > (uint32_t)kTmaRing ? kTmaRing - o : 0u;
    if (tail + skip + bytes - head > (uint32_t)kTmaRing || qi - qc >= (uint32_t)kTmaQ) return false;
    tail += skip;
    o = tail % kTmaRing;
    const int slot = qi % kTmaQ;
    if (lane == 0) {
      s_poff[warp][slot] = o;
      s_pend[warp][slot] = tail + bytes;
      fence_proxy_async();  // earlier generic reads of this ring space come first
      mbar_expect_tx(&s_bar[warp][slot], bytes);
      tma_load_2d(ring + o, &tmd.tap[st.bw[h] / 2 - 1], st.x[h], st.y[h] + 8 * k, &s_bar[warp][slot]);
    }
    tail += bytes;
    ++qi;
    return true;
  };
  // Release the first `cnt` unconsumed pieces (in order).
  auto release = [&](int cnt) {
    for (int c = 0; c < cnt; ++c) {
      head = s_pend[warp][qc % kTmaQ];
      ++qc;
    }
  };

  int parity = 0;
  for (uint64_t cb = blockIdx.x; cb < nchunks; cb = next_chunk(cb, queue, &s_chunk)) {
  const uint32_t c0 = (uint32_t)(cb * chunk);
  if (c0 + chunk > nvalid) {  // rows the plan rejected: zero output
    const uint32_t b = max(c0, nvalid), e = (uint32_t)min((uint64_t)c0 + chunk, (uint64_t)nvis);
    for (uint32_t r = b + threadIdx.x; r < e; r += blockDim.x) vis_out[sidx[r]] = make_float2(0.f, 0.f);
    if (c0 >= nvalid) continue;
  }
  const uint32_t c1 = min(c0 + chunk, nvalid);
  uint32_t pos = c0;
  while (pos < c1) {
    const SegInfo sg = seg_at(pos, c1, smap, off, g);
    if (threadIdx.x == 0) s_next[parity] = pos;  // published by the barrier in seg_box
    uint32_t *next_row = &s_next[parity];
    // The footprint pass ends in a barrier: every warp has finished the
    // previous segment (its ring drained, its grid reads done).
    const SegBox box = seg_box<NW, 1, false>(sg, pos, smap, sidx, nullptr, nullptr, g, s_red[parity]);
    parity ^= 1;
    const bool direct = seg_direct(box, sg.end - pos);
    const int64_t gplane = (int64_t)sg.ch * g.nw + sg.zg;
    if (!direct) {
      const int gx0 = sg.u0 & ~1, xs = sg.u0 - gx0;  // the copy starts on an even column
      if (threadIdx.x == 0) {
        fence_proxy_async();
        mbar_expect_tx(&s_gbar, (uint32_t)(RW * SG * 8));
        tma_load_3d(ring_all, &tmd.grid, gx0, sg.v0, (int)gplane, &s_gbar);
      }
      if (!mbar_wait(&s_gbar, gphase)) ok = false;
      gphase ^= 1;
      const float2 *raw = reinterpret_cast<const float2 *>(ring_all);
      for (int y = box.y0 + warp; y < box.y1; y += NW)
        for (int x = box.x0 + lane; x < box.x1; x += 32) {
          const float2 v = raw[y * RW + x + xs];
          sub4[y * SG + x] = make_float4(v.x, v.x, v.y, v.y);
        }
      __syncthreads();  // the tile is expanded; the rings may be refilled
    }
    auto row_loop = [&](auto lpr_c) {
      constexpr int LP = decltype(lpr_c)::value;
      constexpr int RP = 32 / LP;
      const int hl = lane & (LP - 1), half = lane / LP;
      // Row metadata of a step starting at r: this lane's own row (m, idx)
      // and the warp-uniform copy geometry of every row.
      auto load_step = [&](uint32_t r, RowMap &m, uint32_t &idx, TmaStep &st) {
        const bool act = r + half < sg.end;
        int np = 0, bw = 2, x = 0, y = 0;
        if (act) {
          m = smap[r + half];
          idx = sidx[r + half];
          const int uf = m.sub & 0xff, vf = (m.sub >> 8) & 0xff, zc = m.sub >> 16;
          const int sz = plane_sz(g, zc), toff = (S - sz) >> 1;
          const int64_t e = sg.ch * g.cf_chan_stride + zc * g.cf_z_stride + (int64_t)(vf * O + uf) * S * S;
          np = (sz + 7) >> 3;
          bw = sz + 2 * (toff & 1);
          x = toff & ~1;
          y = (int)(e / S) + toff;
        }
        st.n = 0;
        st.total = 0;
        st.maxk = 0;
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          const int src = h < RP ? h * LP : 0;
          const int nph = __shfl_sync(0xffffffffu, np, src);
          st.np[h] = h < RP ? nph : 0;
          st.bw[h] = __shfl_sync(0xffffffffu, bw, src);
          st.x[h] = __shfl_sync(0xffffffffu, x, src);
          st.y[h] = __shfl_sync(0xffffffffu, y, src);
          if (h < RP && r + h < sg.end) st.n = h + 1;
          st.total += st.np[h];
          st.maxk = max(st.maxk, st.np[h]);
        }
      };
      uint32_t rbase = 0;
      if (lane == 0) rbase = atomicAdd(next_row, (uint32_t)RP);
      rbase = __shfl_sync(0xffffffffu, rbase, 0);
      RowMap m{};
      uint32_t idx = 0;
      TmaStep cur;
      load_step(rbase, m, idx, cur);
      int ci = 0;  // pieces of cur issued
      while (ci < cur.total && try_issue(cur, ci)) ++ci;
      uint32_t cq0 = qi - ci;  // sequence number of cur's first piece
      __syncwarp();
      while (rbase < sg.end) {
        uint32_t rn = 0;
        if (lane == 0) rn = atomicAdd(next_row, (uint32_t)RP);
        rn = __shfl_sync(0xffffffffu, rn, 0);
        RowMap mn{};
        uint32_t idxn = 0;
        TmaStep nxt;
        load_step(rn, mn, idxn, nxt);
        int ni = 0;
        // the rest of cur, then nxt, as far as the ring allows
        auto refill = [&]() {
          while (ci < cur.total && try_issue(cur, ci)) ++ci;
          if (ci == cur.total)
            while (ni < nxt.total && try_issue(nxt, ni)) ++ni;
          __syncwarp();
        };
        refill();
        const bool act = rbase + half < sg.end;
        const int zc = m.sub >> 16;
        const int sz = act ? plane_sz(g, zc) : 0;
        const int bwr = sz + 2 * (((S - sz) >> 1) & 1), xsr = ((S - sz) >> 1) & 1;
        const int wu = m.pu - (sz >> 1), wv = m.pv - (sz >> 1);
        const int wofs4 = (wv - sg.v0) * SG + (wu - sg.u0) + hl, dg = SG - sz;
        const unsigned char *tj = tab + tap_base(sz > 0 ? sz : 2) + hl;
        unsigned long long pa = 0ull, pb = 0ull;
        for (int k = 0; k < cur.maxk; ++k) {
          // column k of cur must be in flight before anyone waits on it
          while (ci < cur.total && ci <= tma_piece_index(cur, cur.n - 1, k) && try_issue(cur, ci)) ++ci;
          __syncwarp();
          const bool mine = act && k * 8 < sz;
          if (mine) {
            const uint32_t q = cq0 + (uint32_t)tma_piece_index(cur, half, k);
            const int slot = q % kTmaQ;
            if (!mbar_wait(&s_bar[warp][slot], (q / kTmaQ) & 1)) ok = false;
            const float2 *kl = reinterpret_cast<const float2 *>(ring + s_poff[warp][slot]) + xsr - 8 * k * bwr + hl;
            const int dk = bwr - sz;
            const int t1 = min(8 * k + 8, sz) * sz;
            auto group = [&](int t, auto kk, auto masked) {
              constexpr int K = decltype(kk)::value;
              int j[K];
              bool on[K];
              unsigned long long tp[K];
              ulonglong2 gv[K];
#pragma unroll
              for (int u = 0; u < K; ++u) {
                on[u] = !decltype(masked)::value || t + LP * u + hl < t1;
                j[u] = on[u] ? tj[t + LP * u] : 0;
                tp[u] = on[u] ? *reinterpret_cast<const unsigned long long *>(kl + t + LP * u + j[u] * dk) : 0ull;
                gv[u] = on[u] ? *reinterpret_cast<const ulonglong2 *>(sub4 + wofs4 + t + LP * u + j[u] * dg)
                              : make_ulonglong2(0ull, 0ull);
              }
#pragma unroll
              for (int u = 0; u < K; ++u) {
                pa = ffma2(gv[u].x, tp[u], pa);
                pb = ffma2(gv[u].y, tp[u], pb);
              }
            };
            int t = 8 * k * sz;
            for (; t + 4 * LP <= t1; t += 4 * LP) group(t, IntC<4>(), BoolC<false>());
            switch ((t1 - t + LP - 1) / LP) {
              case 1: group(t, IntC<1>(), BoolC<true>()); break;
              case 2: group(t, IntC<2>(), BoolC<true>()); break;
              case 3: group(t, IntC<3>(), BoolC<true>()); break;
              case 4: group(t, IntC<4>(), BoolC<true>()); break;
              default: break;
            }
          }
          __syncwarp();  // every lane is done with column k
          int cnt = 0;
          for (int h = 0; h < cur.n; ++h) cnt += k < cur.np[h];
          release(cnt);
          refill();
        }
        const float2 a2 = *reinterpret_cast<const float2 *>(&pa);
        const float2 b2 = *reinterpret_cast<const float2 *>(&pb);
        float sx = a2.x - b2.y, sy = a2.y + b2.x;
        for (int o = LP / 2; o > 0; o >>= 1) {
          sx += __shfl_xor_sync(0xffffffffu, sx, o);
          sy += __shfl_xor_sync(0xffffffffu, sy, o);
        }
        if (act && hl == 0) vis_out[idx] = make_float2(sx, sy);
        // nxt becomes cur
        cq0 += (uint32_t)cur.total;
        cur = nxt;
        ci = ni;
        m = mn;
        idx = idxn;
        rbase = rn;
      }
    };
    if (direct) {
      // Few rows for the footprint: taps and grid cells straight from global
      // memory, one row per warp.
      const float2 *gp = grid + gplane * plane_elems;
      uint32_t r = 0;
      if (lane == 0) r = atomicAdd(next_row, 1u);
      r = __shfl_sync(0xffffffffu, r, 0);
      while (r < sg.end) {
        const RowMap mr = smap[r];
        const uint32_t ir = sidx[r];
        const int uf = mr.sub & 0xff, vf = (mr.sub >> 8) & 0xff, zc = mr.sub >> 16;
        const int sz = plane_sz(g, zc), toff = (S - sz) >> 1;
        const float2 *kb = cf + sg.ch * g.cf_chan_stride + zc * g.cf_z_stride +
                           ((int64_t)(vf * O + uf) * S + toff) * S + toff;
        const int wu = mr.pu - (sz >> 1), wv = mr.pv - (sz >> 1);
        float ax = 0.f, ay = 0.f;
        for (int t = lane; t < sz * sz; t += 32) {
          const int j = t / sz, i = t - j * sz;
          const float2 tp = kb[j * S + i];
          const float2 gv = gp[(int64_t)(wv + j) * g.nx + wu + i];
          ax += gv.x * tp.x - gv.y * tp.y;
          ay += gv.x * tp.y + gv.y * tp.x;
        }
        for (int o = 16; o > 0; o >>= 1) {
          ax += __shfl_xor_sync(0xffffffffu, ax, o);
          ay += __shfl_xor_sync(0xffffffffu, ay, o);
        }
        if (lane == 0) vis_out[ir] = make_float2(ax, ay);
        if (lane == 0) r = atomicAdd(next_row, 1u);
        r = __shfl_sync(0xffffffffu, r, 0);
      }
    } else if (box.sz <= 8) {
      row_loop(IntC<8>());
    } else if (box.sz <= 16) {
      row_loop(IntC<16>());
    } else {
      row_loop(IntC<32>());
    }
    pos = sg.end;
  }
  }
  // Leave no copy in flight: every piece this warp issued has completed
  // (immediate unless a wait above gave up).
  if (lane == 0)
    for (uint32_t q = qi > (uint32_t)kTmaQ ? qi - kTmaQ : 0u; q < qi; ++q)
      if (!mbar_wait(&s_bar[warp][q % kTmaQ], (q / kTmaQ) & 1)) ok = false;
  if (!ok) atomicOr(err, 1u);
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
static double rcp(double x) { return 1.0 / x; }

int make_geom(const arlgpu_grid_desc *gd, const arlgpu_cf_desc *cd, int precision, Geom *g) {
  if (!gd || !cd) return fail(ARLGPU_ERR_INVALID, "null descriptor");
  if (precision != ARLGPU_FP32C && precision != ARLGPU_FP64)
    return fail(ARLGPU_ERR_INVALID, "precision must be ARLGPU_FP32C or ARLGPU_FP64");
  if (gd->nchan < 1 || gd->npol < 1 || gd->nw < 1 || gd->ny < 2 || gd->nx < 2)
    return fail(ARLGPU_ERR_INVALID, "bad grid shape");
  if (gd->npol > 4) return fail(ARLGPU_ERR_UNSUPPORTED, "npol > 4");
  if (cd->npol != gd->npol && !(cd->npol == 1 && cd->pol_stride == 0))
    return fail(ARLGPU_ERR_INVALID, "cf npol %d != grid npol %d", cd->npol, gd->npol);
  if (cd->oversampling < 1 || cd->oversampling > 256) return fail(ARLGPU_ERR_UNSUPPORTED, "oversampling must be 1..256");
  if (cd->support < 2 || (cd->support & 1)) return fail(ARLGPU_ERR_UNSUPPORTED, "support must be even (ARL slices v-S/2:v+S/2)");
  if (cd->support > 64) return fail(ARLGPU_ERR_UNSUPPORTED, "support > 64");
  if (cd->nz < 1 || cd->nz > 65535 || gd->nw > 65535 || gd->nchan > 65535)
    return fail(ARLGPU_ERR_UNSUPPORTED, "nz, nw and nchan must be < 65536");
  if (gd->ny > (1 << 20) || gd->nx > (1 << 20)) return fail(ARLGPU_ERR_UNSUPPORTED, "grid too large");
  memset(g, 0, sizeof *g);
  g->nchan = gd->nchan;
  g->npol = gd->npol;
  g->nw = gd->nw;
  g->ny = gd->ny;
  g->nx = gd->nx;
  g->cf_nchan = cd->nchan;
  g->cf_npol = cd->npol;
  g->nz = cd->nz;
  g->O = cd->oversampling;
  g->S = cd->support;
  g->cf_chan_stride = cd->chan_stride;
  g->cf_pol_stride = cd->pol_stride;
  g->cf_z_stride = (int64_t)cd->oversampling * cd->oversampling * cd->support * cd->support;
  g->gu = gd->u;
  g->gv = gd->v;
  g->gw = gd->w;
  g->gf = gd->f;
  g->cdu = cd->du;
  g->cdv = cd->dv;
  g->cz = cd->z;
  g->rcp_gu = rcp(gd->u.cdelt);
  g->rcp_gv = rcp(gd->v.cdelt);
  g->rcp_gw = rcp(gd->w.cdelt);
  g->rcp_gf = rcp(gd->f.cdelt);
  g->rcp_cdu = rcp(cd->du.cdelt);
  g->rcp_cdv = rcp(cd->dv.cdelt);
  g->rcp_cz = rcp(cd->z.cdelt);
  g->plane_support = cd->plane_support;
  g->tap_absmax = cd->tap_absmax > 0.0 && cd->tap_absmax < 1e30 ? (float)cd->tap_absmax : 0.f;
  {
    // The fast u/v mapping needs zero crvals, integer crpixes and the cf's
    // sub-pixel cdelt equal to the grid cdelt / O (ARL builds both from one
    // image, so this is the usual case).
    auto integral = [](double x) { return x == (double)(long long)x; };
    g->fast_uv = gd->u.crval == 0.0 && gd->v.crval == 0.0 && cd->du.crval == 0.0 && cd->dv.crval == 0.0 &&
                 integral(gd->u.crpix) && integral(gd->v.crpix) && integral(cd->du.crpix) &&
                 integral(cd->dv.crpix) && cd->du.cdelt == gd->u.cdelt / cd->oversampling &&
                 cd->dv.cdelt == gd->v.cdelt / cd->oversampling && fabs(gd->u.crpix) < 1e9 &&
                 fabs(gd->v.crpix) < 1e9;
    const int O = cd->oversampling;
    g->pow2O = g->fast_uv && O >= 2 && (O & (O - 1)) == 0 && O <= 256 && cd->du.crpix - 1.0 == (double)(O / 2) &&
               cd->dv.crpix - 1.0 == (double)(O / 2);
    g->log2O = 0;
    while ((1 << g->log2O) < O) ++g->log2O;
    // X = fma(u, rcp * O, (crpix - 1) O) is within ~2.2e-16 (|X| + |cO|) of the
    // exact value and NumPy's sequence within a few ulps of it: tol has a
    // 10x margin over both for every |X| < Xlim.
    g->rOu = g->rcp_gu * O;
    g->rOv = g->rcp_gv * O;
    g->cOu = (gd->u.crpix - 1.0) * O;
    g->cOv = (gd->v.crpix - 1.0) * O;
    g->Xlim_u = ((double)gd->nx + 2.0 * cd->support + 4.0) * O + fabs(g->cOu);
    g->Xlim_v = ((double)gd->ny + 2.0 * cd->support + 4.0) * O + fabs(g->cOv);
    g->tolX_u = 1e-14 * (g->Xlim_u + fabs(g->cOu) + 2.0 * O);
    g->tolX_v = 1e-14 * (g->Xlim_v + fabs(g->cOv) + 2.0 * O);
    if (g->Xlim_u > 1e9 || g->Xlim_v > 1e9) g->pow2O = 0;  // keep floor(X) within int range
  }
  // Fixed tolerances of the nearest-plane axes, valid for |P| < Plim (the
  // per-row tolerance 1e-14 (|P| + |crpix| + 2) of the exact-fallback test,
  // bounded over that range).
  g->Plim_w = (double)gd->nw + 2.0;
  g->tol_w = 1e-14 * (g->Plim_w + fabs(gd->w.crpix) + 2.0);
  g->Plim_z = (double)cd->nz + 2.0;
  g->tol_z = 1e-14 * (g->Plim_z + fabs(cd->z.crpix) + 2.0);
  g->Plim_f = (double)gd->nchan + 2.0;
  g->tol_f = 1e-14 * (g->Plim_f + fabs(gd->f.crpix) + 2.0);
  {
    auto tq = [](double tol) { return (int32_t)std::min(ceil(tol * 1048576.0) + 1.0, 1e9); };
    g->tq_u = tq(g->tolX_u);
    g->tq_v = tq(g->tolX_v);
    g->tq_w = tq(g->tol_w);
    g->tq_z = tq(g->tol_z);
    g->tq_f = tq(g->tol_f);
    const double lim = 536870912.0;  // 2^29
    // world interval covered by planes [0, n) of a nearest-plane axis
    auto span = [](const arlgpu_axis &a, int n, double *lo, double *hi) {
      const double e0 = a.crval + (0.5 - a.crpix) * a.cdelt, e1 = a.crval + ((double)n + 0.5 - a.crpix) * a.cdelt;
      *lo = std::min(e0, e1);
      *hi = std::max(e0, e1);
    };
    double glo, ghi, zlo, zhi;
    span(gd->w, gd->nw, &glo, &ghi);
    span(cd->z, cd->nz, &zlo, &zhi);
    auto inside = [](double alo, double ahi, double blo, double bhi) {  // [alo, ahi] well inside [blo, bhi]
      const double m = 1e-9 * ((bhi - blo) + fabs(blo) + fabs(bhi));
      return std::isfinite(alo) && std::isfinite(ahi) && alo > blo + m && ahi < bhi - m;
    };
    g->skip_zg = gd->nw == 1 && inside(zlo, zhi, glo, ghi);
    g->skip_zc = cd->nz == 1 && inside(glo, ghi, zlo, zhi);
    g->fixmap = g->pow2O && g->Xlim_u < lim && g->Xlim_v < lim && g->Plim_w < lim && g->Plim_z < lim &&
                g->Plim_f < lim && g->tq_u < (1 << 18) && g->tq_v < (1 << 18) && g->tq_w < (1 << 18) &&
                g->tq_z < (1 << 18) && g->tq_f < (1 << 18);
  }
  // Subgrid edge: 64 cells when npol planes of it (with the FP32 compensation
  // words) fit in 64 KiB of shared memory, else 32.
  const size_t cell = precision == ARLGPU_FP64 ? 16 : 16;  // c128, or c64 sum + c64 comp
  int SG = g_tune_subgrid.load();
  if (SG <= 0) {
    SG = 48;  // the C2 autotuning optimum for supports 8..32
    if ((size_t)g->npol * SG * SG * cell > 64 * 1024) SG = 32;
  }
  if (SG - g->S < 8) SG = ((g->S + 8 + 7) / 8) * 8;
  SG = (SG + 7) & ~7;  // a multiple of the band-owner warp count
  if ((size_t)g->npol * SG * fx_pitch(SG) * cell > 200 * 1024)
    return fail(ARLGPU_ERR_UNSUPPORTED, "support %d with %d polarisations needs more shared memory than a CTA has",
                g->S, g->npol);
  g->SG = SG;
  g->T = SG - g->S;
  g->ntu = (g->nx + g->T - 1) / g->T;
  g->ntv = (g->ny + g->T - 1) / g->T;
  uint64_t nb = (uint64_t)g->nchan * g->nw * g->ntv * g->ntu;
  if (nb >= 0x7fffffffull) return fail(ARLGPU_ERR_UNSUPPORTED, "too many bins");
  g->nbins = (uint32_t)nb;
  return ARLGPU_OK;
}

static size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

// Shares per (channel, plane) run for the plane-mean sums: about 4096 blocks
// in all.
static uint32_t wpart_shares(const Geom &g) {
  const uint64_t runs = (uint64_t)g.nchan * g.nw;
  return runs >= 4096 ? 1u : (uint32_t)(4096 / runs);
}
uint32_t plan_wpart_items(const Geom &g) { return (uint32_t)g.nchan * g.nw * wpart_shares(g); }

size_t plan_bytes(int64_t nvis, const Geom &g) {
  size_t n = (size_t)nvis;
  return align_up(n * 4) + align_up(n * sizeof(RowMap)) + align_up(n * 4) + align_up(n * sizeof(RowMap)) +
         align_up(((size_t)g.nbins + 1) * 4) + align_up(((size_t)g.nbins + 2) * 4) +
         align_up((size_t)plan_wpart_items(g) * 8) + align_up(16);
}

int plan_carve(void *ws, size_t bytes, int64_t nvis, const Geom &g, PlanBufs *b) {
  size_t need = plan_bytes(nvis, g);
  if (!ws || bytes < need)
    return fail(ARLGPU_ERR_WORKSPACE, "workspace of %zu bytes is smaller than the %zu needed", bytes, need);
  // the plan kernels move row maps as 128-bit loads and stores
  if (reinterpret_cast<uintptr_t>(ws) & 15)
    return fail(ARLGPU_ERR_INVALID, "workspace must start on a 16-byte boundary");
  char *p = static_cast<char *>(ws);
  size_t n = (size_t)nvis;
  b->keys = reinterpret_cast<uint32_t *>(p);
  p += align_up(n * 4);
  b->maps = reinterpret_cast<RowMap *>(p);
  p += align_up(n * sizeof(RowMap));
  b->sidx = reinterpret_cast<uint32_t *>(p);
  p += align_up(n * 4);
  b->smap = reinterpret_cast<RowMap *>(p);
  p += align_up(n * sizeof(RowMap));
  b->hist = reinterpret_cast<uint32_t *>(p);
  p += align_up(((size_t)g.nbins + 1) * 4);
  b->offsets = reinterpret_cast<uint32_t *>(p);
  p += align_up(((size_t)g.nbins + 2) * 4);
  b->wpart = reinterpret_cast<double *>(p);
  p += align_up((size_t)plan_wpart_items(g) * 8);
  b->queue = reinterpret_cast<uint32_t *>(p);
  return ARLGPU_OK;
}

static int num_sms() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 152;
  }
  return n;
}

int plan_build(const double *uvw, const double *freq, int64_t nvis, const Geom &g, const PlanBufs &b,
               int64_t *n_bad_dev, cudaStream_t st) {
  const uint32_t nh = g.nbins + 1;
  ARL_CUDA(cudaMemsetAsync(b.hist, 0, (size_t)nh * 4, st));
  if (nvis > 0) {
    int blocks = (int)std::min<int64_t>((nvis + 255) / 256, (int64_t)num_sms() * 16);
    k_map<<<blocks, 256, 0, st>>>(uvw, freq, nvis, g, b.keys, b.maps, b.hist);
    ARL_LAUNCH_CHECK();
    count_launch(1);
  }
  const uint32_t ntiles = (nh + kScanTile - 1) / kScanTile;
  if (ntiles <= 4 || ntiles > 8192 || (size_t)plan_wpart_items(g) * 2 < ntiles) {
    k_scan<<<1, 1024, 0, st>>>(b.hist, nh, b.offsets, n_bad_dev, g.nbins);
    ARL_LAUNCH_CHECK();
    count_launch(1);
  } else {
    // the plane-mean partials' area is free while the plan is built
    uint32_t *tile_sum = reinterpret_cast<uint32_t *>(b.wpart);
    k_scan_tiles<<<ntiles, 1024, 0, st>>>(b.hist, nh, b.offsets, tile_sum);
    ARL_LAUNCH_CHECK();
    k_scan_totals<<<1, 1024, 0, st>>>(tile_sum, ntiles, b.offsets, nh, n_bad_dev, b.hist, g.nbins);
    ARL_LAUNCH_CHECK();
    k_scan_add<<<(nh + 255) / 256, 256, 0, st>>>(b.offsets, nh, tile_sum);
    ARL_LAUNCH_CHECK();
    count_launch(3);
  }
  ARL_CUDA(cudaMemsetAsync(b.hist, 0, (size_t)nh * 4, st));
  if (nvis > 0) {
    int blocks = (int)std::min<int64_t>((nvis + 255) / 256, (int64_t)num_sms() * 16);
    k_scatter<<<blocks, 256, 0, st>>>(b.keys, b.maps, nvis, b.offsets, b.hist, b.sidx, b.smap);
    ARL_LAUNCH_CHECK();
    count_launch(1);
  }
  return ARLGPU_OK;
}

static constexpr int kWarps = 8;
static inline uint32_t chunk_rows() { return (uint32_t)g_tune_chunk.load(); }

// Grid of a chunk-looping kernel: one CTA per chunk, or (persistent) as many
// CTAs as can be resident, each taking every gridDim.x-th chunk.  The
// persistent grid builds each CTA's tap table and clears its subgrid once
// instead of once per chunk.
template <typename K>
static unsigned chunk_grid(K kern, size_t smem, int64_t nvis, uint32_t chunk) {
  const int64_t nchunks = (nvis + chunk - 1) / chunk;
  if (nchunks <= 0) return 0;
  if (g_tune_persistent.load() != 0) {
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kWarps * 32, smem) == cudaSuccess && occ > 0) {
      const int64_t resident = (int64_t)occ * num_sms();
      return (unsigned)(nchunks < resident ? nchunks : resident);
    }
  }
  return (unsigned)nchunks;
}

// Lanes per row of the FP32C gridder / packed degridder: the tuning key
// lanes_per_row when set (8, 16 or 32 for every segment); else, for supports
// up to 8, 32 / small_rows (gridder) or 32 / small_rows_degrid (degridder);
// else 0, the per-segment choice.
static int lanes_per_row(const Geom &g, bool degrid = false) {
  const int fixed = g_tune_lanes.load();
  if (fixed) return fixed;
  if (g.S <= 8) return 32 / (degrid ? g_tune_small_rows_dg.load() : g_tune_small_rows.load());
  return 0;
}

// The device work-queue word of a chunk-looping launch (0: gridder, 1:
// degridder) when the persistent grid takes its chunks dynamically
// (tuning "persistent" = 2), else null (static every-gridDim-th chunk).
static uint32_t *work_queue(const PlanBufs &b, int which, cudaStream_t) {
  return g_tune_persistent.load() == 2 ? b.queue + which : nullptr;
}

// Elements of the cf table the geometry addresses.
static int64_t cf_elems(const Geom &g) {
  return (int64_t)(g.cf_nchan - 1) * g.cf_chan_stride + (int64_t)(g.cf_npol - 1) * g.cf_pol_stride +
         (int64_t)g.nz * g.cf_z_stride;
}

static int launch_grid_fx(const Geom &g, const PlanBufs &b, int64_t nvis, const void *vis, const void *wt,
                          const void *cf, void *grid, double *sumwt, bool resid, cudaStream_t st) {
  const size_t smem = (size_t)(resid ? 4 : 2) * g.npol * g.SG * fx_pitch(g.SG) * 4 + tap_table_bytes(g.S);
  if (smem > 227 * 1024) return fail(ARLGPU_ERR_UNSUPPORTED, "gridder needs %zu bytes of shared memory", smem);
  void (*kern)(Geom, const RowMap *, const uint32_t *, const uint32_t *, uint32_t, const float2 *, const float *,
               const float2 *, float2 *, double *, uint32_t *);
  // Lanes per row: the tuning key lanes_per_row (8, 16 or 32 for every
  // segment), else for supports up to 8 (64 taps) 32 / small_rows, else
  // chosen per segment (0).
  const int lpr = lanes_per_row(g);
  // The default subgrid edge (48, or 32 with four polarisations) runs a
  // compile-time-edge instantiation; other edges (autotuner trials) the
  // runtime-edge one, with lanes per row chosen per segment.
  const bool csg = g.SG == (g.npol == 4 ? 32 : 48);
  // One polarisation: vis and weight copied into bin order first (into the
  // plan's dead mapping scratch: 8 + 4 bytes per row against its 20) and
  // read by sorted position (the SORTED instantiations).
  const bool sorted = g.npol == 1 && g_tune_gather.load() != 0;
  // With sorted rows, chunks of at most kStashRows rows and a cf table
  // addressable in 32 bits: the row set-up comes from the footprint pass (as
  // in the packed degridder, which takes it for supports above 8 only).
  const bool stash = sorted && g_tune_stash.load() != 0 && chunk_rows() <= (uint32_t)kStashRows &&
                     cf_elems(g) < 0x7fffffffll;
  // Four polarisations (rows gathered through the sort index): the stash
  // carries each row's index too.
  const bool stash4 = g.npol == 4 && g_tune_stash.load() != 0 && chunk_rows() <= (uint32_t)kStashRows &&
                      cf_elems(g) < 0x7fffffffll;
  auto pick = [&](auto resid_c) {
    constexpr bool RS = decltype(resid_c)::value;
    auto by_lpr = [&](auto npol_c, auto sg_c, auto sorted_c, auto stash_c) {
      constexpr int NP = decltype(npol_c)::value, SGV = decltype(sg_c)::value;
      constexpr bool SO = decltype(sorted_c)::value, ST = decltype(stash_c)::value;
      return lpr == 8 ? k_grid_fx<NP, kWarps, RS, 8, SGV, SO, ST>
                      : lpr == 16 ? k_grid_fx<NP, kWarps, RS, 16, SGV, SO, ST>
                                  : lpr == 32 ? k_grid_fx<NP, kWarps, RS, 32, SGV, SO, ST>
                                              : k_grid_fx<NP, kWarps, RS, 0, SGV, SO, ST>;
    };
    if (csg) {
      if (g.npol == 4)
        return stash4 ? by_lpr(IntC<4>(), IntC<32>(), BoolC<false>(), BoolC<true>())
                      : by_lpr(IntC<4>(), IntC<32>(), BoolC<false>(), BoolC<false>());
      if (g.npol == 2) return by_lpr(IntC<2>(), IntC<48>(), BoolC<false>(), BoolC<false>());
      if (!sorted) return by_lpr(IntC<1>(), IntC<48>(), BoolC<false>(), BoolC<false>());
      return stash ? by_lpr(IntC<1>(), IntC<48>(), BoolC<true>(), BoolC<true>())
                   : by_lpr(IntC<1>(), IntC<48>(), BoolC<true>(), BoolC<false>());
    }
    if (g.npol == 1) return sorted ? k_grid_fx<1, kWarps, RS, 0, 0, true> : k_grid_fx<1, kWarps, RS>;
    return g.npol == 2 ? k_grid_fx<2, kWarps, RS> : k_grid_fx<4, kWarps, RS>;
  };
  kern = resid ? pick(BoolC<true>()) : pick(BoolC<false>());
  ARL_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const uint32_t chunk = chunk_rows();
  const unsigned blocks = chunk_grid(kern, smem, nvis, chunk);
  if (blocks == 0) return ARLGPU_OK;
  uint32_t *queue = work_queue(b, 0, st);
  if (queue) ARL_CUDA(cudaMemsetAsync(queue, 0, 4, st));
  const void *vis_k = vis, *wt_k = wt;
  if (sorted) {
    float2 *vis_s = reinterpret_cast<float2 *>(b.maps);
    float *wt_s = reinterpret_cast<float *>(b.keys);
    const int gblocks = (int)std::min<int64_t>((nvis + 255) / 256, (int64_t)num_sms() * 8);
    k_gather_rows<<<gblocks, 256, 0, st>>>(b.sidx, b.offsets, g.nbins, static_cast<const float2 *>(vis),
                                           static_cast<const float *>(wt), vis_s, wt_s);
    ARL_LAUNCH_CHECK();
    count_launch(1);
    vis_k = vis_s;
    wt_k = wt_s;
  }
  kern<<<blocks, kWarps * 32, smem, st>>>(g, b.smap, b.sidx, b.offsets, chunk, static_cast<const float2 *>(vis_k),
                                          static_cast<const float *>(wt_k), static_cast<const float2 *>(cf),
                                          static_cast<float2 *>(grid), sumwt, queue);
  ARL_LAUNCH_CHECK();
  count_launch(1);
  return ARLGPU_OK;
}

template <typename R>
static int launch_grid(const Geom &g, const PlanBufs &b, int64_t nvis, const void *vis, const void *wt,
                       const void *cf, void *grid, double *sumwt, cudaStream_t st) {
  size_t smem = (size_t)g.npol * g.SG * g.SG * sizeof(typename Cplx<R>::T) * SmemAcc<R>::kWords;
  auto kern = k_grid<R, kWarps>;
  if (g_tune_grid_kernel.load() == 1) {
    kern = k_grid_band<R, kWarps>;
    smem += sizeof(StagedRow<typename Cplx<R>::T>) * kWarps * 32;
  } else if (g_tune_grid_kernel.load() == 2) {
    kern = g.npol == 1 ? k_grid_lean<R, 1, kWarps> : g.npol == 2 ? k_grid_lean<R, 2, kWarps>
                                                                  : k_grid_lean<R, 4, kWarps>;
    if (g.npol == 3) return fail(ARLGPU_ERR_UNSUPPORTED, "the lean gridder handles 1, 2 or 4 polarisations");
    smem += tap_table_bytes(g.S);
  } else if (g_tune_grid_kernel.load() == 3) {
    kern = g.npol == 1 ? k_grid_lean<R, 1, kWarps, PlainAcc<R>>
                       : g.npol == 2 ? k_grid_lean<R, 2, kWarps, PlainAcc<R>> : k_grid_lean<R, 4, kWarps, PlainAcc<R>>;
    if (g.npol == 3) return fail(ARLGPU_ERR_UNSUPPORTED, "the lean gridder handles 1, 2 or 4 polarisations");
    smem = (size_t)g.npol * g.SG * g.SG * sizeof(typename Cplx<R>::T) + tap_table_bytes(g.S);
  } else if (g_tune_grid_kernel.load() >= 4) {
    if (g.npol == 3) return fail(ARLGPU_ERR_UNSUPPORTED, "the lean gridder handles 1, 2 or 4 polarisations");
    if (sizeof(R) == 4 && g.tap_absmax > 0.f)
      return launch_grid_fx(g, b, nvis, vis, wt, cf, grid, sumwt, g_tune_grid_kernel.load() == 4, st);
    // FP64, or no tap bound: the compensated float variant
    kern = g.npol == 1 ? k_grid_lean<R, 1, kWarps> : g.npol == 2 ? k_grid_lean<R, 2, kWarps>
                                                                  : k_grid_lean<R, 4, kWarps>;
    smem += tap_table_bytes(g.S);
  }
  // The lean variants' planar subgrid has the same size as the interleaved one.
  if (smem > 227 * 1024) return fail(ARLGPU_ERR_UNSUPPORTED, "gridder needs %zu bytes of shared memory", smem);
  ARL_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const uint32_t chunk = chunk_rows();
  const bool loops = g_tune_grid_kernel.load() >= 2;  // the lean kernels loop over chunks
  const unsigned blocks = loops ? chunk_grid(kern, smem, nvis, chunk) : (unsigned)((nvis + chunk - 1) / chunk);
  if (blocks == 0) return ARLGPU_OK;
  uint32_t *queue = loops ? work_queue(b, 0, st) : nullptr;
  if (queue) ARL_CUDA(cudaMemsetAsync(queue, 0, 4, st));
  kern<<<blocks, kWarps * 32, smem, st>>>(g, b.smap, b.sidx, b.offsets, chunk,
                                          static_cast<const typename VisT<R>::C *>(vis),
                                          static_cast<const typename VisT<R>::W *>(wt),
                                          static_cast<const typename Cplx<R>::T *>(cf),
                                          static_cast<typename Cplx<R>::T *>(grid), sumwt, queue);
  ARL_LAUNCH_CHECK();
  count_launch(1);
  return ARLGPU_OK;
}

// The driver's tensor-map encoder, looked up once through the runtime (no
// link against libcuda).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

// Tensor maps of the TMA degridder, or false when this call cannot take it
// (alignment, sizes, or no encoder).
static bool make_tma_desc(const Geom &g, const void *cf, const void *grid, TmaDesc *d) {
  EncodeTiledFn enc = encode_tiled();
  if (!enc) return false;
  if ((reinterpret_cast<uintptr_t>(cf) & 15) || (reinterpret_cast<uintptr_t>(grid) & 15)) return false;
  // Row strides of both tables a multiple of 16 bytes (S and nx even), and
  // every sub-kernel starting on a table row (channel stride a multiple of S).
  if (g.S > kTmaMaxS || g.S < 2 || (g.S & 1) || g.cf_chan_stride < 0 || (g.cf_chan_stride % g.S) != 0 ||
      (g.nx & 1))
    return false;
  const int64_t elems = (int64_t)(g.cf_nchan - 1) * g.cf_chan_stride + (int64_t)(g.cf_npol - 1) * g.cf_pol_stride +
                        (int64_t)g.nz * g.cf_z_stride;
  const int64_t rows = elems / g.S;
  if (rows < 1 || rows > 0x7fffffffll) return false;
  memset(d, 0, sizeof *d);
  for (int m = 0; m < 16; ++m) {
    const int bw = 2 * m + 2;
    if (bw > g.S) break;
    const cuuint64_t dims[2] = {(cuuint64_t)g.S, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)g.S * 8};
    const cuuint32_t box[2] = {(cuuint32_t)bw, 8};
    const cuuint32_t es[2] = {1, 1};
    if (enc(&d->tap[m], CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, const_cast<void *>(cf), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return false;
  }
  const int64_t planes = (int64_t)g.nchan * g.npol * g.nw;
  const cuuint64_t gdims[3] = {(cuuint64_t)g.nx, (cuuint64_t)g.ny, (cuuint64_t)planes};
  const cuuint64_t gstr[2] = {(cuuint64_t)g.nx * 8, (cuuint64_t)g.nx * g.ny * 8};
  const cuuint32_t gbox[3] = {(cuuint32_t)(kTmaSG + 2), (cuuint32_t)kTmaSG, 1};
  const cuuint32_t ges[3] = {1, 1, 1};
  return enc(&d->grid, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, const_cast<void *>(grid), gdims, gstr, gbox, ges,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// degrid_kernel 4: the TMA degridder where it applies (FP32C, one
// polarisation, support <= 32, subgrid edge 48, aligned tables); *launched
// stays false (nothing launched) otherwise, and the caller runs the packed one.
static int launch_degrid_tma(const Geom &g, const PlanBufs &b, int64_t nvis, const void *cf, const void *grid,
                             void *vis_out, cudaStream_t st, bool *launched) {
  *launched = false;
  if (g.npol != 1 || g.SG != kTmaSG || g.S > kTmaMaxS) return ARLGPU_OK;
  TmaDesc d;
  if (!make_tma_desc(g, cf, grid, &d)) return ARLGPU_OK;
  auto kern = k_degrid_tma<kWarps>;
  const size_t smem = 128 + (size_t)kTmaSG * kTmaSG * 16 + (size_t)kWarps * kTmaRing + tap_table_bytes(g.S);
  ARL_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const uint32_t chunk = chunk_rows();
  const unsigned blocks = chunk_grid(kern, smem, nvis, chunk);
  if (blocks == 0) {
    *launched = true;
    return ARLGPU_OK;
  }
  uint32_t *queue = work_queue(b, 1, st);
  if (queue) ARL_CUDA(cudaMemsetAsync(queue, 0, 4, st));
  ARL_CUDA(cudaMemsetAsync(b.queue + 2, 0, 4, st));
  kern<<<blocks, kWarps * 32, smem, st>>>(d, g, b.smap, b.sidx, b.offsets, chunk, nvis,
                                          static_cast<const float2 *>(cf), static_cast<const float2 *>(grid),
                                          static_cast<float2 *>(vis_out), queue, b.queue + 2);
  ARL_LAUNCH_CHECK();
  count_launch(1);
  *launched = true;
  return ARLGPU_OK;
}

template <typename R>
static int launch_degrid(const Geom &g, const PlanBufs &b, int64_t nvis, const void *cf, const void *grid,
                         void *vis_out, cudaStream_t st) {
  if constexpr (sizeof(R) == 4) {
    if (g_tune_degrid_kernel.load() == 4) {
      bool launched = false;
      ARL_TRY(launch_degrid_tma(g, b, nvis, cf, grid, vis_out, st, &launched));
      if (launched) return ARLGPU_OK;
    }
  }
  size_t smem = (size_t)g.npol * g.SG * g.SG * sizeof(typename Cplx<R>::T);
  auto kern = k_degrid<R, kWarps>;
  if (g_tune_degrid_kernel.load() == 1) {
    kern = k_degrid_batch<R, kWarps>;
  } else if (g_tune_degrid_kernel.load() == 2 || (g_tune_degrid_kernel.load() >= 3 && sizeof(R) == 8)) {
    if (g.npol == 3) return fail(ARLGPU_ERR_UNSUPPORTED, "the lean degridder handles 1, 2 or 4 polarisations");
    kern = g.npol == 1 ? k_degrid_lean<R, 1, kWarps> : g.npol == 2 ? k_degrid_lean<R, 2, kWarps>
                                                                    : k_degrid_lean<R, 4, kWarps>;
    smem += tap_table_bytes(g.S);
  } else if (g_tune_degrid_kernel.load() >= 3) {  // FP32: packed multiply-adds (and where TMA does not apply)
    if (g.npol == 3) return fail(ARLGPU_ERR_UNSUPPORTED, "the lean degridder handles 1, 2 or 4 polarisations");
    // Lanes per row as in the gridder (small_rows_degrid for supports up to 8).
    const int lpr = lanes_per_row(g, true);
    bool done = false;
    if constexpr (sizeof(R) == 4) {
      // the default subgrid edge as a compile-time constant (see the gridder)
      if (g.SG == (g.npol == 4 ? 32 : 48)) {
        done = true;
        auto by_lpr = [&](auto npol_c, auto sg_c, auto stash_c) {
          constexpr int NP = decltype(npol_c)::value, SGV = decltype(sg_c)::value;
          constexpr bool ST = decltype(stash_c)::value;
          return lpr == 8 ? k_degrid_lean<R, NP, kWarps, true, 8, SGV, ST>
                          : lpr == 16 ? k_degrid_lean<R, NP, kWarps, true, 16, SGV, ST>
                                      : lpr == 32 ? k_degrid_lean<R, NP, kWarps, true, 32, SGV, ST>
                                                  : k_degrid_lean<R, NP, kWarps, true, 0, SGV, ST>;
        };
        // One polarisation, chunks of at most kStashRows rows and a cf table
        // addressable in 32 bits: the row set-up comes from the footprint pass.
        // (Supports above 8: with four rows per warp the set-up is already shared.)
        const bool stash = g.npol == 1 && g.S > 8 && g_tune_stash.load() != 0 &&
                           chunk_rows() <= (uint32_t)kStashRows && cf_elems(g) < 0x7fffffffll;
        if (g.npol == 4)
          kern = by_lpr(IntC<4>(), IntC<32>(), BoolC<false>());
        else if (g.npol == 2)
          kern = by_lpr(IntC<2>(), IntC<48>(), BoolC<false>());
        else
          kern = stash ? by_lpr(IntC<1>(), IntC<48>(), BoolC<true>()) : by_lpr(IntC<1>(), IntC<48>(), BoolC<false>());
      }
    }
    if (!done)  // runtime edge: rows per warp chosen per segment only
      kern = g.npol == 1 ? k_degrid_lean<R, 1, kWarps, sizeof(R) == 4>
                         : g.npol == 2 ? k_degrid_lean<R, 2, kWarps, sizeof(R) == 4>
                                       : k_degrid_lean<R, 4, kWarps, sizeof(R) == 4>;
    smem = (size_t)g.npol * g.SG * g.SG * 16 + tap_table_bytes(g.S);
  }
  if (smem > 227 * 1024) return fail(ARLGPU_ERR_UNSUPPORTED, "degridder needs %zu bytes of shared memory", smem);
  ARL_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const uint32_t chunk = chunk_rows();
  const bool loops = g_tune_degrid_kernel.load() >= 2;  // the lean kernels loop over chunks
  const unsigned blocks = loops ? chunk_grid(kern, smem, nvis, chunk) : (unsigned)((nvis + chunk - 1) / chunk);
  if (blocks == 0) return ARLGPU_OK;
  uint32_t *queue = loops ? work_queue(b, 1, st) : nullptr;
  if (queue) ARL_CUDA(cudaMemsetAsync(queue, 0, 4, st));
  kern<<<blocks, kWarps * 32, smem, st>>>(g, b.smap, b.sidx, b.offsets, chunk, nvis,
                                          static_cast<const typename Cplx<R>::T *>(cf),
                                          static_cast<const typename Cplx<R>::T *>(grid),
                                          static_cast<typename VisT<R>::C *>(vis_out), queue);
  ARL_LAUNCH_CHECK();
  count_launch(1);
  return ARLGPU_OK;
}

static int check_rows(int64_t nvis) {
  if (nvis < 0) return fail(ARLGPU_ERR_INVALID, "nvis < 0");
  if (nvis >= 0xffffffffll) return fail(ARLGPU_ERR_UNSUPPORTED, "nvis must be < 2^32 per call");
  return ARLGPU_OK;
}

}  // namespace arlgpu

using namespace arlgpu;

extern "C" const char *arlgpu_version(void) { return "arlgpu 0.1 (sm_103a)"; }
extern "C" const char *arlgpu_last_error(void) { return arlgpu::last_error(); }

extern "C" int arlgpu_convolution_mapping(const double *uvw, const double *frequency, int64_t nvis,
                                          const arlgpu_grid_desc *gd, const arlgpu_cf_desc *cd, int32_t *pu,
                                          int32_t *pu_off, int32_t *pv, int32_t *pv_off, int32_t *pwg,
                                          int32_t *pwc, int32_t *pfreq, int64_t *n_bad_host, void *stream) {
  Geom g;
  ARL_TRY(make_geom(gd, cd, ARLGPU_FP64, &g));
  ARL_TRY(check_rows(nvis));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned long long *d_bad = nullptr;
  ARL_CUDA(cudaMallocAsync(&d_bad, sizeof(unsigned long long), st));
  ARL_CUDA(cudaMemsetAsync(d_bad, 0, sizeof(unsigned long long), st));
  if (nvis > 0) {
    int blocks = (int)std::min<int64_t>((nvis + 255) / 256, (int64_t)num_sms() * 16);
    k_map_export<<<blocks, 256, 0, st>>>(uvw, frequency, nvis, g, pu, pu_off, pv, pv_off, pwg, pwc, pfreq, d_bad);
    ARL_LAUNCH_CHECK();
  }
  unsigned long long h = 0;
  ARL_CUDA(cudaMemcpyAsync(&h, d_bad, sizeof h, cudaMemcpyDeviceToHost, st));
  ARL_CUDA(cudaFreeAsync(d_bad, st));
  ARL_CUDA(cudaStreamSynchronize(st));
  if (n_bad_host) *n_bad_host = (int64_t)h;
  return ARLGPU_OK;
}

extern "C" int arlgpu_plan_workspace_bytes(int64_t nvis, const arlgpu_grid_desc *gd, const arlgpu_cf_desc *cd,
                                           size_t *bytes_host) {
  Geom g;
  ARL_TRY(make_geom(gd, cd, ARLGPU_FP32C, &g));
  ARL_TRY(check_rows(nvis));
  if (!bytes_host) return fail(ARLGPU_ERR_INVALID, "null bytes_host");
  *bytes_host = plan_bytes(nvis, g);
  return ARLGPU_OK;
}

extern "C" int arlgpu_plan_build(const double *uvw, const double *frequency, int64_t nvis,
                                 const arlgpu_grid_desc *gd, const arlgpu_cf_desc *cd, void *workspace,
                                 size_t workspace_bytes, int64_t *n_bad_dev, void *stream) {
  Geom g;
  ARL_TRY(make_geom(gd, cd, ARLGPU_FP32C, &g));
  ARL_TRY(check_rows(nvis));
  if (nvis > 0 && (!uvw || !frequency)) return fail(ARLGPU_ERR_INVALID, "null uvw / frequency");
  PlanBufs b;
  ARL_TRY(plan_carve(workspace, workspace_bytes, nvis, g, &b));
  return plan_build(uvw, frequency, nvis, g, b, n_bad_dev, static_cast<cudaStream_t>(stream));
}

extern "C" int arlgpu_grid_planned(const void *vis, const void *weight, int64_t nvis, int precision, const void *cf,
                                   const arlgpu_cf_desc *cd, void *grid, const arlgpu_grid_desc *gd, double *sumwt,
                                   const void *workspace, size_t workspace_bytes, void *stream) {
  Geom g;
  ARL_TRY(make_geom(gd, cd, precision, &g));
  ARL_TRY(check_rows(nvis));
  if (!grid || !sumwt || !cf || (nvis > 0 && (!vis || !weight))) return fail(ARLGPU_ERR_INVALID, "null array argument");
  PlanBufs b;
  ARL_TRY(plan_carve(const_cast<void *>(workspace), workspace_bytes, nvis, g, &b));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t csz = precision == ARLGPU_FP64 ? 16 : 8;
  ARL_CUDA(cudaMemsetAsync(grid, 0, (size_t)g.nchan * g.npol * g.nw * g.ny * g.nx * csz, st));
  ARL_CUDA(cudaMemsetAsync(sumwt, 0, (size_t)g.nchan * g.npol * sizeof(double), st));
  if (precision == ARLGPU_FP64) return launch_grid<double>(g, b, nvis, vis, weight, cf, grid, sumwt, st);
  return launch_grid<float>(g, b, nvis, vis, weight, cf, grid, sumwt, st);
}

extern "C" int arlgpu_degrid_planned(int64_t nvis, int precision, const void *cf, const arlgpu_cf_desc *cd,
                                     const void *grid, const arlgpu_grid_desc *gd, void *vis_out,
                                     const void *workspace, size_t workspace_bytes, void *stream) {
  Geom g;
  ARL_TRY(make_geom(gd, cd, precision, &g));
  ARL_TRY(check_rows(nvis));
  if (!grid || !cf || (nvis > 0 && !vis_out)) return fail(ARLGPU_ERR_INVALID, "null array argument");
  PlanBufs b;
  ARL_TRY(plan_carve(const_cast<void *>(workspace), workspace_bytes, nvis, g, &b));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (precision == ARLGPU_FP64) return launch_degrid<double>(g, b, nvis, cf, grid, vis_out, st);
  return launch_degrid<float>(g, b, nvis, cf, grid, vis_out, st);
}

extern "C" int arlgpu_grid(const double *uvw, const double *frequency, const void *vis, const void *weight,
                           int64_t nvis, int precision, const void *cf, const arlgpu_cf_desc *cd, void *grid,
                           const arlgpu_grid_desc *gd, double *sumwt, int64_t *n_bad_dev, void *workspace,
                           size_t workspace_bytes, void *stream) {
  ARL_TRY(arlgpu_plan_build(uvw, frequency, nvis, gd, cd, workspace, workspace_bytes, n_bad_dev, stream));
  return arlgpu_grid_planned(vis, weight, nvis, precision, cf, cd, grid, gd, sumwt, workspace, workspace_bytes,
                             stream);
}

extern "C" int arlgpu_degrid(const double *uvw, const double *frequency, int64_t nvis, int precision,
                             const void *cf, const arlgpu_cf_desc *cd, const void *grid,
                             const arlgpu_grid_desc *gd, void *vis_out, int64_t *n_bad_dev, void *workspace,
                             size_t workspace_bytes, void *stream) {
  ARL_TRY(arlgpu_plan_build(uvw, frequency, nvis, gd, cd, workspace, workspace_bytes, n_bad_dev, stream));
  return arlgpu_degrid_planned(nvis, precision, cf, cd, grid, gd, vis_out, workspace, workspace_bytes, stream);
}

extern "C" int arlgpu_plan_plane_mean_w(const double *uvw, int64_t nvis, const arlgpu_grid_desc *gd,
                                        const arlgpu_cf_desc *cd, void *workspace, size_t workspace_bytes,
                                        double *wmean, void *stream) {
  Geom g;
  ARL_TRY(make_geom(gd, cd, ARLGPU_FP32C, &g));
  ARL_TRY(check_rows(nvis));
  if (!wmean || (nvis > 0 && !uvw)) return fail(ARLGPU_ERR_INVALID, "null array argument");
  PlanBufs b;
  ARL_TRY(plan_carve(workspace, workspace_bytes, nvis, g, &b));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const uint32_t P = wpart_shares(g);
  k_plane_wsum<<<plan_wpart_items(g), 256, 0, st>>>(uvw, b.sidx, b.offsets, g, P, b.wpart);
  ARL_LAUNCH_CHECK();
  k_plane_wmean<<<(g.nw + 127) / 128, 128, 0, st>>>(b.wpart, b.offsets, g, P, wmean);
  ARL_LAUNCH_CHECK();
  count_launch(2);
  return ARLGPU_OK;
}

extern "C" int arlgpu_plan_flags(int64_t nvis, const arlgpu_grid_desc *gd, const arlgpu_cf_desc *cd,
                                 const void *workspace, size_t workspace_bytes, uint32_t *flags_host, void *stream) {
  Geom g;
  ARL_TRY(make_geom(gd, cd, ARLGPU_FP32C, &g));
  ARL_TRY(check_rows(nvis));
  if (!flags_host) return fail(ARLGPU_ERR_INVALID, "null flags_host");
  PlanBufs b;
  ARL_TRY(plan_carve(const_cast<void *>(workspace), workspace_bytes, nvis, g, &b));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  ARL_CUDA(cudaMemcpyAsync(flags_host, b.queue + 2, 4, cudaMemcpyDeviceToHost, st));
  ARL_CUDA(cudaStreamSynchronize(st));
  return ARLGPU_OK;
}

extern "C" int arlgpu_set_tuning(const char *key, int value) {
  if (!key) return fail(ARLGPU_ERR_INVALID, "null key");
  const std::string k(key);
  if (k == "grid_kernel" && value >= 0 && value <= 5) g_tune_grid_kernel = value;
  else if (k == "degrid_kernel" && value >= 0 && value <= 4) g_tune_degrid_kernel = value;
  else if (k == "subgrid" && (value == 0 || (value >= 16 && value <= 128))) g_tune_subgrid = value;
  else if (k == "chunk" && value >= 32 && value <= (1 << 20)) g_tune_chunk = value;
  else if (k == "persistent" && value >= 0 && value <= 2) g_tune_persistent = value;
  else if (k == "dsfft" && (value == 0 || value == 1)) g_tune_dsfft = value;
  else if (k == "small_rows" && (value == 1 || value == 2 || value == 4)) g_tune_small_rows = value;
  else if (k == "small_rows_degrid" && (value == 1 || value == 2 || value == 4)) g_tune_small_rows_dg = value;
  else if (k == "lanes_per_row" && (value == 0 || value == 8 || value == 16 || value == 32)) g_tune_lanes = value;
  else if (k == "gather_rows" && (value == 0 || value == 1)) g_tune_gather = value;
  else if (k == "stash_rows" && (value == 0 || value == 1)) g_tune_stash = value;
  else return fail(ARLGPU_ERR_INVALID, "unknown tuning key or value: %s = %d", key, value);
  return ARLGPU_OK;
}

extern "C" int arlgpu_get_tuning(const char *key, int *value) {
  if (!key || !value) return fail(ARLGPU_ERR_INVALID, "null argument");
  const std::string k(key);
  if (k == "grid_kernel") *value = g_tune_grid_kernel;
  else if (k == "degrid_kernel") *value = g_tune_degrid_kernel;
  else if (k == "subgrid") *value = g_tune_subgrid;
  else if (k == "chunk") *value = g_tune_chunk;
  else if (k == "persistent") *value = g_tune_persistent;
  else if (k == "dsfft") *value = g_tune_dsfft;
  else if (k == "small_rows") *value = g_tune_small_rows;
  else if (k == "small_rows_degrid") *value = g_tune_small_rows_dg;
  else if (k == "lanes_per_row") *value = g_tune_lanes;
  else if (k == "gather_rows") *value = g_tune_gather;
  else if (k == "stash_rows") *value = g_tune_stash;
  else return fail(ARLGPU_ERR_INVALID, "unknown tuning key: %s", key);
  return ARLGPU_OK;
}

extern "C" unsigned long long arlgpu_kernel_launches(void) { return g_launches.load(); }
