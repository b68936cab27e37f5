// Double-single inverse 2-D FFT for the FP32C path (K5 / K9 transforms).
//
// Reference behaviour:
//   ifft (centred inverse transform)  processing_library/fourier_transforms/fft_support.py:41-89
//   fft_griddata_to_image             processing_components/griddata/gridding.py:270-289
//   w-stack slice sum                 processing_components/imaging/wstack_single.py:26-60 with
//                                     workflows/serial/imaging/imaging_serial.py:186-197
//
// The grid correction multiplies transform rounding by up to max(gcf)/min(gcf)
// (~6e4 at the edge of a PSWF-corrected field), so the inverse transform must
// be much more accurate than FP32.  GB300 runs FP64 at 1/64 of its FP32 rate,
// which makes cuFFT's FP64 transform of an 8192^2 plane compute-bound at
// ~14 ms.  Here every complex value is a pair of double-single numbers
// (float4: re.hi, re.lo, im.hi, im.lo; ~48-bit significands) and all
// arithmetic runs on the FP32 pipes.
//
// Layout: a plane of ny x nx points, row-major.  Three passes per plane:
//   rows   one CTA per 4096 points (4096 / nx rows, or half of an
//          8192-point row): FP32 grid (w-planes summed, chk sign) -> row
//          DFTs in shared memory -> DS buffer
//   cols1  ny = N1 * N2: DFTs of length N1 over rows n2 + N2 n1 of 32 or 64
//          adjacent columns, times exp(2 pi i n2 k1 / ny), in place
//   cols2  DFTs of length N2 over rows N2 k1 + n2 -> row k1 + N1 k2, with the
//          epilogue fused: image write (invert_2d) or the w-screen product
//          summed over the slices of the group (w-stacking)
// Each DFT is a Stockham radix-4 (one radix-2 pass for odd log2) sequence in
// shared memory: the first pass reads global memory, the last writes the
// epilogue, both coalesced.  Twiddles come from one DS table of
// exp(2 pi i m / 16384) computed once per device in FP64.
#include <atomic>

#include "common.cuh"
#include "dsmath.cuh"

namespace arlgpu {

void count_launch(unsigned n);

constexpr int kLog2Tw = 14;
constexpr int kTw = 1 << kLog2Tw;
__device__ float4 g_tw[kTw];  // exp(+2 pi i m / 16384): (cos hi, cos lo, sin hi, sin lo)

__global__ void k_tw_init() {
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < kTw; m += gridDim.x * blockDim.x) {
    double s, c;
    sincospi((double)m / (double)(kTw / 2), &s, &c);
    const dsf cc = ds_from_double(c), ss = ds_from_double(s);
    g_tw[m] = make_float4(cc.hi, cc.lo, ss.hi, ss.lo);
  }
}

static std::atomic<unsigned> g_tw_ready{0};

// The table is filled once per device on a stream that is not capturing
// (synchronised so that every later stream sees it); under capture the fill
// is recorded into the graph instead, every time, so a graph never relies on
// a fill that did not run.
static int ensure_twiddles(cudaStream_t st) {
  int dev = 0;
  ARL_CUDA(cudaGetDevice(&dev));
  const unsigned bit = 1u << (dev & 31);
  if (g_tw_ready.load() & bit) return ARLGPU_OK;
  k_tw_init<<<16, 256, 0, st>>>();
  ARL_LAUNCH_CHECK();
  count_launch(1);
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  ARL_CUDA(cudaStreamIsCapturing(st, &cs));
  if (cs == cudaStreamCaptureStatusNone) {
    ARL_CUDA(cudaStreamSynchronize(st));
    g_tw_ready.fetch_or(bit);
  }
  return ARLGPU_OK;
}

// ---------------------------------------------------------------------------
// Complex double-single arithmetic on float4 (re.hi, re.lo, im.hi, im.lo).
// ---------------------------------------------------------------------------
__device__ __forceinline__ float4 c_add_nr(float4 a, float4 b) {  // unnormalised sum
  const dsf r = two_sum(a.x, b.x), i = two_sum(a.z, b.z);
  return make_float4(r.hi, __fadd_rn(r.lo, __fadd_rn(a.y, b.y)), i.hi, __fadd_rn(i.lo, __fadd_rn(a.w, b.w)));
}
__device__ __forceinline__ float4 c_neg(float4 a) { return make_float4(-a.x, -a.y, -a.z, -a.w); }
__device__ __forceinline__ float4 c_norm(float4 a) {
  const dsf r = quick_two_sum(a.x, a.y), i = quick_two_sum(a.z, a.w);
  return make_float4(r.hi, r.lo, i.hi, i.lo);
}
// i * a
__device__ __forceinline__ float4 c_muli(float4 a) { return make_float4(-a.z, -a.w, a.x, a.y); }

// a * w (w a unit twiddle).
__device__ __forceinline__ float4 c_mul(float4 a, float4 w) {
  const dsf p1 = two_prod(a.x, w.x), p2 = two_prod(a.z, w.z);
  const dsf s1 = two_sum(p1.hi, -p2.hi);
  float e1 = __fadd_rn(s1.lo, __fsub_rn(p1.lo, p2.lo));
  e1 = __fmaf_rn(a.x, w.y, e1);
  e1 = __fmaf_rn(a.y, w.x, e1);
  e1 = __fmaf_rn(-a.z, w.w, e1);
  e1 = __fmaf_rn(-a.w, w.z, e1);
  const dsf p3 = two_prod(a.x, w.z), p4 = two_prod(a.z, w.x);
  const dsf s2 = two_sum(p3.hi, p4.hi);
  float e2 = __fadd_rn(s2.lo, __fadd_rn(p3.lo, p4.lo));
  e2 = __fmaf_rn(a.x, w.w, e2);
  e2 = __fmaf_rn(a.y, w.z, e2);
  e2 = __fmaf_rn(a.z, w.y, e2);
  e2 = __fmaf_rn(a.w, w.x, e2);
  const dsf r = quick_two_sum(s1.hi, e1), i = quick_two_sum(s2.hi, e2);
  return make_float4(r.hi, r.lo, i.hi, i.lo);
}

// exp(+2 pi i m / 2^log2n) for 0 <= m < 2^log2n <= 16384
__device__ __forceinline__ float4 twiddle(int m, int log2n) { return __ldg(&g_tw[m << (kLog2Tw - log2n)]); }

// 16-byte global -> shared copies that bypass the registers, all in flight
// before one wait (the column passes stage their 64 KiB tiles this way).
__device__ __forceinline__ void cp_async16(float4 *smem, const float4 *gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// ---------------------------------------------------------------------------
// In-place radix-2^2 decimation-in-frequency transform (inverse sign) of
// S = 2^log2S sequences of L = 2^log2L points held in shared memory at
// pos(n, q): natural order in, bit-reversed order out.  Each butterfly reads
// and writes the same four slots, so a thread holds one butterfly at a time
// and a pass needs one barrier.  Two radix-2 stages of spans h and h/2 fuse
// into one butterfly on the points n0 + {0, h/2, h, 3h/2} of a block of 2h:
//   a = x0 + x2, b = x0 - x2, c = x1 + x3, d = i (x1 - x3), w = exp(2 pi i j / 2h)
//   y0 = a + c, y1 = (a - c) w^2, y2 = (b + d) w, y3 = (b - d) w^3
// and an odd log2 L ends with one radix-2 stage of span 1.  Sums are left
// unnormalised (hi + lo still equals the value; the next error-free sum or
// twiddle product absorbs it), which NumPy float32 emulation shows costs
// nothing measurable (7.9e-15 against 7.4e-15 of the scale at 8192 points).
// tw(m, lw) = exp(2 pi i m / 2^lw).
// ---------------------------------------------------------------------------
template <int T, typename Pos, typename Tw>
__device__ __forceinline__ void ds_dif_cta(float4 *sm, int log2L, int log2S, bool seqfast, Pos pos, Tw tw) {
  const int S1 = (1 << log2S) - 1;
  const int nb4 = 1 << (log2L - 2 + log2S);
  int log2h = log2L - 1;
  for (; log2h >= 1; log2h -= 2) {
    const int lq = log2h - 1, J1 = (1 << lq) - 1;
    const int lblk = log2L - log2h - 1;  // log2 of the blocks per sequence
    for (int bb = threadIdx.x; bb < nb4; bb += T) {
      int q, jp, blk;
      if (seqfast) {
        q = bb & S1;
        const int rest = bb >> log2S;
        jp = rest & J1;
        blk = rest >> lq;
      } else {
        jp = bb & J1;
        const int rest = bb >> lq;
        blk = rest & ((1 << lblk) - 1);
        q = rest >> lblk;
      }
      const int n0 = (blk << (log2h + 1)) + jp, hh = 1 << lq;
      const int i0 = pos(n0, q), i1 = pos(n0 + hh, q), i2 = pos(n0 + 2 * hh, q), i3 = pos(n0 + 3 * hh, q);
      const float4 x0 = sm[i0], x1 = sm[i1], x2 = sm[i2], x3 = sm[i3];
      const float4 a = c_add_nr(x0, x2), b = c_add_nr(x0, c_neg(x2));
      const float4 c = c_add_nr(x1, x3), d = c_muli(c_add_nr(x1, c_neg(x3)));
      float4 y1 = c_add_nr(a, c_neg(c)), y2 = c_add_nr(b, d), y3 = c_add_nr(b, c_neg(d));
      if (jp) {
        const int lw = log2h + 1;
        y2 = c_mul(y2, tw(jp, lw));
        y1 = c_mul(y1, tw(2 * jp, lw));
        y3 = c_mul(y3, tw(3 * jp, lw));
      }
      sm[i0] = c_add_nr(a, c);
      sm[i1] = y1;
      sm[i2] = y2;
      sm[i3] = y3;
    }
    __syncthreads();
  }
  if (log2h == 0) {
    const int nb2 = 1 << (log2L - 1 + log2S), lb = log2L - 1, B1 = (1 << lb) - 1;
    for (int bb = threadIdx.x; bb < nb2; bb += T) {
      const int q = seqfast ? (bb & S1) : (bb >> lb), i = seqfast ? (bb >> log2S) : (bb & B1);
      const int i0 = pos(2 * i, q), i1 = pos(2 * i + 1, q);
      const float4 x0 = sm[i0], x1 = sm[i1];
      sm[i0] = c_add_nr(x0, x1);
      sm[i1] = c_add_nr(x0, c_neg(x1));
    }
    __syncthreads();
  }
}

// Global table lookup, for the row transforms.
struct TwGlobal {
  __device__ __forceinline__ float4 operator()(int m, int lw) const { return twiddle(m, lw); }
};
// exp(2 pi i m / L) for m < L <= 128 staged in shared memory by the column
// kernels (the only twiddles their transforms use).
struct TwShared {
  const float4 *t;
  int log2L;
  __device__ __forceinline__ float4 operator()(int m, int lw) const { return t[m << (log2L - lw)]; }
};
__device__ __forceinline__ void stage_twiddles(float4 *t, int log2L) {
  for (int m = threadIdx.x; m < (1 << log2L); m += blockDim.x) t[m] = twiddle(m, log2L);
}

__device__ __forceinline__ int brev(int k, int log2L) { return (int)(__brev((unsigned)k) >> (32 - log2L)); }

// ---------------------------------------------------------------------------
// Pass 1: row transforms.  Logical plane q of the input is the sum over
// z < nsum of grid[q * qstride + z * plane]; rows of planes [q0, q0 + np) go to
// buf[(q - q0) * plane + y * nx + x] with the chk sign applied on input.  One
// CTA holds PTS points (PTS / nx rows).  For rows of 512 points or more the
// slot of point n within its row has its low three bits XORed with a function
// of bits 3-5 and of the top three bits of n: the small-span butterflies
// (strides 2, 4 and 16 slots) and the bit-reversed reads of the epilogue then
// touch eight different 16-byte bank groups per quarter warp.
// ---------------------------------------------------------------------------
constexpr int kColT = 512, kColPts = 4096, kColNPT = kColPts / kColT, kColSmem = (kColPts + 256) * 16,
              kColSmem2 = (2 * kColPts + 128) * 16 + kColPts * 8;

template <int PTS, int T>
__global__ void __launch_bounds__(T, 1024 / T)
k_dsfft_rows(const float2 *__restrict__ grid, int64_t qstride, int nsum, int64_t q0, int np, int log2ny, int log2nx,
             float4 *__restrict__ buf) {
  extern __shared__ float4 sm[];
  constexpr int LOG2PTS = PTS == 8192 ? 13 : 12;
  const int ny = 1 << log2ny;
  const int64_t plane = (int64_t)ny << log2nx;
  const int log2S = LOG2PTS - log2nx;  // rows per CTA
  const int64_t row0 = (int64_t)blockIdx.x << log2S;
  const int64_t nrows = (int64_t)np << log2ny;
  const bool swz = log2nx >= 9;
  auto pos = [&](int n, int q) {
    int m = n;
    if (swz) {
      const int j = (n >> 3) & 7;
      m = n ^ ((j & 3) | ((j & 2) << 1)) ^ ((n >> (log2nx - 3)) & 7);
    }
    return (q << log2nx) + m;
  };
  if (nsum == 1) {
    // all loads of the thread in flight before the first shared store
    constexpr int K = PTS / T;
    float2 gv[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int t = threadIdx.x + k * T;
      const int q = t >> log2nx, x = t & ((1 << log2nx) - 1);
      const int64_t R = row0 + q;
      gv[k] = make_float2(0.f, 0.f);
      if (R < nrows)
        gv[k] = grid[(q0 + (R >> log2ny)) * qstride + ((int64_t)(R & (ny - 1)) << log2nx) + x];
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int t = threadIdx.x + k * T;
      const int q = t >> log2nx, x = t & ((1 << log2nx) - 1);
      const int y = (int)((row0 + q) & (ny - 1));
      const float sg = ((x + y) & 1) ? -1.f : 1.f;
      sm[pos(x, q)] = make_float4(sg * gv[k].x, 0.f, sg * gv[k].y, 0.f);
    }
  } else {
  for (int t = threadIdx.x; t < PTS; t += T) {
    const int q = t >> log2nx, x = t & ((1 << log2nx) - 1);
    const int64_t R = row0 + q;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (R < nrows) {
      const int64_t pl = R >> log2ny;
      const int y = (int)(R & (ny - 1));
      const float2 *src = grid + (q0 + pl) * qstride + ((int64_t)y << log2nx) + x;
      float2 g = src[0];
      dsf re = {g.x, 0.f}, im = {g.y, 0.f};
      for (int z = 1; z < nsum; ++z) {
        g = src[z * plane];
        re = ds_add(re, {g.x, 0.f});
        im = ds_add(im, {g.y, 0.f});
      }
      const float sg = ((x + y) & 1) ? -1.f : 1.f;
      v = make_float4(sg * re.hi, sg * re.lo, sg * im.hi, sg * im.lo);
    }
    sm[pos(x, q)] = v;
  }
  }
  // An all-zero tile (whole empty grid rows, common in w-stack slices)
  // transforms to zero: write zeros and skip the arithmetic.
  bool nz = false;
  for (int t = threadIdx.x; t < PTS && !nz; t += T) {
    const float4 v = sm[pos(t & ((1 << log2nx) - 1), t >> log2nx)];
    nz = v.x != 0.f || v.z != 0.f;
  }
  if (!__syncthreads_or(nz)) {
    for (int t = threadIdx.x; t < PTS; t += T) {
      const int64_t R = row0 + (t >> log2nx);
      if (R < nrows) buf[(R << log2nx) + (t & ((1 << log2nx) - 1))] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    return;
  }
  ds_dif_cta<T>(sm, log2nx, log2S, false, pos, TwGlobal());
  for (int t = threadIdx.x; t < PTS; t += T) {
    const int q = t >> log2nx, x = t & ((1 << log2nx) - 1);
    const int64_t R = row0 + q;
    if (R < nrows) buf[(R << log2nx) + x] = sm[pos(brev(x, log2nx), q)];
  }
}

// 8192-point rows as two 4096-point halves on two CTAs (64 KiB of shared
// memory each, so that two CTAs share an SM): the first decimation-in-
// frequency stage, span 4096, is done while loading, CTA h = 0 taking
// x[n] + x[n + 4096] (whose DFT is X[2k]) and h = 1 taking
// (x[n] - x[n + 4096]) exp(2 pi i n / 8192) (DFT X[2k + 1]); each writes its
// 4096 outputs to the even or odd positions of the row.
__global__ void __launch_bounds__(512, 2)
k_dsfft_rows_split(const float2 *__restrict__ grid, int64_t qstride, int nsum, int64_t q0, int np, int log2ny,
                   float4 *__restrict__ buf) {
  extern __shared__ float4 sm[];
  constexpr int LX = 13, LH = 12, H = 1 << LH;
  const int ny = 1 << log2ny;
  const int64_t plane = (int64_t)ny << LX;
  const int64_t R = blockIdx.x >> 1;
  const int half = blockIdx.x & 1;
  auto pos = [&](int n, int) {
    const int j = (n >> 3) & 7;
    return n ^ ((j & 3) | ((j & 2) << 1)) ^ ((n >> (LH - 3)) & 7);
  };
  const int64_t pl = R >> log2ny;
  const int y = (int)(R & (ny - 1));
  const float2 *src = grid + (q0 + pl) * qstride + ((int64_t)y << LX);
  auto in = [&](int x) -> float4 {
    float2 g = src[x];
    dsf re = {g.x, 0.f}, im = {g.y, 0.f};
    for (int z = 1; z < nsum; ++z) {
      g = src[z * plane + x];
      re = ds_add(re, {g.x, 0.f});
      im = ds_add(im, {g.y, 0.f});
    }
    const float sg = ((x + y) & 1) ? -1.f : 1.f;
    return make_float4(sg * re.hi, sg * re.lo, sg * im.hi, sg * im.lo);
  };
  if (nsum == 1) {
    constexpr int K = H / 512;
    float2 ga[K], gb[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      ga[k] = src[threadIdx.x + k * 512];
      gb[k] = src[threadIdx.x + k * 512 + H];
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int n = threadIdx.x + k * 512;
      const float sg = ((n + y) & 1) ? -1.f : 1.f;  // n and n + 4096 have the same parity
      const float4 a = make_float4(sg * ga[k].x, 0.f, sg * ga[k].y, 0.f);
      const float4 b = make_float4(sg * gb[k].x, 0.f, sg * gb[k].y, 0.f);
      float4 v;
      if (half == 0) {
        v = c_add_nr(a, b);
      } else {
        v = c_add_nr(a, c_neg(b));
        if (n) v = c_mul(v, twiddle(n, LX));
      }
      sm[pos(n, 0)] = v;
    }
  } else {
  for (int n = threadIdx.x; n < H; n += 512) {
    const float4 a = in(n), b = in(n + H);
    float4 v;
    if (half == 0) {
      v = c_add_nr(a, b);
    } else {
      v = c_add_nr(a, c_neg(b));
      if (n) v = c_mul(v, twiddle(n, LX));
    }
    sm[pos(n, 0)] = v;
  }
  }
  // An all-zero half (a whole empty grid row) transforms to zero.
  bool nz = false;
  for (int n = threadIdx.x; n < H && !nz; n += 512) {
    const float4 v = sm[pos(n, 0)];
    nz = v.x != 0.f || v.z != 0.f;
  }
  float4 *out = buf + (R << LX) + half;
  if (!__syncthreads_or(nz)) {
    for (int k = threadIdx.x; k < H; k += 512) out[2 * k] = make_float4(0.f, 0.f, 0.f, 0.f);
    return;
  }
  ds_dif_cta<512>(sm, LH, 0, false, pos, TwGlobal());
  for (int k = threadIdx.x; k < H; k += 512) out[2 * k] = sm[pos(brev(k, LH), 0)];
}

// ---------------------------------------------------------------------------
// Column decomposition ny = N1 N2 (N1 <= N2 <= 128) and the CTA tiles.
// ---------------------------------------------------------------------------
struct ColGeom {
  int log2N1, log2N2;
  int log2G1, log2WC1;  // cols1: n2 values x columns per CTA
  int log2G2, log2WC2;  // cols2: k1 values x columns per CTA
};

static bool col_geom(int log2ny, int log2nx, ColGeom *c) {
  c->log2N1 = log2ny / 2;
  c->log2N2 = log2ny - c->log2N1;
  if (c->log2N2 > 7 || c->log2N1 < 2) return false;
  const int lp = 12;  // log2 of the points per column CTA
  c->log2G1 = std::min(7 - c->log2N1, c->log2N2);
  c->log2WC1 = lp - c->log2N1 - c->log2G1;
  c->log2G2 = std::min(7 - c->log2N2, c->log2N1);
  c->log2WC2 = lp - c->log2N2 - c->log2G2;
  return c->log2WC1 <= log2nx && c->log2WC2 <= log2nx && c->log2WC1 >= 5 && c->log2WC2 >= 5;
}

// Pass 2: length-N1 DFTs over rows n2 + N2 n1, twiddled, in place.
__global__ void __launch_bounds__(kColT)
k_dsfft_cols1(float4 *__restrict__ buf, int log2ny, int log2nx, ColGeom cg, int64_t ntile_pl) {
  extern __shared__ float4 sm[];
  const int64_t pl = blockIdx.x / ntile_pl;
  const int64_t t0 = blockIdx.x - pl * ntile_pl;
  const int ntx = 1 << (log2nx - cg.log2WC1);
  const int n2_0 = (int)(t0 / ntx) << cg.log2G1, x0 = (int)(t0 % ntx) << cg.log2WC1;
  float4 *p = buf + (pl << (log2ny + log2nx));
  const int WC1 = (1 << cg.log2WC1) - 1, log2S = cg.log2G1 + cg.log2WC1;
  auto addr = [&](int n1, int q) {
    const int n2 = n2_0 + (q >> cg.log2WC1);
    return ((int64_t)(n2 + (n1 << cg.log2N2)) << log2nx) + x0 + (q & WC1);
  };
  auto pos = [&](int n, int q) { return (n << log2S) + q; };
  float4 *stw = sm + kColPts;
  stage_twiddles(stw, cg.log2N1);
  // the 4-step twiddles exp(2 pi i n2 k1 / ny) of this CTA's G1 x N1 outputs
  float4 *stw2 = stw + 128;
  for (int e = threadIdx.x; e < (1 << (cg.log2G1 + cg.log2N1)); e += kColT)
    stw2[e] = twiddle((n2_0 + (e >> cg.log2N1)) * (e & ((1 << cg.log2N1) - 1)), log2ny);
  for (int t = threadIdx.x; t < kColPts; t += kColT) cp_async16(sm + t, p + addr(t >> log2S, t & ((1 << log2S) - 1)));
  cp_async_wait_all();
  __syncthreads();
  ds_dif_cta<kColT>(sm, cg.log2N1, log2S, true, pos, TwShared{stw, cg.log2N1});
  for (int t = threadIdx.x; t < kColPts; t += kColT) {
    const int k1 = t >> log2S, q = t & ((1 << log2S) - 1);
    const int g = q >> cg.log2WC1;
    const float4 v = sm[pos(brev(k1, cg.log2N1), q)];
    p[addr(k1, q)] = (n2_0 + g && k1) ? c_mul(v, stw2[(g << cg.log2N1) + k1]) : v;
  }
}

// Pass 3 for invert_2d: length-N2 DFTs over rows N2 k1 + n2 -> row k1 + N1 k2;
// image = part(v * chk * s0) * gcf [/ sumwt].  Plane pl is image b = b0 + pl.
__global__ void __launch_bounds__(kColT)
k_dsfft_cols2_image(const float4 *__restrict__ buf, int log2ny, int log2nx, ColGeom cg, int64_t ntile_pl, int64_t b0,
                    float s0, const double *__restrict__ gcf, const double *__restrict__ sumwt,
                    double *__restrict__ im_re, double *__restrict__ im_im) {
  extern __shared__ float4 sm[];
  const int64_t pl = blockIdx.x / ntile_pl;
  const int64_t t0 = blockIdx.x - pl * ntile_pl;
  const int ntx = 1 << (log2nx - cg.log2WC2);
  const int k1_0 = (int)(t0 / ntx) << cg.log2G2, x0 = (int)(t0 % ntx) << cg.log2WC2;
  const float4 *p = buf + (pl << (log2ny + log2nx));
  const int WC2 = (1 << cg.log2WC2) - 1, log2S = cg.log2G2 + cg.log2WC2, S1 = (1 << log2S) - 1;
  const int64_t b = b0 + pl;
  const int64_t obase = b << (log2ny + log2nx);
  auto pos = [&](int n, int q) { return (n << log2S) + q; };
  for (int t = threadIdx.x; t < kColPts; t += kColT) {
    const int n2 = t >> log2S, q = t & S1;
    const int k1 = k1_0 + (q >> cg.log2WC2);
    cp_async16(sm + t, p + ((int64_t)((k1 << cg.log2N2) + n2) << log2nx) + x0 + (q & WC2));
  }
  cp_async_wait_all();
  float4 *stw = sm + kColPts;
  stage_twiddles(stw, cg.log2N2);
  __syncthreads();
  ds_dif_cta<kColT>(sm, cg.log2N2, log2S, true, pos, TwShared{stw, cg.log2N2});
  double inv = 1.0;
  bool zero = false;
  if (sumwt) {
    const double w = sumwt[b];
    zero = !(w > 0.0);
    inv = zero ? 0.0 : 1.0 / w;
  }
  for (int t = threadIdx.x; t < kColPts; t += kColT) {
    const int k2 = t >> log2S, q = t & S1;
    const float4 v = sm[pos(brev(k2, cg.log2N2), q)];
    const int k = k1_0 + (q >> cg.log2WC2) + (k2 << cg.log2N1), x = x0 + (q & WC2);
    const int64_t o = obase + ((int64_t)k << log2nx) + x;
    const double f = (double)((((x + k) & 1) ? -1.f : 1.f) * s0) * gcf[o];
    double re = ds_to_double({v.x, v.y}) * f, im = ds_to_double({v.z, v.w}) * f;
    if (sumwt) {
      re = zero ? 0.0 : re * inv;
      im = zero ? 0.0 : im * inv;
    }
    im_re[o] = re;
    if (im_im) im_im[o] = im;
  }
}

// Pass 3 for w-stacking: planes [p0, p1) of the flattened (image b, slice s)
// order, buf holding them from p0.  Each CTA sums Re(wb_s v) over the slices
// of its tile into double-single accumulators and adds them to the image's DS
// slots (image memory viewed as float2; the group holding slice 0 of image b
// writes them).
__global__ void __launch_bounds__(kColT)
k_dsfft_cols2_wstack(const float4 *__restrict__ buf, int log2ny, int log2nx, ColGeom cg, int64_t p0, int64_t p1,
                     int K, double fov, const double *__restrict__ wmean, float2 *__restrict__ slots) {
  extern __shared__ float4 sm[];
  const int ntx = 1 << (log2nx - cg.log2WC2);
  const int k1_0 = (int)(blockIdx.x / ntx) << cg.log2G2, x0 = (int)(blockIdx.x % ntx) << cg.log2WC2;
  const int WC2 = (1 << cg.log2WC2) - 1, log2S = cg.log2G2 + cg.log2WC2, S1 = (1 << log2S) - 1;
  const int n = 1 << log2nx;
  const dsf c2 = ds_from_double(fov * fov / ((double)n * n));
  auto pos = [&](int k, int q) { return (k << log2S) + q; };
  // Two tiles: the next slice's tile is copied in while this one is
  // transformed.
  float4 *stw = sm + 2 * kColPts;
  stage_twiddles(stw, cg.log2N2);  // ordered before first use by the barrier after the first load
  float2 *snt = reinterpret_cast<float2 *>(stw + 128);  // kColPts per-pixel w-screen terms
  auto issue = [&](int64_t pp, float4 *dst) {
    const float4 *p = buf + ((pp - p0) << (log2ny + log2nx));
    for (int t = threadIdx.x; t < kColPts; t += kColT) {
      const int n2 = t >> log2S, q = t & S1;
      const int k1 = k1_0 + (q >> cg.log2WC2);
      cp_async16(dst + t, p + ((int64_t)((k1 << cg.log2N2) + n2) << log2nx) + x0 + (q & WC2));
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  };
  dsf acc[kColNPT];
#pragma unroll
  for (int m = 0; m < kColNPT; ++m) acc[m] = {0.f, 0.f};
  issue(p0, sm);
  for (int64_t pp = p0; pp < p1; ++pp) {
    const int64_t b = pp / K;
    const int s = (int)(pp - b * K);
    float4 *cur = ((pp - p0) & 1) ? sm + kColPts : sm;
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    __syncthreads();  // this tile has landed, and every thread is done with the other one
    if (pp + 1 < p1) issue(pp + 1, ((pp - p0) & 1) ? sm : sm + kColPts);
    ds_dif_cta<kColT>(cur, cg.log2N2, log2S, true, pos, TwShared{stw, cg.log2N2});
    const dsf w = ds_from_double(wmean[s]);
#pragma unroll
    for (int m = 0; m < kColNPT; ++m) {
      const int t = threadIdx.x + m * kColT;
      const int k2 = t >> log2S, q = t & S1;
      const float4 v = cur[pos(brev(k2, cg.log2N2), q)];
      // w-screen term of this thread's pixel t, formed at the first slice and
      // kept in the thread's own shared slot: nterm, or hi = -1 where r^2 >= 1
      if (pp == p0) {
        const int k = k1_0 + (q >> cg.log2WC2) + (k2 << cg.log2N1), x = x0 + (q & WC2);
        const DsPix px = ds_wpix(k, x, n, c2);
        snt[t] = px.state == 2 ? make_float2(-1.f, 0.f) : make_float2(px.nterm.hi, px.nterm.lo);
      }
      const float2 nt = snt[t];
      DsPix px;
      px.state = nt.x < 0.f ? 2 : 1;
      px.nterm = {nt.x, nt.y};
      const float2 wb = ds_wbeam(px, w);
      // Re(wb v) = wb.re v.re - wb.im v.im
      acc[m] = ds_add(acc[m], ds_sub(ds_mul_f({v.x, v.y}, wb.x), ds_mul_f({v.z, v.w}, wb.y)));
    }
    if (pp + 1 == p1 || (pp + 1) / K != b) {
      const bool first = p0 <= b * K;
      float2 *out = slots + (b << (log2ny + log2nx));
#pragma unroll
      for (int m = 0; m < kColNPT; ++m) {
        const int t = threadIdx.x + m * kColT;
        const int k2 = t >> log2S, q = t & S1;
        const int k = k1_0 + (q >> cg.log2WC2) + (k2 << cg.log2N1), x = x0 + (q & WC2);
        float2 *o = out + ((int64_t)k << log2nx) + x;
        dsf v = acc[m];
        if (!first) {
          const float2 old = *o;
          v = ds_add(v, {old.x, old.y});
        }
        *o = make_float2(v.hi, v.lo);
        acc[m] = {0.f, 0.f};
      }
    }
  }
}

// image[b, y, x] = DS slot * chk * s0 * gcf / sumwt[b] (0 where sumwt <= 0), in
// place over the slots.
__global__ void k_ds_wstack_finish(double *image, int64_t nb, int log2ny, int log2nx, float s0,
                                   const double *__restrict__ gcf, const double *__restrict__ sumwt) {
  const int64_t plane = (int64_t)1 << (log2ny + log2nx), tot = nb * plane;
  const int nx1 = (1 << log2nx) - 1;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i >> (log2ny + log2nx);
    const int y = (int)((i >> log2nx) & ((1 << log2ny) - 1)), x = (int)(i & nx1);
    const float2 sl = reinterpret_cast<const float2 *>(image)[i];
    const double w = sumwt[b];
    const double sg = (double)((((x + y) & 1) ? -1.f : 1.f) * s0);
    image[i] = w > 0.0 ? ds_to_double({sl.x, sl.y}) * sg * gcf[i] / w : 0.0;
  }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
static int ilog2_exact(int n) {
  if (n <= 0 || (n & (n - 1))) return -1;
  int l = 0;
  while ((1 << l) < n) ++l;
  return l;
}

bool dsfft_supported(int ny, int nx) {
  const int ly = ilog2_exact(ny), lx = ilog2_exact(nx);
  if (ly < 6 || lx < 6 || lx > 13 || ly > 14) return false;
  ColGeom cg;
  return col_geom(ly, lx, &cg);
}

// Function attributes belong to each device's context: set once per device.
static int set_smem() {
  static std::atomic<unsigned> done{0};
  int dev = 0;
  ARL_CUDA(cudaGetDevice(&dev));
  const unsigned bit = 1u << (dev & 31);
  if (done.load() & bit) return ARLGPU_OK;
  ARL_CUDA(cudaFuncSetAttribute(k_dsfft_rows_split, cudaFuncAttributeMaxDynamicSharedMemorySize, 4096 * 16));
  ARL_CUDA(cudaFuncSetAttribute(k_dsfft_rows<4096, 512>, cudaFuncAttributeMaxDynamicSharedMemorySize, 4096 * 16));
  ARL_CUDA(cudaFuncSetAttribute(k_dsfft_cols1, cudaFuncAttributeMaxDynamicSharedMemorySize, kColSmem));
  ARL_CUDA(cudaFuncSetAttribute(k_dsfft_cols2_image, cudaFuncAttributeMaxDynamicSharedMemorySize, kColSmem));
  ARL_CUDA(cudaFuncSetAttribute(k_dsfft_cols2_wstack, cudaFuncAttributeMaxDynamicSharedMemorySize, kColSmem2));
  done.fetch_or(bit);
  return ARLGPU_OK;
}

// Rows and first column pass of logical planes [q0, q0 + np) into buf.
static int rows_cols1(const float2 *grid, int64_t qstride, int nsum, int64_t q0, int64_t np, int ly, int lx,
                      const ColGeom &cg, float4 *buf, cudaStream_t st) {
  const int64_t nrows = np << ly;
  if (lx == 13) {
    k_dsfft_rows_split<<<(unsigned)(2 * nrows), 512, 4096 * 16, st>>>(grid, qstride, nsum, q0, (int)np, ly, buf);
  } else {
    const int log2S = 12 - lx;
    const int64_t rblocks = (nrows + ((int64_t)1 << log2S) - 1) >> log2S;
    k_dsfft_rows<4096, 512><<<(unsigned)rblocks, 512, 4096 * 16, st>>>(grid, qstride, nsum, q0, (int)np, ly, lx, buf);
  }
  ARL_LAUNCH_CHECK();
  const int64_t ntile = ((int64_t)1 << (cg.log2N2 - cg.log2G1)) << (lx - cg.log2WC1);
  k_dsfft_cols1<<<(unsigned)(np * ntile), kColT, kColSmem, st>>>(buf, ly, lx, cg, ntile);
  ARL_LAUNCH_CHECK();
  count_launch(2);
  return ARLGPU_OK;
}

// invert_2d: grid [nb][nw][ny][nx] FP32 complex -> image (real part, and the
// imaginary part when im_im is set); buf holds nb planes of float4.
int dsfft_g2i_2d(const float2 *grid, int nb, int nw, int ny, int nx, const double *gcf, const double *sumwt,
                 double *im_re, double *im_im, void *buf, cudaStream_t st) {
  const int ly = ilog2_exact(ny), lx = ilog2_exact(nx);
  ColGeom cg;
  if (!dsfft_supported(ny, nx) || !col_geom(ly, lx, &cg)) return fail(ARLGPU_ERR_UNSUPPORTED, "dsfft size");
  ARL_TRY(ensure_twiddles(st));
  ARL_TRY(set_smem());
  const int64_t plane = (int64_t)ny * nx;
  float4 *b4 = static_cast<float4 *>(buf);
  ARL_TRY(rows_cols1(grid, plane * nw, nw, 0, nb, ly, lx, cg, b4, st));
  const int64_t ntile = ((int64_t)1 << (cg.log2N1 - cg.log2G2)) << (lx - cg.log2WC2);
  const float s0 = (((nx / 2) + (ny / 2)) & 1) ? -1.f : 1.f;
  k_dsfft_cols2_image<<<(unsigned)(nb * ntile), kColT, kColSmem, st>>>(b4, ly, lx, cg, ntile, 0, s0, gcf, sumwt,
                                                                          im_re, im_im);
  ARL_LAUNCH_CHECK();
  count_launch(1);
  return ARLGPU_OK;
}

// w-stacking: grid [nb][K][ny][nx] FP32 complex; planes go through buf
// (room for G planes of float4) a group at a time; the image accumulates in
// double-single slots and is finished in place.
int dsfft_g2i_wstack(const float2 *grid, int nb, int K, int ny, int nx, double fov, const double *wmean,
                     const double *gcf, const double *sumwt, double *image, void *buf, int64_t G, cudaStream_t st) {
  const int ly = ilog2_exact(ny), lx = ilog2_exact(nx);
  ColGeom cg;
  if (!dsfft_supported(ny, nx) || !col_geom(ly, lx, &cg)) return fail(ARLGPU_ERR_UNSUPPORTED, "dsfft size");
  if (G < 1) return fail(ARLGPU_ERR_INVALID, "empty FFT group");
  ARL_TRY(ensure_twiddles(st));
  ARL_TRY(set_smem());
  const int64_t plane = (int64_t)ny * nx, nplanes = (int64_t)nb * K;
  float4 *b4 = static_cast<float4 *>(buf);
  const int64_t ntile = ((int64_t)1 << (cg.log2N1 - cg.log2G2)) << (lx - cg.log2WC2);
  for (int64_t p0 = 0; p0 < nplanes; p0 += G) {
    const int64_t np = std::min(G, nplanes - p0);
    ARL_TRY(rows_cols1(grid, plane, 1, p0, np, ly, lx, cg, b4, st));
    k_dsfft_cols2_wstack<<<(unsigned)ntile, kColT, kColSmem2, st>>>(b4, ly, lx, cg, p0, p0 + np, K, fov, wmean,
                                                                      reinterpret_cast<float2 *>(image));
    ARL_LAUNCH_CHECK();
    count_launch(1);
  }
  const float s0 = (((nx / 2) + (ny / 2)) & 1) ? -1.f : 1.f;
  const int64_t tot = nb * plane;
  const int blocks = (int)std::min<int64_t>((tot + 255) / 256, 152 * 32);
  k_ds_wstack_finish<<<blocks, 256, 0, st>>>(image, nb, ly, lx, s0, gcf, sumwt);
  ARL_LAUNCH_CHECK();
  count_launch(1);
  return ARLGPU_OK;
}

}  // namespace arlgpu
