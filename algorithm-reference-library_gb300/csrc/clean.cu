// Hogbom CLEAN on the GPU.
//
// Reference behaviour:
//   hogbom, overlapIndices    processing_library/arrays/cleaners.py:12-69, :134-154
//   hogbom_complex            processing_library/arrays/cleaners.py:72-131
//   deconvolve_cube('hogbom') processing_components/image/deconvolution.py:43-300
//
// Each minor-cycle iteration is two launches on one stream, with no host
// round trip:
//   k_hog_find  argmax of |res * window| (or |res|) over the image, first
//               index on ties as numpy.argmax; the last block to finish
//               (counted with an atomic, no waiting) reduces the per-block
//               maxima, forms mval = res[peak] * gain / pmax and adds it to the
//               component image;
//   k_hog_sub   res[overlap] -= psf[overlap] * mval, and the stopping test
//               |res[peak]| < 0.9 * threshold on the updated peak.
// A set stop flag turns the remaining launches into no-ops; the host reads
// the flag every kCheck iterations to stop launching.  All arithmetic is FP64
// with each operation rounded on its own (no FMA contraction), in the
// reference's order, so the result equals NumPy's bit for bit.
#include "common.cuh"

namespace arlgpu {

void count_launch(unsigned n);

struct HogState {
  double mval;
  long long peak;  // flat index of the peak, row-major [nx][ny]
  int stop;
  int iters;
  unsigned int counter;
};

struct Best {
  double v;
  long long i;
};

__device__ __forceinline__ Best better(Best a, Best b) {
  // larger value wins; on equal values the smaller index (numpy.argmax)
  if (b.v > a.v || (b.v == a.v && b.i < a.i)) return b;
  return a;
}

constexpr int kFindThreads = 256;

__global__ void __launch_bounds__(kFindThreads)
k_hog_find(const double *__restrict__ res, const double *__restrict__ window, long long n, double gain, double pmax,
           double *__restrict__ comps, Best *__restrict__ partial, HogState *__restrict__ st) {
  if (st->stop) return;
  __shared__ Best s_best[kFindThreads / 32];
  __shared__ bool s_last;
  Best b{-1.0, 0x7fffffffffffffffll};
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double a = window ? fabs(__dmul_rn(res[i], window[i])) : fabs(res[i]);
    b = better(b, Best{a, i});
  }
  for (int o = 16; o > 0; o >>= 1) {
    Best c;
    c.v = __shfl_xor_sync(0xffffffffu, b.v, o);
    c.i = __shfl_xor_sync(0xffffffffu, b.i, o);
    b = better(b, c);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) s_best[warp] = b;
  __syncthreads();
  if (threadIdx.x == 0) {
    Best t = s_best[0];
    for (int k = 1; k < kFindThreads / 32; ++k) t = better(t, s_best[k]);
    partial[blockIdx.x] = t;
    __threadfence();
    s_last = atomicAdd(&st->counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last) return;
  // Last block: reduce the per-block maxima.
  __threadfence();
  Best t{-1.0, 0x7fffffffffffffffll};
  for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) {
    Best q;  // other blocks' results: read past L1
    q.v = __ldcg(&partial[k].v);
    q.i = __ldcg(&partial[k].i);
    t = better(t, q);
  }
  for (int o = 16; o > 0; o >>= 1) {
    Best c;
    c.v = __shfl_xor_sync(0xffffffffu, t.v, o);
    c.i = __shfl_xor_sync(0xffffffffu, t.i, o);
    t = better(t, c);
  }
  if (lane == 0) s_best[warp] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    Best f = s_best[0];
    for (int k = 1; k < kFindThreads / 32; ++k) f = better(f, s_best[k]);
    const double mval = __ddiv_rn(__dmul_rn(res[f.i], gain), pmax);
    comps[f.i] = __dadd_rn(comps[f.i], mval);
    st->mval = mval;
    st->peak = f.i;
    st->counter = 0;
  }
}

// res[overlap] -= psf[overlap] * mval (overlapIndices of the reference), then
// the stopping test on the updated peak.
__global__ void k_hog_sub(double *__restrict__ res, int nx, int ny, const double *__restrict__ psf, int pnx, int pny,
                          double stop_level, HogState *__restrict__ st) {
  if (st->stop) return;
  const long long peak = st->peak;
  const int mx = (int)(peak / ny), my = (int)(peak - (long long)mx * ny);
  const double mval = st->mval;
  const int wx = pnx / 2, wy = pny / 2;
  const int r0 = max(0, mx - wx), r1 = min(nx, mx + wx);
  const int c0 = max(0, my - wy), c1 = min(my + wy, ny);
  const int p0 = max(0, wx + (r0 - mx)), q0 = max(0, wy + (c0 - my));
  const int p1 = min(pnx, wx + (r1 - mx)), q1 = min(wy + (c1 - my), pny);
  // numpy slices of unequal length would raise; the extents agree for every
  // peak inside the image, so the patch is (r1 - r0) x (c1 - c0)
  const int h = min(r1 - r0, p1 - p0), w = min(c1 - c0, q1 - q0);
  const long long total = (long long)h * w;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < total;
       k += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(k / w), j = (int)(k - (long long)i * w);
    const long long ri = (long long)(r0 + i) * ny + (c0 + j);
    const double nv = __dsub_rn(res[ri], __dmul_rn(psf[(long long)(p0 + i) * pny + (q0 + j)], mval));
    res[ri] = nv;
    if (ri == peak) {
      st->iters += 1;
      if (fabs(nv) < stop_level) st->stop = 1;
    }
  }
}

// ---------------------------------------------------------------------------
// Complex Hogbom CLEAN of Q + iU (processing_library/arrays/cleaners.py:72-131):
// the same two launches per iteration on a residual held as two planes
// (real, imaginary).  The peak is the first largest |res * window| (or |res|)
// with |.| the hypotenuse of the two parts, as numpy.absolute; the component
// res[peak] * gain / pmax and the PSF subtraction are taken part by part
// (the PSF is real), and the loop stops when |res[peak]| after the
// subtraction falls below the threshold itself (no 0.9 factor here).
// ---------------------------------------------------------------------------
struct HogCState {
  double mre, mim;
  long long peak;
  int stop;
  int iters;
  unsigned int counter;
};

__global__ void __launch_bounds__(kFindThreads)
k_hogc_find(const double *__restrict__ rre, const double *__restrict__ rim, const double *__restrict__ window,
            long long n, double gain, double pmax, double *__restrict__ cre, double *__restrict__ cim,
            Best *__restrict__ partial, HogCState *__restrict__ st) {
  if (st->stop) return;
  __shared__ Best s_best[kFindThreads / 32];
  __shared__ bool s_last;
  Best b{-1.0, 0x7fffffffffffffffll};
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double a = window ? hypot(__dmul_rn(rre[i], window[i]), __dmul_rn(rim[i], window[i])) : hypot(rre[i], rim[i]);
    b = better(b, Best{a, i});
  }
  for (int o = 16; o > 0; o >>= 1) {
    Best c;
    c.v = __shfl_xor_sync(0xffffffffu, b.v, o);
    c.i = __shfl_xor_sync(0xffffffffu, b.i, o);
    b = better(b, c);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) s_best[warp] = b;
  __syncthreads();
  if (threadIdx.x == 0) {
    Best t = s_best[0];
    for (int k = 1; k < kFindThreads / 32; ++k) t = better(t, s_best[k]);
    partial[blockIdx.x] = t;
    __threadfence();
    s_last = atomicAdd(&st->counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  Best t{-1.0, 0x7fffffffffffffffll};
  for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) {
    Best q;
    q.v = __ldcg(&partial[k].v);
    q.i = __ldcg(&partial[k].i);
    t = better(t, q);
  }
  for (int o = 16; o > 0; o >>= 1) {
    Best c;
    c.v = __shfl_xor_sync(0xffffffffu, t.v, o);
    c.i = __shfl_xor_sync(0xffffffffu, t.i, o);
    t = better(t, c);
  }
  if (lane == 0) s_best[warp] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    Best f = s_best[0];
    for (int k = 1; k < kFindThreads / 32; ++k) f = better(f, s_best[k]);
    const double mre = __ddiv_rn(__dmul_rn(rre[f.i], gain), pmax);
    const double mim = __ddiv_rn(__dmul_rn(rim[f.i], gain), pmax);
    cre[f.i] = __dadd_rn(cre[f.i], mre);
    cim[f.i] = __dadd_rn(cim[f.i], mim);
    st->mre = mre;
    st->mim = mim;
    st->peak = f.i;
    st->counter = 0;
  }
}

__global__ void k_hogc_sub(double *__restrict__ rre, double *__restrict__ rim, int nx, int ny,
                           const double *__restrict__ psf, int pnx, int pny, double stop_level,
                           HogCState *__restrict__ st) {
  if (st->stop) return;
  const long long peak = st->peak;
  const int mx = (int)(peak / ny), my = (int)(peak - (long long)mx * ny);
  const double mre = st->mre, mim = st->mim;
  const int wx = pnx / 2, wy = pny / 2;
  const int r0 = max(0, mx - wx), r1 = min(nx, mx + wx);
  const int c0 = max(0, my - wy), c1 = min(my + wy, ny);
  const int p0 = max(0, wx + (r0 - mx)), q0 = max(0, wy + (c0 - my));
  const int p1 = min(pnx, wx + (r1 - mx)), q1 = min(wy + (c1 - my), pny);
  const int h = min(r1 - r0, p1 - p0), w = min(c1 - c0, q1 - q0);
  const long long total = (long long)h * w;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < total;
       k += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(k / w), j = (int)(k - (long long)i * w);
    const long long ri = (long long)(r0 + i) * ny + (c0 + j);
    const double pv = psf[(long long)(p0 + i) * pny + (q0 + j)];
    const double nre = __dsub_rn(rre[ri], __dmul_rn(pv, mre));
    const double nim = __dsub_rn(rim[ri], __dmul_rn(pv, mim));
    rre[ri] = nre;
    rim[ri] = nim;
    if (ri == peak) {
      st->iters += 1;
      if (hypot(nre, nim) < stop_level) st->stop = 1;
    }
  }
}

// ---------------------------------------------------------------------------
// Multi-scale multi-frequency CLEAN minor cycle (processing_library/arrays/
// cleaners.py:469-600 with find_global_optimum :601-634,
// update_scale_moment_residual :636-646, update_moment_model :648-661,
// calculate_scale_moment_principal_solution :722-735 and
// find_optimum_scale_zero_moment :738-767).  Inputs from the set-up: the
// scale-moment residual smres [ns][nm][n0][n1], the scale-scale-moment-moment
// PSF ssm [ns][ns][nm][nm][p0][p1], the PSF-sized scale images pscale
// [ns][p0][p1], an optional window stack [ns][n0][n1] and the moment-moment
// Hessian and its inverse [ns][nm][nm].  Per iteration:
//   k_mfs_find  for each scale, the principal solution
//               smpsol[s][n] = sum_m ih[s][m][n] smres[s][m] at every pixel and
//               the search image (ARL: smpsol[s][0] smres[s][0]; Algorithm1:
//               smpsol[s][0]; CASA: the chi^2 change); the scale whose search
//               image has the largest |. * window| (first scale on ties, 0 if
//               none exceeds 0) wins, at the first largest signed (unwindowed)
//               search value -- the reference's argmax; the last block forms
//               mval = smpsol[scale][:, peak] and stops the loop when
//               max |mval| falls below the threshold;
//   k_mfs_sub   smres[:, :, lhs] -= gain * sum_q ssm[scale, :, :, q, rhs] mval[q]
//               and model[t, lhs] += pscale[scale, rhs] * gain * mval[t].
// FP64 with each operation rounded on its own, in the reference's order.
// ---------------------------------------------------------------------------
constexpr int kMfsMaxScales = 16, kMfsMaxMoments = 8;

struct MfsState {
  double mval[kMfsMaxMoments];
  long long peak;
  int scale;
  int stop;
  int iters;
  unsigned int counter;
};

struct MfsBest {
  double absmax;  // largest |search * window| (value only)
  Best vmax;      // first largest signed search value
};

__device__ __forceinline__ void mfs_solution(const double *__restrict__ smres, const double *__restrict__ ihess,
                                             int s, int nm, long long plane, long long i, double *sol) {
  // einsum("smn,smxy->snxy"): sum over m in order
  for (int n = 0; n < nm; ++n) {
    double acc = 0.0;
    for (int m = 0; m < nm; ++m)
      acc = __dadd_rn(acc, __dmul_rn(ihess[(s * nm + m) * nm + n], smres[((long long)s * nm + m) * plane + i]));
    sol[n] = acc;
  }
}

__device__ __forceinline__ double mfs_search(const double *__restrict__ smres, const double *__restrict__ hess,
                                             const double *sol, int s, int nm, long long plane, long long i,
                                             int findpeak) {
  if (findpeak == 1) return sol[0];  // Algorithm1
  if (findpeak == 2) {               // CASA: dchisq
    double d = 0.0;
    for (int m1 = 0; m1 < nm; ++m1) {
      d = __dadd_rn(d, __dmul_rn(__dmul_rn(2.0, sol[m1]), smres[((long long)s * nm + m1) * plane + i]));
      for (int m2 = 0; m2 < nm; ++m2)
        d = __dsub_rn(d, __dmul_rn(__dmul_rn(hess[(s * nm + m1) * nm + m2], sol[m1]), sol[m2]));
    }
    return d;
  }
  return __dmul_rn(sol[0], smres[(long long)s * nm * plane + i]);  // ARL
}

__global__ void __launch_bounds__(kFindThreads)
k_mfs_find(const double *__restrict__ smres, const double *__restrict__ windowstack, const double *__restrict__ hess,
           const double *__restrict__ ihess, int ns, int nm, long long plane, int findpeak, double absthresh,
           MfsBest *__restrict__ partial, MfsState *__restrict__ st) {
  if (st->stop) return;
  __shared__ double s_abs[kFindThreads / 32];
  __shared__ Best s_best[kFindThreads / 32];
  __shared__ bool s_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double sol[kMfsMaxMoments];
  for (int s = 0; s < ns; ++s) {
    double am = 0.0;
    Best b{-INFINITY, 0x7fffffffffffffffll};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < plane;
         i += (long long)gridDim.x * blockDim.x) {
      mfs_solution(smres, ihess, s, nm, plane, i, sol);
      const double v = mfs_search(smres, hess, sol, s, nm, plane, i, findpeak);
      const double vw = windowstack ? __dmul_rn(v, windowstack[(long long)s * plane + i]) : v;
      am = fmax(am, fabs(vw));
      b = better(b, Best{v, i});
    }
    for (int o = 16; o > 0; o >>= 1) {
      am = fmax(am, __shfl_xor_sync(0xffffffffu, am, o));
      Best c;
      c.v = __shfl_xor_sync(0xffffffffu, b.v, o);
      c.i = __shfl_xor_sync(0xffffffffu, b.i, o);
      b = better(b, c);
    }
    if (lane == 0) {
      s_abs[warp] = am;
      s_best[warp] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      MfsBest t{s_abs[0], s_best[0]};
      for (int k = 1; k < kFindThreads / 32; ++k) {
        t.absmax = fmax(t.absmax, s_abs[k]);
        t.vmax = better(t.vmax, s_best[k]);
      }
      partial[(long long)blockIdx.x * ns + s] = t;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(&st->counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last || threadIdx.x != 0) return;
  // Last block, one thread: per scale the reduction over blocks, then the
  // scale search of find_optimum_scale_zero_moment.
  __threadfence();
  double optimum = 0.0;
  int sscale = 0;
  long long sidx = 0;
  for (int s = 0; s < ns; ++s) {
    double am = 0.0;
    Best b{-INFINITY, 0x7fffffffffffffffll};
    for (int k = 0; k < (int)gridDim.x; ++k) {
      const MfsBest *q = &partial[(long long)k * ns + s];
      am = fmax(am, __ldcg(&q->absmax));
      b = better(b, Best{__ldcg(&q->vmax.v), __ldcg(&q->vmax.i)});
    }
    if (am > optimum) {
      optimum = am;
      sscale = s;
      sidx = b.i;
    }
  }
  mfs_solution(smres, ihess, sscale, nm, plane, sidx, sol);
  double peak = 0.0;
  for (int n = 0; n < nm; ++n) {
    st->mval[n] = sol[n];
    peak = fmax(peak, fabs(sol[n]));
  }
  st->scale = sscale;
  st->peak = sidx;
  st->counter = 0;
  st->iters += 1;
  if (peak < absthresh) st->stop = 2;  // stop before this iteration's update
}

__global__ void k_mfs_sub(double *__restrict__ smres, double *__restrict__ model, const double *__restrict__ ssm,
                          const double *__restrict__ pscale, int ns, int nm, int n0, int n1, int p0n, int p1n,
                          double gain, MfsState *__restrict__ st) {
  if (st->stop) return;
  const long long peak = st->peak;
  const int mx = (int)(peak / n1), my = (int)(peak - (long long)mx * n1);
  const int ms = st->scale;
  const int wx = p0n / 2, wy = p1n / 2;
  const int r0 = max(0, mx - wx), r1 = min(n0, mx + wx);
  const int c0 = max(0, my - wy), c1 = min(my + wy, n1);
  const int q0 = max(0, wx + (r0 - mx)), s0 = max(0, wy + (c0 - my));
  const int q1 = min(p0n, wx + (r1 - mx)), s1 = min(wy + (c1 - my), p1n);
  const int h = min(r1 - r0, q1 - q0), w = min(c1 - c0, s1 - s0);
  const long long plane = (long long)n0 * n1, pplane = (long long)p0n * p1n;
  const long long total = (long long)h * w;
  double mv[kMfsMaxMoments];
  for (int t = 0; t < nm; ++t) mv[t] = st->mval[t];
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < total;
       k += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(k / w), j = (int)(k - (long long)i * w);
    const long long ri = (long long)(r0 + i) * n1 + (c0 + j);
    const long long pi = (long long)(q0 + i) * p1n + (s0 + j);
    for (int s = 0; s < ns; ++s)
      for (int t = 0; t < nm; ++t) {
        double acc = 0.0;  // einsum("stqxy,q->stxy"): sum over q in order
        for (int q = 0; q < nm; ++q)
          acc = __dadd_rn(acc, __dmul_rn(ssm[((((long long)ms * ns + s) * nm + t) * nm + q) * pplane + pi], mv[q]));
        double *r = smres + ((long long)s * nm + t) * plane + ri;
        *r = __dsub_rn(*r, __dmul_rn(gain, acc));
      }
    const double ps = pscale[(long long)ms * pplane + pi];
    for (int t = 0; t < nm; ++t) {
      double *m = model + (long long)t * plane + ri;
      *m = __dadd_rn(*m, __dmul_rn(__dmul_rn(ps, gain), mv[t]));
    }
  }
}

// ---------------------------------------------------------------------------
// Multiscale CLEAN (processing_library/arrays/cleaners.py:165-280): the
// minor-cycle loop over the scale stack.  The scale images, the twice-
// convolved PSF stack and the coupling matrix come from the caller (the
// reference forms them with NumPy FFTs).  Per iteration:
//   k_ms_find  argmax over scales and pixels of |stack_s * window_s / c_ss|,
//              ties to the lower scale, then the lower index (the reference
//              scans scales in order and keeps a strictly larger value); the
//              last block applies the stopping tests (|stack[peak]| below
//              0.9 * threshold, or a zero component) and forms mval;
//   k_ms_sub   stack_s[overlap] -= psf_ss[s, mscale][overlap] * gain * mval for
//              every scale, comps[overlap] += pscale[mscale][overlap] * gain * mval.
// ---------------------------------------------------------------------------
struct MsState {
  double mval;
  long long peak;  // flat pixel index
  int mscale;
  int stop;
  int iters;
  unsigned int counter;
};

struct BestS {
  double v;
  long long key;  // scale * npix + pixel: lower key wins ties
};

__device__ __forceinline__ BestS better_s(BestS a, BestS b) {
  if (b.v > a.v || (b.v == a.v && b.key < a.key)) return b;
  return a;
}

__global__ void __launch_bounds__(kFindThreads)
k_ms_find(const double *__restrict__ stack, const double *__restrict__ wstack, const double *__restrict__ coupling,
          int ns, long long npix, double stop_level, BestS *__restrict__ partial, MsState *__restrict__ st) {
  if (st->stop) return;
  __shared__ BestS s_best[kFindThreads / 32];
  __shared__ bool s_last;
  BestS b{-1.0, 0x7fffffffffffffffll};
  const long long total = (long long)ns * npix;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < total;
       k += (long long)gridDim.x * blockDim.x) {
    const int sc = (int)(k / npix);
    const double c = coupling[sc * ns + sc];
    const double v = wstack ? __dmul_rn(stack[k], wstack[k]) : stack[k];
    b = better_s(b, BestS{fabs(__ddiv_rn(v, c)), k});
  }
  for (int o = 16; o > 0; o >>= 1) {
    BestS c;
    c.v = __shfl_xor_sync(0xffffffffu, b.v, o);
    c.key = __shfl_xor_sync(0xffffffffu, b.key, o);
    b = better_s(b, c);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) s_best[warp] = b;
  __syncthreads();
  if (threadIdx.x == 0) {
    BestS t = s_best[0];
    for (int k = 1; k < kFindThreads / 32; ++k) t = better_s(t, s_best[k]);
    partial[blockIdx.x] = t;
    __threadfence();
    s_last = atomicAdd(&st->counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  BestS t{-1.0, 0x7fffffffffffffffll};
  for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) {
    BestS q;  // other blocks' results: read past L1
    q.v = __ldcg(&partial[k].v);
    q.key = __ldcg(&partial[k].key);
    t = better_s(t, q);
  }
  for (int o = 16; o > 0; o >>= 1) {
    BestS c;
    c.v = __shfl_xor_sync(0xffffffffu, t.v, o);
    c.key = __shfl_xor_sync(0xffffffffu, t.key, o);
    t = better_s(t, c);
  }
  if (lane == 0) s_best[warp] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    BestS f = s_best[0];
    for (int k = 1; k < kFindThreads / 32; ++k) f = better_s(f, s_best[k]);
    const int sc = (int)(f.key / npix);
    const double r = stack[f.key];
    const double mval = __ddiv_rn(r, coupling[sc * ns + sc]);
    st->counter = 0;
    st->iters += 1;
    if (fabs(r) < stop_level || !(fabs(mval) > 0.0)) {
      st->stop = 1;
      return;
    }
    st->mval = mval;
    st->mscale = sc;
    st->peak = f.key - (long long)sc * npix;
  }
}

__global__ void k_ms_sub(double *__restrict__ stack, double *__restrict__ comps, int ns, int nx, int ny,
                         const double *__restrict__ psf_ss, const double *__restrict__ pscale, int pnx, int pny,
                         double gain, MsState *__restrict__ st) {
  if (st->stop) return;
  const long long peak = st->peak;
  const int mscale = st->mscale;
  const int mx = (int)(peak / ny), my = (int)(peak - (long long)mx * ny);
  const double mval = st->mval;
  const int wx = pnx / 2, wy = pny / 2;
  const int r0 = max(0, mx - wx), r1 = min(nx, mx + wx);
  const int c0 = max(0, my - wy), c1 = min(my + wy, ny);
  const int p0 = max(0, wx + (r0 - mx)), q0 = max(0, wy + (c0 - my));
  const int p1 = min(pnx, wx + (r1 - mx)), q1 = min(wy + (c1 - my), pny);
  const int h = min(r1 - r0, p1 - p0), w = min(c1 - c0, q1 - q0);
  const long long patch = (long long)h * w, total = patch * (ns + 1);
  const long long npix = (long long)nx * ny, ppix = (long long)pnx * pny;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < total;
       k += (long long)gridDim.x * blockDim.x) {
    const int slot = (int)(k / patch);
    const long long e = k - (long long)slot * patch;
    const int i = (int)(e / w), j = (int)(e - (long long)i * w);
    const long long ri = (long long)(r0 + i) * ny + (c0 + j);
    const long long pi = (long long)(p0 + i) * pny + (q0 + j);
    if (slot < ns) {
      const double d = __dmul_rn(__dmul_rn(psf_ss[((long long)slot * ns + mscale) * ppix + pi], gain), mval);
      stack[slot * npix + ri] = __dsub_rn(stack[slot * npix + ri], d);
    } else {
      const double d = __dmul_rn(__dmul_rn(pscale[(long long)mscale * ppix + pi], gain), mval);
      comps[ri] = __dadd_rn(comps[ri], d);
    }
  }
}

static int nblk(long long n, int cap) {
  long long b = (n + 255) / 256;
  return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace arlgpu

using namespace arlgpu;

extern "C" int arlgpu_hogbom(const double *dirty, const double *psf, const double *window, int32_t nx, int32_t ny,
                             int32_t psf_nx, int32_t psf_ny, double gain, double thresh, int32_t niter,
                             double fracthresh, double dirty_absmax, double psf_max, double *comps, double *res,
                             int32_t *iterations, void *stream) {
  if (!dirty || !psf || !comps || !res || !iterations) return fail(ARLGPU_ERR_INVALID, "null array argument");
  if (nx < 1 || ny < 1 || psf_nx < 2 || psf_ny < 2) return fail(ARLGPU_ERR_INVALID, "bad image or psf shape");
  if (!(gain > 0.0 && gain < 2.0)) return fail(ARLGPU_ERR_INVALID, "gain must be in (0, 2)");
  if (niter < 1) return fail(ARLGPU_ERR_INVALID, "niter must be > 0");
  if (!(psf_max > 0.0)) return fail(ARLGPU_ERR_INVALID, "psf maximum must be > 0");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const long long n = (long long)nx * ny;
  const int fblocks = nblk(n, 152 * 4);
  const int sblocks = nblk((long long)psf_nx * psf_ny, 152 * 8);
  HogState *state = nullptr;
  Best *partial = nullptr;
  ARL_CUDA(cudaMallocAsync(&state, sizeof(HogState), st));
  int rc = ARLGPU_OK;
  if (cudaMallocAsync(&partial, sizeof(Best) * fblocks, st) != cudaSuccess) {
    cudaFreeAsync(state, st);
    return fail(ARLGPU_ERR_CUDA, "cudaMallocAsync failed");
  }
  const double absthresh = fmax(thresh, fracthresh * dirty_absmax);
  const double stop_level = 0.9 * absthresh;
  constexpr int kCheck = 64;
  int it = 0;
  HogState hs{};
  do {
    if (cudaMemsetAsync(state, 0, sizeof(HogState), st) != cudaSuccess ||
        cudaMemcpyAsync(res, dirty, sizeof(double) * n, cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
        cudaMemsetAsync(comps, 0, sizeof(double) * n, st) != cudaSuccess) {
      rc = fail(ARLGPU_ERR_CUDA, "hogbom set-up failed");
      break;
    }
    while (it < niter) {
      const int batch = niter - it < kCheck ? niter - it : kCheck;
      for (int k = 0; k < batch; ++k) {
        k_hog_find<<<fblocks, kFindThreads, 0, st>>>(res, window, n, gain, psf_max, comps, partial, state);
        k_hog_sub<<<sblocks, 256, 0, st>>>(res, nx, ny, psf, psf_nx, psf_ny, stop_level, state);
      }
      count_launch(2 * batch);
      it += batch;
      if (cudaGetLastError() != cudaSuccess) {
        rc = fail(ARLGPU_ERR_CUDA, "hogbom launch failed");
        break;
      }
      if (cudaMemcpyAsync(&hs, state, sizeof hs, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
          cudaStreamSynchronize(st) != cudaSuccess) {
        rc = fail(ARLGPU_ERR_CUDA, "hogbom state read failed");
        break;
      }
      if (hs.stop) break;
    }
  } while (false);
  *iterations = hs.iters;
  cudaFreeAsync(partial, st);
  cudaFreeAsync(state, st);
  return rc;
}

extern "C" int arlgpu_hogbom_complex(const double *dirty_q, const double *dirty_u, const double *psf,
                                     const double *window, int32_t nx, int32_t ny, int32_t psf_nx, int32_t psf_ny,
                                     double gain, double thresh, int32_t niter, double fracthresh,
                                     double dirty_absmax, double psf_max, double *comps_q, double *comps_u,
                                     double *res_q, double *res_u, int32_t *iterations, void *stream) {
  if (!dirty_q || !dirty_u || !psf || !comps_q || !comps_u || !res_q || !res_u || !iterations)
    return fail(ARLGPU_ERR_INVALID, "null array argument");
  if (nx < 1 || ny < 1 || psf_nx < 2 || psf_ny < 2) return fail(ARLGPU_ERR_INVALID, "bad image or psf shape");
  if (!(gain > 0.0 && gain < 2.0)) return fail(ARLGPU_ERR_INVALID, "gain must be in (0, 2)");
  if (niter < 1) return fail(ARLGPU_ERR_INVALID, "niter must be > 0");
  if (!(psf_max > 0.0)) return fail(ARLGPU_ERR_INVALID, "psf maximum must be > 0");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const long long n = (long long)nx * ny;
  const int fblocks = nblk(n, 152 * 4);
  const int sblocks = nblk((long long)psf_nx * psf_ny, 152 * 8);
  HogCState *state = nullptr;
  Best *partial = nullptr;
  ARL_CUDA(cudaMallocAsync(&state, sizeof(HogCState), st));
  int rc = ARLGPU_OK;
  if (cudaMallocAsync(&partial, sizeof(Best) * fblocks, st) != cudaSuccess) {
    cudaFreeAsync(state, st);
    return fail(ARLGPU_ERR_CUDA, "cudaMallocAsync failed");
  }
  const double absthresh = fmax(thresh, fracthresh * dirty_absmax);
  constexpr int kCheck = 64;
  int it = 0;
  HogCState hs{};
  do {
    if (cudaMemsetAsync(state, 0, sizeof(HogCState), st) != cudaSuccess ||
        cudaMemcpyAsync(res_q, dirty_q, sizeof(double) * n, cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(res_u, dirty_u, sizeof(double) * n, cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
        cudaMemsetAsync(comps_q, 0, sizeof(double) * n, st) != cudaSuccess ||
        cudaMemsetAsync(comps_u, 0, sizeof(double) * n, st) != cudaSuccess) {
      rc = fail(ARLGPU_ERR_CUDA, "hogbom_complex set-up failed");
      break;
    }
    while (it < niter) {
      const int batch = niter - it < kCheck ? niter - it : kCheck;
      for (int k = 0; k < batch; ++k) {
        k_hogc_find<<<fblocks, kFindThreads, 0, st>>>(res_q, res_u, window, n, gain, psf_max, comps_q, comps_u,
                                                       partial, state);
        k_hogc_sub<<<sblocks, 256, 0, st>>>(res_q, res_u, nx, ny, psf, psf_nx, psf_ny, absthresh, state);
      }
      count_launch(2 * batch);
      it += batch;
      if (cudaGetLastError() != cudaSuccess) {
        rc = fail(ARLGPU_ERR_CUDA, "hogbom_complex launch failed");
        break;
      }
      if (cudaMemcpyAsync(&hs, state, sizeof hs, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
          cudaStreamSynchronize(st) != cudaSuccess) {
        rc = fail(ARLGPU_ERR_CUDA, "hogbom_complex state read failed");
        break;
      }
      if (hs.stop) break;
    }
  } while (false);
  *iterations = hs.iters;
  cudaFreeAsync(partial, st);
  cudaFreeAsync(state, st);
  return rc;
}

extern "C" int arlgpu_msmfsclean(double *smres, const double *ssm, const double *pscale, const double *windowstack,
                                 const double *hess, const double *ihess, int32_t nscales, int32_t nmoment,
                                 int32_t n0, int32_t n1, int32_t psf_n0, int32_t psf_n1, double gain, double absthresh,
                                 int32_t niter, int32_t findpeak, double *model, int32_t *iterations, void *stream) {
  if (!smres || !ssm || !pscale || !hess || !ihess || !model || !iterations)
    return fail(ARLGPU_ERR_INVALID, "null array argument");
  if (nscales < 1 || nscales > kMfsMaxScales || nmoment < 1 || nmoment > kMfsMaxMoments)
    return fail(ARLGPU_ERR_UNSUPPORTED, "msmfsclean takes 1..%d scales and 1..%d moments", kMfsMaxScales,
                kMfsMaxMoments);
  if (n0 < 1 || n1 < 1 || psf_n0 < 2 || psf_n1 < 2) return fail(ARLGPU_ERR_INVALID, "bad image or psf shape");
  if (!(gain > 0.0 && gain < 2.0)) return fail(ARLGPU_ERR_INVALID, "gain must be in (0, 2)");
  if (niter < 1) return fail(ARLGPU_ERR_INVALID, "niter must be > 0");
  if (findpeak < 0 || findpeak > 2) return fail(ARLGPU_ERR_INVALID, "findpeak must be 0 (ARL), 1 (Algorithm1), 2 (CASA)");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const long long plane = (long long)n0 * n1;
  const int fblocks = nblk(plane, 152 * 2);
  const int sblocks = nblk((long long)psf_n0 * psf_n1, 152 * 8);
  MfsState *state = nullptr;
  MfsBest *partial = nullptr;
  ARL_CUDA(cudaMallocAsync(&state, sizeof(MfsState), st));
  int rc = ARLGPU_OK;
  if (cudaMallocAsync(&partial, sizeof(MfsBest) * fblocks * nscales, st) != cudaSuccess) {
    cudaFreeAsync(state, st);
    return fail(ARLGPU_ERR_CUDA, "cudaMallocAsync failed");
  }
  constexpr int kCheck = 32;
  int it = 0;
  MfsState hs{};
  do {
    if (cudaMemsetAsync(state, 0, sizeof(MfsState), st) != cudaSuccess ||
        cudaMemsetAsync(model, 0, sizeof(double) * plane * nmoment, st) != cudaSuccess) {
      rc = fail(ARLGPU_ERR_CUDA, "msmfsclean set-up failed");
      break;
    }
    while (it < niter) {
      const int batch = niter - it < kCheck ? niter - it : kCheck;
      for (int k = 0; k < batch; ++k) {
        k_mfs_find<<<fblocks, kFindThreads, 0, st>>>(smres, windowstack, hess, ihess, nscales, nmoment, plane,
                                                      findpeak, absthresh, partial, state);
        k_mfs_sub<<<sblocks, 256, 0, st>>>(smres, model, ssm, pscale, nscales, nmoment, n0, n1, psf_n0, psf_n1,
                                           gain, state);
      }
      count_launch(2 * batch);
      it += batch;
      if (cudaGetLastError() != cudaSuccess) {
        rc = fail(ARLGPU_ERR_CUDA, "msmfsclean launch failed");
        break;
      }
      if (cudaMemcpyAsync(&hs, state, sizeof hs, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
          cudaStreamSynchronize(st) != cudaSuccess) {
        rc = fail(ARLGPU_ERR_CUDA, "msmfsclean state read failed");
        break;
      }
      if (hs.stop) break;
    }
  } while (false);
  *iterations = hs.iters;
  cudaFreeAsync(partial, st);
  cudaFreeAsync(state, st);
  return rc;
}

extern "C" int arlgpu_msclean(double *stack, const double *psf_ss, const double *pscale, const double *windowstack,
                              const double *coupling, int32_t nscales, int32_t nx, int32_t ny, int32_t psf_nx,
                              int32_t psf_ny, double gain, double absthresh, int32_t niter, double *comps,
                              int32_t *iterations, void *stream) {
  if (!stack || !psf_ss || !pscale || !coupling || !comps || !iterations)
    return fail(ARLGPU_ERR_INVALID, "null array argument");
  if (nscales < 1 || nx < 1 || ny < 1 || psf_nx < 2 || psf_ny < 2) return fail(ARLGPU_ERR_INVALID, "bad shapes");
  if (!(gain > 0.0 && gain < 2.0)) return fail(ARLGPU_ERR_INVALID, "gain must be in (0, 2)");
  if (niter < 1) return fail(ARLGPU_ERR_INVALID, "niter must be > 0");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const long long npix = (long long)nx * ny;
  const int fblocks = nblk((long long)nscales * npix, 152 * 4);
  const int sblocks = nblk((long long)psf_nx * psf_ny * (nscales + 1), 152 * 8);
  MsState *state = nullptr;
  BestS *partial = nullptr;
  ARL_CUDA(cudaMallocAsync(&state, sizeof(MsState), st));
  if (cudaMallocAsync(&partial, sizeof(BestS) * fblocks, st) != cudaSuccess) {
    cudaFreeAsync(state, st);
    return fail(ARLGPU_ERR_CUDA, "cudaMallocAsync failed");
  }
  const double stop_level = 0.9 * absthresh;
  constexpr int kCheck = 64;
  int rc = ARLGPU_OK;
  MsState hs{};
  if (cudaMemsetAsync(state, 0, sizeof(MsState), st) != cudaSuccess ||
      cudaMemsetAsync(comps, 0, sizeof(double) * npix, st) != cudaSuccess) {
    rc = fail(ARLGPU_ERR_CUDA, "msclean set-up failed");
  }
  for (int it = 0; rc == ARLGPU_OK && it < niter;) {
    const int batch = niter - it < kCheck ? niter - it : kCheck;
    for (int k = 0; k < batch; ++k) {
      k_ms_find<<<fblocks, kFindThreads, 0, st>>>(stack, windowstack, coupling, nscales, npix, stop_level, partial,
                                                  state);
      k_ms_sub<<<sblocks, 256, 0, st>>>(stack, comps, nscales, nx, ny, psf_ss, pscale, psf_nx, psf_ny, gain, state);
    }
    count_launch(2 * batch);
    it += batch;
    if (cudaGetLastError() != cudaSuccess) {
      rc = fail(ARLGPU_ERR_CUDA, "msclean launch failed");
      break;
    }
    if (cudaMemcpyAsync(&hs, state, sizeof hs, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      rc = fail(ARLGPU_ERR_CUDA, "msclean state read failed");
      break;
    }
    if (hs.stop) break;
  }
  *iterations = hs.iters;
  cudaFreeAsync(partial, st);
  cudaFreeAsync(state, st);
  return rc;
}
