// Row-wise visibility operators on the path (K10, K11).
//
// Reference behaviour:
//   phaserotate_visibility (tangent=True)   processing_components/visibility/base.py:295-334
//   simulate_point                          processing_library/util/coordinate_support.py:192-212
//   apply_gaintable, scalar gains           processing_components/calibration/operations.py:79-164 (:134-137)
#include "common.cuh"

namespace arlgpu {

void count_launch(unsigned n);

// vis *= exp(-2 pi i s.uvw) (inverse) or its conjugate; s = (l, m, n - 1).
template <typename CT>
__global__ void k_phaserotate(CT *vis, const double *uvw, int64_t nvis, int npol, double l, double m, double n1,
                              int inverse) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nvis; r += (int64_t)gridDim.x * blockDim.x) {
    const double ph = -2.0 * M_PI * (uvw[3 * r] * l + uvw[3 * r + 1] * m + uvw[3 * r + 2] * n1);
    double s, c;
    sincos(ph, &s, &c);
    if (!inverse) s = -s;
    for (int p = 0; p < npol; ++p) {
      CT v = vis[r * npol + p];
      const double re = (double)v.x * c - (double)v.y * s, im = (double)v.x * s + (double)v.y * c;
      v.x = re;
      v.y = im;
      vis[r * npol + p] = v;
    }
  }
}

// Row of baseline (a1, a2), stored at [a2, a1]: V *= g[a2] conj(g[a1]).
// inverse uses 1/g where |g| > 0 and 1 elsewhere (operations.py:128-131).
template <typename CT>
__global__ void k_gains(CT *vis, int64_t nvis, int npol, const int32_t *a1, const int32_t *a2, const double2 *g,
                        int inverse) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nvis; r += (int64_t)gridDim.x * blockDim.x) {
    double2 ga = g[a2[r]], gb = g[a1[r]];
    if (inverse) {
      double na = ga.x * ga.x + ga.y * ga.y, nb = gb.x * gb.x + gb.y * gb.y;
      ga = na > 0.0 ? make_double2(ga.x / na, -ga.y / na) : make_double2(1.0, 0.0);
      gb = nb > 0.0 ? make_double2(gb.x / nb, -gb.y / nb) : make_double2(1.0, 0.0);
    }
    // m = ga * conj(gb)
    const double mr = ga.x * gb.x + ga.y * gb.y, mi = ga.y * gb.x - ga.x * gb.y;
    for (int p = 0; p < npol; ++p) {
      CT v = vis[r * npol + p];
      const double re = (double)v.x * mr - (double)v.y * mi, im = (double)v.x * mi + (double)v.y * mr;
      v.x = re;
      v.y = im;
      vis[r * npol + p] = v;
    }
  }
}

// chi^2 = sum_r,p w |Vobs - g[a2] conj(g[a1]) M|^2 and its conjugate-Wirtinger
// derivatives (row of baseline (a1, a2) stored at [a2, a1], the convention of
// apply_gaintable, calibration/operations.py:134-137):
//   d/d conj(M)     = -w conj(g2) g1 R
//   d/d conj(g[a2]) = -w R g1 conj(M)        (summed over rows and pols)
//   d/d conj(g[a1]) = -w conj(R) g2 M
// with R = Vobs - g2 conj(g1) M.  Per-antenna sums go through shared memory,
// then one global atomic per antenna and block.
template <typename CT>
__global__ void k_gain_chi2(const CT *__restrict__ vobs, const CT *__restrict__ m, const double *__restrict__ wt,
                            int64_t nvis, int npol, const int32_t *__restrict__ a1, const int32_t *__restrict__ a2,
                            const double2 *__restrict__ g, int nant, double *__restrict__ chi2,
                            CT *__restrict__ grad_m, double2 *__restrict__ grad_g) {
  extern __shared__ double sg[];  // 2 * nant: re, im of the per-antenna sums
  for (int i = threadIdx.x; i < 2 * nant; i += blockDim.x) sg[i] = 0.0;
  __syncthreads();
  double local = 0.0;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nvis; r += (int64_t)gridDim.x * blockDim.x) {
    const int i1 = a1[r], i2 = a2[r];
    const double2 g1 = g[i1], g2 = g[i2];
    const double gr = g2.x * g1.x + g2.y * g1.y, gi = g2.y * g1.x - g2.x * g1.y;  // g2 conj(g1)
    double d2r = 0.0, d2i = 0.0, d1r = 0.0, d1i = 0.0;
    for (int p = 0; p < npol; ++p) {
      const int64_t k = r * npol + p;
      const double w = wt ? wt[k] : 1.0;
      const double mr = m[k].x, mi = m[k].y;
      const double rr = (double)vobs[k].x - (gr * mr - gi * mi);
      const double ri = (double)vobs[k].y - (gr * mi + gi * mr);
      local += w * (rr * rr + ri * ri);
      if (grad_m) {
        // -w conj(g2 conj(g1)) R
        CT o;
        o.x = -w * (gr * rr + gi * ri);
        o.y = -w * (gr * ri - gi * rr);
        grad_m[k] = o;
      }
      // -w R g1 conj(M)
      const double tr = g1.x * mr + g1.y * mi, ti = g1.y * mr - g1.x * mi;  // g1 conj(M)
      d2r -= w * (rr * tr - ri * ti);
      d2i -= w * (rr * ti + ri * tr);
      // -w conj(R) g2 M
      const double ur = g2.x * mr - g2.y * mi, ui = g2.x * mi + g2.y * mr;  // g2 M
      d1r -= w * (rr * ur + ri * ui);
      d1i -= w * (rr * ui - ri * ur);
    }
    if (grad_g) {
      atomicAdd(&sg[2 * i2], d2r);
      atomicAdd(&sg[2 * i2 + 1], d2i);
      atomicAdd(&sg[2 * i1], d1r);
      atomicAdd(&sg[2 * i1 + 1], d1i);
    }
  }
  for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(chi2, local);
  __syncthreads();
  if (grad_g)
    for (int i = threadIdx.x; i < nant; i += blockDim.x)
      if (sg[2 * i] != 0.0 || sg[2 * i + 1] != 0.0) {
        atomicAdd(&grad_g[i].x, sg[2 * i]);
        atomicAdd(&grad_g[i].y, sg[2 * i + 1]);
      }
}

// apply_gaintable with scalar gains on a BlockVisibility (one polarisation):
// cell [t][i][j][c] of the block, for a time t with a gain-table row
// k = time_row[t] >= 0, becomes V * g[k][i][c] conj(g[k][j][c]), where g is the
// gain or, for the inverse, 1/gain where |gain| > 0 and 1 elsewhere
// (operations.py:124-137); the cell is zeroed where the product of the two
// antennas' gain weights is 0 (:138-140).  Times with time_row[t] < 0 are
// left as they are.
template <typename CT>
__global__ void k_gaintable(CT *vis, int ntimes, int nant, int nchan, const int32_t *__restrict__ time_row,
                            const double2 *__restrict__ g, const double *__restrict__ gw, int inverse) {
  const int64_t ncell = (int64_t)ntimes * nant * nant * nchan;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < ncell; q += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(q % nchan);
    int64_t r = q / nchan;
    const int j = (int)(r % nant);
    r /= nant;
    const int i = (int)(r % nant);
    const int t = (int)(r / nant);
    const int k = time_row[t];
    if (k < 0) continue;
    const int64_t gi = ((int64_t)k * nant + i) * nchan + c, gj = ((int64_t)k * nant + j) * nchan + c;
    double2 ga = g[gi], gb = g[gj];
    if (inverse) {
      const double na = ga.x * ga.x + ga.y * ga.y, nb = gb.x * gb.x + gb.y * gb.y;
      ga = na > 0.0 ? make_double2(ga.x / na, -ga.y / na) : make_double2(1.0, 0.0);
      gb = nb > 0.0 ? make_double2(gb.x / nb, -gb.y / nb) : make_double2(1.0, 0.0);
    }
    CT v = vis[q];
    if (gw[gi] * gw[gj] == 0.0) {
      v.x = 0;
      v.y = 0;
    } else {
      // m = ga conj(gb), then V m
      const double mr = ga.x * gb.x + ga.y * gb.y, mi = ga.y * gb.x - ga.x * gb.y;
      const double re = (double)v.x * mr - (double)v.y * mi, im = (double)v.x * mi + (double)v.y * mr;
      v.x = re;
      v.y = im;
    }
    vis[q] = v;
  }
}

static int nblk(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)(b < 1 ? 1 : (b > 152 * 32 ? 152 * 32 : b));
}

}  // namespace arlgpu

using namespace arlgpu;

extern "C" int arlgpu_phaserotate(void *vis, const double *uvw, int64_t nvis, int32_t npol, int precision, double l,
                                  double m, int inverse, void *stream) {
  if (nvis < 0 || npol < 1 || (nvis > 0 && (!vis || !uvw))) return fail(ARLGPU_ERR_INVALID, "bad arguments");
  if (nvis == 0) return ARLGPU_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const double n1 = sqrt(1.0 - l * l - m * m) - 1.0;
  if (precision == ARLGPU_FP64)
    k_phaserotate<double2><<<nblk(nvis), 256, 0, st>>>(static_cast<double2 *>(vis), uvw, nvis, npol, l, m, n1, inverse);
  else if (precision == ARLGPU_FP32C)
    k_phaserotate<float2><<<nblk(nvis), 256, 0, st>>>(static_cast<float2 *>(vis), uvw, nvis, npol, l, m, n1, inverse);
  else
    return fail(ARLGPU_ERR_INVALID, "bad precision");
  ARL_LAUNCH_CHECK();
  count_launch(1);
  return ARLGPU_OK;
}

extern "C" int arlgpu_apply_gains(void *vis, int64_t nvis, int32_t npol, int precision, const int32_t *a1,
                                  const int32_t *a2, const void *gains, int inverse, void *stream) {
  if (nvis < 0 || npol < 1 || (nvis > 0 && (!vis || !a1 || !a2 || !gains))) return fail(ARLGPU_ERR_INVALID, "bad arguments");
  if (nvis == 0) return ARLGPU_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const double2 *g = static_cast<const double2 *>(gains);
  if (precision == ARLGPU_FP64)
    k_gains<double2><<<nblk(nvis), 256, 0, st>>>(static_cast<double2 *>(vis), nvis, npol, a1, a2, g, inverse);
  else if (precision == ARLGPU_FP32C)
    k_gains<float2><<<nblk(nvis), 256, 0, st>>>(static_cast<float2 *>(vis), nvis, npol, a1, a2, g, inverse);
  else
    return fail(ARLGPU_ERR_INVALID, "bad precision");
  ARL_LAUNCH_CHECK();
  count_launch(1);
  return ARLGPU_OK;
}

extern "C" int arlgpu_apply_gaintable(void *vis, int32_t ntimes, int32_t nants, int32_t nchan, int precision,
                                      const int32_t *time_row, const void *gain, const double *gain_weight,
                                      int inverse, void *stream) {
  if (ntimes < 0 || nants < 1 || nchan < 1) return fail(ARLGPU_ERR_INVALID, "bad block shape");
  const int64_t ncell = (int64_t)ntimes * nants * nants * nchan;
  if (ncell == 0) return ARLGPU_OK;
  if (!vis || !time_row || !gain || !gain_weight) return fail(ARLGPU_ERR_INVALID, "null array argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const double2 *g = static_cast<const double2 *>(gain);
  if (precision == ARLGPU_FP64)
    k_gaintable<double2><<<nblk(ncell), 256, 0, st>>>(static_cast<double2 *>(vis), ntimes, nants, nchan, time_row, g,
                                                      gain_weight, inverse);
  else if (precision == ARLGPU_FP32C)
    k_gaintable<float2><<<nblk(ncell), 256, 0, st>>>(static_cast<float2 *>(vis), ntimes, nants, nchan, time_row, g,
                                                     gain_weight, inverse);
  else
    return fail(ARLGPU_ERR_INVALID, "bad precision");
  ARL_LAUNCH_CHECK();
  count_launch(1);
  return ARLGPU_OK;
}

extern "C" int arlgpu_gain_chi2(const void *vobs, const void *model, const double *weight, int64_t nvis, int32_t npol,
                                int precision, const int32_t *a1, const int32_t *a2, const void *gains, int32_t nant,
                                double *chi2, void *grad_model, void *grad_gains, void *stream) {
  if (nvis < 0 || npol < 1 || nant < 1 || !chi2 || (nvis > 0 && (!vobs || !model || !a1 || !a2 || !gains)))
    return fail(ARLGPU_ERR_INVALID, "bad arguments");
  if (nant > 4096) return fail(ARLGPU_ERR_UNSUPPORTED, "more than 4096 antennas");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  ARL_CUDA(cudaMemsetAsync(chi2, 0, sizeof(double), st));
  if (grad_gains) ARL_CUDA(cudaMemsetAsync(grad_gains, 0, sizeof(double2) * nant, st));
  if (nvis == 0) return ARLGPU_OK;
  const size_t smem = 2 * sizeof(double) * nant;
  const int blocks = nblk(nvis) < 152 * 4 ? nblk(nvis) : 152 * 4;
  const double2 *g = static_cast<const double2 *>(gains);
  if (precision == ARLGPU_FP64)
    k_gain_chi2<double2><<<blocks, 256, smem, st>>>(static_cast<const double2 *>(vobs),
                                                     static_cast<const double2 *>(model), weight, nvis, npol, a1, a2, g,
                                                     nant, chi2, static_cast<double2 *>(grad_model),
                                                     static_cast<double2 *>(grad_gains));
  else if (precision == ARLGPU_FP32C)
    k_gain_chi2<float2><<<blocks, 256, smem, st>>>(static_cast<const float2 *>(vobs), static_cast<const float2 *>(model),
                                                    weight, nvis, npol, a1, a2, g, nant, chi2,
                                                    static_cast<float2 *>(grad_model),
                                                    static_cast<double2 *>(grad_gains));
  else
    return fail(ARLGPU_ERR_INVALID, "bad precision");
  ARL_LAUNCH_CHECK();
  count_launch(1);
  return ARLGPU_OK;
}
