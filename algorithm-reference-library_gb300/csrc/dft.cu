// Direct Fourier transform of point components, and its adjoint.
//
// Reference behaviour:
//   predict_skycomponent_visibility   processing_components/imaging/base.py:192-244
//   simulate_point                    processing_library/util/coordinate_support.py:192-212
//
// vis[r, p] += sum_k flux[k, chan[r], p] exp(-2 pi i (u l_k + v m_k + w n_k)),
// n_k = sqrt(1 - l_k^2 - m_k^2) - 1 supplied by the caller.  The phase in
// turns is formed in FP64 (|u l| reaches 1e4 turns on long baselines) and
// reduced to [-1/2, 1/2] before the sine and cosine: FP64 sincospi on the
// FP64 path, FP32 sincospif on the FP32C path (phase error below 1e-7 rad).
//
// The adjoint, image[k, p] += Re sum_r conj(exp(...)) x[r, p] (for rows of
// one channel map), gives the gradient of a DFT-predicted chi^2 with respect
// to the component fluxes; the gradient checks use it as a dense reference.
#include "common.cuh"

namespace arlgpu {

void count_launch(unsigned n);

constexpr int kTile = 128;  // components staged per shared-memory tile

template <typename R> struct Phasor;
template <> struct Phasor<float> {
  __device__ static __forceinline__ void at(double turns, float *c, float *s) {
    const float t = (float)(turns - rint(turns));
    sincospif(-2.f * t, s, c);
  }
};
template <> struct Phasor<double> {
  __device__ static __forceinline__ void at(double turns, double *c, double *s) {
    sincospi(-2.0 * (turns - rint(turns)), s, c);
  }
};

template <typename R, int NPOL>
__global__ void __launch_bounds__(256)
k_dft_predict(const double *__restrict__ uvw, const int32_t *__restrict__ chan, int64_t nvis,
              const double *__restrict__ lmn, const double *__restrict__ flux, int ncomp, int nchan,
              typename Cplx<R>::T *__restrict__ vis) {
  __shared__ double s_lmn[kTile][3];
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = r < nvis;
  double u = 0, v = 0, w = 0;
  int c = 0;
  if (live) {
    u = uvw[3 * r];
    v = uvw[3 * r + 1];
    w = uvw[3 * r + 2];
    c = chan ? chan[r] : 0;
  }
  R ar[NPOL], ai[NPOL];
#pragma unroll
  for (int p = 0; p < NPOL; ++p) ar[p] = ai[p] = 0;
  for (int k0 = 0; k0 < ncomp; k0 += kTile) {
    const int nk = min(kTile, ncomp - k0);
    __syncthreads();
    for (int i = threadIdx.x; i < nk * 3; i += blockDim.x) s_lmn[i / 3][i % 3] = lmn[3 * k0 + i];
    __syncthreads();
    if (!live) continue;
    for (int k = 0; k < nk; ++k) {
      const double turns = fma(u, s_lmn[k][0], fma(v, s_lmn[k][1], w * s_lmn[k][2]));
      R cs, sn;
      Phasor<R>::at(turns, &cs, &sn);
      const double *fk = flux + ((int64_t)(k0 + k) * nchan + c) * NPOL;
#pragma unroll
      for (int p = 0; p < NPOL; ++p) {
        const R f = (R)fk[p];
        ar[p] += f * cs;
        ai[p] += f * sn;
      }
    }
  }
  if (!live) return;
#pragma unroll
  for (int p = 0; p < NPOL; ++p) {
    typename Cplx<R>::T o = vis[r * NPOL + p];
    o.x += ar[p];
    o.y += ai[p];
    vis[r * NPOL + p] = o;
  }
}

// image[k, p] += Re sum_r conj(phasor_rk) x[r, p]: one warp per component,
// lanes over rows, shuffle reduction.
template <typename R, int NPOL>
__global__ void __launch_bounds__(256)
k_dft_adjoint(const double *__restrict__ uvw, int64_t nvis, const double *__restrict__ lmn, int ncomp,
              const typename Cplx<R>::T *__restrict__ x, double *__restrict__ image) {
  const int lane = threadIdx.x & 31;
  const int64_t k = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (k >= ncomp) return;
  const double l = lmn[3 * k], m = lmn[3 * k + 1], n = lmn[3 * k + 2];
  double acc[NPOL];
#pragma unroll
  for (int p = 0; p < NPOL; ++p) acc[p] = 0.0;
  for (int64_t r = lane; r < nvis; r += 32) {
    const double turns = fma(uvw[3 * r], l, fma(uvw[3 * r + 1], m, uvw[3 * r + 2] * n));
    R cs, sn;
    Phasor<R>::at(turns, &cs, &sn);
#pragma unroll
    for (int p = 0; p < NPOL; ++p) {
      const typename Cplx<R>::T xv = x[r * NPOL + p];
      acc[p] += (double)(cs * xv.x + sn * xv.y);  // Re(conj(c + i s) x)
    }
  }
#pragma unroll
  for (int p = 0; p < NPOL; ++p) {
    double s = acc[p];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) image[k * NPOL + p] += s;
  }
}

template <typename R>
static int launch_predict(const double *uvw, const int32_t *chan, int64_t nvis, const double *lmn,
                          const double *flux, int ncomp, int nchan, int npol, void *vis, cudaStream_t st) {
  const int blocks = (int)((nvis + 255) / 256);
  using CT = typename Cplx<R>::T;
  CT *o = static_cast<CT *>(vis);
  switch (npol) {
    case 1: k_dft_predict<R, 1><<<blocks, 256, 0, st>>>(uvw, chan, nvis, lmn, flux, ncomp, nchan, o); break;
    case 2: k_dft_predict<R, 2><<<blocks, 256, 0, st>>>(uvw, chan, nvis, lmn, flux, ncomp, nchan, o); break;
    case 4: k_dft_predict<R, 4><<<blocks, 256, 0, st>>>(uvw, chan, nvis, lmn, flux, ncomp, nchan, o); break;
    default: return fail(ARLGPU_ERR_UNSUPPORTED, "npol must be 1, 2 or 4");
  }
  ARL_LAUNCH_CHECK();
  count_launch(1);
  return ARLGPU_OK;
}

template <typename R>
static int launch_adjoint(const double *uvw, int64_t nvis, const double *lmn, int ncomp, int npol, const void *x,
                          double *image, cudaStream_t st) {
  const int64_t threads = (int64_t)ncomp * 32;
  const int blocks = (int)((threads + 255) / 256);
  using CT = typename Cplx<R>::T;
  const CT *xi = static_cast<const CT *>(x);
  switch (npol) {
    case 1: k_dft_adjoint<R, 1><<<blocks, 256, 0, st>>>(uvw, nvis, lmn, ncomp, xi, image); break;
    case 2: k_dft_adjoint<R, 2><<<blocks, 256, 0, st>>>(uvw, nvis, lmn, ncomp, xi, image); break;
    case 4: k_dft_adjoint<R, 4><<<blocks, 256, 0, st>>>(uvw, nvis, lmn, ncomp, xi, image); break;
    default: return fail(ARLGPU_ERR_UNSUPPORTED, "npol must be 1, 2 or 4");
  }
  ARL_LAUNCH_CHECK();
  count_launch(1);
  return ARLGPU_OK;
}

}  // namespace arlgpu

using namespace arlgpu;

extern "C" int arlgpu_dft_predict(const double *uvw, const int32_t *row_chan, int64_t nvis, const double *lmn,
                                  const double *flux, int32_t ncomp, int32_t nchan, int32_t npol, int precision,
                                  void *vis, void *stream) {
  if (precision != ARLGPU_FP32C && precision != ARLGPU_FP64) return fail(ARLGPU_ERR_INVALID, "bad precision");
  if (nvis < 0 || ncomp < 0 || nchan < 1) return fail(ARLGPU_ERR_INVALID, "bad sizes");
  if (nvis == 0 || ncomp == 0) return ARLGPU_OK;
  if (!uvw || !lmn || !flux || !vis) return fail(ARLGPU_ERR_INVALID, "null array argument");
  if (nchan > 1 && !row_chan) return fail(ARLGPU_ERR_INVALID, "row_chan is required when nchan > 1");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (precision == ARLGPU_FP64) return launch_predict<double>(uvw, row_chan, nvis, lmn, flux, ncomp, nchan, npol, vis, st);
  return launch_predict<float>(uvw, row_chan, nvis, lmn, flux, ncomp, nchan, npol, vis, st);
}

extern "C" int arlgpu_dft_adjoint(const double *uvw, int64_t nvis, const double *lmn, int32_t ncomp, int32_t npol,
                                  int precision, const void *x, double *image, void *stream) {
  if (precision != ARLGPU_FP32C && precision != ARLGPU_FP64) return fail(ARLGPU_ERR_INVALID, "bad precision");
  if (nvis < 0 || ncomp < 0) return fail(ARLGPU_ERR_INVALID, "bad sizes");
  if (nvis == 0 || ncomp == 0) return ARLGPU_OK;
  if (!uvw || !lmn || !x || !image) return fail(ARLGPU_ERR_INVALID, "null array argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (precision == ARLGPU_FP64) return launch_adjoint<double>(uvw, nvis, lmn, ncomp, npol, x, image, st);
  return launch_adjoint<float>(uvw, nvis, lmn, ncomp, npol, x, image, st);
}
