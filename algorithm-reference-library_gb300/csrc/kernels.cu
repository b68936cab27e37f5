// One-time FP64 kernel generation on the GPU (K7 / K8).
//
// Reference behaviour:
//   grdsf                               processing_library/fourier_transforms/convolutional_gridding.py:72-117
//   w_beam                              convolutional_gridding.py:120-188
//   create_pswf_convolutionfunction     processing_components/griddata/kernels.py:52-97
//   create_awterm_convolutionfunction   processing_components/griddata/kernels.py:100-200
//                                       (use_aaf=True, no primary beam)
//   create_w_term_like / pad_image / fft_image
//                                       processing_library/image/operations.py:269-408
#include <cufft.h>

#include <vector>

#include "common.cuh"

namespace arlgpu {

void count_launch(unsigned n);

int get_plan(int ny, int nx, int batch, long long dist, cufftType type, cufftHandle *out);

// Schwab's rational approximation of the m=6, alpha=1 prolate spheroidal
// function (Indirect Imaging, 1984): P/Q on [0, 0.75) and [0.75, 1].
__constant__ double c_sph_p[2][5] = {{8.203343e-2, -3.644705e-1, 6.278660e-1, -5.335581e-1, 2.312756e-1},
                                     {4.028559e-3, -3.697768e-2, 1.021332e-1, -1.201436e-1, 6.412774e-2}};
__constant__ double c_sph_q[2][3] = {{1.0000000e0, 8.212018e-1, 2.078043e-1}, {1.0000000e0, 9.599102e-1, 2.918724e-1}};

// Returns grdsf(nu); *taper = (1 - nu^2) grdsf(nu).
__device__ double grdsf(double nu, double *taper) {
  nu = fabs(nu);
  const int part = nu >= 0.75 ? 1 : 0;
  const double nuend = part ? 1.0 : 0.75;
  const double d = nu * nu - nuend * nuend;
  double top = c_sph_p[part][0], bot = c_sph_q[part][0];
  double dk = d;
  for (int k = 1; k < 5; ++k) {
    top += c_sph_p[part][k] * dk;
    if (k < 3) bot += c_sph_q[part][k] * dk;
    dk *= d;
  }
  double g = bot > 0.0 ? top / bot : 0.0;
  if (nu > 1.0) g = 0.0;
  if (taper) *taper = (1.0 - nu * nu) * g;
  return g;
}

// 1-D PSWF kernel table k[s][g] (unnormalised), O x S.
__global__ void k_pswf1d(int O, int S, double *k) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < O * S; t += gridDim.x * blockDim.x) {
    const int s = t / S, g = t - s * S;
    const double nu = ((double)(g - S / 2) - (double)(s - O / 2) / (double)O) / (double)(S / 2);
    double taper;
    grdsf(nu, &taper);
    k[t] = taper;
  }
}

// Normalise k by the sum of its centre row, then the outer-product norm
// sum_ij k[0][j] k[0][i]; both sums in a fixed order (one thread).
__global__ void k_pswf_norm(int O, int S, double *k, double *norm2) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int g = 0; g < S; ++g) s += k[(O / 2) * S + g];
  for (int t = 0; t < O * S; ++t) k[t] /= s;
  double n2 = 0.0;
  for (int j = 0; j < S; ++j)
    for (int i = 0; i < S; ++i) n2 += k[j] * k[i];
  *norm2 = n2;
}

// cf[y][x][j][i] = k[y][j] k[x][i] / norm2 (complex128, imaginary zero)
__global__ void k_pswf_outer(int O, int S, const double *k, const double *norm2, double2 *cf) {
  const int64_t n = (int64_t)O * O * S * S;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % S), j = (int)((t / S) % S), x = (int)((t / S / S) % O), y = (int)(t / S / S / O);
    cf[t] = make_double2(k[y * S + j] * k[x * S + i] / *norm2, 0.0);
  }
}

// g1[x] = grdsf(|2 (x - n/2) / n|)
__global__ void k_gcf1d(int n, double *g1) {
  for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < n; x += gridDim.x * blockDim.x)
    g1[x] = grdsf(fabs(2.0 * ((double)(x - n / 2) / (double)n)), nullptr);
}

__global__ void k_max1(int n, const double *g1, double *mx) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double m = 0.0;
  for (int x = 0; x < n; ++x) m = fmax(m, g1[x]);
  *mx = m * m;
}

// gcf[y][x] = max / (g1[y] g1[x]) where positive (ARL keeps non-positive values)
__global__ void k_gcf2d(int n, const double *g1, const double *mx, double *gcf) {
  const int64_t tot = (int64_t)n * n;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (int64_t)gridDim.x * blockDim.x) {
    const double v = g1[t / n] * g1[t % n];
    gcf[t] = v > 0.0 ? *mx / v : v;
  }
}

// Padded w-screen planes for a batch of w values, multiplied by norm = 1/gcf
// (qnx x qnx, centred in nx x nx), and pre-multiplied by the checkerboard so
// that an inverse cuFFT yields the centred ifft.
__global__ void k_wscreen(int nb, int z0, int nw, double wstep, int qnx, int nx, double fov, const double *norm,
                          double2 *pad) {
  const int64_t plane = (int64_t)nx * nx;
  const int64_t tot = (int64_t)nb * plane;
  const int off = nx / 2 - qnx / 2;
  const double c = (double)(qnx / 2);
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(t / plane);
    const int64_t yx = t - (int64_t)b * plane;
    const int y = (int)(yx / nx), x = (int)(yx - (int64_t)y * nx);
    const int qy = y - off, qx = x - off;
    double2 val = make_double2(0.0, 0.0);
    if (qy >= 0 && qy < qnx && qx >= 0 && qx < qnx) {
      // w = pix2world0(z) on the cf WW axis: ((z + 1) - (nw//2 + 1)) * wstep
      const double w = ((double)(z0 + b) + 1.0 - (double)(nw / 2 + 1)) * wstep;
      const double ly = ((double)qy - c) / (double)qnx, mx = ((double)qx - c) / (double)qnx;
      const double r2 = fov * fov * (ly * ly + mx * mx);
      if (r2 == 0.0) {
        val = make_double2(1.0, 0.0);
      } else if (r2 < 1.0) {
        const double ph = -2.0 * M_PI * w * (1.0 - sqrt(1.0 - r2));
        double s, co;
        sincos(ph, &s, &co);
        val = make_double2(co, s);
      }
      if (norm) {  // the anti-aliasing function's inverse (use_aaf)
        const double nv = norm[qy * qnx + qx];
        val.x *= nv;
        val.y *= nv;
      }
    }
    const double sg = ((x + y) & 1) ? -1.0 : 1.0;
    pad[t] = make_double2(val.x * sg, val.y * sg);
  }
}

// Strided decimation of the transformed planes into cf[z][y][x][j][i]
//   cf = pad[ybeg - j O, xbeg - i O] * chk * s / nx^2,
//   ybeg = y + nx/2 + (S O)/2 - O/2  (kernels.py:176-186).
__global__ void k_decimate(int nb, int z0, int O, int S, int nx, double2 *pad, double2 *cf) {
  const int64_t per = (int64_t)O * O * S * S;
  const int64_t tot = (int64_t)nb * per;
  const double s = (((nx / 2) + (nx / 2)) & 1) ? -1.0 : 1.0;
  const double scale = 1.0 / ((double)nx * (double)nx);
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(t / per);
    int64_t r = t - (int64_t)b * per;
    const int i = (int)(r % S), j = (int)((r / S) % S), x = (int)((r / S / S) % O), y = (int)(r / S / S / O);
    const int cen = nx / 2;
    const int yy = y + cen + (S * O) / 2 - O / 2 - j * O;
    const int xx = x + cen + (S * O) / 2 - O / 2 - i * O;
    double2 v = pad[(int64_t)b * nx * nx + (int64_t)yy * nx + xx];
    const double sg = (((xx + yy) & 1) ? -1.0 : 1.0) * s * scale;
    cf[(int64_t)(z0 + b) * per + r] = make_double2(v.x * sg, v.y * sg);
  }
}

// Sum of the real part of the centre plane's centre sub-kernel (one thread).
__global__ void k_wnorm(int nw, int O, int S, const double2 *cf, double *norm) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int64_t per = (int64_t)O * O * S * S;
  const double2 *p = cf + (int64_t)(nw / 2) * per + ((int64_t)(O / 2) * O + O / 2) * S * S;
  double s = 0.0;
  for (int t = 0; t < S * S; ++t) s += p[t].x;
  *norm = s;
}

// cf = conj(cf / norm)
__global__ void k_wfinal(int64_t n, const double *norm, double2 *cf) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    double2 v = cf[t];
    cf[t] = make_double2(v.x / *norm, -(v.y / *norm));
  }
}

// x = 1 / x  (kernels.py:155, norm = 1.0 / this_pswf_gcf.data)
__global__ void k_recip(int64_t n, double *x) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    x[t] = 1.0 / x[t];
}

static int nblk(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)(b < 1 ? 1 : (b > 152 * 32 ? 152 * 32 : b));
}

int make_gcf(int n, double *gcf, double *scratch /* n + 1 doubles */, cudaStream_t st) {
  k_gcf1d<<<nblk(n), 256, 0, st>>>(n, scratch);
  count_launch(1);
  ARL_LAUNCH_CHECK();
  k_max1<<<1, 32, 0, st>>>(n, scratch, scratch + n);
  count_launch(1);
  ARL_LAUNCH_CHECK();
  k_gcf2d<<<nblk((int64_t)n * n), 256, 0, st>>>(n, scratch, scratch + n, gcf);
  count_launch(1);
  ARL_LAUNCH_CHECK();
  return ARLGPU_OK;
}

}  // namespace arlgpu

using namespace arlgpu;

extern "C" int arlgpu_make_pswf(int32_t oversampling, int32_t support, int32_t ny, int32_t nx, void *cf_out,
                                double *gcf_out, void *stream) {
  if (oversampling < 1 || support < 2 || (support & 1)) return fail(ARLGPU_ERR_INVALID, "bad oversampling/support");
  if (gcf_out && (ny != nx || nx < 2)) return fail(ARLGPU_ERR_UNSUPPORTED, "ARL's gcf needs a square image");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double *tmp = nullptr;
  const size_t n1 = (size_t)oversampling * support + 1 + (size_t)nx + 1;
  ARL_CUDA(cudaMallocAsync(&tmp, n1 * sizeof(double), st));
  double *k = tmp, *norm2 = tmp + (size_t)oversampling * support, *g1 = norm2 + 1;
  int rc = ARLGPU_OK;
  if (cf_out) {
    k_pswf1d<<<nblk((int64_t)oversampling * support), 256, 0, st>>>(oversampling, support, k);
  count_launch(1);
    k_pswf_norm<<<1, 32, 0, st>>>(oversampling, support, k, norm2);
  count_launch(1);
    k_pswf_outer<<<nblk((int64_t)oversampling * oversampling * support * support), 256, 0, st>>>(
        oversampling, support, k, norm2, static_cast<double2 *>(cf_out));
  count_launch(1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = cuda_fail(e, "pswf kernels", __FILE__, __LINE__);
  }
  if (rc == ARLGPU_OK && gcf_out) rc = make_gcf(nx, gcf_out, g1, st);
  cudaError_t e = cudaFreeAsync(tmp, st);
  if (rc == ARLGPU_OK && e != cudaSuccess) rc = cuda_fail(e, "cudaFreeAsync", __FILE__, __LINE__);
  return rc;
}

extern "C" int arlgpu_make_wkernels(int32_t nw, double wstep, int32_t oversampling, int32_t support,
                                    int32_t maxsupport, int32_t image_nx, double cdelt_ra_deg, int32_t use_aaf,
                                    void *cf_out, void *stream) {
  if (nw < 1 || oversampling < 1 || support < 2 || (support & 1) || image_nx < 2 || !cf_out)
    return fail(ARLGPU_ERR_INVALID, "bad w-kernel arguments");
  const int nx = maxsupport > 2 * oversampling * support ? maxsupport : 2 * oversampling * support;
  if (nx % oversampling) return fail(ARLGPU_ERR_UNSUPPORTED, "padded size not a multiple of oversampling");
  const int qnx = nx / oversampling;
  if ((nx & 1) || (qnx & 1)) return fail(ARLGPU_ERR_UNSUPPORTED, "odd padded sizes are not supported");
  const double d2r = M_PI / 180.0;
  const double ccell = image_nx * fabs(d2r * cdelt_ra_deg) / qnx;
  const double sub_cell = fabs(-ccell / d2r) * M_PI / 180.0;
  const double fov = qnx * sub_cell;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // norm = 1 / gcf_pswf(qnx) with use_aaf, else 1 (kernels.py:153-156)
  const int batch = 8;
  double *norm = nullptr, *scratch = nullptr;
  double2 *pad = nullptr;
  ARL_CUDA(cudaMallocAsync(&norm, (size_t)qnx * qnx * sizeof(double), st));
  ARL_CUDA(cudaMallocAsync(&scratch, (size_t)(qnx + 2) * sizeof(double), st));
  ARL_CUDA(cudaMallocAsync(&pad, (size_t)batch * nx * nx * sizeof(double2), st));
  int rc = use_aaf ? make_gcf(qnx, norm, scratch, st) : ARLGPU_OK;
  if (rc == ARLGPU_OK && use_aaf) {
    k_recip<<<nblk((int64_t)qnx * qnx), 256, 0, st>>>((int64_t)qnx * qnx, norm);
  count_launch(1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = cuda_fail(e, "k_recip", __FILE__, __LINE__);
  }
  cufftHandle h;
  if (rc == ARLGPU_OK) rc = get_plan(nx, nx, batch, (long long)nx * nx, CUFFT_Z2Z, &h);
  if (rc == ARLGPU_OK) {
    cufftResult r = cufftSetStream(h, st);
    if (r != CUFFT_SUCCESS) rc = fail(ARLGPU_ERR_CUFFT, "cufftSetStream failed (%d)", (int)r);
  }
  for (int z0 = 0; rc == ARLGPU_OK && z0 < nw; z0 += batch) {
    const int nb = nw - z0 < batch ? nw - z0 : batch;
    k_wscreen<<<nblk((int64_t)batch * nx * nx), 256, 0, st>>>(batch, z0, nw, wstep, qnx, nx, fov,
                                                              use_aaf ? norm : nullptr, pad);
  count_launch(1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      rc = cuda_fail(e, "k_wscreen", __FILE__, __LINE__);
      break;
    }
    cufftResult r = cufftExecZ2Z(h, reinterpret_cast<cufftDoubleComplex *>(pad),
                                 reinterpret_cast<cufftDoubleComplex *>(pad), CUFFT_INVERSE);
    if (r != CUFFT_SUCCESS) {
      rc = fail(ARLGPU_ERR_CUFFT, "cufftExecZ2Z failed (%d)", (int)r);
      break;
    }
    k_decimate<<<nblk((int64_t)nb * oversampling * oversampling * support * support), 256, 0, st>>>(
        nb, z0, oversampling, support, nx, pad, static_cast<double2 *>(cf_out));
  count_launch(1);
    e = cudaGetLastError();
    if (e != cudaSuccess) rc = cuda_fail(e, "k_decimate", __FILE__, __LINE__);
  }
  if (rc == ARLGPU_OK) {
    k_wnorm<<<1, 32, 0, st>>>(nw, oversampling, support, static_cast<double2 *>(cf_out), scratch);
  count_launch(1);
    const int64_t n = (int64_t)nw * oversampling * oversampling * support * support;
    k_wfinal<<<nblk(n), 256, 0, st>>>(n, scratch, static_cast<double2 *>(cf_out));
  count_launch(1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = cuda_fail(e, "w-kernel normalisation", __FILE__, __LINE__);
  }
  cudaFreeAsync(pad, st);
  cudaFreeAsync(scratch, st);
  cudaFreeAsync(norm, st);
  return rc;
}
