// FFT stages of invert_2d / predict_2d (K5 + K6).
//
// Reference behaviour:
//   fft / ifft                 processing_library/fourier_transforms/fft_support.py:21-89
//   fft_griddata_to_image      processing_components/griddata/gridding.py:270-289
//   fft_image_to_griddata      processing_components/griddata/gridding.py:292-302
//   normalize_sumwt            processing_components/imaging/base.py:84-101
//
// The centred transform fftshift(F(ifftshift(a))) for even N equals
// s * chk * F(chk * a) with chk[y, x] = (-1)^(x + y) and s = (-1)^(nx/2 + ny/2),
// and also F(z) with z[y, x] = chk(y, x) a[y + ny/2, x + nx/2] (indices mod N),
// so the shifts cost nothing: the sign flips are fused into the passes that
// also sum the w-planes, apply the grid correction and the sumwt
// normalisation (the forward direction needs no pass after the transform).
// The transforms are cuFFT (batched over chan, pol) or, for the FP32C
// inverse, the double-single transform of dsfft.cu.
#include <cufft.h>

#include <map>
#include <mutex>
#include <tuple>

#include "common.cuh"

namespace arlgpu {

void count_launch(unsigned n);
bool tune_dsfft();
bool dsfft_supported(int ny, int nx);
int dsfft_g2i_2d(const float2 *grid, int nb, int nw, int ny, int nx, const double *gcf, const double *sumwt,
                 double *im_re, double *im_im, void *buf, cudaStream_t st);

static int cufft_fail(cufftResult r, const char *what) {
  return fail(ARLGPU_ERR_CUFFT, "%s failed with cufftResult %d", what, (int)r);
}

// Plan cache keyed on (ny, nx, batch, batch distance, type, device).
struct PlanKey {
  int ny, nx, batch;
  long long dist;
  int type, dev;
  bool operator<(const PlanKey &o) const {
    return std::tie(ny, nx, batch, dist, type, dev) < std::tie(o.ny, o.nx, o.batch, o.dist, o.type, o.dev);
  }
};
static std::mutex g_plan_mu;
static std::map<PlanKey, cufftHandle> g_plans;

int get_plan(int ny, int nx, int batch, long long dist, cufftType type, cufftHandle *out) {
  int dev = 0;
  ARL_CUDA(cudaGetDevice(&dev));
  PlanKey k{ny, nx, batch, dist, (int)type, dev};
  std::lock_guard<std::mutex> lk(g_plan_mu);
  auto it = g_plans.find(k);
  if (it != g_plans.end()) {
    *out = it->second;
    return ARLGPU_OK;
  }
  cufftHandle h;
  int n[2] = {ny, nx};
  cufftResult r = cufftPlanMany(&h, 2, n, nullptr, 1, (long long)dist, nullptr, 1, (long long)dist, type, batch);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftPlanMany");
  g_plans[k] = h;
  *out = h;
  return ARLGPU_OK;
}

__device__ __forceinline__ float chk_sign(int y, int x) { return ((x + y) & 1) ? -1.f : 1.f; }

template <typename CT> __device__ __forceinline__ CT cmk(double a, double b);
template <> __device__ __forceinline__ float2 cmk<float2>(double a, double b) { return make_float2((float)a, (float)b); }
template <> __device__ __forceinline__ double2 cmk<double2>(double a, double b) { return make_double2(a, b); }

// buf[b, y, x] = chk * sum_z grid[b, z, y, x], summed and stored in FP64
template <typename CT>
__global__ void k_pre_g2i(const CT *__restrict__ grid, int nb, int nw, int ny, int nx, double2 *__restrict__ buf) {
  const int64_t plane = (int64_t)ny * nx;
  const int64_t total = (int64_t)nb * plane;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / plane, yx = i - b * plane;
    const int y = (int)(yx / nx), x = (int)(yx - (int64_t)y * nx);
    const CT *src = grid + b * nw * plane + yx;
    double sx = src[0].x, sy = src[0].y;
    for (int z = 1; z < nw; ++z) {
      sx += (double)src[z * plane].x;
      sy += (double)src[z * plane].y;
    }
    const double sg = chk_sign(y, x);
    buf[i] = make_double2(sx * sg, sy * sg);
  }
}

// image = part(buf * chk * s) * gcf  [/ sumwt]
__global__ void k_post_g2i(const double2 *__restrict__ buf, int nb, int ny, int nx, float s, const double *__restrict__ gcf,
                           const double *__restrict__ sumwt, double *__restrict__ im_re, double *__restrict__ im_im) {
  const int64_t plane = (int64_t)ny * nx;
  const int64_t total = (int64_t)nb * plane;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / plane, yx = i - b * plane;
    const int y = (int)(yx / nx), x = (int)(yx - (int64_t)y * nx);
    const double sg = (double)(chk_sign(y, x) * s);
    const double g = gcf[i];
    double re = buf[i].x * sg * g;
    double im = buf[i].y * sg * g;
    if (sumwt) {
      const double w = sumwt[b];
      if (w > 0.0) {
        re = re / w;
        im = im / w;
      } else {
        re = 0.0;
        im = 0.0;
      }
    }
    im_re[i] = re;
    if (im_im) im_im[i] = im;
  }
}

// grid plane 0 of each (chan, pol), ready for a plain forward transform: the
// centred transform of an even-sized a equals F(z) with
// z[y, x] = chk(y, x) a[(y + ny/2) mod ny, (x + nx/2) mod nx], a = image * gcf.
template <typename CT>
__global__ void k_pre_i2g(const double *__restrict__ image, const double *__restrict__ gcf, int nb, int nw, int ny,
                          int nx, CT *__restrict__ grid) {
  const int64_t plane = (int64_t)ny * nx;
  const int64_t total = (int64_t)nb * plane;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / plane, yx = i - b * plane;
    const int y = (int)(yx / nx), x = (int)(yx - (int64_t)y * nx);
    const int ys = y + ny / 2 - (y >= ny - ny / 2 ? ny : 0), xs = x + nx / 2 - (x >= nx - nx / 2 ? nx : 0);
    const int64_t src = b * plane + (int64_t)ys * nx + xs;
    grid[b * nw * plane + yx] = cmk<CT>(image[src] * gcf[src] * (double)chk_sign(y, x), 0.0);
  }
}

// grid[b, z] = grid[b, 0] for z = 1 .. nw - 1 (every w-plane holds the same
// transform, as ARL's fft_image_to_griddata writes it)
template <typename CT>
__global__ void k_post_i2g(CT *__restrict__ grid, int nb, int nw, int ny, int nx) {
  const int64_t plane = (int64_t)ny * nx;
  const int64_t total = (int64_t)nb * plane;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / plane, yx = i - b * plane;
    CT *p = grid + b * nw * plane + yx;
    const CT v = p[0];
    for (int z = 1; z < nw; ++z) p[z * plane] = v;
  }
}

static int grid_blocks(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)(b < 152 * 32 ? (b < 1 ? 1 : b) : 152 * 32);
}

template <typename CT>
static int exec_c2c(cufftHandle h, CT *data, int dir);
template <>
int exec_c2c<float2>(cufftHandle h, float2 *data, int dir) {
  cufftResult r = cufftExecC2C(h, reinterpret_cast<cufftComplex *>(data), reinterpret_cast<cufftComplex *>(data), dir);
  return r == CUFFT_SUCCESS ? ARLGPU_OK : cufft_fail(r, "cufftExecC2C");
}
template <>
int exec_c2c<double2>(cufftHandle h, double2 *data, int dir) {
  cufftResult r =
      cufftExecZ2Z(h, reinterpret_cast<cufftDoubleComplex *>(data), reinterpret_cast<cufftDoubleComplex *>(data), dir);
  return r == CUFFT_SUCCESS ? ARLGPU_OK : cufft_fail(r, "cufftExecZ2Z");
}

// The inverse transform is never FP32: the grid correction multiplies the
// transform's rounding error by up to max(gcf) / min(gcf) (~6e4 at the edge
// of a PSWF-corrected image), so an FP32 transform would leave ~1e-3 relative
// errors in the image whatever the gridder's accuracy.  FP64 path: cuFFT Z2Z.
// FP32C path: the double-single transform (dsfft.cu) for power-of-two sizes
// 64..8192, else cuFFT Z2Z.
template <typename CT>
static int g2i(const CT *grid, const arlgpu_grid_desc *gd, const double *gcf, const double *sumwt, double *re,
               double *im, double2 *buf, cudaStream_t st) {
  const int nb = gd->nchan * gd->npol, ny = gd->ny, nx = gd->nx;
  if (sizeof(CT) == 8 && tune_dsfft() && dsfft_supported(ny, nx))
    return dsfft_g2i_2d(reinterpret_cast<const float2 *>(grid), nb, gd->nw, ny, nx, gcf, sumwt, re, im, buf, st);
  const int64_t total = (int64_t)nb * ny * nx;
  cufftHandle h;
  ARL_TRY(get_plan(ny, nx, nb, (long long)ny * nx, CUFFT_Z2Z, &h));
  k_pre_g2i<CT><<<grid_blocks(total), 256, 0, st>>>(grid, nb, gd->nw, ny, nx, buf);
  count_launch(1);
  ARL_LAUNCH_CHECK();
  cufftResult r = cufftSetStream(h, st);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftSetStream");
  ARL_TRY(exec_c2c<double2>(h, buf, CUFFT_INVERSE));
  const float s = (((nx / 2) + (ny / 2)) & 1) ? -1.f : 1.f;
  k_post_g2i<<<grid_blocks(total), 256, 0, st>>>(buf, nb, ny, nx, s, gcf, sumwt, re, im);
  count_launch(1);
  ARL_LAUNCH_CHECK();
  return ARLGPU_OK;
}

template <typename CT>
static int i2g(const double *image, const double *gcf, const arlgpu_grid_desc *gd, CT *grid, cudaStream_t st) {
  const int nb = gd->nchan * gd->npol, nw = gd->nw, ny = gd->ny, nx = gd->nx;
  const int64_t total = (int64_t)nb * ny * nx;
  cufftHandle h;
  ARL_TRY(get_plan(ny, nx, nb, (long long)nw * ny * nx, sizeof(CT) == 8 ? CUFFT_C2C : CUFFT_Z2Z, &h));
  k_pre_i2g<CT><<<grid_blocks(total), 256, 0, st>>>(image, gcf, nb, nw, ny, nx, grid);
  count_launch(1);
  ARL_LAUNCH_CHECK();
  cufftResult r = cufftSetStream(h, st);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftSetStream");
  ARL_TRY(exec_c2c<CT>(h, grid, CUFFT_FORWARD));
  if (nw > 1) {
    k_post_i2g<CT><<<grid_blocks(total), 256, 0, st>>>(grid, nb, nw, ny, nx);
    count_launch(1);
    ARL_LAUNCH_CHECK();
  }
  return ARLGPU_OK;
}

static int check_fft_desc(const arlgpu_grid_desc *gd, int precision) {
  if (!gd) return fail(ARLGPU_ERR_INVALID, "null grid descriptor");
  if (precision != ARLGPU_FP32C && precision != ARLGPU_FP64) return fail(ARLGPU_ERR_INVALID, "bad precision");
  if (gd->nchan < 1 || gd->npol < 1 || gd->nw < 1 || gd->ny < 2 || gd->nx < 2)
    return fail(ARLGPU_ERR_INVALID, "bad grid shape");
  if ((gd->ny & 1) || (gd->nx & 1)) return fail(ARLGPU_ERR_UNSUPPORTED, "odd image sizes are not supported");
  return ARLGPU_OK;
}

}  // namespace arlgpu

using namespace arlgpu;

extern "C" int arlgpu_fft_grid_to_image(const void *grid, const arlgpu_grid_desc *gd, int precision,
                                        const double *gcf, const double *sumwt, double *image_real,
                                        double *image_imag, void *fftbuf, void *stream) {
  ARL_TRY(check_fft_desc(gd, precision));
  if (!grid || !gcf || !image_real || !fftbuf) return fail(ARLGPU_ERR_INVALID, "null array argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (precision == ARLGPU_FP64)
    return g2i<double2>(static_cast<const double2 *>(grid), gd, gcf, sumwt, image_real, image_imag,
                        static_cast<double2 *>(fftbuf), st);
  return g2i<float2>(static_cast<const float2 *>(grid), gd, gcf, sumwt, image_real, image_imag,
                     static_cast<double2 *>(fftbuf), st);
}

extern "C" int arlgpu_fft_image_to_grid(const double *image, const double *gcf, const arlgpu_grid_desc *gd,
                                        int precision, void *grid, void *stream) {
  ARL_TRY(check_fft_desc(gd, precision));
  if (!grid || !gcf || !image) return fail(ARLGPU_ERR_INVALID, "null array argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (precision == ARLGPU_FP64) return i2g<double2>(image, gcf, gd, static_cast<double2 *>(grid), st);
  return i2g<float2>(image, gcf, gd, static_cast<float2 *>(grid), st);
}
