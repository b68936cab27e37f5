// Batched w-stacking (K9): every w-slice gridded into its own plane of one
// [nchan][npol][K][ny][nx] grid by a single gridder launch, one batched cuFFT
// over all planes, and one pass that applies each slice's w-beam and sums the
// slices into the image.
//
// Reference behaviour:
//   vis_wslice_iter                       processing_components/visibility/iterators.py:91-109
//   invert_wstack_single / predict_wstack_single
//                                         processing_components/imaging/wstack_single.py:26-96
//   w_beam / create_w_term_like           processing_library/fourier_transforms/convolutional_gridding.py:120-188,
//                                         processing_library/image/operations.py:364-408
//   invert_list_serial_workflow (sum of sumwt-weighted slice images, normalisation)
//                                         workflows/serial/imaging/imaging_serial.py:186-197
//
// invert: slice s contributes sumwt_s * Re(wb_s * I_s) with I_s = ifft(grid_s) gcf N^2 / sumwt_s,
//         so the image is gcf * sum_s Re(wb_s * U_s) / sum_s sumwt_s, U_s the unnormalised
//         centred inverse transform of grid_s.
// predict: V = P(Re(wb) M) - i P(Im(wb) M) = P(conj(wb) M) by linearity, so plane s of the
//          grid is fft(conj(wb_s) M gcf) and one degrid over all rows reads plane s for the
//          rows of slice s.
#include <cufft.h>

#include <algorithm>

#include "common.cuh"
#include "dsmath.cuh"

namespace arlgpu {

void count_launch(unsigned n);
int get_plan(int ny, int nx, int batch, long long dist, cufftType type, cufftHandle *out);
bool tune_dsfft();
bool dsfft_supported(int ny, int nx);
int dsfft_g2i_wstack(const float2 *grid, int nb, int K, int ny, int nx, double fov, const double *wmean,
                     const double *gcf, const double *sumwt, double *image, void *buf, int64_t G, cudaStream_t st);

// w-screen of create_w_term_like at one pixel of an n x n image centred on
// (n/2, n/2): exp(-2 pi i w (1 - sqrt(1 - r^2))), zero for r^2 >= 1, one at
// r^2 == 0.  The pixel part, nterm = 1 - sqrt(1 - r^2), is computed once per
// pixel (FP64) and shared by all slices.
struct Pix {
  double nterm;
  int state;  // 0: r^2 == 0 (value 1), 1: inside, 2: r^2 >= 1 (value 0)
};
__device__ __forceinline__ Pix wpix(int y, int x, int n, double fov) {
  const double c = (double)(n / 2);
  const double ly = ((double)y - c) / (double)n, mx = ((double)x - c) / (double)n;
  const double r2 = fov * fov * (ly * ly + mx * mx);
  Pix p;
  p.state = r2 == 0.0 ? 0 : (r2 >= 1.0 ? 2 : 1);
  p.nterm = p.state == 1 ? 1.0 - sqrt(1.0 - r2) : 0.0;
  return p;
}

// FP64 path: exp(-2 pi i w nterm) with an FP64 sincos.
__device__ __forceinline__ double2 wb64(const Pix &p, double w) {
  if (p.state == 0) return make_double2(1.0, 0.0);
  if (p.state == 2) return make_double2(0.0, 0.0);
  double s, co;
  sincos(-2.0 * M_PI * w * p.nterm, &s, &co);
  return make_double2(co, s);
}

// FP32C path: the phase in turns t = w nterm is formed in FP64 and reduced to
// [-1/2, 1/2] before an FP32 sincospi, so the phase error stays at FP32
// rounding of the reduced argument (< 1e-7 rad) for any w.
__device__ __forceinline__ double2 wb32(const Pix &p, double w) {
  if (p.state == 0) return make_double2(1.0, 0.0);
  if (p.state == 2) return make_double2(0.0, 0.0);
  const double t = w * p.nterm;
  const float f = (float)(t - rint(t));
  float s, co;
  sincospif(-2.f * f, &s, &co);
  return make_double2(co, s);
}

template <typename CT> struct WB;
template <> struct WB<float2> {
  __device__ static __forceinline__ double2 at(const Pix &p, double w) { return wb32(p, w); }
};
template <> struct WB<double2> {
  __device__ static __forceinline__ double2 at(const Pix &p, double w) { return wb64(p, w); }
};

// pre-invert: every plane into the FP64 FFT buffer with the chk sign (the
// centred-transform trick)
template <typename CT>
__global__ void k_chk_planes(const CT *grid, int64_t nplanes, int ny, int nx, double2 *buf) {
  const int64_t plane = (int64_t)ny * nx, tot = nplanes * plane;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t yx = i % plane;
    const int y = (int)(yx / nx), x = (int)(yx - (int64_t)y * nx);
    const double sg = ((x + y) & 1) ? -1.0 : 1.0;
    buf[i] = make_double2(sg * (double)grid[i].x, sg * (double)grid[i].y);
  }
}

// image[b, y, x] (+)= gcf * sum_s Re(wb_s * U_s * chk * s0) / sumwt[b] over the
// slices of flattened planes [p0, p1) (plane index b * K + s); buf holds those
// planes' FP64 transforms.  The group holding slice 0 of image b writes it,
// later groups add to it.  U_s in FP64, the w-beam in the precision of the
// path (CT).
template <typename CT>
__global__ void k_wstack_combine(const double2 *__restrict__ buf, int64_t p0, int64_t p1, int K, int ny, int nx,
                                 float s0, double fov, const double *__restrict__ wmean,
                                 const double *__restrict__ gcf, const double *__restrict__ sumwt,
                                 double *__restrict__ image) {
  const int64_t plane = (int64_t)ny * nx;
  const int64_t b0 = p0 / K, b1 = (p1 - 1) / K;
  const int64_t tot = (b1 - b0 + 1) * plane;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = b0 + i / plane, yx = i % plane;
    const int y = (int)(yx / nx), x = (int)(yx - (int64_t)y * nx);
    const double sg = (((x + y) & 1) ? -1.0 : 1.0) * (double)s0;
    const Pix px = wpix(y, x, nx, fov);
    const int sa = (int)max((int64_t)0, p0 - b * K), sb = (int)min((int64_t)K, p1 - b * K);
    double acc = 0.0;
    for (int s = sa; s < sb; ++s) {
      const double2 u = buf[(b * K + s - p0) * plane + yx];
      const double2 wb = WB<CT>::at(px, wmean[s]);
      acc += wb.x * u.x - wb.y * u.y;
    }
    const int64_t o = b * plane + yx;
    const double w = sumwt[b];
    const double v = w > 0.0 ? acc * sg * gcf[o] / w : 0.0;
    image[o] = sa == 0 ? v : image[o] + v;
  }
}

// Plane s of image b, ready for a plain forward transform: the centred
// transform fftshift(F(ifftshift(a))) of an even-sized a equals F(z) with
// z[y, x] = chk(y, x) a[(y + ny/2) mod ny, (x + nx/2) mod nx], so
//   grid[b, s, y, x] = chk(y, x) conj(wb_s) image gcf   at the shifted pixel
// and no pass after the transform is needed.
// FP64 path: FP64 w-screen.  FP32C path: double-single w-screen (no FP64
// square root or per-slice FP64 phase), FP32 sincospi.
__global__ void k_wstack_pre_predict64(const double *__restrict__ image, const double *__restrict__ gcf, int nb, int K,
                                       int ny, int nx, double fov, const double *__restrict__ wmean,
                                       double2 *__restrict__ grid) {
  const int64_t plane = (int64_t)ny * nx, tot = (int64_t)nb * plane;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / plane, yx = i - b * plane;
    const int y = (int)(yx / nx), x = (int)(yx - (int64_t)y * nx);
    const int ys = y + ny / 2 - (y >= ny - ny / 2 ? ny : 0), xs = x + nx / 2 - (x >= nx - nx / 2 ? nx : 0);
    const int64_t src = b * plane + (int64_t)ys * nx + xs;
    const double m = image[src] * gcf[src] * (((x + y) & 1) ? -1.0 : 1.0);
    const Pix px = wpix(ys, xs, nx, fov);
    for (int s = 0; s < K; ++s) {
      const double2 wb = wb64(px, wmean[s]);
      grid[(b * K + s) * plane + yx] = make_double2(wb.x * m, -wb.y * m);
    }
  }
}

__global__ void k_wstack_pre_predict32(const double *__restrict__ image, const double *__restrict__ gcf, int nb, int K,
                                       int ny, int nx, double fov, const double *__restrict__ wmean,
                                       float2 *__restrict__ grid) {
  extern __shared__ dsf s_w[];
  for (int s = threadIdx.x; s < K; s += blockDim.x) s_w[s] = ds_from_double(wmean[s]);
  __syncthreads();
  const dsf c2 = ds_from_double(fov * fov / ((double)nx * nx));
  const int64_t plane = (int64_t)ny * nx, tot = (int64_t)nb * plane;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / plane, yx = i - b * plane;
    const int y = (int)(yx / nx), x = (int)(yx - (int64_t)y * nx);
    const int ys = y + ny / 2 - (y >= ny - ny / 2 ? ny : 0), xs = x + nx / 2 - (x >= nx - nx / 2 ? nx : 0);
    const int64_t src = b * plane + (int64_t)ys * nx + xs;
    const float m = (float)(image[src] * gcf[src]) * (((x + y) & 1) ? -1.f : 1.f);
    const DsPix px = ds_wpix(ys, xs, nx, c2);
    for (int s = 0; s < K; ++s) {
      const float2 wb = ds_wbeam(px, s_w[s]);
      grid[(b * K + s) * plane + yx] = make_float2(wb.x * m, -wb.y * m);
    }
  }
}

static int nblk(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)(b < 1 ? 1 : (b > 152 * 64 ? 152 * 64 : b));
}

template <typename CT>
static int exec(cufftHandle h, CT *d, int dir) {
  cufftResult r = sizeof(CT) == 8
                      ? cufftExecC2C(h, reinterpret_cast<cufftComplex *>(d), reinterpret_cast<cufftComplex *>(d), dir)
                      : cufftExecZ2Z(h, reinterpret_cast<cufftDoubleComplex *>(d),
                                     reinterpret_cast<cufftDoubleComplex *>(d), dir);
  return r == CUFFT_SUCCESS ? ARLGPU_OK : fail(ARLGPU_ERR_CUFFT, "cuFFT exec failed (%d)", (int)r);
}

// Planes per transform group: at most kGroupBytes of 16-byte cells (complex128
// or double-single complex), so the FFT scratch (fftbuf) and cuFFT's own work
// area stay bounded for large grids (an 8192^2 plane is 1 GiB).
constexpr int64_t kGroupBytes = (int64_t)4 << 30;

int64_t group_planes(int64_t nplanes, int ny, int nx) {
  int64_t g = kGroupBytes / ((int64_t)ny * nx * (int64_t)sizeof(double2));
  if (g < 1) g = 1;
  return g < nplanes ? g : nplanes;
}

// The inverse transforms run in FP64 for both precisions (the grid correction
// amplifies transform rounding by up to max(gcf) / min(gcf)).  Planes go
// through the FP64 buffer a group at a time; with precision FP64 and the grid
// passed as fftbuf, each group is transformed where it lies in the grid.
template <typename CT>
static int g2i(const CT *grid, const arlgpu_grid_desc *gd, const double *gcf, const double *wmean, double fov,
               const double *sumwt, double *image, double2 *fftbuf, cudaStream_t st) {
  const int nb = gd->nchan * gd->npol, K = gd->nw, ny = gd->ny, nx = gd->nx;
  const int64_t nplanes = (int64_t)nb * K, plane = (int64_t)ny * nx;
  if (nplanes > 0x7fffffff) return fail(ARLGPU_ERR_UNSUPPORTED, "too many planes");
  const bool inplace = (const void *)grid == (const void *)fftbuf;
  const int64_t G = group_planes(nplanes, ny, nx);
  if (sizeof(CT) == 8 && !inplace && tune_dsfft() && dsfft_supported(ny, nx))
    return dsfft_g2i_wstack(reinterpret_cast<const float2 *>(grid), nb, K, ny, nx, fov, wmean, gcf, sumwt, image,
                            fftbuf, G, st);
  const float s0 = (((nx / 2) + (ny / 2)) & 1) ? -1.f : 1.f;
  for (int64_t p0 = 0; p0 < nplanes; p0 += G) {
    const int64_t np = std::min(G, nplanes - p0);
    double2 *buf = inplace ? fftbuf + p0 * plane : fftbuf;
    cufftHandle h;
    ARL_TRY(get_plan(ny, nx, (int)np, (long long)plane, CUFFT_Z2Z, &h));
    k_chk_planes<CT><<<nblk(np * plane), 256, 0, st>>>(grid + p0 * plane, np, ny, nx, buf);
    ARL_LAUNCH_CHECK();
    count_launch(1);
    cufftResult r = cufftSetStream(h, st);
    if (r != CUFFT_SUCCESS) return fail(ARLGPU_ERR_CUFFT, "cufftSetStream failed (%d)", (int)r);
    ARL_TRY(exec<double2>(h, buf, CUFFT_INVERSE));
    const int64_t nbt = (p0 + np - 1) / K - p0 / K + 1;
    k_wstack_combine<CT><<<nblk(nbt * plane), 256, 0, st>>>(buf, p0, p0 + np, K, ny, nx, s0, fov, wmean, gcf,
                                                             sumwt, image);
    ARL_LAUNCH_CHECK();
    count_launch(1);
  }
  return ARLGPU_OK;
}

template <typename CT>
static int i2g(const double *image, const double *gcf, const double *wmean, double fov, const arlgpu_grid_desc *gd,
               CT *grid, cudaStream_t st) {
  const int nb = gd->nchan * gd->npol, K = gd->nw, ny = gd->ny, nx = gd->nx;
  const int64_t nplanes = (int64_t)nb * K, plane = (int64_t)ny * nx;
  if (nplanes > 0x7fffffff) return fail(ARLGPU_ERR_UNSUPPORTED, "too many planes");
  if (sizeof(CT) == 16)
    k_wstack_pre_predict64<<<nblk((int64_t)nb * plane), 256, 0, st>>>(image, gcf, nb, K, ny, nx, fov, wmean,
                                                                      reinterpret_cast<double2 *>(grid));
  else
    k_wstack_pre_predict32<<<nblk((int64_t)nb * plane), 256, K * sizeof(dsf), st>>>(
        image, gcf, nb, K, ny, nx, fov, wmean, reinterpret_cast<float2 *>(grid));
  ARL_LAUNCH_CHECK();
  count_launch(1);
  const int64_t G = group_planes(nplanes, ny, nx);
  for (int64_t p0 = 0; p0 < nplanes; p0 += G) {
    const int64_t np = std::min(G, nplanes - p0);
    cufftHandle h;
    ARL_TRY(get_plan(ny, nx, (int)np, (long long)plane, sizeof(CT) == 8 ? CUFFT_C2C : CUFFT_Z2Z, &h));
    cufftResult r = cufftSetStream(h, st);
    if (r != CUFFT_SUCCESS) return fail(ARLGPU_ERR_CUFFT, "cufftSetStream failed (%d)", (int)r);
    ARL_TRY(exec<CT>(h, grid + p0 * plane, CUFFT_FORWARD));
  }
  return ARLGPU_OK;
}

static int check(const arlgpu_grid_desc *gd, int precision) {
  if (!gd) return fail(ARLGPU_ERR_INVALID, "null grid descriptor");
  if (precision != ARLGPU_FP32C && precision != ARLGPU_FP64) return fail(ARLGPU_ERR_INVALID, "bad precision");
  if (gd->nchan < 1 || gd->npol < 1 || gd->nw < 1 || gd->ny < 2 || gd->nx < 2)
    return fail(ARLGPU_ERR_INVALID, "bad grid shape");
  if (gd->ny != gd->nx || (gd->nx & 1)) return fail(ARLGPU_ERR_UNSUPPORTED, "w-stacking needs a square, even image");
  return ARLGPU_OK;
}

}  // namespace arlgpu

using namespace arlgpu;

extern "C" int arlgpu_wstack_grid_to_image(const void *grid, const arlgpu_grid_desc *gd, int precision,
                                           const double *gcf, const double *wmean, double cellsize,
                                           const double *sumwt, double *image, void *fftbuf, void *stream) {
  ARL_TRY(check(gd, precision));
  if (!grid || !gcf || !wmean || !sumwt || !image || !fftbuf) return fail(ARLGPU_ERR_INVALID, "null array argument");
  const double fov = gd->nx * cellsize;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double2 *buf = static_cast<double2 *>(fftbuf);
  if (precision == ARLGPU_FP64)
    return g2i<double2>(static_cast<const double2 *>(grid), gd, gcf, wmean, fov, sumwt, image, buf, st);
  return g2i<float2>(static_cast<const float2 *>(grid), gd, gcf, wmean, fov, sumwt, image, buf, st);
}

extern "C" int arlgpu_wstack_fftbuf_bytes(const arlgpu_grid_desc *gd, size_t *bytes) {
  ARL_TRY(check(gd, ARLGPU_FP64));
  if (!bytes) return fail(ARLGPU_ERR_INVALID, "null bytes");
  const int64_t nplanes = (int64_t)gd->nchan * gd->npol * gd->nw;
  *bytes = (size_t)group_planes(nplanes, gd->ny, gd->nx) * gd->ny * gd->nx * sizeof(double2);
  return ARLGPU_OK;
}

extern "C" int arlgpu_wstack_image_to_grid(const double *image, const double *gcf, const double *wmean,
                                           double cellsize, const arlgpu_grid_desc *gd, int precision, void *grid,
                                           void *stream) {
  ARL_TRY(check(gd, precision));
  if (!grid || !gcf || !wmean || !image) return fail(ARLGPU_ERR_INVALID, "null array argument");
  const double fov = gd->nx * cellsize;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (precision == ARLGPU_FP64) return i2g<double2>(image, gcf, wmean, fov, gd, static_cast<double2 *>(grid), st);
  return i2g<float2>(image, gcf, wmean, fov, gd, static_cast<float2 *>(grid), st);
}
