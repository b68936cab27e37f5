// Multiscale CLEAN set-up on the GPU: everything msclean computes before its
// minor cycle.
//
// Reference behaviour (processing_library/arrays/cleaners.py):
//   msclean, up to the loop       :165-212
//   create_scalestack             :283-316
//   convolve_scalestack           :319-335
//   convolve_convolve_scalestack  :338-360
//   spheroidal_function           :398-440
//
// Steps, all on one stream:
//   pmax = max(psf); every later use of dirty / psf divides by it;
//   scale basis images for the dirty and the PSF shapes (Schwab's spheroidal
//   rational approximation times (1 - r^2), clipped at 0, normalised to unit
//   sum; scale 0 is a unit spike at the centre);
//   centred transforms F = fft2(fftshift(a)) with cuFFT (complex128), batched
//   over the scales.  The reference transforms fftshift(fft2(fftshift(a))),
//   multiplies, and applies ifftshift before ifft2: the two outer shifts
//   cancel, so the products are formed in cuFFT's order and only the input
//   (fftshift) and output (ifftshift) permutations remain, folded into the
//   gather and scatter passes around the transforms;
//   residual stack[s] = Re ifftshift(ifft2(Fd conj(Fs[s])));
//   psf stack[s][p] = Re ifftshift(ifft2(Fp Fps[p] conj(Fps[s])));
//   window stack[s] = 1 where the window convolved with scale s exceeds 0.9;
//   coupling[s][p] = max psf stack[s][p]; and the largest |stack[0]|.
// The inverse transform's 1/(n0 n1) is one multiply after cuFFT's
// unnormalised inverse.
#include <cufft.h>

#include "common.cuh"

namespace arlgpu {

void count_launch(unsigned n);
int get_plan(int ny, int nx, int batch, long long dist, cufftType type, cufftHandle *out);

// Schwab's rational approximation (m = 6, alpha = 1) of the spheroidal
// function, the coefficient table of cleaners.py:411-418.
__constant__ double c_sph_p[2][5] = {{8.203343e-2, -3.644705e-1, 6.278660e-1, -5.335581e-1, 2.312756e-1},
                                     {4.028559e-3, -3.697768e-2, 1.021332e-1, -1.201436e-1, 6.412774e-2}};
__constant__ double c_sph_q[2][3] = {{1.0000000, 8.212018e-1, 2.078043e-1}, {1.0000000, 9.599102e-1, 2.918724e-1}};

__device__ double spheroidal(double vnu) {
  int part;
  double nuend;
  if (vnu >= 0.0 && vnu < 0.75) {
    part = 0;
    nuend = 0.75;
  } else if (vnu >= 0.75 && vnu <= 1.0) {
    part = 1;
    nuend = 1.0;
  } else {
    return 0.0;
  }
  const double d = vnu * vnu - nuend * nuend;
  double top = c_sph_p[part][0], bot = c_sph_q[part][0], dk = 1.0;
  for (int k = 1; k < 5; ++k) {
    dk *= d;
    top += c_sph_p[part][k] * dk;
  }
  dk = 1.0;
  for (int k = 1; k < 3; ++k) {
    dk *= d;
    bot += c_sph_q[part][k] * dk;
  }
  const double v = bot != 0.0 ? top / bot : 0.0;
  return v >= 0.0 ? v : 0.0;
}

// Scale basis images into a zeroed stack [ns][n0][n1] (rows x, columns y as
// the reference indexes basis[iscale, x, y]), then normalised by
// k_scale_norm.  One block per scale; its threads walk the square window
// x, y in [c - h - 1, c + h + 1), h = ceil(scale / 2), c = ceil(n / 2).
__global__ void k_scale_basis(const double *__restrict__ scales, int n0, int n1, double *__restrict__ basis) {
  const int s = blockIdx.x;
  double *b = basis + (int64_t)s * n0 * n1;
  const double sc = scales[s];
  const int xc = (n0 + 1) / 2, yc = (n1 + 1) / 2;
  if (!(sc > 0.0)) {
    if (threadIdx.x == 0) b[(int64_t)xc * n1 + yc] = 1.0;
    return;
  }
  const int h = (int)ceil(sc / 2.0);
  const double rs2 = 1.0 / ((sc / 2.0) * (sc / 2.0));
  const int w = 2 * h + 2;
  for (int t = threadIdx.x; t < w * w; t += blockDim.x) {
    const int x = xc - h - 1 + t / w, y = yc - h - 1 + t % w;
    const double fx = (double)(x - xc), fy = (double)(y - yc);
    const double r = sqrt(rs2 * (fx * fx + fy * fy));
    const double v = spheroidal(r) * (1.0 - r * r);
    // negative window indices wrap, as NumPy indexing does
    const int xi = x < 0 ? x + n0 : x, yi = y < 0 ? y + n1 : y;
    b[(int64_t)xi * n1 + yi] = v > 0.0 ? v : 0.0;
  }
}

// basis[s] /= sum(basis[s]) over its window (every other cell is 0); one block
// per scale, fixed per-thread order and a fixed tree: deterministic.
__global__ void k_scale_norm(const double *__restrict__ scales, int n0, int n1, double *__restrict__ basis) {
  __shared__ double red[256];
  const int s = blockIdx.x;
  const double sc = scales[s];
  if (!(sc > 0.0)) return;
  double *b = basis + (int64_t)s * n0 * n1;
  const int xc = (n0 + 1) / 2, yc = (n1 + 1) / 2;
  const int h = (int)ceil(sc / 2.0), w = 2 * h + 2;
  double sum = 0.0;
  for (int t = threadIdx.x; t < w * w; t += blockDim.x) {
    const int x = xc - h - 1 + t / w, y = yc - h - 1 + t % w;
    const int xi = x < 0 ? x + n0 : x, yi = y < 0 ? y + n1 : y;
    sum += b[(int64_t)xi * n1 + yi];
  }
  red[threadIdx.x] = sum;
  __syncthreads();
  for (int d = blockDim.x / 2; d > 0; d >>= 1) {
    if (threadIdx.x < d) red[threadIdx.x] += red[threadIdx.x + d];
    __syncthreads();
  }
  const double tot = red[0];
  for (int t = threadIdx.x; t < w * w; t += blockDim.x) {
    const int x = xc - h - 1 + t / w, y = yc - h - 1 + t % w;
    const int xi = x < 0 ? x + n0 : x, yi = y < 0 ? y + n1 : y;
    b[(int64_t)xi * n1 + yi] /= tot;
  }
}

// dst[b][k0][k1] = src[b][(k0 - n0/2) mod n0][(k1 - n1/2) mod n1] / div (fftshift
// as a gather), imaginary part 0; div = *pdiv, or 1 when pdiv is null.
__global__ void k_shift_in(const double *__restrict__ src, int nb, int n0, int n1, const double *__restrict__ pdiv,
                           double2 *__restrict__ dst) {
  const int64_t plane = (int64_t)n0 * n1, tot = plane * nb;
  const double div = pdiv ? *pdiv : 1.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / plane, k = i - b * plane;
    const int k0 = (int)(k / n1), k1 = (int)(k - (int64_t)k0 * n1);
    int s0 = k0 - n0 / 2, s1 = k1 - n1 / 2;
    s0 += s0 < 0 ? n0 : 0;
    s1 += s1 < 0 ? n1 : 0;
    const double v = src[b * plane + (int64_t)s0 * n1 + s1];
    dst[i] = make_double2(pdiv ? v / div : v, 0.0);
  }
}

// prod[b][k] = a[k] conj(f[b][k])            (three == nullptr)
// prod[b][k] = a[k] f[b][k] conj(three[k])   (the double convolution; a[k]
//                                             f[b][k] first, as the reference)
__global__ void k_spectra(const double2 *__restrict__ a, const double2 *__restrict__ f,
                          const double2 *__restrict__ three, int nb, int64_t plane, double2 *__restrict__ prod) {
  const int64_t tot = plane * nb;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = i % plane;
    const double2 x = a[k], y = f[i];
    double2 r;
    if (!three) {
      r = make_double2(x.x * y.x + x.y * y.y, x.y * y.x - x.x * y.y);
    } else {
      const double2 t = make_double2(x.x * y.x - x.y * y.y, x.x * y.y + x.y * y.x);
      const double2 z = three[k];
      r = make_double2(t.x * z.x + t.y * z.y, t.y * z.x - t.x * z.y);
    }
    prod[i] = r;
  }
}

// out[b][k0][k1] = Re src[b][(k0 + n0/2) mod n0][(k1 + n1/2) mod n1] * scale
// (ifftshift as a gather); with thresh >= 0 the output is 1 where that value
// exceeds thresh and 0 elsewhere.
__global__ void k_shift_out(const double2 *__restrict__ src, int nb, int n0, int n1, double scale, double thresh,
                            double *__restrict__ out) {
  const int64_t plane = (int64_t)n0 * n1, tot = plane * nb;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / plane, k = i - b * plane;
    const int k0 = (int)(k / n1), k1 = (int)(k - (int64_t)k0 * n1);
    int s0 = k0 + n0 / 2, s1 = k1 + n1 / 2;
    s0 -= s0 >= n0 ? n0 : 0;
    s1 -= s1 >= n1 ? n1 : 0;
    const double v = src[b * plane + (int64_t)s0 * n1 + s1].x * scale;
    out[i] = thresh >= 0.0 ? (v > thresh ? 1.0 : 0.0) : v;
  }
}

// out[p] = max over plane p of x (or of |x| with absval); one block per plane.
__global__ void k_plane_max(const double *__restrict__ x, int64_t plane, int absval, double *__restrict__ out) {
  __shared__ double red[256];
  const double *a = x + (int64_t)blockIdx.x * plane;
  double m = -INFINITY;
  for (int64_t i = threadIdx.x; i < plane; i += blockDim.x) m = fmax(m, absval ? fabs(a[i]) : a[i]);
  red[threadIdx.x] = m;
  __syncthreads();
  for (int d = blockDim.x / 2; d > 0; d >>= 1) {
    if (threadIdx.x < d) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + d]);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

static int nblk(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)(b < 1 ? 1 : (b > 152 * 32 ? 152 * 32 : b));
}

static size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

static size_t setup_bytes(int n0, int n1, int p0, int p1, int ns) {
  const size_t d = (size_t)n0 * n1, p = (size_t)p0 * p1;
  return al(16 * d) + 2 * al(16 * d * ns) + al(16 * p) + 2 * al(16 * p * ns) + al(8 * d * ns) + al(8 * (size_t)ns);
}

static int fft_z2z(double2 *data, int n0, int n1, int batch, int dir, cudaStream_t st) {
  cufftHandle h;
  ARL_TRY(get_plan(n0, n1, batch, (long long)n0 * n1, CUFFT_Z2Z, &h));
  cufftResult r = cufftSetStream(h, st);
  if (r != CUFFT_SUCCESS) return fail(ARLGPU_ERR_CUFFT, "cufftSetStream failed (%d)", (int)r);
  r = cufftExecZ2Z(h, reinterpret_cast<cufftDoubleComplex *>(data), reinterpret_cast<cufftDoubleComplex *>(data), dir);
  if (r != CUFFT_SUCCESS) return fail(ARLGPU_ERR_CUFFT, "cufftExecZ2Z failed (%d)", (int)r);
  return ARLGPU_OK;
}

}  // namespace arlgpu

using namespace arlgpu;

extern "C" int arlgpu_msclean_setup_bytes(int32_t nx, int32_t ny, int32_t psf_nx, int32_t psf_ny, int32_t nscales,
                                          size_t *bytes_host) {
  if (nx < 1 || ny < 1 || psf_nx < 1 || psf_ny < 1 || nscales < 1 || !bytes_host)
    return fail(ARLGPU_ERR_INVALID, "bad msclean set-up shape");
  *bytes_host = setup_bytes(nx, ny, psf_nx, psf_ny, nscales);
  return ARLGPU_OK;
}

extern "C" int arlgpu_msclean_setup(const double *dirty, int32_t nx, int32_t ny, const double *psf, int32_t psf_nx,
                                    int32_t psf_ny, const double *window, const double *scales_host,
                                    int32_t nscales, double *stack, double *psf_ss,
                                    double *pscale, double *windowstack, double *coupling, double *scalars,
                                    void *workspace, size_t workspace_bytes, void *stream) {
  if (nx < 1 || ny < 1 || psf_nx < 1 || psf_ny < 1 || nscales < 1 || nscales > 64)
    return fail(ARLGPU_ERR_INVALID, "bad msclean set-up shape");
  if (!dirty || !psf || !scales_host || !stack || !psf_ss || !pscale || !coupling || !scalars ||
      (window && !windowstack))
    return fail(ARLGPU_ERR_INVALID, "null array argument");
  // Each scale's window of 2 ceil(scale / 2) + 2 cells must fit in both images
  // (wider windows would wrap onto themselves).
  for (int s = 0; s < nscales; ++s) {
    const double sc = scales_host[s];
    if (!(sc >= 0.0) || sc > 1e6) return fail(ARLGPU_ERR_INVALID, "scale %d is %g", s, sc);
    const int w = sc > 0.0 ? 2 * (int)ceil(sc / 2.0) + 2 : 1;
    if (w > nx || w > ny || w > psf_nx || w > psf_ny)
      return fail(ARLGPU_ERR_UNSUPPORTED, "scale %g is wider than the image or the PSF", sc);
  }
  const size_t need = setup_bytes(nx, ny, psf_nx, psf_ny, nscales);
  if (!workspace || workspace_bytes < need)
    return fail(ARLGPU_ERR_WORKSPACE, "msclean set-up needs %zu bytes of workspace, got %zu", need, workspace_bytes);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int64_t d = (int64_t)nx * ny, p = (int64_t)psf_nx * psf_ny;
  char *w = static_cast<char *>(workspace);
  double2 *fd = reinterpret_cast<double2 *>(w);
  w += al(16 * d);
  double2 *fs = reinterpret_cast<double2 *>(w);
  w += al(16 * d * nscales);
  double2 *td = reinterpret_cast<double2 *>(w);
  w += al(16 * d * nscales);
  double2 *fp = reinterpret_cast<double2 *>(w);
  w += al(16 * p);
  double2 *fps = reinterpret_cast<double2 *>(w);
  w += al(16 * p * nscales);
  double2 *tp = reinterpret_cast<double2 *>(w);
  w += al(16 * p * nscales);
  double *ss = reinterpret_cast<double *>(w);
  w += al(8 * d * nscales);
  double *scales = reinterpret_cast<double *>(w);
  double *pmax = scalars;  // scalars[0] = max(psf), scalars[1] = max |stack[0]|

  // the scales go up from the caller's host array (staged before this call returns)
  ARL_CUDA(cudaMemcpyAsync(scales, scales_host, sizeof(double) * nscales, cudaMemcpyHostToDevice, st));
  unsigned launches = 0;
  k_plane_max<<<1, 256, 0, st>>>(psf, p, 0, pmax);
  ++launches;
  // scale stacks for the dirty and the PSF shapes
  ARL_CUDA(cudaMemsetAsync(ss, 0, sizeof(double) * d * nscales, st));
  ARL_CUDA(cudaMemsetAsync(pscale, 0, sizeof(double) * p * nscales, st));
  k_scale_basis<<<nscales, 256, 0, st>>>(scales, nx, ny, ss);
  k_scale_norm<<<nscales, 256, 0, st>>>(scales, nx, ny, ss);
  k_scale_basis<<<nscales, 256, 0, st>>>(scales, psf_nx, psf_ny, pscale);
  k_scale_norm<<<nscales, 256, 0, st>>>(scales, psf_nx, psf_ny, pscale);
  launches += 4;
  ARL_LAUNCH_CHECK();
  // residual stack
  k_shift_in<<<nblk(d), 256, 0, st>>>(dirty, 1, nx, ny, pmax, fd);
  k_shift_in<<<nblk(d * nscales), 256, 0, st>>>(ss, nscales, nx, ny, nullptr, fs);
  launches += 2;
  ARL_LAUNCH_CHECK();
  ARL_TRY(fft_z2z(fd, nx, ny, 1, CUFFT_FORWARD, st));
  ARL_TRY(fft_z2z(fs, nx, ny, nscales, CUFFT_FORWARD, st));
  k_spectra<<<nblk(d * nscales), 256, 0, st>>>(fd, fs, nullptr, nscales, d, td);
  ++launches;
  ARL_LAUNCH_CHECK();
  ARL_TRY(fft_z2z(td, nx, ny, nscales, CUFFT_INVERSE, st));
  const double sd = (1.0 / nx) * (1.0 / ny), sp = (1.0 / psf_nx) * (1.0 / psf_ny);
  k_shift_out<<<nblk(d * nscales), 256, 0, st>>>(td, nscales, nx, ny, sd, -1.0, stack);
  k_plane_max<<<1, 256, 0, st>>>(stack, d, 1, scalars + 1);
  launches += 2;
  ARL_LAUNCH_CHECK();
  // window stack: the window convolved with each scale, above 0.9
  if (window) {
    k_shift_in<<<nblk(d), 256, 0, st>>>(window, 1, nx, ny, nullptr, fd);
    ++launches;
    ARL_LAUNCH_CHECK();
    ARL_TRY(fft_z2z(fd, nx, ny, 1, CUFFT_FORWARD, st));
    k_spectra<<<nblk(d * nscales), 256, 0, st>>>(fd, fs, nullptr, nscales, d, td);
    ++launches;
    ARL_LAUNCH_CHECK();
    ARL_TRY(fft_z2z(td, nx, ny, nscales, CUFFT_INVERSE, st));
    k_shift_out<<<nblk(d * nscales), 256, 0, st>>>(td, nscales, nx, ny, sd, 0.9, windowstack);
    ++launches;
    ARL_LAUNCH_CHECK();
  }
  // PSF scale-scale stack and the coupling matrix
  k_shift_in<<<nblk(p), 256, 0, st>>>(psf, 1, psf_nx, psf_ny, pmax, fp);
  k_shift_in<<<nblk(p * nscales), 256, 0, st>>>(pscale, nscales, psf_nx, psf_ny, nullptr, fps);
  launches += 2;
  ARL_LAUNCH_CHECK();
  ARL_TRY(fft_z2z(fp, psf_nx, psf_ny, 1, CUFFT_FORWARD, st));
  ARL_TRY(fft_z2z(fps, psf_nx, psf_ny, nscales, CUFFT_FORWARD, st));
  for (int s = 0; s < nscales; ++s) {
    k_spectra<<<nblk(p * nscales), 256, 0, st>>>(fp, fps, fps + (int64_t)s * p, nscales, p, tp);
    ++launches;
    ARL_LAUNCH_CHECK();
    ARL_TRY(fft_z2z(tp, psf_nx, psf_ny, nscales, CUFFT_INVERSE, st));
    k_shift_out<<<nblk(p * nscales), 256, 0, st>>>(tp, nscales, psf_nx, psf_ny, sp, -1.0,
                                                    psf_ss + (int64_t)s * nscales * p);
    ++launches;
    ARL_LAUNCH_CHECK();
  }
  k_plane_max<<<nscales * nscales, 256, 0, st>>>(psf_ss, p, 0, coupling);
  ++launches;
  ARL_LAUNCH_CHECK();
  count_launch(launches);
  return ARLGPU_OK;
}

// ---------------------------------------------------------------------------
// Building blocks of the multi-scale multi-frequency CLEAN set-up
// (cleaners.py:469-540): scale basis stacks of any shape, and images
// convolved once (convolve_scalestack, :319-335) or twice
// (convolve_convolve_scalestack, :338-360) with a given stack, through the
// same shift / transform / spectra passes as the msclean set-up above.
// ---------------------------------------------------------------------------
extern "C" int arlgpu_scale_stack(const double *scales_host, int32_t nscales, int32_t n0, int32_t n1, double *stack,
                                  void *stream) {
  if (!scales_host || !stack) return fail(ARLGPU_ERR_INVALID, "null array argument");
  if (n0 < 1 || n1 < 1 || nscales < 1 || nscales > 64) return fail(ARLGPU_ERR_INVALID, "bad scale-stack shape");
  for (int s = 0; s < nscales; ++s) {
    const double sc = scales_host[s];
    if (!(sc >= 0.0) || sc > 1e6) return fail(ARLGPU_ERR_INVALID, "scale %d is %g", s, sc);
    const int w = sc > 0.0 ? 2 * (int)ceil(sc / 2.0) + 2 : 1;
    if (w > n0 || w > n1) return fail(ARLGPU_ERR_UNSUPPORTED, "scale %g is wider than the image", sc);
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double *scales = nullptr;
  ARL_CUDA(cudaMallocAsync(&scales, sizeof(double) * nscales, st));
  int rc = ARLGPU_OK;
  if (cudaMemcpyAsync(scales, scales_host, sizeof(double) * nscales, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemsetAsync(stack, 0, sizeof(double) * n0 * n1 * nscales, st) != cudaSuccess) {
    rc = fail(ARLGPU_ERR_CUDA, "scale-stack set-up failed");
  } else {
    k_scale_basis<<<nscales, 256, 0, st>>>(scales, n0, n1, stack);
    k_scale_norm<<<nscales, 256, 0, st>>>(scales, n0, n1, stack);
    if (cudaGetLastError() != cudaSuccess) rc = fail(ARLGPU_ERR_CUDA, "scale-stack launch failed");
    count_launch(2);
  }
  // the caller's host array is staged before cudaMemcpyAsync returns; the
  // device copy is freed in stream order
  cudaFreeAsync(scales, st);
  return rc;
}

static size_t conv_bytes(int n0, int n1, int ns) {
  const size_t d = (size_t)n0 * n1;
  return al(16 * d) + 2 * al(16 * d * ns);
}

extern "C" int arlgpu_scale_convolve_bytes(int32_t n0, int32_t n1, int32_t nscales, size_t *bytes_host) {
  if (n0 < 1 || n1 < 1 || nscales < 1 || !bytes_host) return fail(ARLGPU_ERR_INVALID, "bad scale-convolve shape");
  *bytes_host = conv_bytes(n0, n1, nscales);
  return ARLGPU_OK;
}

extern "C" int arlgpu_scale_convolve(const double *img, int32_t nimg, int32_t n0, int32_t n1, const double *stack,
                                     int32_t nscales, int32_t twice, double thresh, double *out, void *workspace,
                                     size_t workspace_bytes, void *stream) {
  if (!img || !stack || !out) return fail(ARLGPU_ERR_INVALID, "null array argument");
  if (nimg < 1 || n0 < 1 || n1 < 1 || nscales < 1 || nscales > 64) return fail(ARLGPU_ERR_INVALID, "bad shapes");
  const size_t need = conv_bytes(n0, n1, nscales);
  if (!workspace || workspace_bytes < need)
    return fail(ARLGPU_ERR_WORKSPACE, "scale convolution needs %zu bytes of workspace, got %zu", need,
                workspace_bytes);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int64_t d = (int64_t)n0 * n1;
  char *w = static_cast<char *>(workspace);
  double2 *fd = reinterpret_cast<double2 *>(w);
  w += al(16 * d);
  double2 *fs = reinterpret_cast<double2 *>(w);
  w += al(16 * d * nscales);
  double2 *td = reinterpret_cast<double2 *>(w);
  const double sd = (1.0 / n0) * (1.0 / n1);
  unsigned launches = 0;
  k_shift_in<<<nblk(d * nscales), 256, 0, st>>>(stack, nscales, n0, n1, nullptr, fs);
  ++launches;
  ARL_LAUNCH_CHECK();
  ARL_TRY(fft_z2z(fs, n0, n1, nscales, CUFFT_FORWARD, st));
  for (int i = 0; i < nimg; ++i) {
    k_shift_in<<<nblk(d), 256, 0, st>>>(img + (int64_t)i * d, 1, n0, n1, nullptr, fd);
    ++launches;
    ARL_LAUNCH_CHECK();
    ARL_TRY(fft_z2z(fd, n0, n1, 1, CUFFT_FORWARD, st));
    const int nouter = twice ? nscales : 1;
    for (int s = 0; s < nouter; ++s) {
      k_spectra<<<nblk(d * nscales), 256, 0, st>>>(fd, fs, twice ? fs + (int64_t)s * d : nullptr, nscales, d, td);
      ++launches;
      ARL_LAUNCH_CHECK();
      ARL_TRY(fft_z2z(td, n0, n1, nscales, CUFFT_INVERSE, st));
      double *o = out + ((int64_t)i * nouter + s) * nscales * d;
      k_shift_out<<<nblk(d * nscales), 256, 0, st>>>(td, nscales, n0, n1, sd, twice ? -1.0 : thresh, o);
      ++launches;
      ARL_LAUNCH_CHECK();
    }
  }
  count_launch(launches);
  return ARLGPU_OK;
}

