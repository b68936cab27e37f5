/*
 * arlgpu.h -- C ABI of libarlgpu.so, the GB300 (sm_103a) implementation of
 * ARL's convolutional gridding / degridding imaging path.
 *
 * Conventions
 *   - Every entry point returns an int status (ARLGPU_OK = 0).  The message of
 *     the last failure on the calling thread is available from
 *     arlgpu_last_error().
 *   - All array arguments are DEVICE pointers owned by the caller unless a
 *     parameter name ends in _host.  No entry point keeps a pointer after it
 *     returns; the library caches only FFT plans.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *     Work is enqueued asynchronously; results are valid once the stream has
 *     been synchronised.
 *   - Scratch memory comes from the caller through `workspace` /
 *     `workspace_bytes`, sized by arlgpu_plan_workspace_bytes().  A plan
 *     workspace starts on a 16-byte boundary (cudaMalloc and the PyTorch
 *     allocator give 256); an unaligned one is rejected with
 *     ARLGPU_ERR_INVALID before any GPU work.
 *   - Array layouts are ARL's (row-major, C order):
 *       uvw        [nvis][3]            float64, wavelengths
 *       frequency  [nvis]               float64, Hz
 *       vis        [nvis][npol]         complex (see precision)
 *       weight     [nvis][npol]         real    (see precision)
 *       grid       [nchan][npol][nw][ny][nx]          complex
 *       cf         [nchan][npol][nz][O][O][S][S]      complex (strides below)
 *       image      [nchan][npol][ny][nx]              float64
 *   - Precision: ARLGPU_FP32C uses complex64 vis / grid / cf taps and float32
 *     weights with compensated FP32 accumulation; ARLGPU_FP64 uses complex128 /
 *     float64 throughout.  uvw -> pixel mapping is FP64 in both.
 */
#ifndef ARLGPU_H
#define ARLGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  ARLGPU_OK = 0,
  ARLGPU_ERR_INVALID = 1,       /* bad argument (shape, pointer, precision) */
  ARLGPU_ERR_CUDA = 2,          /* a CUDA runtime call failed */
  ARLGPU_ERR_OUT_OF_GRID = 3,   /* rows whose kernel window leaves the grid */
  ARLGPU_ERR_UNSUPPORTED = 4,   /* valid ARL input this library does not handle */
  ARLGPU_ERR_WORKSPACE = 5,     /* workspace missing or too small */
  ARLGPU_ERR_CUFFT = 6          /* a cuFFT call failed */
};

enum { ARLGPU_FP32C = 0, ARLGPU_FP64 = 1 };

/* One linear FITS axis: world = ((pix0 + 1) - crpix) * cdelt + crval. */
typedef struct {
  double crval, crpix, cdelt;
} arlgpu_axis;

/* GridData geometry (ARL GridData: processing_components/griddata/operations.py:91-145). */
typedef struct {
  int32_t nchan, npol, nw, ny, nx;
  arlgpu_axis u, v, w, f;       /* grid_wcs axes UU, VV, WW and FREQ */
} arlgpu_grid_desc;

/* ConvolutionFunction geometry (convolution_functions.py:62-147).  The table is
 * [nchan][npol][nz][O][O][S][S]; chan_stride / pol_stride are element strides
 * between channel / polarisation blocks (0 = the same kernel for all).
 * plane_support, if not NULL, is a device array of nz even supports <= S: plane
 * z then uses only the central plane_support[z] x plane_support[z] taps.
 * tap_absmax is an upper bound of |Re| and |Im| over every tap of the table, or
 * 0 when the caller does not know one.  With a bound the FP32C gridder can sum
 * each tile exactly in fixed point (grid_kernel 4); without one it uses the
 * compensated float variant.  A bound that is too small gives wrong grids. */
typedef struct {
  int32_t nchan, npol, nz, oversampling, support;
  int64_t chan_stride, pol_stride;
  arlgpu_axis du, dv, z;        /* cf grid_wcs axes DUU, DVV and WW */
  const int32_t *plane_support;
  double tap_absmax;
} arlgpu_cf_desc;

/* Library version string and the message of the last failure on this thread. */
const char *arlgpu_version(void);
const char *arlgpu_last_error(void);

/* Number of kernels this library has launched in the process (its own kernels,
 * not cuFFT's), for launch accounting. */
unsigned long long arlgpu_kernel_launches(void);

/* Kernel-variant selection (the autotuner's knobs; process-wide):
 *   "grid_kernel"   0 = shared-memory atomics with TwoSum compensation,
 *                   1 = band owner: each warp owns a band of the subgrid, plain
 *                       read-modify-write with a per-cell Kahan term,
 *                   2 = as 0, specialised on npol with 32-bit incremental offsets,
 *                   3 = as 2 without the compensation (measurement only: FP32C
 *                       promises compensated sums, so the autotuner never picks it),
 *                   4 = FP32C tiles summed in two-limb 32-bit fixed point: the rounded
 *                       contributions and their rounding residuals (default; needs cf
 *                       tap_absmax; FP64 and an unknown bound use 2),
 *                   5 = as 4 without the residual plane (measurement only)
 *   "degrid_kernel" 0 = one warp per row, 1 = 32-row batches per warp,
 *                   2 = one warp per row, specialised on npol, groups of four steps,
 *                   3 = as 2 with the staged cells duplicated (re, re, im, im) so each tap is
 *                       two packed FP32 multiply-adds (default; FP32C, FP64 uses 2),
 *                   4 = as 3 with the grid tile and each row's kernel taps brought into shared
 *                       memory by TMA tensor copies (FP32C, one polarisation, support <= 32,
 *                       subgrid 48, 16-byte aligned tables, even nx; otherwise 3)
 *   "subgrid"       subgrid edge in cells (16..128), 0 = automatic (48, or 32 when 4 pols)
 *   "chunk"         sorted rows per gridder / degridder CTA (32..2^20, default 512)
 *   "persistent"    1 = the lean and fixed-point kernels run as one grid of resident CTAs,
 *                   each looping over every gridDim-th chunk; 2 = the same resident grid fed by
 *                   a device work queue (each CTA takes the next unclaimed chunk with one
 *                   atomic; the default); 0 = one CTA per chunk, which the hardware schedules
 *                   dynamically
 *   "dsfft"         FP32C inverse transforms (invert_2d and w-stacking): 1 = double-single
 *                   FFT on the FP32 pipes for power-of-two sizes 64..8192 (default),
 *                   0 = cuFFT complex128
 *   "small_rows"    rows per warp (1, 2 or 4; default 2) in the FP32C fixed-point gridder when the
 *                   largest support is at most 8 (64 taps) and the subgrid edge is the default
 *   "small_rows_degrid"  the same for the packed degridder (default 4)
 *   "lanes_per_row" 0 = lanes per row (threads per visibility) chosen per segment and support
 *                   (default); 8, 16 or 32 = that many lanes per row in every segment of the
 *                   FP32C fixed-point gridder and packed degridder at the default subgrid edge
 *                   Otherwise both kernels choose per segment: two rows per warp when the
 *                   segment's largest support is at most 16, four (degridder) at most 8.
 *   "gather_rows"   1 = the FP32C fixed-point gridder with one polarisation first copies the
 *                   rows' vis and weight into bin order, into the plan workspace's mapping
 *                   scratch, and reads them contiguously (default); 0 = it gathers them
 *                   through the sort index in its row loop.  Either way the grid is the same.
 *   "stash_rows"    1 = with one or four polarisations and chunks of at most 512 rows, the
 *                   FP32C fixed-point gridder (and, for one polarisation and supports above 8,
 *                   the packed degridder) take
 *                   each row's set-up (kernel-window offset, window origin, support, row index)
 *                   from the footprint pass, which computes it one row per lane, instead of
 *                   a whole warp computing it per row (default); 0 = per row in the row loop.
 * No reference counterpart (ARL has one Python loop per function). */
int arlgpu_set_tuning(const char *key, int value);
int arlgpu_get_tuning(const char *key, int *value);

/* ---- a1: convolution_mapping (processing_components/griddata/gridding.py:24-96) ----
 * Writes pu, pu_off, pv, pv_off, pwg, pwc, pfreq (int32 [nvis] each) and the
 * number of rows whose S x S window, plane or channel falls outside the grid /
 * cf into *n_bad_host (the rows ARL's asserts reject).  Synchronises `stream`. */
int arlgpu_convolution_mapping(const double *uvw, const double *frequency, int64_t nvis,
                               const arlgpu_grid_desc *gd, const arlgpu_cf_desc *cd,
                               int32_t *pu, int32_t *pu_off, int32_t *pv, int32_t *pv_off,
                               int32_t *pwg, int32_t *pwc, int32_t *pfreq,
                               int64_t *n_bad_host, void *stream);

/* Scratch bytes needed by arlgpu_grid / arlgpu_degrid for nvis rows. */
int arlgpu_plan_workspace_bytes(int64_t nvis, const arlgpu_grid_desc *gd,
                                const arlgpu_cf_desc *cd, size_t *bytes_host);

/* ---- a2: grid_visibility_to_griddata (gridding.py:99-133) ----
 * grid is zeroed, then grid[c,:,zg,v-S/2:v+S/2,u-S/2:u+S/2] += conj(cf[c,:,zc,dv,du]) * vis*weight;
 * sumwt [nchan][npol] float64 receives the summed weights.  n_bad_dev (device
 * int64, may be NULL) receives the count of rejected rows, which are skipped. */
int arlgpu_grid(const double *uvw, const double *frequency, const void *vis, const void *weight,
                int64_t nvis, int precision, const void *cf, const arlgpu_cf_desc *cd,
                void *grid, const arlgpu_grid_desc *gd, double *sumwt, int64_t *n_bad_dev,
                void *workspace, size_t workspace_bytes, void *stream);

/* ---- Plans: the mapping and tile binning of a set of rows, built once and
 * shared by the planned gridder and degridder (ARL recomputes the mapping in
 * each of grid_visibility_to_griddata and degrid_visibility_from_griddata,
 * gridding.py:113-114,243-244).  The plan lives in `workspace`; the planned
 * calls must be given the same nvis, gd and cd as arlgpu_plan_build.  The
 * planned gridder writes scratch into the workspace (bin-order row copies,
 * work-queue words), so planned calls that share a workspace must not overlap
 * on the GPU: order them on one stream. */
int arlgpu_plan_build(const double *uvw, const double *frequency, int64_t nvis, const arlgpu_grid_desc *gd,
                      const arlgpu_cf_desc *cd, void *workspace, size_t workspace_bytes, int64_t *n_bad_dev,
                      void *stream);
int arlgpu_grid_planned(const void *vis, const void *weight, int64_t nvis, int precision, const void *cf,
                        const arlgpu_cf_desc *cd, void *grid, const arlgpu_grid_desc *gd, double *sumwt,
                        const void *workspace, size_t workspace_bytes, void *stream);
int arlgpu_degrid_planned(int64_t nvis, int precision, const void *cf, const arlgpu_cf_desc *cd, const void *grid,
                          const arlgpu_grid_desc *gd, void *vis_out, const void *workspace,
                          size_t workspace_bytes, void *stream);

/* Status flags the kernels of the last planned call left in the plan's
 * workspace (same nvis / gd / cd as the plan): bit 0 = a bounded wait of the TMA
 * degridder (degrid_kernel 4) gave up, so that call's output is not to be
 * trusted.  Synchronises `stream`.  No reference counterpart. */
int arlgpu_plan_flags(int64_t nvis, const arlgpu_grid_desc *gd, const arlgpu_cf_desc *cd, const void *workspace,
                      size_t workspace_bytes, uint32_t *flags_host, void *stream);

/* Mean w of the rows that a plan assigned to each grid w-plane (the slice mean
 * numpy.average(vis.w) of invert/predict_wstack_single, wstack_single.py:43,83);
 * wmean: [gd->nw] float64 (0 for empty planes).  Same nvis / gd / cd as the plan.
 * The plan's row order is read, and a small partial-sum area of the workspace is
 * written; the result is deterministic (fixed summation order). */
int arlgpu_plan_plane_mean_w(const double *uvw, int64_t nvis, const arlgpu_grid_desc *gd, const arlgpu_cf_desc *cd,
                             void *workspace, size_t workspace_bytes, double *wmean, void *stream);

/* ---- Gridding without any device allocation (no counterpart in the reference,
 * whose gridder is a NumPy loop) ----
 * For callers that cannot allocate device memory when they grid: hosts whose
 * device memory is all owned by another framework's pool, and real-time code
 * that allocates only at start-up.  Same arguments and results as arlgpu_grid,
 * minus the workspace: the row plan lives in a fixed device array of ~22.0 MB
 * that the library holds on every GPU it runs on until the process exits.  At
 * most 524,288 rows and 65,536 plan bins (channel x w-plane x uv-tile) per call;
 * larger calls fail with ARLGPU_ERR_WORKSPACE before any GPU work.  All calls
 * share the array, which keeps the last call's contents: calls whose GPU work
 * overlaps (other streams or threads) race on it.  The first call on each device
 * looks up the array's address; make it before any stream capture begins, and
 * do not use this entry point across a cudaDeviceReset.  No cudaMalloc /
 * cudaFree is called. */
int arlgpu_grid_noalloc(const double *uvw, const double *frequency, const void *vis, const void *weight,
                        int64_t nvis, int precision, const void *cf, const arlgpu_cf_desc *cd, void *grid,
                        const arlgpu_grid_desc *gd, double *sumwt, int64_t *n_bad_dev, void *stream);

/* ---- a3: degrid_visibility_from_griddata (gridding.py:233-267) ----
 * vis_out[r,p] = sum_ij grid[c,p,zg,v-S/2+j,u-S/2+i] * cf[c,p,zc,dv,du,j,i]; rejected rows get 0. */
int arlgpu_degrid(const double *uvw, const double *frequency, int64_t nvis, int precision,
                  const void *cf, const arlgpu_cf_desc *cd, const void *grid,
                  const arlgpu_grid_desc *gd, void *vis_out, int64_t *n_bad_dev,
                  void *workspace, size_t workspace_bytes, void *stream);

/* ---- a4: fft_griddata_to_image (gridding.py:270-289) + normalize_sumwt (imaging/base.py:84-101) ----
 * image = Re/Im[ fftshift(ifft2(ifftshift(sum_w grid))) ] * gcf * nx*ny, divided by
 * sumwt[c,p] when sumwt != NULL (zero where sumwt <= 0).  image_imag may be NULL.
 * `fftbuf` is caller scratch of nchan*npol*ny*nx complex128 elements: the transform
 * runs in FP64 for both precisions, because the grid correction multiplies its
 * rounding error by up to max(gcf)/min(gcf).  With precision FP64 and nw == 1 the
 * grid itself may be passed as fftbuf (it is then destroyed). */
int arlgpu_fft_grid_to_image(const void *grid, const arlgpu_grid_desc *gd, int precision,
                             const double *gcf, const double *sumwt, double *image_real,
                             double *image_imag, void *fftbuf, void *stream);

/* ---- a5: fft_image_to_griddata (gridding.py:292-302) ----
 * grid[c,p,z] = fftshift(fft2(ifftshift(image * gcf))) for every w-plane z. */
int arlgpu_fft_image_to_grid(const double *image, const double *gcf, const arlgpu_grid_desc *gd,
                             int precision, void *grid, void *stream);

/* ---- a14: w-stacking, all slices at once (imaging/wstack_single.py:26-96,
 * workflows/serial/imaging/imaging_serial.py:186-197) ----
 * The grid holds one w-plane per slice (gd->nw = number of slices, gridded with a
 * plan whose WW axis bins rows into slices); wmean[s] is slice s's mean w and
 * cellsize the image cell (radians).
 * arlgpu_wstack_grid_to_image: image = gcf * sum_s Re(wbeam(wmean[s]) * ifft_s) * nx*ny / sumwt,
 *   i.e. the sumwt-weighted sum of the slices' invert_wstack_single images divided by
 *   the total sumwt [nchan][npol].  fftbuf: complex128 scratch of
 *   arlgpu_wstack_fftbuf_bytes() bytes (the transforms run in FP64, on groups of
 *   planes of at most 2 GiB of complex128 each); with precision FP64 the grid itself
 *   may be passed instead (it is then destroyed).
 * arlgpu_wstack_image_to_grid: plane s = fft(conj(wbeam(wmean[s])) * image * gcf), so one
 *   degrid over all rows is predict_wstack_single summed over the slices.
 * arlgpu_wstack_fftbuf_bytes: bytes of fftbuf for a grid of shape gd (no reference
 *   counterpart: the reference transforms one slice at a time in NumPy). */
int arlgpu_wstack_fftbuf_bytes(const arlgpu_grid_desc *gd, size_t *bytes);
int arlgpu_wstack_grid_to_image(const void *grid, const arlgpu_grid_desc *gd, int precision, const double *gcf,
                                const double *wmean, double cellsize, const double *sumwt, double *image,
                                void *fftbuf, void *stream);
int arlgpu_wstack_image_to_grid(const double *image, const double *gcf, const double *wmean, double cellsize,
                                const arlgpu_grid_desc *gd, int precision, void *grid, void *stream);

/* ---- (f1) uniform weighting: grid_weight_to_griddata (gridding.py:161-183),
 * griddata_reweight (gridding.py:213-230), as weight_visibility (imaging/weighting.py:19-40)
 * calls them ----
 * arlgpu_grid_weights: wgrid [nchan][npol][nw][ny][nx] float64 and sumwt [nchan][npol]
 *   are zeroed, then each row's weight [nvis][npol] (float32 for FP32C, float64 for FP64)
 *   is added to its nearest cell and to sumwt.  Rows whose cell, w-plane, cf plane or
 *   channel is out of range are counted in *n_bad_dev (ARL asserts) and skipped.
 * arlgpu_reweight: each row's weights are divided by its cells when every
 *   polarisation's cell is non-zero (the reference's `real(cell).all() > 0`). */
int arlgpu_grid_weights(const double *uvw, const double *frequency, const void *weight, int64_t nvis,
                        int precision, const arlgpu_cf_desc *cd, double *wgrid, const arlgpu_grid_desc *gd,
                        double *sumwt, int64_t *n_bad_dev, void *stream);
int arlgpu_reweight(const double *uvw, const double *frequency, void *weight, int64_t nvis, int precision,
                    const arlgpu_cf_desc *cd, const double *wgrid, const arlgpu_grid_desc *gd, void *stream);

/* ---- (f2) BlockVisibility -> Visibility: convert_blocks (visibility/coalesce.py:331-443)
 * and the copy-back of decoalesce_visibility (coalesce.py:112-143) ----
 * arlgpu_convert_blocks: block arrays [ntimes][nant][nant][nchan][npol] (vis complex,
 *   weights real, both of the precision; block_uvw [ntimes][nant][nant][3] float64 in
 *   metres; frequency [nchan]) -> rows ordered (time, a2, a1, channel) over a2 > a1:
 *   vis, uvw [nrows][3] in wavelengths (uvw * (f / c)), weight, imaging_weight,
 *   row_frequency, antenna1, antenna2, time_index; nrows = ntimes nant (nant-1)/2 nchan.
 *   cindex [ntimes][nant][nant][nchan] int64 (may be NULL): the row of each block cell,
 *   0 for cells with i <= j.
 * arlgpu_decoalesce: one column (elem_bytes 4, 8 or 16 per element) of rows
 *   [nrows][npol] back into block [ntimes][nant][nant][nchan][npol] with the reference
 *   loop's result (flat[i:i+npol] = row[cindex[i]] for every cell i, overlapping when
 *   npol > 1; positions past ncell + npol - 2 keep their values).  Indices outside
 *   [0, nrows) are counted in *n_bad_dev and skipped. */
int arlgpu_convert_blocks(const void *block_vis, const double *block_uvw, const void *block_weight,
                          const void *block_imaging_weight, const double *frequency, int32_t ntimes,
                          int32_t nant, int32_t nchan, int32_t npol, int precision, void *vis, double *uvw,
                          void *weight, void *imaging_weight, double *row_frequency, int32_t *antenna1,
                          int32_t *antenna2, int32_t *time_index, int64_t *cindex, void *stream);
int arlgpu_decoalesce(const void *rows, int64_t nrows, const int64_t *cindex, int32_t ntimes, int32_t nant,
                      int32_t nchan, int32_t npol, int elem_bytes, void *block, int64_t *n_bad_dev,
                      void *stream);

/* ---- (f3) DFT predict: predict_skycomponent_visibility (imaging/base.py:192-244) with
 * simulate_point (util/coordinate_support.py:192-212) ----
 * arlgpu_dft_predict: vis[r][p] += sum_k flux[k][row_chan[r]][p] exp(-2 pi i (u l + v m + w n))
 *   for uvw [nvis][3] (wavelengths), lmn [ncomp][3] = (l, m, sqrt(1-l^2-m^2) - 1), flux
 *   [ncomp][nchan][npol] float64, vis [nvis][npol] complex of the precision (updated in
 *   place).  row_chan [nvis] int32 may be NULL when nchan == 1.  Phases in FP64.
 * arlgpu_dft_adjoint: image[k][p] += Re sum_r conj(exp(-2 pi i uvw_r . lmn_k)) x[r][p], the
 *   adjoint for one channel (no reference counterpart; the dense gradient reference). */
int arlgpu_dft_predict(const double *uvw, const int32_t *row_chan, int64_t nvis, const double *lmn,
                       const double *flux, int32_t ncomp, int32_t nchan, int32_t npol, int precision, void *vis,
                       void *stream);
int arlgpu_dft_adjoint(const double *uvw, int64_t nvis, const double *lmn, int32_t ncomp, int32_t npol,
                       int precision, const void *x, double *image, void *stream);

/* ---- (f4) deconvolution: hogbom (processing_library/arrays/cleaners.py:12-69), as
 * deconvolve_cube(algorithm='hogbom') (image/deconvolution.py:43-300) calls it ----
 * One plane: dirty [nx][ny], psf [psf_nx][psf_ny], window [nx][ny] or NULL, all float64
 * device arrays; comps and res [nx][ny] are written (res starts as a copy of dirty).
 * dirty_absmax = max|dirty| and psf_max = max(psf) are the caller's (exact maxima).
 * Stops after niter iterations or when |res[peak]| < 0.9 max(thresh, fracthresh *
 * dirty_absmax); *iterations (host) receives the count.  FP64 in the reference's
 * operation order: the result equals NumPy's bit for bit. */
int arlgpu_hogbom(const double *dirty, const double *psf, const double *window, int32_t nx, int32_t ny,
                  int32_t psf_nx, int32_t psf_ny, double gain, double thresh, int32_t niter, double fracthresh,
                  double dirty_absmax, double psf_max, double *comps, double *res, int32_t *iterations,
                  void *stream);

/* ---- (f4) hogbom_complex (processing_library/arrays/cleaners.py:72-131): CLEAN of Q + iU ----
 * dirty_q, dirty_u, comps_q, comps_u, res_q, res_u [nx][ny] (device, FP64): the residual
 * Q + iU starts as the dirty pair and the components at zero; psf [psf_nx][psf_ny] is
 * the (common, real) PSF; window [nx][ny] or NULL.  The peak is the first largest
 * |res * window| (|.| the hypotenuse); the loop stops after niter iterations or when
 * |res[peak]| < max(thresh, fracthresh * dirty_absmax), dirty_absmax = max |Q + iU|.
 * *iterations (host) receives the count. */
int arlgpu_hogbom_complex(const double *dirty_q, const double *dirty_u, const double *psf, const double *window,
                          int32_t nx, int32_t ny, int32_t psf_nx, int32_t psf_ny, double gain, double thresh,
                          int32_t niter, double fracthresh, double dirty_absmax, double psf_max, double *comps_q,
                          double *comps_u, double *res_q, double *res_u, int32_t *iterations, void *stream);

/* ---- (f4) msmfsclean (processing_library/arrays/cleaners.py:469-600): the minor cycle ----
 * smres [nscales][nmoment][n0][n1] is the scale-moment residual (updated in place), ssm
 * [nscales][nscales][nmoment][nmoment][psf_n0][psf_n1] the scale-scale-moment-moment PSF,
 * pscale [nscales][psf_n0][psf_n1] the PSF-sized scale images, windowstack [nscales][n0][n1]
 * or NULL, hess / ihess [nscales][nmoment][nmoment] the moment-moment Hessian at the PSF
 * centre and its inverse; model [nmoment][n0][n1] is written.  findpeak: 0 'ARL', 1
 * 'Algorithm1', 2 'CASA' (find_global_optimum, cleaners.py:601-634).  At most 16 scales and
 * 8 moments.  Stops after niter iterations or when max |mval| < absthresh. */
int arlgpu_msmfsclean(double *smres, const double *ssm, const double *pscale, const double *windowstack,
                      const double *hess, const double *ihess, int32_t nscales, int32_t nmoment, int32_t n0,
                      int32_t n1, int32_t psf_n0, int32_t psf_n1, double gain, double absthresh, int32_t niter,
                      int32_t findpeak, double *model, int32_t *iterations, void *stream);

/* Scale basis stack [nscales][n0][n1] (create_scalestack, cleaners.py:283-316) from the
 * caller's host array of scales (pixels). */
int arlgpu_scale_stack(const double *scales_host, int32_t nscales, int32_t n0, int32_t n1, double *stack,
                       void *stream);

/* img [nimg][n0][n1] convolved with every plane of stack [nscales][n0][n1]:
 * convolve_scalestack (cleaners.py:319-335) into out [nimg][nscales][n0][n1], or with twice
 * != 0 convolve_convolve_scalestack (:338-360) into out [nimg][nscales][nscales][n0][n1].
 * thresh >= 0 (once only) writes 1 where the result exceeds thresh and 0 elsewhere, as the
 * window stacks are made.  Device workspace of arlgpu_scale_convolve_bytes. */
int arlgpu_scale_convolve_bytes(int32_t n0, int32_t n1, int32_t nscales, size_t *bytes_host);
int arlgpu_scale_convolve(const double *img, int32_t nimg, int32_t n0, int32_t n1, const double *stack,
                          int32_t nscales, int32_t twice, double thresh, double *out, void *workspace,
                          size_t workspace_bytes, void *stream);

/* ---- (f4) msclean (processing_library/arrays/cleaners.py:165-280): the minor cycle ----
 * stack [nscales][nx][ny] is the scale-convolved residual (updated in place), psf_ss
 * [nscales][nscales][psf_nx][psf_ny] the twice-convolved PSF stack, pscale [nscales]
 * [psf_nx][psf_ny] the PSF-sized scale images, windowstack [nscales][nx][ny] or NULL,
 * coupling [nscales][nscales]; comps [nx][ny] is written.  arlgpu_msclean_setup forms
 * these; the caller applies the final pmax scaling. */
int arlgpu_msclean(double *stack, const double *psf_ss, const double *pscale, const double *windowstack,
                   const double *coupling, int32_t nscales, int32_t nx, int32_t ny, int32_t psf_nx, int32_t psf_ny,
                   double gain, double absthresh, int32_t niter, double *comps, int32_t *iterations, void *stream);

/* ---- (f4) msclean set-up (processing_library/arrays/cleaners.py:165-212, with
 * create_scalestack :283-316, convolve_scalestack :319-335,
 * convolve_convolve_scalestack :338-360, spheroidal_function :398-440) ----
 * From dirty [nx][ny], psf [psf_nx][psf_ny] and window [nx][ny] (or NULL), float64
 * device arrays, and the nscales scale sizes (host array, pixels): pscale
 * [nscales][psf_nx][psf_ny] (the PSF-sized scale images), stack [nscales][nx][ny]
 * (dirty / max(psf) convolved with each dirty-sized scale image), psf_ss
 * [nscales][nscales][psf_nx][psf_ny] (psf / max(psf) convolved with scale p and
 * correlated with scale s), windowstack [nscales][nx][ny] (1 where the window
 * convolved with a scale exceeds 0.9; needed only with a window), coupling
 * [nscales][nscales] (the maximum of each psf_ss plane) and scalars[2] = {max(psf),
 * max|stack[0]|}, all device arrays.  Convolutions are complex128 cuFFT transforms;
 * workspace bytes come from arlgpu_msclean_setup_bytes.  A scale whose window
 * (2 ceil(scale / 2) + 2 pixels) is wider than the image or the PSF is rejected. */
int arlgpu_msclean_setup_bytes(int32_t nx, int32_t ny, int32_t psf_nx, int32_t psf_ny, int32_t nscales,
                               size_t *bytes_host);
int arlgpu_msclean_setup(const double *dirty, int32_t nx, int32_t ny, const double *psf, int32_t psf_nx,
                         int32_t psf_ny, const double *window, const double *scales_host, int32_t nscales,
                         double *stack, double *psf_ss, double *pscale, double *windowstack, double *coupling,
                         double *scalars, void *workspace, size_t workspace_bytes, void *stream);

/* ---- a7/a8: create_pswf_convolutionfunction (griddata/kernels.py:52-97), FP64 ----
 * cf_out: [O][O][S][S] complex128 (one plane; ARL broadcasts it over chan/pol);
 * gcf_out: [ny][nx] float64. */
int arlgpu_make_pswf(int32_t oversampling, int32_t support, int32_t ny, int32_t nx,
                     void *cf_out, double *gcf_out, void *stream);

/* ---- a9: create_awterm_convolutionfunction without primary beam
 * (griddata/kernels.py:100-200), FP64 ----
 * cf_out: [nw][O][O][S][S] complex128; image_nx / cdelt_ra_deg describe the image
 * template; maxsupport as in ARL (512); use_aaf != 0 divides the w-screens by the
 * PSWF grid correction of the padded sub-image (ARL's default), 0 leaves them as they are. */
int arlgpu_make_wkernels(int32_t nw, double wstep, int32_t oversampling, int32_t support,
                         int32_t maxsupport, int32_t image_nx, double cdelt_ra_deg, int32_t use_aaf,
                         void *cf_out, void *stream);

/* ---- a17: apply_gaintable, scalar gains (calibration/operations.py:134-137) ----
 * vis[r,p] *= g[a2[r]] * conj(g[a1[r]])  (inverse: 1/g), complex128 gains [nant]. */
int arlgpu_apply_gains(void *vis, int64_t nvis, int32_t npol, int precision, const int32_t *a1,
                       const int32_t *a2, const void *gains, int inverse, void *stream);

/* ---- a17: apply_gaintable on a BlockVisibility, scalar gains
 * (calibration/operations.py:79-164, the scalar branch :124-140) ----
 * vis: the block [ntimes][nants][nants][nchan] (one polarisation; complex64 for
 * FP32C, complex128 for FP64).  time_row [ntimes] int32: the gain-table row of
 * each block time, or -1 to leave that time alone.  gain [rows][nants][nchan]
 * complex128 and gain_weight [rows][nants][nchan] float64.  Cell [t][i][j][c]
 * becomes V * g[i] conj(g[j]) with g the row's gains (inverse: 1/gain where
 * |gain| > 0, else 1), and 0 where the two antennas' gain weights multiply to 0. */
int arlgpu_apply_gaintable(void *vis, int32_t ntimes, int32_t nants, int32_t nchan, int precision,
                           const int32_t *time_row, const void *gain, const double *gain_weight,
                           int inverse, void *stream);

/* ---- a13: phaserotate_visibility, tangent plane (visibility/base.py:295-334) ----
 * vis[r,:] *= exp(+/-2 pi i (u l + v m + w (n - 1))), n = sqrt(1 - l^2 - m^2); inverse selects +. */
int arlgpu_phaserotate(void *vis, const double *uvw, int64_t nvis, int32_t npol, int precision,
                       double l, double m, int inverse, void *stream);

/* ---- chi^2 of a gain-corrupted model and its gradients (the g_i g_j* convention
 * of apply_gaintable, calibration/operations.py:134-137; no reference counterpart
 * for the derivatives) ----
 * chi2 = sum w |vobs - g[a2] conj(g[a1]) model|^2 (weight may be NULL = 1), written
 * to the device double *chi2.  grad_model (may be NULL) = d chi2 / d conj(model)
 * [nvis][npol] in the precision's complex type; grad_gains (may be NULL) =
 * d chi2 / d conj(g) [nant] complex128.  gains: [nant] complex128. */
int arlgpu_gain_chi2(const void *vobs, const void *model, const double *weight, int64_t nvis, int32_t npol,
                     int precision, const int32_t *a1, const int32_t *a2, const void *gains, int32_t nant,
                     double *chi2, void *grad_model, void *grad_gains, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* ARLGPU_H */
