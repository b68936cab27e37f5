// BlockVisibility <-> Visibility on the device.
//
// Reference behaviour:
//   convert_blocks / convert_blockvisibility_to_visibility
//                             processing_components/visibility/coalesce.py:331-443, :456-474
//   decoalesce_visibility     processing_components/visibility/coalesce.py:112-143
//
// The block holds [ntimes][nant][nant][nchan][npol] with baseline (a1 < a2)
// at [a2][a1].  Rows come out ordered (time, a2, a1, channel) over the
// baselines a2 > a1, with uvw converted from metres to wavelengths as
// uvw * (f / c) (the reference divides f by c first), and cindex maps every
// block cell [t][i][j][chan] to its row (0 for cells with i <= j, as the
// reference's zero-initialised index leaves them).
//
// The reverse copies rows back into the block.  The reference's loop writes
// flat[i : i + npol] = row[cindex[i]] for i over the block's cells, so with
// npol > 1 the slices overlap: position k ends up holding element k - i* of
// row cindex[i*], i* = min(k, ncells - 1), and positions beyond
// ncells + npol - 2 keep the block's previous values.  That result is
// reproduced as written.
#include "common.cuh"

namespace arlgpu {

void count_launch(unsigned n);

constexpr double kLightSpeed = 299792458.0;  // m/s, as astropy.constants.c

template <typename CT, typename W>
__global__ void k_convert_blocks(const CT *__restrict__ bvis, const double *__restrict__ buvw,
                                 const W *__restrict__ bwt, const W *__restrict__ biwt,
                                 const double *__restrict__ freq, int ntimes, int nant, int nchan, int npol,
                                 CT *__restrict__ vis, double *__restrict__ uvw, W *__restrict__ wt,
                                 W *__restrict__ iwt, double *__restrict__ rfreq, int32_t *__restrict__ a1o,
                                 int32_t *__restrict__ a2o, int32_t *__restrict__ tix) {
  const int64_t nbl = (int64_t)nant * (nant - 1) / 2;
  const int64_t nrows = (int64_t)ntimes * nbl * nchan;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = r / (nbl * nchan), rem = r - t * nbl * nchan;
    const int64_t b = rem / nchan;
    const int c = (int)(rem - b * nchan);
    // baseline b = a2 (a2 - 1) / 2 + a1 with 0 <= a1 < a2
    int a2 = (int)((1.0 + sqrt(1.0 + 8.0 * (double)b)) * 0.5);
    while ((int64_t)a2 * (a2 - 1) / 2 > b) --a2;
    while ((int64_t)(a2 + 1) * a2 / 2 <= b) ++a2;
    const int a1 = (int)(b - (int64_t)a2 * (a2 - 1) / 2);
    const int64_t cellbl = ((int64_t)t * nant + a2) * nant + a1;  // [t][a2][a1]
    const int64_t cell = cellbl * nchan + c;                      // [t][a2][a1][chan]
    const double k = freq[c] / kLightSpeed;
    for (int d = 0; d < 3; ++d) uvw[3 * r + d] = buvw[3 * cellbl + d] * k;
    for (int p = 0; p < npol; ++p) {
      vis[r * npol + p] = bvis[cell * npol + p];
      wt[r * npol + p] = bwt[cell * npol + p];
      iwt[r * npol + p] = biwt[cell * npol + p];
    }
    rfreq[r] = freq[c];
    a1o[r] = a1;
    a2o[r] = a2;
    tix[r] = (int32_t)t;
  }
}

// cindex over every block cell (nant * nant per time and channel).
__global__ void k_block_index(int ntimes, int nant, int nchan, int64_t *__restrict__ cindex) {
  const int64_t nbl = (int64_t)nant * (nant - 1) / 2;
  const int64_t ncell = (int64_t)ntimes * nant * nant * nchan;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < ncell; k += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(k % nchan);
    const int64_t tij = k / nchan;
    const int j = (int)(tij % nant), i = (int)((tij / nant) % nant);
    const int64_t t = tij / ((int64_t)nant * nant);
    cindex[k] = i > j ? (t * nbl + (int64_t)i * (i - 1) / 2 + j) * nchan + c : 0;
  }
}

// One column back into the block with the reference loop's result.  An
// index outside [0, nrows) is counted in nbad and its positions are left
// unwritten (the reference asserts max(cindex) < nrows first).
template <typename T>
__global__ void k_decoalesce(const T *__restrict__ rows, int64_t nrows, const int64_t *__restrict__ cindex,
                             int64_t ncell, int npol, T *__restrict__ block, unsigned long long *__restrict__ nbad) {
  const int64_t total = ncell * npol, last = ncell + npol - 1;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < total && k < last;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = k < ncell - 1 ? k : ncell - 1;
    const int64_t row = cindex[i];
    if (row < 0 || row >= nrows) {
      atomicAdd(nbad, 1ull);
      continue;
    }
    block[k] = rows[row * npol + (k - i)];
  }
}

static int nblk(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)(b < 1 ? 1 : (b > 152 * 32 ? 152 * 32 : b));
}

}  // namespace arlgpu

using namespace arlgpu;

extern "C" int arlgpu_convert_blocks(const void *block_vis, const double *block_uvw, const void *block_weight,
                                     const void *block_imaging_weight, const double *frequency, int32_t ntimes,
                                     int32_t nant, int32_t nchan, int32_t npol, int precision, void *vis,
                                     double *uvw, void *weight, void *imaging_weight, double *row_frequency,
                                     int32_t *antenna1, int32_t *antenna2, int32_t *time_index, int64_t *cindex,
                                     void *stream) {
  if (precision != ARLGPU_FP32C && precision != ARLGPU_FP64) return fail(ARLGPU_ERR_INVALID, "bad precision");
  if (ntimes < 0 || nant < 0 || nchan < 0 || npol < 1) return fail(ARLGPU_ERR_INVALID, "bad block shape");
  const int64_t nrows = (int64_t)ntimes * nant * (nant > 0 ? nant - 1 : 0) / 2 * nchan;
  const int64_t ncell = (int64_t)ntimes * nant * nant * nchan;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (nrows > 0) {
    if (!block_vis || !block_uvw || !block_weight || !block_imaging_weight || !frequency || !vis || !uvw ||
        !weight || !imaging_weight || !row_frequency || !antenna1 || !antenna2 || !time_index)
      return fail(ARLGPU_ERR_INVALID, "null array argument");
    if (precision == ARLGPU_FP64)
      k_convert_blocks<double2, double><<<nblk(nrows), 256, 0, st>>>(
          static_cast<const double2 *>(block_vis), block_uvw, static_cast<const double *>(block_weight),
          static_cast<const double *>(block_imaging_weight), frequency, ntimes, nant, nchan, npol,
          static_cast<double2 *>(vis), uvw, static_cast<double *>(weight), static_cast<double *>(imaging_weight),
          row_frequency, antenna1, antenna2, time_index);
    else
      k_convert_blocks<float2, float><<<nblk(nrows), 256, 0, st>>>(
          static_cast<const float2 *>(block_vis), block_uvw, static_cast<const float *>(block_weight),
          static_cast<const float *>(block_imaging_weight), frequency, ntimes, nant, nchan, npol,
          static_cast<float2 *>(vis), uvw, static_cast<float *>(weight), static_cast<float *>(imaging_weight),
          row_frequency, antenna1, antenna2, time_index);
    ARL_LAUNCH_CHECK();
    count_launch(1);
  }
  if (cindex && ncell > 0) {
    k_block_index<<<nblk(ncell), 256, 0, st>>>(ntimes, nant, nchan, cindex);
    ARL_LAUNCH_CHECK();
    count_launch(1);
  }
  return ARLGPU_OK;
}

extern "C" int arlgpu_decoalesce(const void *rows, int64_t nrows, const int64_t *cindex, int32_t ntimes, int32_t nant,
                                 int32_t nchan, int32_t npol, int elem_bytes, void *block, int64_t *n_bad_dev,
                                 void *stream) {
  if (npol < 1 || ntimes < 0 || nant < 0 || nchan < 0) return fail(ARLGPU_ERR_INVALID, "bad block shape");
  const int64_t ncell = (int64_t)ntimes * nant * nant * nchan;
  if (!n_bad_dev) return fail(ARLGPU_ERR_INVALID, "null n_bad_dev");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  ARL_CUDA(cudaMemsetAsync(n_bad_dev, 0, sizeof(int64_t), st));
  if (ncell == 0) return ARLGPU_OK;
  if (!rows || !cindex || !block) return fail(ARLGPU_ERR_INVALID, "null array argument");
  if (nrows < 1) return fail(ARLGPU_ERR_INVALID, "no rows to decoalesce");
  const int64_t n = ncell * npol;
  unsigned long long *nb = reinterpret_cast<unsigned long long *>(n_bad_dev);
  switch (elem_bytes) {
    case 4:
      k_decoalesce<float><<<nblk(n), 256, 0, st>>>(static_cast<const float *>(rows), nrows, cindex, ncell, npol,
                                                    static_cast<float *>(block), nb);
      break;
    case 8:
      k_decoalesce<double><<<nblk(n), 256, 0, st>>>(static_cast<const double *>(rows), nrows, cindex, ncell, npol,
                                                     static_cast<double *>(block), nb);
      break;
    case 16:
      k_decoalesce<double2><<<nblk(n), 256, 0, st>>>(static_cast<const double2 *>(rows), nrows, cindex, ncell,
                                                      npol, static_cast<double2 *>(block), nb);
      break;
    default:
      return fail(ARLGPU_ERR_INVALID, "elem_bytes must be 4, 8 or 16");
  }
  ARL_LAUNCH_CHECK();
  count_launch(1);
  return ARLGPU_OK;
}
