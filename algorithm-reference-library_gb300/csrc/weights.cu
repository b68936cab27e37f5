// Uniform weighting on the GPU.
//
// Reference behaviour:
//   grid_weight_to_griddata   processing_components/griddata/gridding.py:161-183
//   griddata_reweight         processing_components/griddata/gridding.py:213-230
//   weight_visibility         processing_components/imaging/weighting.py:19-40
//
// grid_weight_to_griddata adds each row's imaging weight (one value per
// polarisation) to its nearest grid cell grid[chan, :, pwg, pv, pu] and to
// sumwt[chan, :]; griddata_reweight then divides each row's weights by the
// real part of that cell when every polarisation's cell is non-zero.  The
// weight grid is real FP64 here (ARL keeps it in the real part of a complex
// grid); the row weights keep the precision of the path.
#include "common.cuh"
#include "mapping.cuh"

namespace arlgpu {

void count_launch(unsigned n);

// Nearest-cell mapping of one row.  ARL's convolution_mapping asserts that
// the pixel, the w-plane, the cf plane and the channel are in range; the
// sub-pixel index is not used here.
__device__ __forceinline__ bool map_cell(const double *uvw, const double *freq, int64_t r, const Geom &g,
                                         int *ch, int64_t *cell0) {
  const RawMap m = map_raw(uvw[3 * r], uvw[3 * r + 1], uvw[3 * r + 2], freq[r], g);
  const bool ok = m.pu >= 0.0 && m.pu < g.nx && m.pv >= 0.0 && m.pv < g.ny && m.zg >= 0.0 && m.zg < g.nw &&
                  m.zc >= 0.0 && m.zc < g.nz && m.ch >= 0.0 && m.ch < g.nchan && m.ch < g.cf_nchan;
  if (!ok) return false;
  *ch = (int)m.ch;
  // cell of polarisation 0; polarisation p is p * nw * ny * nx further
  *cell0 = (((int64_t)*ch * g.npol) * g.nw + (int64_t)m.zg) * g.ny * g.nx + (int64_t)m.pv * g.nx + (int64_t)m.pu;
  return true;
}

// K10a: weights onto the weight grid; sumwt summed per block in shared memory
// when [nchan][npol] fits, else directly.
template <typename W>
__global__ void k_grid_weight(const double *__restrict__ uvw, const double *__restrict__ freq,
                              const W *__restrict__ wt, int64_t nvis, Geom g, double *__restrict__ wgrid,
                              double *__restrict__ sumwt, unsigned long long *__restrict__ nbad, int shared_sum) {
  extern __shared__ double s_sum[];
  const int nsum = g.nchan * g.npol;
  if (shared_sum) {
    for (int k = threadIdx.x; k < nsum; k += blockDim.x) s_sum[k] = 0.0;
    __syncthreads();
  }
  const int64_t pstride = (int64_t)g.nw * g.ny * g.nx;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nvis; r += (int64_t)gridDim.x * blockDim.x) {
    int ch;
    int64_t c0;
    if (!map_cell(uvw, freq, r, g, &ch, &c0)) {
      atomicAdd(nbad, 1ull);
      continue;
    }
    for (int p = 0; p < g.npol; ++p) {
      const double w = (double)wt[r * g.npol + p];
      atomicAdd(&wgrid[c0 + p * pstride], w);
      if (shared_sum)
        atomicAdd(&s_sum[ch * g.npol + p], w);
      else
        atomicAdd(&sumwt[ch * g.npol + p], w);
    }
  }
  if (shared_sum) {
    __syncthreads();
    for (int k = threadIdx.x; k < nsum; k += blockDim.x)
      if (s_sum[k] != 0.0) atomicAdd(&sumwt[k], s_sum[k]);
  }
}

// K10b: each row's weights divided by its cells when all are non-zero.
template <typename W>
__global__ void k_reweight(const double *__restrict__ uvw, const double *__restrict__ freq, W *__restrict__ wt,
                           int64_t nvis, Geom g, const double *__restrict__ wgrid) {
  const int64_t pstride = (int64_t)g.nw * g.ny * g.nx;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nvis; r += (int64_t)gridDim.x * blockDim.x) {
    int ch;
    int64_t c0;
    if (!map_cell(uvw, freq, r, g, &ch, &c0)) continue;
    bool all = true;
    for (int p = 0; p < g.npol; ++p) all = all && wgrid[c0 + p * pstride] != 0.0;
    if (!all) continue;
    for (int p = 0; p < g.npol; ++p) wt[r * g.npol + p] = (W)((double)wt[r * g.npol + p] / wgrid[c0 + p * pstride]);
  }
}

static int blocks_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)(b < 1 ? 1 : (b > 152 * 32 ? 152 * 32 : b));
}

}  // namespace arlgpu

using namespace arlgpu;

extern "C" int arlgpu_grid_weights(const double *uvw, const double *frequency, const void *weight, int64_t nvis,
                                   int precision, const arlgpu_cf_desc *cd, double *wgrid, const arlgpu_grid_desc *gd,
                                   double *sumwt, int64_t *n_bad_dev, void *stream) {
  Geom g;
  ARL_TRY(make_geom(gd, cd, precision, &g));
  if (nvis < 0) return fail(ARLGPU_ERR_INVALID, "nvis < 0");
  if (!wgrid || !sumwt || !n_bad_dev || (nvis > 0 && (!uvw || !frequency || !weight)))
    return fail(ARLGPU_ERR_INVALID, "null array argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t cells = (size_t)g.nchan * g.npol * g.nw * g.ny * g.nx;
  ARL_CUDA(cudaMemsetAsync(wgrid, 0, cells * sizeof(double), st));
  ARL_CUDA(cudaMemsetAsync(sumwt, 0, (size_t)g.nchan * g.npol * sizeof(double), st));
  ARL_CUDA(cudaMemsetAsync(n_bad_dev, 0, sizeof(int64_t), st));
  if (nvis == 0) return ARLGPU_OK;
  const int nsum = g.nchan * g.npol;
  const int shared_sum = nsum <= 4096;
  const size_t smem = shared_sum ? (size_t)nsum * sizeof(double) : 0;
  unsigned long long *nb = reinterpret_cast<unsigned long long *>(n_bad_dev);
  if (precision == ARLGPU_FP64)
    k_grid_weight<double><<<blocks_for(nvis), 256, smem, st>>>(uvw, frequency, static_cast<const double *>(weight),
                                                                nvis, g, wgrid, sumwt, nb, shared_sum);
  else
    k_grid_weight<float><<<blocks_for(nvis), 256, smem, st>>>(uvw, frequency, static_cast<const float *>(weight),
                                                               nvis, g, wgrid, sumwt, nb, shared_sum);
  ARL_LAUNCH_CHECK();
  count_launch(1);
  return ARLGPU_OK;
}

extern "C" int arlgpu_reweight(const double *uvw, const double *frequency, void *weight, int64_t nvis, int precision,
                               const arlgpu_cf_desc *cd, const double *wgrid, const arlgpu_grid_desc *gd,
                               void *stream) {
  Geom g;
  ARL_TRY(make_geom(gd, cd, precision, &g));
  if (nvis < 0) return fail(ARLGPU_ERR_INVALID, "nvis < 0");
  if (nvis == 0) return ARLGPU_OK;
  if (!uvw || !frequency || !weight || !wgrid) return fail(ARLGPU_ERR_INVALID, "null array argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (precision == ARLGPU_FP64)
    k_reweight<double><<<blocks_for(nvis), 256, 0, st>>>(uvw, frequency, static_cast<double *>(weight), nvis, g,
                                                          wgrid);
  else
    k_reweight<float><<<blocks_for(nvis), 256, 0, st>>>(uvw, frequency, static_cast<float *>(weight), nvis, g,
                                                         wgrid);
  ARL_LAUNCH_CHECK();
  count_launch(1);
  return ARLGPU_OK;
}
