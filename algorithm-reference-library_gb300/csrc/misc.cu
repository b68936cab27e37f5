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
