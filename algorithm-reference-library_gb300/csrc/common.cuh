// Internal helpers shared by the libarlgpu translation units.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include "../../include/arlgpu.h"

namespace arlgpu {

int fail(int code, const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what, const char *file, int line);

#define ARL_CUDA(call)                                                         \
  do {                                                                         \
    cudaError_t _e = (call);                                                   \
    if (_e != cudaSuccess) return ::arlgpu::cuda_fail(_e, #call, __FILE__, __LINE__); \
  } while (0)

#define ARL_LAUNCH_CHECK() ARL_CUDA(cudaGetLastError())

#define ARL_TRY(expr)                 \
  do {                                \
    int _s = (expr);                  \
    if (_s != ARLGPU_OK) return _s;   \
  } while (0)

template <typename R> struct Cplx;
template <> struct Cplx<float> { using T = float2; };
template <> struct Cplx<double> { using T = double2; };

// Per-row result of the uvw -> grid mapping, 16 bytes.
//   pu, pv : nearest grid pixel (ARL pu_grid / pv_grid)
//   sub    : pu_off | pv_off << 8 | pwc << 16
//   cz     : pfreq | pwg << 16
struct RowMap {
  int32_t pu, pv;
  uint32_t sub, cz;
};

// 128-bit copies of a row map, for the plan kernels: the scatter writes each
// row's map to a random slot in bin order, where four 32-bit stores cost four
// L2 requests instead of one.  The plan's arrays start on 16-byte boundaries
// (the workspace must), so every element is 16-byte aligned.  The gridding
// kernels keep plain struct loads: 128-bit loads there made the degridder's
// four-rows-per-warp variant 7 % slower on C5.
__device__ __forceinline__ RowMap ld_map16(const RowMap *p) {
  const uint4 v = *reinterpret_cast<const uint4 *>(p);
  return RowMap{(int32_t)v.x, (int32_t)v.y, v.z, v.w};
}
__device__ __forceinline__ void st_map16(RowMap *p, const RowMap &m) {
  *reinterpret_cast<uint4 *>(p) = make_uint4((uint32_t)m.pu, (uint32_t)m.pv, m.sub, m.cz);
}

// Geometry handed to the device kernels by value.
// Row pitch of the fixed-point gridder's shared-memory subgrid.  An edge that
// is a multiple of 32 four-byte words puts every row of a kernel window on the
// same 32 banks, so the integer atomics of the rows a warp covers collide;
// 8 words of padding shift consecutive rows by 8 banks, which lays four rows
// of an 8-wide window (PSWF support 8) on distinct banks.
__host__ __device__ constexpr int fx_pitch(int sg) { return sg % 32 == 0 ? sg + 8 : sg; }

struct Geom {
  int32_t nchan, npol, nw, ny, nx;     // grid
  int32_t cf_nchan, cf_npol, nz, O, S; // cf
  int64_t cf_chan_stride, cf_pol_stride, cf_z_stride;
  arlgpu_axis gu, gv, gw, gf, cdu, cdv, cz;
  double rcp_gu, rcp_gv, rcp_gw, rcp_gf, rcp_cdu, rcp_cdv, rcp_cz;
  const int32_t *plane_support;        // device, may be null
  float tap_absmax;                    // bound of |Re|, |Im| over the cf taps (0: unknown)
  int32_t fast_uv;                     // 1: u/v mapping may use the one-FMA fast path
  // Sub-pixel fast path (fast_uv with a power-of-two O): X = P * O by one FMA,
  // pixel and sub-pixel index from floor(X) by integer shifts.
  int32_t pow2O, log2O;
  double rOu, cOu, rOv, cOv;           // X = fma(u, rOu, cOu)
  double Xlim_u, Xlim_v, tolX_u, tolX_v;
  // Nearest-plane axes (WW grid, WW cf, FREQ): |P| < Plim uses the fixed tolerance
  double Plim_w, tol_w, Plim_z, tol_z, Plim_f, tol_f;
  // Fixed-point decisions (pow2O and every limit below 2^29): the tolerances
  // above in units of 2^-20, plus one.
  int32_t fixmap, tq_u, tq_v, tq_w, tq_z, tq_f;
  // One grid w-plane whose interval contains every cf plane's (w-projection),
  // or one cf plane whose interval contains every grid plane's (w-stacking,
  // 2-D): that index is 0 for every row the other axis accepts, so the fast
  // path does not compute it.
  int32_t skip_zg, skip_zc;
  // binning
  int32_t T;       // tile edge (grid pixels)
  int32_t SG;      // staged subgrid edge = T + S
  int32_t ntu, ntv;
  uint32_t nbins;  // nchan * nw * ntv * ntu; key == nbins marks a rejected row
};

int make_geom(const arlgpu_grid_desc *gd, const arlgpu_cf_desc *cd, int precision, Geom *g);

// Workspace carve-up for a plan over nvis rows.
struct PlanBufs {
  uint32_t *keys;
  RowMap *maps;
  uint32_t *sidx;
  RowMap *smap;
  uint32_t *hist;     // nbins + 1
  uint32_t *offsets;  // nbins + 2
  double *wpart;      // per-plane partial w sums (plan_wpart_items entries)
  uint32_t *queue;    // device work-queue words of the gridder [0] and degridder [1]
};
uint32_t plan_wpart_items(const Geom &g);
size_t plan_bytes(int64_t nvis, const Geom &g);
int plan_carve(void *ws, size_t bytes, int64_t nvis, const Geom &g, PlanBufs *b);
int plan_build(const double *uvw, const double *freq, int64_t nvis, const Geom &g, const PlanBufs &b,
               int64_t *n_bad_dev, cudaStream_t st);

}  // namespace arlgpu
