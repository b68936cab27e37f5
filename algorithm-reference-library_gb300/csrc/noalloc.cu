// arlgpu_grid_noalloc: the gridder for callers that cannot allocate device
// memory.
//
// Some callers of this library have no way to obtain scratch memory at the
// moment they want to grid: hosts whose device memory is entirely owned by
// another framework's pool (the pool hands out only the buffers it was asked
// for at start-up), and real-time pipelines that allocate everything once
// when they start and forbid allocation, with its possible implicit
// synchronisation, afterwards.  For them this file keeps the gridder's
// scratch (the row plan: mapping, bin keys, sorted row ids, bin histogram and
// offsets) in a fixed file-scope device array, so the entry point needs
// nothing beyond the caller's inputs and outputs.
//
// Costs and limits of that choice:
//   * every GPU that loads the library holds kScratchBytes (about 22.0 MB) of
//     device memory for this array until the process exits;
//   * one call handles at most kMaxRows rows and a plan of at most kMaxBins
//     (channel x w-plane x uv-tile) bins; larger calls are rejected with
//     ARLGPU_ERR_WORKSPACE before any GPU work is queued;
//   * all calls share the one array, and it keeps whatever the previous call
//     left in it: the plan build clears the bin histogram itself before use,
//     and every other part is fully rewritten by each call.  Two calls whose
//     GPU work overlaps in time (different streams, or different host threads)
//     race on the array and corrupt each other's results; callers must order
//     them on one stream or synchronise between them;
//   * the device address of the array is looked up once per device (with
//     cudaGetSymbolAddress), the first time the entry point runs with that
//     device current.  Make that first call before any stream capture begins.
//     The cached address belongs to the device's context at that time: after
//     cudaDeviceReset the module is loaded again at another address, so this
//     entry point must not be used across a device reset.
#include <mutex>

#include "common.cuh"

namespace {

constexpr int64_t kMaxRows = 1 << 19;  // 524,288 rows per call
constexpr int64_t kMaxBins = 1 << 16;  // 65,536 bins per call

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Same carve-up as the workspace of arlgpu_grid (keys, RowMap, sorted ids,
// sorted RowMap, histogram, offsets) at the maximum sizes above.
constexpr size_t kScratchBytes = align256(kMaxRows * 4) + align256(kMaxRows * 16) + align256(kMaxRows * 4) +
                                 align256(kMaxRows * 16) + align256((kMaxBins + 1) * 4) +
                                 align256((kMaxBins + 2) * 4) + align256(kMaxBins * 8) +  // plane-mean partials
                                 align256(16);                                            // work-queue words

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_scratch_ptr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (looked up once).
int scratch_for_current_device(void **out) {
  int dev = 0;
  ARL_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices)
    return arlgpu::fail(ARLGPU_ERR_UNSUPPORTED, "device ordinal %d is beyond the %d this entry point tracks", dev,
                        kMaxDevices);
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    ARL_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return ARLGPU_OK;
}

}  // namespace

using namespace arlgpu;

extern "C" int arlgpu_grid_noalloc(const double *uvw, const double *frequency, const void *vis, const void *weight,
                                   int64_t nvis, int precision, const void *cf, const arlgpu_cf_desc *cd, void *grid,
                                   const arlgpu_grid_desc *gd, double *sumwt, int64_t *n_bad_dev, void *stream) {
  if (nvis > kMaxRows)
    return fail(ARLGPU_ERR_WORKSPACE,
                "arlgpu_grid_noalloc takes at most %lld rows per call (got %lld); use arlgpu_grid with a workspace",
                (long long)kMaxRows, (long long)nvis);
  Geom g;
  ARL_TRY(make_geom(gd, cd, precision, &g));
  if ((int64_t)g.nbins > kMaxBins)
    return fail(ARLGPU_ERR_WORKSPACE,
                "arlgpu_grid_noalloc takes a plan of at most %lld bins per call (this grid has %u channel x "
                "w-plane x uv-tile bins); use arlgpu_grid with a workspace",
                (long long)kMaxBins, g.nbins);
  size_t need = 0;
  ARL_TRY(arlgpu_plan_workspace_bytes(nvis, gd, cd, &need));
  if (need > kScratchBytes)
    return fail(ARLGPU_ERR_WORKSPACE,
                "arlgpu_grid_noalloc: this grid needs %zu bytes of plan scratch, more than its fixed %zu bytes "
                "(at most %lld rows and %lld bins); use arlgpu_grid with a workspace",
                need, kScratchBytes, (long long)kMaxRows, (long long)kMaxBins);
  void *scratch = nullptr;
  ARL_TRY(scratch_for_current_device(&scratch));
  return arlgpu_grid(uvw, frequency, vis, weight, nvis, precision, cf, cd, grid, gd, sumwt, n_bad_dev, scratch,
                     kScratchBytes, stream);
}
