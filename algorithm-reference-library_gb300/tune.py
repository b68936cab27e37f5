"""Autotuner for the gridding kernels.

Times each candidate (gridder variant, degridder variant, subgrid edge) on the
caller's own rows with CUDA events -- plan + grid + degrid, as a step runs --
and leaves the fastest one selected in the library (``arlgpu_set_tuning``).
The subgrid edge changes the tile binning, so every candidate builds its own
plan.
"""
import ctypes
import itertools

import torch

from . import _native as nat
from . import device as dv

GRID_KERNELS = (0, 1)      # shared atomics + TwoSum, band owner + Kahan
DEGRID_KERNELS = (0, 1)    # warp per row, 32-row batches
SUBGRIDS = (32, 48, 64, 96)


def set_tuning(**kw):
    lib = nat.load()
    for k, v in kw.items():
        nat.check(lib.arlgpu_set_tuning(k.encode(), int(v)))


def get_tuning():
    lib = nat.load()
    out = {}
    for k in ('grid_kernel', 'degrid_kernel', 'subgrid'):
        v = ctypes.c_int()
        nat.check(lib.arlgpu_get_tuning(k.encode(), ctypes.byref(v)))
        out[k] = v.value
    return out


def _time_step(uvw, freq, vis, wt, cf_t, cd, gd, precision, reps):
    n = uvw.shape[0]
    dev = uvw.device
    lib = nat.load()
    P = nat.PRECISIONS[precision]
    nbytes = dv.plan_bytes(n, gd, cd)
    ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    grid = torch.empty((gd.nchan, gd.npol, gd.nw, gd.ny, gd.nx), dtype=dv.CDTYPE[precision], device=dev)
    sumwt = torch.empty((gd.nchan, gd.npol), dtype=torch.float64, device=dev)
    out = torch.empty((n, gd.npol), dtype=dv.CDTYPE[precision], device=dev)
    st = torch.cuda.current_stream()
    sp = ctypes.c_void_p(st.cuda_stream)

    def step():
        nat.check(lib.arlgpu_plan_build(nat.ptr(uvw), nat.ptr(freq), n, ctypes.byref(gd), ctypes.byref(cd),
                                        nat.ptr(ws), ws.numel(), None, sp))
        nat.check(lib.arlgpu_grid_planned(nat.ptr(vis), nat.ptr(wt), n, P, nat.ptr(cf_t), ctypes.byref(cd),
                                          nat.ptr(grid), ctypes.byref(gd), nat.ptr(sumwt), nat.ptr(ws), ws.numel(),
                                          sp))
        nat.check(lib.arlgpu_degrid_planned(n, P, nat.ptr(cf_t), ctypes.byref(cd), nat.ptr(grid), ctypes.byref(gd),
                                            nat.ptr(out), nat.ptr(ws), ws.numel(), sp))

    step()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        step()
    e1.record(st)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def stage_times(uvw, freq, vis, wt, cf_t, cd, gd, precision, reps=3):
    """(plan, grid, degrid) milliseconds of one step with the current setting."""
    n = uvw.shape[0]
    dev = uvw.device
    lib = nat.load()
    P = nat.PRECISIONS[precision]
    ws = torch.empty(dv.plan_bytes(n, gd, cd), dtype=torch.uint8, device=dev)
    grid = torch.empty((gd.nchan, gd.npol, gd.nw, gd.ny, gd.nx), dtype=dv.CDTYPE[precision], device=dev)
    sumwt = torch.empty((gd.nchan, gd.npol), dtype=torch.float64, device=dev)
    out = torch.empty((n, gd.npol), dtype=dv.CDTYPE[precision], device=dev)
    st = torch.cuda.current_stream()
    sp = ctypes.c_void_p(st.cuda_stream)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    acc = [0.0, 0.0, 0.0]
    for r in range(reps + 1):
        ev[0].record(st)
        nat.check(lib.arlgpu_plan_build(nat.ptr(uvw), nat.ptr(freq), n, ctypes.byref(gd), ctypes.byref(cd),
                                        nat.ptr(ws), ws.numel(), None, sp))
        ev[1].record(st)
        nat.check(lib.arlgpu_grid_planned(nat.ptr(vis), nat.ptr(wt), n, P, nat.ptr(cf_t), ctypes.byref(cd),
                                          nat.ptr(grid), ctypes.byref(gd), nat.ptr(sumwt), nat.ptr(ws), ws.numel(),
                                          sp))
        ev[2].record(st)
        nat.check(lib.arlgpu_degrid_planned(n, P, nat.ptr(cf_t), ctypes.byref(cd), nat.ptr(grid), ctypes.byref(gd),
                                            nat.ptr(out), nat.ptr(ws), ws.numel(), sp))
        ev[3].record(st)
        torch.cuda.synchronize()
        if r:
            for i in range(3):
                acc[i] += ev[i].elapsed_time(ev[i + 1]) / reps
    return tuple(acc)


def autotune(uvw, freq, vis, wt, cf_t, cd, gd, precision, reps=2, subgrids=SUBGRIDS, grid_kernels=GRID_KERNELS,
             degrid_kernels=DEGRID_KERNELS):
    """Pick the fastest (grid_kernel, degrid_kernel, subgrid) for these rows;
    returns (best setting, {setting: ms per step})."""
    results = {}
    for sg, gk, dk in itertools.product(subgrids, grid_kernels, degrid_kernels):
        try:
            set_tuning(grid_kernel=gk, degrid_kernel=dk, subgrid=sg)
            ms = _time_step(uvw, freq, vis, wt, cf_t, cd, gd, precision, reps)
        except nat.ArlGpuError:
            continue
        results[(gk, dk, sg)] = ms
    best = min(results, key=results.get)
    set_tuning(grid_kernel=best[0], degrid_kernel=best[1], subgrid=best[2])
    return dict(grid_kernel=best[0], degrid_kernel=best[1], subgrid=best[2]), results
