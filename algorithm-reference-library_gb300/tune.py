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

GRID_KERNELS = (0, 1, 2, 4)  # shared atomics + TwoSum, band owner + Kahan, lean atomics, fixed point
DEGRID_KERNELS = (0, 1, 2, 3)  # warp per row, 32-row batches, lean warp per row, lean packed FMA
SUBGRIDS = (32, 48, 64)
CHUNKS = (512, 2048)


def set_tuning(**kw):
    lib = nat.load()
    for k, v in kw.items():
        nat.check(lib.arlgpu_set_tuning(k.encode(), int(v)))


def get_tuning():
    lib = nat.load()
    out = {}
    for k in ('grid_kernel', 'degrid_kernel', 'subgrid', 'chunk', 'persistent', 'dsfft', 'small_rows', 'small_rows_degrid'):
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


def autotune(uvw, freq, vis, wt, cf_t, cd, gd, precision, reps=2, subgrids=SUBGRIDS, chunks=CHUNKS,
             grid_kernels=GRID_KERNELS, degrid_kernels=DEGRID_KERNELS):
    """Pick the fastest (subgrid, chunk) and, for it, the fastest gridder and
    degridder variants, timing plan, grid and degrid separately on these rows.
    Returns (best setting, {setting string: (plan, grid, degrid) ms})."""
    results = {}
    best, best_ms = None, float('inf')
    for sg, ch in itertools.product(subgrids, chunks):
        g_ms, d_ms, plan = {}, {}, None
        for k in sorted(set(grid_kernels) | set(degrid_kernels)):
            try:
                set_tuning(subgrid=sg, chunk=ch, grid_kernel=k if k in grid_kernels else grid_kernels[0],
                           degrid_kernel=k if k in degrid_kernels else degrid_kernels[0])
                t = stage_times(uvw, freq, vis, wt, cf_t, cd, gd, precision, reps)
            except nat.ArlGpuError:
                continue
            plan = t[0] if plan is None else min(plan, t[0])
            if k in grid_kernels:
                g_ms[k] = t[1]
            if k in degrid_kernels:
                d_ms[k] = t[2]
            results['sg%d/chunk%d/kernel%d' % (sg, ch, k)] = tuple(round(x, 4) for x in t)
        if not g_ms or not d_ms:
            continue
        gk = min(g_ms, key=g_ms.get)
        dk = min(d_ms, key=d_ms.get)
        total = plan + g_ms[gk] + d_ms[dk]
        if total < best_ms:
            best_ms = total
            best = dict(grid_kernel=gk, degrid_kernel=dk, subgrid=sg, chunk=ch)
    # persistent grid (resident CTAs looping over chunks) or one CTA per chunk
    step_ms = {}
    for pers in (1, 0):
        set_tuning(persistent=pers, **best)
        t = stage_times(uvw, freq, vis, wt, cf_t, cd, gd, precision, reps)
        results['best/persistent%d' % pers] = tuple(round(x, 4) for x in t)
        step_ms[pers] = sum(t)
    best['persistent'] = min(step_ms, key=step_ms.get)
    best_ms = step_ms[best['persistent']]
    set_tuning(**best)
    best['ms_per_step'] = round(best_ms, 4)
    return best, results
