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
DEGRID_KERNELS = (0, 1, 2, 3, 4)  # warp per row, 32-row batches, lean warp per row, lean packed FMA, TMA-staged
SUBGRIDS = (32, 48, 64)
CHUNKS = (512, 2048)
LANES = (0, 8, 16, 32)                          # lanes per row: per segment, or fixed
SMALL_ROWS = ((1, 1), (2, 2), (4, 4), (2, 4))   # (gridder, degridder) rows per warp, supports <= 8


def set_tuning(**kw):
    lib = nat.load()
    for k, v in kw.items():
        nat.check(lib.arlgpu_set_tuning(k.encode(), int(v)))


def get_tuning():
    lib = nat.load()
    out = {}
    for k in ('grid_kernel', 'degrid_kernel', 'subgrid', 'chunk', 'persistent', 'dsfft', 'small_rows', 'small_rows_degrid',
              'lanes_per_row', 'gather_rows', 'stash_rows'):
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
    degridder variants, then lanes per row (threads per visibility; rows per
    warp for supports up to 8) and the chunk assignment (hardware scheduling,
    a static resident grid, or the device work queue), timing plan, grid and
    degrid separately on these rows.  Returns (best setting, {setting string:
    (plan, grid, degrid) ms})."""
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
    # Lanes per row (threads per visibility): chosen per segment by its
    # largest support (0), or fixed for every segment; for supports up to 8
    # also the rows-per-warp keys.  Gridder and degridder are timed apart, so
    # each keeps its own best.
    set_tuning(persistent=2, **best)
    lanes_opts = [dict(lanes_per_row=v) for v in LANES]
    if cd.support <= 8:
        lanes_opts += [dict(lanes_per_row=0, small_rows=a, small_rows_degrid=b) for a, b in SMALL_ROWS]
    g_best, d_best = None, None
    for opt in lanes_opts:
        full = dict(dict(lanes_per_row=0, small_rows=2, small_rows_degrid=4), **opt)
        set_tuning(**full)
        t = stage_times(uvw, freq, vis, wt, cf_t, cd, gd, precision, reps)
        results['lanes/' + '/'.join('%s%d' % (k, v) for k, v in sorted(opt.items()))] = tuple(round(x, 4) for x in t)
        if g_best is None or t[1] < g_best[0]:
            g_best = (t[1], full)
        if d_best is None or t[2] < d_best[0]:
            d_best = (t[2], full)
    # One lanes_per_row key serves both kernels: keep the one whose grid +
    # degrid sum is smallest among the two winners.
    cands = {}
    for _, full in (g_best, d_best):
        set_tuning(**full)
        t = stage_times(uvw, freq, vis, wt, cf_t, cd, gd, precision, reps)
        cands[tuple(sorted(full.items()))] = t[1] + t[2]
    best.update(dict(min(cands, key=cands.get)))
    # Chunk assignment: one CTA per chunk (hardware block scheduling, 0), a
    # resident grid taking every gridDim-th chunk (1), or a resident grid fed
    # by the device work queue (2).
    step_ms = {}
    for pers in (0, 1, 2):
        set_tuning(persistent=pers, **best)
        t = stage_times(uvw, freq, vis, wt, cf_t, cd, gd, precision, reps)
        results['best/persistent%d' % pers] = tuple(round(x, 4) for x in t)
        step_ms[pers] = sum(t)
    best['persistent'] = min(step_ms, key=step_ms.get)
    best_ms = step_ms[best['persistent']]
    set_tuning(**best)
    best['ms_per_step'] = round(best_ms, 4)
    return best, results
