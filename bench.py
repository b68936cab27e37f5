"""Benchmark of ARL's gridding hot path on GB300.

Workload (default, --workload C2): W-projection grid + degrid of the C2
observation -- 256 antennas in a 5 km-radius disk, 4 channels 100-120 MHz, 120
times over +/-2 h, 1024 x 1024 x 4-channel grid, cellsize 5e-4 rad, 64 w-planes
with support growing 8 -> 32 with |w|, oversampling 8, 50 point sources.  Rows
whose 32 x 32 window would leave the grid are cut (4.34 M of 15.67 M rows stay).

One step = map + bin the rows (FP64), grid them (zeroed grid), degrid them:
arlgpu_plan_build + arlgpu_grid_planned + arlgpu_degrid_planned on device
tensors.  `value` = rows / step time (vis/s), FP32C path.  The FP64 path, the
end-to-end figure through the C ABI with pinned host buffers, the roofline of
the dominant kernel, clocks and the CPU baseline are reported alongside.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

With --gpus N > 1 (launched by torch.distributed.run) every rank runs its own
replica of the workload (no data-path collective); value = N * rows / max time.
"""
import argparse
import ctypes
import importlib
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "vis/s grid+degrid FP32 vs FP64 GPU path at ≤1e-5 rel err; % of HBM roofline"
L2_FLUSH_BYTES = 256 << 20
FALLBACK_HBM_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=10)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--workload', default='C2')
    ap.add_argument('--no-fp64', action='store_true', help='skip the FP64 comparison arm')
    ap.add_argument('--no-cpu', action='store_true', help='skip the CPU baseline')
    ap.add_argument('--cpu-seconds', type=float, default=12.0, help='CPU-baseline time budget')
    ap.add_argument('--no-tune', action='store_true', help='keep the library\'s default kernel variants')
    ap.add_argument('--no-c5', action='store_true',
                    help='skip the sub-record of the largest single-GPU workload (C5 w-stacking)')
    ap.add_argument('--no-stages', action='store_true',
                    help='skip the invert_2d / predict_2d / gradient-step rates')
    ap.add_argument('--profile-rows', type=int, default=0,
                    help='profiling case for ncu: the workload subsampled to this many rows, --warmup + --steps '
                         'untimed steps with the library defaults, no other arms')
    ap.add_argument('--tuning', action='append', default=[], metavar='KEY=VALUE',
                    help='profiling case only: a kernel-variant setting (arlgpu_set_tuning) to profile instead of '
                         'the default, e.g. degrid_kernel=4; repeatable')
    ap.add_argument('--wstack-profile', action='store_true',
                    help='profiling case for ncu: a 2,000,000-row PSWF w-stack invert onto 4 slices of 4096^2 '
                         '(FP32C, 2.3 GB on the device), run --warmup + --steps times, no other arms')
    ap.add_argument('--transform', type=int, default=0, metavar='N',
                    help='time the FP32C inverse 2-D transform with grid correction alone on two random N^2 '
                         'planes: the double-single FFT against cuFFT complex128 (also a small ncu case)')
    return ap.parse_args()


# ---------------------------------------------------------------------------
# Distributed plumbing (replicas only)
# ---------------------------------------------------------------------------
def dist_setup(torch):
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    if world > 1:
        import torch.distributed as tdist
        backend = 'nccl' if torch.cuda.is_available() else 'gloo'
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        tdist.init_process_group(backend)
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return world, rank, local


def barrier(torch, world):
    if world > 1:
        import torch.distributed as tdist
        if torch.cuda.is_available():
            tdist.barrier(device_ids=[torch.cuda.current_device()])
        else:
            tdist.barrier()


def max_over_ranks(torch, world, x, device=None):
    if world == 1:
        return x
    import torch.distributed as tdist
    if device is None:
        device = 'cuda' if torch.cuda.is_available() else 'cpu'
    t = torch.tensor([x], dtype=torch.float64, device=device)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# Clocks sampled during the timed region
# ---------------------------------------------------------------------------
class Clocks:
    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
         'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
         'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu_index, period_ms=50):
        self.idx = gpu_index
        self.f = tempfile.NamedTemporaryFile('w+', suffix='.csv', delete=False)
        try:
            self.p = subprocess.Popen(['nvidia-smi', '-i', str(gpu_index), '--query-gpu=' + self.Q,
                                       '--format=csv,noheader,nounits', '-lms', str(period_ms)],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.p = None
        self._wait_lines(1, 5.0)  # sampling is running before the caller's timed region starts

    def _lines(self):
        with open(self.f.name) as fh:
            return sum(1 for line in fh if line.count(',') >= 8)

    def _wait_lines(self, n, seconds):
        t0 = time.time()
        while self.p is not None and self.p.poll() is None and time.time() - t0 < seconds:
            if self._lines() >= n:
                return
            time.sleep(0.01)

    def stop(self):
        if self.p is None:
            return None
        self._wait_lines(self._lines() + 1, 1.0)  # one sample after the timed region ends
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(',')]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == 'active':
                    reasons.add(n)
        os.unlink(self.f.name)
        if not sm:
            return None
        return {'sm_mhz': statistics.median(sm), 'sm_max_mhz': max(mx), 'reasons': sorted(reasons),
                'samples': len(sm)}


def measured_hbm():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            return float(json.load(f)['hbm_gbs']), 'measured'
    except (OSError, ValueError, KeyError):
        return FALLBACK_HBM_GBS, 'fallback'


def launch_insts(kernel, nrows):
    """Warp instructions of one `kernel` launch over nrows rows from the
    committed one-pass ncu capture (profiles/ncu_inst.txt), scaled by rows when
    the capture ran on a different row count; None when absent."""
    path = os.path.join(ROOT, 'profiles', 'ncu_inst.txt')
    try:
        for line in open(path):
            parts = line.split()
            if len(parts) == 3 and parts[0] == kernel:
                rows, k = float(parts[1]), float(parts[2])
                return {'inst': k * nrows / rows, 'captured_rows': int(rows), 'scaled': rows != nrows}
    except (OSError, ValueError):
        pass
    return None


def launch_traffic(kernel, nrows):
    """DRAM bytes of one `kernel` launch over nrows rows from the committed ncu
    summary (profiles/ncu_dram.txt: kernel, rows captured, bytes), scaled by
    rows when the capture ran on a row subsample; None when absent."""
    path = os.path.join(ROOT, 'profiles', 'ncu_dram.txt')
    try:
        for line in open(path):
            parts = line.split()
            if len(parts) == 3 and parts[0] == kernel:
                rows, b = float(parts[1]), float(parts[2])
                return {'bytes': b * nrows / rows, 'captured_rows': int(rows),
                        'scaled': rows != nrows}
    except (OSError, ValueError):
        pass
    return None


def issue_roofline(torch, kernel, nrows, kms, clk):
    """The dominant kernel against the instruction-issue ceiling (one warp
    instruction per cycle per scheduler, 4 per SM, at the SM clock sampled
    during the timed region): its ncu instruction count per launch over the
    CUDA-event launch time measured here."""
    ins = launch_insts(kernel, nrows)
    if ins is None or not torch.cuda.is_available():
        return None
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    mhz = (clk or {}).get('sm_mhz') or 2070.0
    peak = sms * 4 * mhz * 1e6
    achieved = ins['inst'] / (kms / 1e3)
    return {'bound': 'issue', 'kernel': kernel, 'achieved': achieved, 'peak': peak, 'unit': 'warp-inst/s',
            'frac': achieved / peak, 'inst_per_launch': ins['inst'],
            'inst_source': 'ncu smsp__inst_executed.sum (one pass), %d-row capture%s' %
                           (ins['captured_rows'], ', scaled by rows' if ins['scaled'] else ''),
            'peak_source': '%d SMs x 4 schedulers x %.0f MHz' % (sms, mhz)}


# ---------------------------------------------------------------------------
# Workload
# ---------------------------------------------------------------------------
def build_context(arl, torch, w, precision, device):
    dv = arl.device
    if w['kernel'] == 'wproj':
        # C2: one image channel per visibility channel
        im = arl.create_image(npixel=w['npixel'], cellsize=w['cellsize'], frequency=numpy.asarray(w['freqs']),
                              channel_bandwidth=numpy.array([w['channel_bandwidth']]),
                              phasecentre=arl.PhaseCentre(0.0, -45.0))
    else:
        # PSWF workloads: the workload's own (MFS) image with its polarisations
        im = arl.simulation.workload_image(arl, w)
    if w['kernel'] == 'wproj':
        gcf, cf = arl.create_awterm_convolutionfunction(im, nw=w['nwplanes'], wstep=w['wstep'],
                                                        oversampling=w['oversampling'], support=w['support'],
                                                        plane_support=w['plane_support'])
    else:
        gcf, cf = arl.create_pswf_convolutionfunction(im, oversampling=w['oversampling'], support=w['support'])
    gd = dv.grid_desc(arl.kernels._grid_wcs(im, 1, 1e15), (im.nchan, im.npol, 1, w['npixel'], w['npixel']))
    cf_t, cs, ps, psup = dv.device_cf(cf, precision, device)
    cd = dv.cf_desc(cf.grid_wcs, cf.data.shape, cs, ps, psup, table=cf_t)
    n = w['uvw'].shape[0]
    npol = w['npol']
    ctx = dict(precision=precision, n=n, gd=gd, cd=cd, cf_t=cf_t, psup=psup, im=im, cf=cf, gcf=gcf)
    ctx['uvw'] = torch.as_tensor(w['uvw'], device=device)
    ctx['freq'] = torch.as_tensor(w['frequency'], device=device)
    ctx['vis'] = w['vis'].to(device=device, dtype=dv.CDTYPE[precision]).contiguous()
    ctx['wt'] = torch.ones((w['uvw'].shape[0], w['npol']), dtype=dv.RDTYPE[precision], device=device)
    ctx['grid'] = torch.empty((gd.nchan, gd.npol, gd.nw, gd.ny, gd.nx), dtype=dv.CDTYPE[precision], device=device)
    ctx['sumwt'] = torch.empty((gd.nchan, gd.npol), dtype=torch.float64, device=device)
    ctx['out'] = torch.empty((n, npol), dtype=dv.CDTYPE[precision], device=device)
    ctx['nbad'] = torch.zeros(1, dtype=torch.int64, device=device)
    nbytes = dv.plan_bytes(n, gd, cd)
    ctx['ws'] = torch.empty(nbytes, dtype=torch.uint8, device=device)
    return ctx


def run_step(arl, ctx, stream, ev=None):
    """plan + grid + degrid; ev = (e0, e1, e2, e3) events recorded between stages."""
    nat = arl._native
    lib = nat.load()
    P = nat.PRECISIONS[ctx['precision']]
    gd, cd, ws = ctx['gd'], ctx['cd'], ctx['ws']
    sp = ctypes.c_void_p(stream.cuda_stream)
    if ev:
        ev[0].record(stream)
    nat.check(lib.arlgpu_plan_build(nat.ptr(ctx['uvw']), nat.ptr(ctx['freq']), ctx['n'], ctypes.byref(gd),
                                    ctypes.byref(cd), nat.ptr(ws), ws.numel(), nat.ptr(ctx['nbad']), sp))
    if ev:
        ev[1].record(stream)
    nat.check(lib.arlgpu_grid_planned(nat.ptr(ctx['vis']), nat.ptr(ctx['wt']), ctx['n'], P, nat.ptr(ctx['cf_t']),
                                      ctypes.byref(cd), nat.ptr(ctx['grid']), ctypes.byref(gd), nat.ptr(ctx['sumwt']),
                                      nat.ptr(ws), ws.numel(), sp))
    if ev:
        ev[2].record(stream)
    nat.check(lib.arlgpu_degrid_planned(ctx['n'], P, nat.ptr(ctx['cf_t']), ctypes.byref(cd), nat.ptr(ctx['grid']),
                                        ctypes.byref(gd), nat.ptr(ctx['out']), nat.ptr(ws), ws.numel(), sp))
    if ev:
        ev[3].record(stream)


def timed_steps(arl, torch, ctx, steps, warmup, world, flush):
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        run_step(arl, ctx, stream)
    torch.cuda.synchronize()
    assert int(ctx['nbad'].item()) == 0
    lib = arl._native.load()
    launches0 = lib.arlgpu_kernel_launches()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(steps)]
    barrier(torch, world)
    torch.cuda.synchronize()
    for k in range(steps):
        flush.zero_()                       # L2 flush, outside the timed events
        run_step(arl, ctx, stream, evs[k])
    torch.cuda.synchronize()
    barrier(torch, world)
    launches = lib.arlgpu_kernel_launches() - launches0
    plan = [e[0].elapsed_time(e[1]) for e in evs]
    grid = [e[1].elapsed_time(e[2]) for e in evs]
    degrid = [e[2].elapsed_time(e[3]) for e in evs]
    total = sum(e[0].elapsed_time(e[3]) for e in evs)
    return dict(total_ms=total, plan_ms=sum(plan) / steps, grid_ms=sum(grid) / steps, degrid_ms=sum(degrid) / steps,
                launches=int(launches))


def e2e_steps(arl, torch, ctx, steps, warmup):
    """Same step through the C ABI from pinned host buffers: H2D of uvw,
    frequency, vis, weight; D2H of the grid and the degridded vis.  The
    copies the next stage does not need yet run on a second stream: vis and
    weight go up after uvw and frequency (so the plan's inputs get the whole
    link) while the plan runs, and the grid comes down while the degridder
    reads it."""
    nat = arl._native
    lib = nat.load()
    host = {k: ctx[k].cpu().pin_memory() for k in ('uvw', 'freq', 'vis', 'wt')}
    gh = torch.empty(ctx['grid'].shape, dtype=ctx['grid'].dtype).pin_memory()
    oh = torch.empty(ctx['out'].shape, dtype=ctx['out'].dtype).pin_memory()
    stream = torch.cuda.current_stream()
    side = torch.cuda.Stream(device=ctx['uvw'].device)
    h2d = sum(t.numel() * t.element_size() for t in host.values())
    d2h = gh.numel() * gh.element_size() + oh.numel() * oh.element_size()
    P = nat.PRECISIONS[ctx['precision']]
    gd, cd, ws = ctx['gd'], ctx['cd'], ctx['ws']
    sp = ctypes.c_void_p(stream.cuda_stream)

    def one():
        ctx['uvw'].copy_(host['uvw'], non_blocking=True)
        ctx['freq'].copy_(host['freq'], non_blocking=True)
        side.wait_stream(stream)  # the previous step is done with vis, wt and the grid; uvw is up
        with torch.cuda.stream(side):
            ctx['vis'].copy_(host['vis'], non_blocking=True)
            ctx['wt'].copy_(host['wt'], non_blocking=True)
            rows_in = torch.cuda.current_stream().record_event()
        nat.check(lib.arlgpu_plan_build(nat.ptr(ctx['uvw']), nat.ptr(ctx['freq']), ctx['n'], ctypes.byref(gd),
                                        ctypes.byref(cd), nat.ptr(ws), ws.numel(), nat.ptr(ctx['nbad']), sp))
        stream.wait_event(rows_in)
        nat.check(lib.arlgpu_grid_planned(nat.ptr(ctx['vis']), nat.ptr(ctx['wt']), ctx['n'], P,
                                          nat.ptr(ctx['cf_t']), ctypes.byref(cd), nat.ptr(ctx['grid']),
                                          ctypes.byref(gd), nat.ptr(ctx['sumwt']), nat.ptr(ws), ws.numel(), sp))
        gridded = stream.record_event()
        with torch.cuda.stream(side):
            torch.cuda.current_stream().wait_event(gridded)
            gh.copy_(ctx['grid'], non_blocking=True)
        nat.check(lib.arlgpu_degrid_planned(ctx['n'], P, nat.ptr(ctx['cf_t']), ctypes.byref(cd),
                                            nat.ptr(ctx['grid']), ctypes.byref(gd), nat.ptr(ctx['out']),
                                            nat.ptr(ws), ws.numel(), sp))
        oh.copy_(ctx['out'], non_blocking=True)
        stream.wait_stream(side)

    for _ in range(warmup):
        one()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        one()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps, h2d, d2h


def e2e_pipelined(arl, torch, ctx, steps, warmup):
    """A stream of steps through the C ABI from pinned host buffers, as a
    caller gridding one batch of rows after another would run it: every step
    uploads its uvw, frequency, vis and weight and reads back its grid and
    degridded vis.  Inputs, outputs and plan workspace are double-buffered on
    the device; consecutive steps run on two compute streams (independent
    batches, so step k + 1's plan and grid can share the SMs with step k's
    degrid), step k + 1's uploads run on one copy stream and step k's
    read-backs on another.  An input set is reused once the gridder of the
    step before last has read it, an output set once its read-back is done.
    Returns (ms per step over the timed steps, first upload to last
    read-back; ms per step of the same two-stream compute with the inputs
    resident and no copies)."""
    nat = arl._native
    lib = nat.load()
    host = {k: ctx[k].cpu().pin_memory() for k in ('uvw', 'freq', 'vis', 'wt')}
    gh = torch.empty(ctx['grid'].shape, dtype=ctx['grid'].dtype).pin_memory()
    oh = torch.empty(ctx['out'].shape, dtype=ctx['out'].dtype).pin_memory()
    keys = ('uvw', 'freq', 'vis', 'wt', 'grid', 'out', 'sumwt', 'ws', 'nbad')
    sets = [{k: ctx[k] for k in keys}, {k: torch.empty_like(ctx[k]) for k in keys}]
    sets[1]['nbad'].zero_()
    cur = torch.cuda.current_stream()
    dev = ctx['uvw'].device
    comp = [torch.cuda.Stream(device=dev), torch.cuda.Stream(device=dev)]
    up, down = torch.cuda.Stream(device=dev), torch.cuda.Stream(device=dev)
    P = nat.PRECISIONS[ctx['precision']]
    gd, cd = ctx['gd'], ctx['cd']
    inputs_free = [None, None]   # event: the gridder that last read the set has run
    outputs_free = [None, None]  # event: the set's last read-back is done

    def compute(b, st, plan_in=None, rows_in=None, free=None):
        sp = ctypes.c_void_p(st.cuda_stream)
        if plan_in is not None:
            st.wait_event(plan_in)
        nat.check(lib.arlgpu_plan_build(nat.ptr(b['uvw']), nat.ptr(b['freq']), ctx['n'], ctypes.byref(gd),
                                        ctypes.byref(cd), nat.ptr(b['ws']), b['ws'].numel(), nat.ptr(b['nbad']), sp))
        if rows_in is not None:
            st.wait_event(rows_in)
        if free is not None:
            st.wait_event(free)
        nat.check(lib.arlgpu_grid_planned(nat.ptr(b['vis']), nat.ptr(b['wt']), ctx['n'], P, nat.ptr(ctx['cf_t']),
                                          ctypes.byref(cd), nat.ptr(b['grid']), ctypes.byref(gd),
                                          nat.ptr(b['sumwt']), nat.ptr(b['ws']), b['ws'].numel(), sp))
        gridded = st.record_event()
        nat.check(lib.arlgpu_degrid_planned(ctx['n'], P, nat.ptr(ctx['cf_t']), ctypes.byref(cd),
                                            nat.ptr(b['grid']), ctypes.byref(gd), nat.ptr(b['out']),
                                            nat.ptr(b['ws']), b['ws'].numel(), sp))
        return gridded, st.record_event()

    def one(k):
        s = k % 2
        b = sets[s]
        with torch.cuda.stream(up):
            if inputs_free[s] is not None:
                up.wait_event(inputs_free[s])
            b['uvw'].copy_(host['uvw'], non_blocking=True)
            b['freq'].copy_(host['freq'], non_blocking=True)
            plan_in = up.record_event()
            b['vis'].copy_(host['vis'], non_blocking=True)
            b['wt'].copy_(host['wt'], non_blocking=True)
            rows_in = up.record_event()
        gridded, degridded = compute(b, comp[s], plan_in, rows_in, outputs_free[s])
        inputs_free[s] = gridded
        with torch.cuda.stream(down):
            down.wait_event(gridded)
            gh.copy_(b['grid'], non_blocking=True)
            down.wait_event(degridded)
            oh.copy_(b['out'], non_blocking=True)
            outputs_free[s] = down.record_event()

    def timed(fn, nsteps):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(cur)
        for st in comp + [up, down]:
            st.wait_stream(cur)
        fn(nsteps)
        for st in comp + [up, down]:
            cur.wait_stream(st)
        e1.record(cur)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / nsteps

    for k in range(warmup):
        one(k)
    ms = timed(lambda m: [one(k) for k in range(warmup, warmup + m)], steps)
    assert int(sets[0]['nbad'].item()) == 0 and int(sets[1]['nbad'].item()) == 0

    def resident(m):
        for k in range(m):
            compute(sets[k % 2], comp[k % 2])
    ms_resident = timed(resident, steps)
    return ms, ms_resident


def _events(torch, n):
    return [torch.cuda.Event(enable_timing=True) for _ in range(n)]


def stage_rates(arl, torch, ctx, steps, warmup, flush):
    """vis/s of invert_2d (plan + grid + inverse transform with grid correction
    and sumwt normalisation: double-single on FP32C, complex128 on FP64) and predict_2d (gcf multiply + forward FFT +
    degrid) on the bench's device-resident rows; L2 flushed between steps."""
    nat = arl._native
    P = nat.PRECISIONS[ctx['precision']]
    gd, cd, ws = ctx['gd'], ctx['cd'], ctx['ws']
    dev = ctx['uvw'].device
    gcf = arl.gridding._gcf_t(ctx['gcf'], dev)
    nb = gd.nchan * gd.npol
    image = torch.empty((gd.nchan, gd.npol, gd.ny, gd.nx), dtype=torch.float64, device=dev)
    fftbuf = torch.empty(nb * gd.ny * gd.nx, dtype=torch.complex128, device=dev)
    model = torch.zeros_like(image)
    model[..., gd.ny // 2 - 40:gd.ny // 2 + 40:7, gd.nx // 2 - 40:gd.nx // 2 + 40:5] = 1.0
    stream = torch.cuda.current_stream()
    sp = nat.stream_ptr()

    def invert():
        nat.call('arlgpu_plan_build', nat.ptr(ctx['uvw']), nat.ptr(ctx['freq']), ctx['n'], ctypes.byref(gd),
                 ctypes.byref(cd), nat.ptr(ws), ws.numel(), nat.ptr(ctx['nbad']), sp)
        nat.call('arlgpu_grid_planned', nat.ptr(ctx['vis']), nat.ptr(ctx['wt']), ctx['n'], P, nat.ptr(ctx['cf_t']),
                 ctypes.byref(cd), nat.ptr(ctx['grid']), ctypes.byref(gd), nat.ptr(ctx['sumwt']), nat.ptr(ws),
                 ws.numel(), sp)
        nat.call('arlgpu_fft_grid_to_image', nat.ptr(ctx['grid']), ctypes.byref(gd), P, nat.ptr(gcf),
                 nat.ptr(ctx['sumwt']), nat.ptr(image), None, nat.ptr(fftbuf), sp)

    def predict():
        nat.call('arlgpu_plan_build', nat.ptr(ctx['uvw']), nat.ptr(ctx['freq']), ctx['n'], ctypes.byref(gd),
                 ctypes.byref(cd), nat.ptr(ws), ws.numel(), nat.ptr(ctx['nbad']), sp)
        nat.call('arlgpu_fft_image_to_grid', nat.ptr(model), nat.ptr(gcf), ctypes.byref(gd), P, nat.ptr(ctx['grid']),
                 sp)
        nat.call('arlgpu_degrid_planned', ctx['n'], P, nat.ptr(ctx['cf_t']), ctypes.byref(cd), nat.ptr(ctx['grid']),
                 ctypes.byref(gd), nat.ptr(ctx['out']), nat.ptr(ws), ws.numel(), sp)

    out = {}
    for name, fn in (('invert_2d', invert), ('predict_2d', predict)):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        ev = [_events(torch, 2) for _ in range(steps)]
        for k in range(steps):
            flush.zero_()
            ev[k][0].record(stream)
            fn()
            ev[k][1].record(stream)
        torch.cuda.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in ev) / steps
        out[name] = {'value': ctx['n'] / (ms / 1e3), 'unit': 'vis/s', 'ms': ms}
    return out


def gradient_step_rate(arl, torch, device, steps, warmup, flush):
    """vis/s of one chi^2 gradient step of the gain-solve workload (C4: 128
    antennas, 8 channels summed onto a 2048^2 image, 240 times, PSWF 8 x 8):
    predict (FFT + degrid), the gain chi^2 with its Wirtinger gradients, and
    the adjoint (grid + FFT) for the image gradient, FP32C."""
    sim = arl.simulation
    w = sim.make_workload('C4')
    im = sim.workload_image(arl, w)
    gcfcf = arl.create_pswf_convolutionfunction(im, oversampling=w['oversampling'], support=w['support'])
    n = w['uvw'].shape[0]
    dvis = arl.DeviceVisibility(torch.as_tensor(w['uvw'], device=device),
                                torch.as_tensor(w['frequency'], device=device),
                                torch.zeros((n, 1), dtype=torch.complex64, device=device),
                                torch.ones((n, 1), dtype=torch.float32, device=device))
    op = arl.autograd.GriddingOperator(dvis, im, gcfcf, precision='fp32c')
    model = torch.as_tensor(w['model_image'], device=device)
    gains = torch.as_tensor(w['gains'], device=device)
    a1 = torch.as_tensor(w['antenna1'].astype(numpy.int32), device=device)
    a2 = torch.as_tensor(w['antenna2'].astype(numpy.int32), device=device)
    vobs = sim.observe(op.predict(model), gains, a1, a2, w['noise'], seed=1004)
    x = 0.7 * model
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        arl.autograd.gain_chi2_step(x, gains, vobs, op, a1, a2)
    torch.cuda.synchronize()
    ev = [_events(torch, 2) for _ in range(steps)]
    for k in range(steps):
        flush.zero_()
        ev[k][0].record(stream)
        arl.autograd.gain_chi2_step(x, gains, vobs, op, a1, a2)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in ev) / steps
    # Error of the timed FP32C step against the same step in complex128 (FP64
    # operator, FP64 inputs), after the timing.
    c32, gx32, gg32 = arl.autograd.gain_chi2_step(x, gains, vobs, op, a1, a2)
    dvis64 = arl.DeviceVisibility(dvis.uvw, dvis.frequency, torch.zeros((n, 1), dtype=torch.complex128, device=device),
                                  torch.ones((n, 1), dtype=torch.float64, device=device))
    op64 = arl.autograd.GriddingOperator(dvis64, im, gcfcf, precision='fp64')
    c64, gx64, gg64 = arl.autograd.gain_chi2_step(x.double(), gains.to(torch.complex128), vobs.to(torch.complex128),
                                                  op64, a1, a2)

    def err(a, b):
        d = (a.to(b.dtype) - b).abs()
        return {'max_rel': float(d.max() / b.abs().max()),
                'rms_rel': float(d.pow(2).mean().sqrt() / b.abs().pow(2).mean().sqrt())}
    errs = {'chi2_rel': float(abs(float(c32) - float(c64)) / abs(float(c64))), 'image_gradient': err(gx32, gx64),
            'gain_gradient': err(gg32, gg64), 'against': 'the same step through the FP64 (complex128) operator'}
    del op64, dvis64
    return {'value': n / (ms / 1e3), 'unit': 'vis/s', 'ms': ms, 'err_vs_fp64': errs,
            'workload': 'C4 gain solve: 128 antennas / 2 km disk, 8 chan 100-120 MHz summed, 240 times, 2048^2, '
                        'PSWF S=8 O=8, %d rows; chi^2 + image and gain gradients, FP32C' % n}


# ---------------------------------------------------------------------------
# CPU baseline: the oracle's reference-faithful per-row loops
# ---------------------------------------------------------------------------
_W = {}


def _cpu_init(cf, img, nz, wstep, O, S):
    """Per-process state of the CPU baseline: the kernel table and geometry."""
    from oracle import arl_oracle as orc
    _W.update(cf=cf, ccf=numpy.conjugate(cf), gax=orc.grid_axes(img),
              cax=orc.cf_axes(img, O, S, nz=nz, zstep=wstep))
    _W['grid'] = numpy.zeros(_W['gax']['shape'], complex)
    _W['sumwt'] = numpy.zeros(_W['gax']['shape'][:2])


def _cpu_worker(args):
    """Grid then degrid rows with the oracle's per-row loops, each for half of
    `budget` seconds; returns (rows gridded, s, rows degridded, s)."""
    uvw, freq, vis, wt, budget = args
    from oracle import arl_oracle as orc
    maps = orc.convolution_mapping(uvw, freq, _W['gax'], _W['cax'])
    n = uvw.shape[0]
    chunk = 256
    t0 = time.perf_counter()
    done_g = 0
    while done_g < n and time.perf_counter() - t0 < budget / 2:
        e = min(done_g + chunk, n)
        orc.grid_loop(vis[done_g:e], wt[done_g:e], tuple(a[done_g:e] for a in maps), _W['cf'], _W['gax']['shape'],
                      out=(_W['grid'], _W['sumwt']), ccf=_W['ccf'])
        done_g = e
    tg = time.perf_counter() - t0
    t1 = time.perf_counter()
    done_d = 0
    while done_d < n and time.perf_counter() - t1 < budget / 2:
        e = min(done_d + chunk, n)
        orc.degrid_loop(_W['grid'], tuple(a[done_d:e] for a in maps), _W['cf'])
        done_d = e
    td = time.perf_counter() - t1
    return done_g, tg, done_d, td


class CpuBaseline:
    """The oracle's reference-faithful loops (complex128, per-row, NumPy FFT)
    on `procs` processes (spawned, so no process inherits a CUDA context)."""

    def __init__(self, w, cf, procs):
        from oracle import arl_oracle as orc
        self.w = w
        self.procs = procs
        img = orc.image_geometry(w['npixel'], w['cellsize'], len(w['freqs']), w['npol'], w['freqs'][0],
                                 w['channel_bandwidth'])
        init = (cf, img, cf.shape[2], float(w.get('wstep', 1e15)), w['oversampling'], w['support'])
        self.vis = w['vis'].cpu().numpy() if hasattr(w['vis'], 'cpu') else numpy.asarray(w['vis'])
        self.rng = numpy.random.default_rng(7)
        if procs == 1:
            _cpu_init(*init)
            self.pool = None
        else:
            self.pool = mp.get_context('spawn').Pool(procs, initializer=_cpu_init, initargs=init)

    def rate(self, budget, sample_rows):
        """Summed rows/s over the processes of grid+degrid, 1/(1/r_grid + 1/r_degrid)."""
        n = self.w['uvw'].shape[0]
        jobs = []
        for _ in range(self.procs):
            sel = numpy.sort(self.rng.choice(n, min(sample_rows, n), replace=False))
            jobs.append((self.w['uvw'][sel], self.w['frequency'][sel], self.vis[sel], self.w['weight'][sel], budget))
        res = [_cpu_worker(jobs[0])] if self.pool is None else self.pool.map(_cpu_worker, jobs)
        rate, rows = 0.0, 0
        for done_g, tg, done_d, td in res:
            rate += 1.0 / (tg / done_g + td / done_d)
            rows += done_g + done_d
        return rate, rows

    def close(self):
        if self.pool is not None:
            self.pool.close()
            self.pool.join()


def cpu_model():
    try:
        for line in open('/proc/cpuinfo'):
            if line.lower().startswith(('model name', 'cpu part')):
                return line.split(':', 1)[1].strip()
    except OSError:
        pass
    return 'unknown'


def _err(a, b):
    """Max-norm and RMS error of a against the oracle result b, each relative
    to b's own max-norm / RMS."""
    return {'max_rel': float(numpy.max(numpy.abs(a - b)) / numpy.max(numpy.abs(b))),
            'rms_rel': float(numpy.sqrt(numpy.mean(numpy.abs(a - b) ** 2)) / numpy.sqrt(numpy.mean(numpy.abs(b) ** 2)))}


def _img_err(a, b, gcf):
    """Image error over the whole image and over the inner region where the
    grid correction is <= 100 (the PSWF correction grows to ~6e4 at the field
    edge and multiplies the FP32 rounding there)."""
    e = _err(a, b)
    inner = numpy.broadcast_to(gcf, b.shape) <= 100.0
    d = numpy.abs(a - b)
    e['inner_max_rel'] = float(d[inner].max() / numpy.max(numpy.abs(b)))
    e['inner_fraction'] = float(inner.mean())
    return e


def oracle_errors(arl, torch, w, ctx, nsub=20000):
    """Max-norm and RMS error against the complex128 oracle, on a seeded row
    subsample of the workload, of every result the bench times on it: the
    grid and the degridded rows (this context's precision, the oracle's own
    w-kernels), the invert_2d image (plan + grid + inverse transform + grid
    correction + sumwt normalisation) and the predict_2d rows of a model image."""
    from oracle import arl_oracle as orc
    dv = arl.device
    rng = numpy.random.default_rng(11)
    n = w['uvw'].shape[0]
    sel = numpy.sort(rng.choice(n, min(nsub, n), replace=False))
    uvw, f = w['uvw'][sel], w['frequency'][sel]
    vis = w['vis'].cpu().numpy()[sel]
    wt = numpy.ones(vis.shape)
    img = orc.image_geometry(w['npixel'], w['cellsize'], len(w['freqs']), w['npol'], w['freqs'][0],
                             w['channel_bandwidth'])
    nz = int(w.get('nwplanes', 1))
    wstep = float(w.get('wstep', 1e15))
    if w['kernel'] == 'wproj':
        ogcf, ocf = orc.create_awterm_cf(img, nw=nz, wstep=wstep, oversampling=w['oversampling'],
                                         support=w['support'])
        ocf = orc.crop_cf_planes(ocf, w['plane_support'])
    else:
        ogcf, ocf = orc.create_pswf_cf(img['nchan'], img['npol'], img['ny'], img['nx'], w['oversampling'],
                                       w['support'])
    gax = orc.grid_axes(img)
    cax = orc.cf_axes(img, w['oversampling'], w['support'], nz=nz, zstep=wstep)
    maps = orc.convolution_mapping(uvw, f, gax, cax)
    g_ref, _ = orc.grid_vec(vis, wt, maps, ocf, gax['shape'])
    d_ref = orc.degrid_vec(g_ref, maps, ocf)
    p = ctx['precision']
    dev = ctx['uvw'].device
    t_uvw = torch.as_tensor(uvw, device=dev)
    t_f = torch.as_tensor(f, device=dev)
    t_v = torch.as_tensor(vis, device=dev).to(dv.CDTYPE[p])
    t_w = torch.as_tensor(wt, device=dev).to(dv.RDTYPE[p])
    g, _, _ = dv.grid(t_uvw, t_f, t_v, t_w, ctx['cf_t'], ctx['cd'], ctx['gd'], p)
    gr = torch.as_tensor(g_ref, device=dev).to(dv.CDTYPE[p])
    d, _ = dv.degrid(t_uvw, t_f, gr, ctx['cf_t'], ctx['cd'], ctx['gd'], p)
    g = g.to(torch.complex128).cpu().numpy()
    d = d.to(torch.complex128).cpu().numpy()
    out = {'rows': int(sel.size), 'precision': p, 'grid': _err(g, g_ref), 'degrid': _err(d, d_ref)}
    # invert_2d and predict_2d through the package's public functions on the
    # same rows (device-resident), against the oracle's invert_2d / predict_2d
    dvis = arl.DeviceVisibility(t_uvw, t_f, t_v, t_w)
    gcfcf = (ctx['gcf'], ctx['cf'])
    dirty, _ = arl.invert_2d(dvis, ctx['im'], gcfcf=gcfcf, precision=p)
    im_ref, _ = orc.invert_2d(uvw, f, vis, wt, img, ogcf, ocf, cax)
    out['invert_2d'] = _img_err(dirty.data.cpu().numpy(), im_ref.real, ogcf)
    model = numpy.zeros((img['nchan'], img['npol'], img['ny'], img['nx']))
    c = img['ny'] // 2
    model[..., c - 40:c + 40:7, c - 40:c + 40:5] = 1.0
    mim = arl.Image(model, ctx['im'].wcs.deepcopy(), ctx['im'].polarisation_frame)
    pv = arl.predict_2d(dvis, mim, gcfcf=gcfcf, precision=p)
    p_ref = orc.predict_2d(uvw, f, model, img, ogcf, ocf, cax)
    out['predict_2d'] = _err(pv.vis.to(torch.complex128).cpu().numpy(), p_ref)
    return out


# ---------------------------------------------------------------------------
# Arms
# ---------------------------------------------------------------------------
def workload_label(w):
    return ('%s W-projection grid+degrid: %d antennas / %.0f km disk, %d chan %.0f-%.0f MHz, %d times, %d^2 grid, '
            'cell %.0e rad, %d w-planes support %d->%d, O=%d, %d rows after uv-cut of %d' %
            (w['name'], w['nants'], w['radius'] / 1e3, len(w['freqs']), w['freqs'][0] / 1e6, w['freqs'][-1] / 1e6,
             w['ntimes'], w['npixel'], w['cellsize'], w.get('nwplanes', 1), w.get('support_min', w['support']),
             w['support'], w['oversampling'], w['uvw'].shape[0], w['nrows_generated']))


def arm_gb300(args, torch, world, rank, local):
    arl = importlib.import_module('algorithm-reference-library_gb300')
    sim = importlib.import_module('algorithm-reference-library_gb300.simulation')
    device = torch.device('cuda', local)
    w = sim.make_workload(args.workload, device=device)
    w['name'] = args.workload
    n = w['uvw'].shape[0]
    tuned = None
    if not args.no_tune:
        # Autotune on this workload before any timing (untimed set-up).
        c0 = build_context(arl, torch, w, 'fp32c', device)
        best, table = arl.tune.autotune(c0['uvw'], c0['freq'], c0['vis'], c0['wt'], c0['cf_t'], c0['cd'], c0['gd'],
                                        'fp32c')
        tuned = {'choice': best, 'stage_ms_plan_grid_degrid': table}
        del c0
    ctx = build_context(arl, torch, w, 'fp32c', device)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=device)
    clocks = Clocks(local)
    r = timed_steps(arl, torch, ctx, args.steps, args.warmup, world, flush)
    clk = clocks.stop()
    t_max = max_over_ranks(torch, world, r['total_ms'])
    ms = t_max / args.steps
    value = world * n / (ms / 1e3)

    out = {}
    if not args.no_fp64:
        ctx64 = build_context(arl, torch, w, 'fp64', device)
        r64 = timed_steps(arl, torch, ctx64, max(3, args.steps // 2), 2, world, flush)
        ms64 = max_over_ranks(torch, world, r64['total_ms']) / max(3, args.steps // 2)
        g32 = ctx['grid'].to(torch.complex128)
        run_step(arl, ctx, torch.cuda.current_stream())
        torch.cuda.synchronize()
        g32 = ctx['grid'].to(torch.complex128)
        run_step(arl, ctx64, torch.cuda.current_stream())
        torch.cuda.synchronize()
        gerr = float((g32 - ctx64['grid']).abs().max() / ctx64['grid'].abs().max())
        derr = float((ctx['out'].to(torch.complex128) - ctx64['out']).abs().max() / ctx64['out'].abs().max())
        out['fp64'] = {'value': world * n / (ms64 / 1e3), 'ms_per_step': ms64, 'plan_ms': r64['plan_ms'],
                       'grid_ms': r64['grid_ms'], 'degrid_ms': r64['degrid_ms'],
                       'fp32c_speedup': ms64 / ms,
                       'fp32c_vs_fp64_max_rel_err': {'grid': gerr, 'degrid': derr}}
        del ctx64
        torch.cuda.empty_cache()

    e2e_seq_ms, h2d, d2h = e2e_steps(arl, torch, ctx, max(3, args.steps // 2), 2)
    e2e_ms, two_stream_ms = e2e_pipelined(arl, torch, ctx, max(3, args.steps), 2)
    stages = None
    if not args.no_stages:
        stages = {'grid': {'value': n / (r['grid_ms'] / 1e3), 'unit': 'vis/s', 'ms': r['grid_ms']},
                  'degrid': {'value': n / (r['degrid_ms'] / 1e3), 'unit': 'vis/s', 'ms': r['degrid_ms']}}
        stages.update(stage_rates(arl, torch, ctx, max(3, args.steps // 2), 2, flush))
        stages['gradient_step'] = gradient_step_rate(arl, torch, device, 3, 2, flush)
    e2e_ms = max_over_ranks(torch, world, e2e_ms)
    e2e_seq_ms = max_over_ranks(torch, world, e2e_seq_ms)

    # Roofline of the dominant kernel (grid or degrid launch), HBM-bound, with
    # the algorithmic bytes of the gridding / degridding stage: each row's uvw
    # (3 x f64), vis (c64 per pol), weight (f32 per pol, gridder only) and
    # channel id (i32) read once, and every cell of the grid written (gridder)
    # or read (degridder) once.
    npol = w['npol']
    gd = ctx['gd']
    grid_bytes = 8 * gd.ny * gd.nx * gd.npol * gd.nchan * gd.nw
    alg = {'grid': n * (24 + 8 * npol + 4 * npol + 4) + grid_bytes, 'degrid': n * (24 + 4 + 8 * npol) + grid_bytes}
    kern = 'grid' if r['grid_ms'] >= r['degrid_ms'] else 'degrid'
    kms = r[kern + '_ms']
    peak, peak_kind = measured_hbm()
    achieved = alg[kern] / (kms / 1e3) / 1e9
    tr = launch_traffic('k_' + kern, n)
    step_alg = n * (24 + 8 * npol + 4 * npol + 4) + grid_bytes + n * (24 + 4 + 8 * npol) + grid_bytes
    line = {
        'metric': METRIC, 'value': value, 'unit': 'vis/s', 'n_gpus': world, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': ms, 'higher_is_better': True, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic (seeded; ARL create_visibility row layout)',
        'config': {'workload': workload_label(w), 'nvis': n, 'precision': 'fp32c (complex64 storage, compensated FP32)',
                   'l2': 'flushed between steps (256 MiB write outside the timed events)',
                   'parallelism': 'replicas' if world > 1 else 'single GPU',
                   'step': 'plan (FP64 map + tile bin) + grid + degrid'},
        'breakdown_ms': {'plan': r['plan_ms'], 'grid': r['grid_ms'], 'degrid': r['degrid_ms']},
        'roofline': {'bound': 'hbm', 'kernel': 'k_' + kern, 'achieved': achieved, 'peak': peak, 'unit': 'GB/s',
                     'frac': achieved / peak, 'peak_source': peak_kind + ' (MEASURED_PEAKS.json hbm_gbs)',
                     'algorithmic_bytes_per_launch': alg[kern],
                     'traffic': None if tr is None else tr['bytes'],
                     'traffic_source': None if tr is None else
                     ('ncu dram__bytes_read.sum + dram__bytes_write.sum, %d-row capture%s' %
                      (tr['captured_rows'], ', scaled by rows' if tr['scaled'] else ''))},
        'roofline_issue': issue_roofline(torch, 'k_' + kern, n, kms, clk),
        'roofline_step': {'algorithmic_bytes': step_alg, 'achieved_gbs': step_alg / (ms / 1e3) / 1e9,
                          'frac': step_alg / (ms / 1e3) / 1e9 / peak},
        'e2e': {'value': world * n / (e2e_ms / 1e3), 'unit': 'vis/s', 'h2d_bytes_per_step': h2d,
                'd2h_bytes_per_step': d2h, 'ms_per_step': e2e_ms, 'path': 'C ABI, pinned host buffers',
                'overlap': 'a stream of steps: inputs, outputs and plan workspace double-buffered on the device, '
                           'consecutive steps on two compute streams, step k+1 uploads (copy stream) and step k '
                           'read-backs (second copy stream) under the compute; every step copies all its inputs '
                           'up and its grid and vis down',
                'two_stream_resident': {'value': world * n / (two_stream_ms / 1e3), 'ms_per_step': two_stream_ms,
                                        'what': 'the same two-stream compute with inputs resident and no copies '
                                                '(value above is one step at a time)'},
                'sequential': {'value': world * n / (e2e_seq_ms / 1e3), 'ms_per_step': e2e_seq_ms,
                               'overlap': 'one step at a time: uvw H2D first, then vis and weight H2D under the '
                                          'plan; grid D2H under the degrid (second stream)'}},
        'gpu_launches': r['launches'],
        'stages': stages,
        'clocks': clk,
        'autotune': tuned,
    }
    line.update(out)
    if rank == 0:
        line['err_vs_oracle_fp32c'] = oracle_errors(arl, torch, w, ctx)
        if not args.no_cpu:
            cb = CpuBaseline(w, ctx['cf'].data, 1)
            rate, rows = cb.rate(args.cpu_seconds, 200000)
            line['cpu_baseline'] = {'value': rate, 'unit': 'vis/s', 'cores': 1, 'kind': 'port',
                                    'sample': '%d rows of the workload through the oracle\'s per-row complex128 '
                                              'grid and degrid loops (%.0f s budget), %s' %
                                              (rows, args.cpu_seconds, cpu_model())}
        if not args.no_c5:
            del ctx
            torch.cuda.empty_cache()
            line['c5'] = wstack_record(torch, device)
    return line


def arm_wstack(args, torch, world, rank, local):
    """The w-stacking workloads (C3: 4 pols, 64 flagged channels, 20 slices,
    4096^2; C5: 1e8 rows, 32 slices, 8192^2): vis/s of the batched w-stack
    invert (plan + grid + inverse transforms with the w-screen sum: double-single
    on FP32C, complex128 on FP64) and predict (w-screens + FFTs + degrid)
    through WStackImager, of the invert replayed as one CUDA graph, and one
    staged pass.  Inputs and grids exceed L2, so no flush is needed."""
    arl = importlib.import_module('algorithm-reference-library_gb300')
    sim = arl.simulation
    device = torch.device('cuda', local)
    w = sim.make_workload(args.workload, device=device)
    n = w['uvw'].shape[0]
    im = sim.workload_image(arl, w)
    gcfcf = arl.create_pswf_convolutionfunction(im, oversampling=w['oversampling'], support=w['support'])
    model = torch.zeros((1, w['npol'], w['npixel'], w['npixel']), dtype=torch.float64, device=device)
    c = w['npixel'] // 2
    model[..., c - 200:c + 200:37, c - 200:c + 200:41] = 1.0
    stream = torch.cuda.current_stream()

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        e = _events(torch, 2)
        e[0].record(stream)
        for _ in range(steps):
            fn()
        e[1].record(stream)
        torch.cuda.synchronize()
        return e[0].elapsed_time(e[1]) / steps

    res, outs = {}, {}
    for prec in (('fp32c',) if args.no_fp64 else ('fp32c', 'fp64')):
        dvis = arl.DeviceVisibility(torch.as_tensor(w['uvw'], device=device),
                                    torch.as_tensor(w['frequency'], device=device),
                                    w['vis'].to(arl.device.CDTYPE[prec]),
                                    torch.ones((n, w['npol']), dtype=arl.device.RDTYPE[prec], device=device))
        imager = arl.WStackImager(dvis, im, w['vis_slices'], gcfcf=gcfcf, precision=prec)
        imager.set_model(model)
        lib = arl._native.load()
        l0 = lib.arlgpu_kernel_launches()
        t_inv = timed(lambda: imager.invert(replan=True), args.steps, args.warmup)
        t_pred = timed(lambda: imager.predict(replan=True), args.steps, args.warmup)
        r = {'invert_ms': t_inv, 'predict_ms': t_pred, 'invert_vis_s': n / (t_inv / 1e3),
             'predict_vis_s': n / (t_pred / 1e3), 'launches': int(lib.arlgpu_kernel_launches() - l0)}
        outs[prec] = (imager.invert(replan=True)[0].clone(), imager.predict(model, replan=True).clone())
        if prec == 'fp32c':
            imager.capture('invert')
            r['invert_graph_ms'] = timed(lambda: imager.replay('invert'), args.steps, 2)
            r['stages_ms'] = wstack_stages(torch, imager, stream)
        res[prec] = r
        del imager, dvis
        torch.cuda.empty_cache()
    f = res['fp32c']
    ms = f['invert_ms'] + f['predict_ms']
    line = {'metric': 'vis/s w-stack invert + predict (%s)' % args.workload, 'value': n / (ms / 1e3),
            'unit': 'vis/s', 'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': ms,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
            'data': 'synthetic (seeded)',
            'config': {'workload': args.workload, 'nvis': n, 'npol': w['npol'], 'npixel': w['npixel'],
                       'vis_slices': w['vis_slices'], 'kernel': 'PSWF S=%d O=%d' % (w['support'], w['oversampling']),
                       'l2': 'rows and grids exceed L2'},
            'fp32c': f}
    if 'fp64' in res:
        line['fp64'] = res['fp64']
        line['fp32c_speedup'] = (res['fp64']['invert_ms'] + res['fp64']['predict_ms']) / ms
        (i32, v32), (i64, v64) = outs['fp32c'], outs['fp64']
        gcf = torch.as_tensor(numpy.asarray(gcfcf[0].data), device=device)
        inner = (gcf <= 100.0).expand_as(i64)
        d, dv_ = (i32 - i64).abs(), (v32.to(torch.complex128) - v64).abs()
        line['err_vs_fp64_fp32c'] = {
            'invert_image': {'max_rel': float(d.max() / i64.abs().max()),
                             'rms_rel': float(d.pow(2).mean().sqrt() / i64.pow(2).mean().sqrt()),
                             'inner_max_rel': float(d[inner].max() / i64.abs().max())},
            'predict_vis': {'max_rel': float(dv_.max() / v64.abs().max()),
                            'rms_rel': float(dv_.pow(2).mean().sqrt() / v64.abs().pow(2).mean().sqrt())},
            'against': 'the same workload through the FP64 (complex128) GPU path'}
    return line


def _wstack_fp64_errors(arl, torch, w, im, gcfcf, model, img32, vis32, device):
    """Max-norm and RMS error of an FP32C w-stack result against the same
    workload through the FP64 (complex128) path on the GPU: the image (over
    the whole field and where the grid correction is <= 100) and the
    predicted rows.  The FP64 path is itself held to the oracle at 1e-10
    (images) and 1e-12 (grids, rows) by the parity tests; at 1e8 rows and
    8192^2 pixels the oracle's own loops are out of reach."""
    n = w['uvw'].shape[0]
    dvis = arl.DeviceVisibility(torch.as_tensor(w['uvw'], device=device),
                                torch.as_tensor(w['frequency'], device=device), w['vis'].to(torch.complex128),
                                torch.ones((n, w['npol']), dtype=torch.float64, device=device))
    im64 = arl.WStackImager(dvis, im, w['vis_slices'], gcfcf=gcfcf, precision='fp64')
    image64, _ = im64.invert(replan=True)
    gcf = torch.as_tensor(numpy.asarray(gcfcf[0].data), device=device)
    inner = (gcf <= 100.0).expand_as(image64)
    d = (img32 - image64).abs()
    mx = image64.abs().max()
    e_img = {'max_rel': float(d.max() / mx), 'rms_rel': float(d.pow(2).mean().sqrt() / image64.pow(2).mean().sqrt()),
             'inner_max_rel': float(d[inner].max() / mx), 'inner_fraction': float(inner.float().mean())}
    v64 = im64.predict(model)
    dv_ = (vis32.to(torch.complex128) - v64).abs()
    e_vis = {'max_rel': float(dv_.max() / v64.abs().max()),
             'rms_rel': float(dv_.pow(2).mean().sqrt() / v64.abs().pow(2).mean().sqrt())}
    del im64, dvis, v64, image64
    torch.cuda.empty_cache()
    return {'invert_image': e_img, 'predict_vis': e_vis,
            'against': 'the same workload through the FP64 (complex128) GPU path'}


def wstack_record(torch, device, name='C5', steps=2, warmup=1, nsub=20000):
    """Sub-record of the default bench for the largest single-GPU workload
    (C5: 100,466,688 rows onto 32 w-stack slices of 8192^2, PSWF 8 x 16),
    FP32C: invert / predict rates, one staged pass with each stage's HBM
    roofline (algorithmic bytes: grid nvis (24 + 12 npol + 4) + 8 N^2 npol P;
    degrid nvis (24 + 4 + 8 npol) + 8 N^2 npol P; each of the P inverse / forward
    transforms 2 x 8 N^2 npol), and the grid and degrid against the oracle on a
    seeded row subsample (the cells the rows touch, and the rows' windows)."""
    from oracle import arl_oracle as orc
    arl = importlib.import_module('algorithm-reference-library_gb300')
    sim = arl.simulation
    w = sim.make_workload(name, device=device)
    n = w['uvw'].shape[0]
    im = sim.workload_image(arl, w)
    gcfcf = arl.create_pswf_convolutionfunction(im, oversampling=w['oversampling'], support=w['support'])
    model = torch.zeros((1, w['npol'], w['npixel'], w['npixel']), dtype=torch.float64, device=device)
    c = w['npixel'] // 2
    model[..., c - 200:c + 200:37, c - 200:c + 200:41] = 1.0
    stream = torch.cuda.current_stream()
    dvis = arl.DeviceVisibility(torch.as_tensor(w['uvw'], device=device),
                                torch.as_tensor(w['frequency'], device=device), w['vis'].to(torch.complex64),
                                torch.ones((n, w['npol']), dtype=torch.float32, device=device))
    imager = arl.WStackImager(dvis, im, w['vis_slices'], gcfcf=gcfcf, precision='fp32c')
    imager.set_model(model)

    def timed(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        e = _events(torch, 2)
        e[0].record(stream)
        for _ in range(steps):
            fn()
        e[1].record(stream)
        torch.cuda.synchronize()
        return e[0].elapsed_time(e[1]) / steps

    t_inv = timed(lambda: imager.invert(replan=True))
    t_pred = timed(lambda: imager.predict(replan=True))
    st = wstack_stages(torch, imager, stream)
    img32 = imager.invert(replan=True)[0].clone()
    vis32 = imager.predict(model, replan=True).clone()
    peak, peak_kind = measured_hbm()
    npol, N, P = w['npol'], w['npixel'], w['vis_slices']
    cells = 8 * N * N * npol * P
    alg = {'grid': n * (24 + 12 * npol + 4) + cells, 'degrid': n * (28 + 8 * npol) + cells,
           'g2i': 2 * cells, 'i2g': 2 * cells}
    roof = {k: {'ms': st[k], 'algorithmic_bytes': b, 'achieved_gbs': b / (st[k] / 1e3) / 1e9,
                'frac': b / (st[k] / 1e3) / 1e9 / peak} for k, b in alg.items()}
    # oracle check on a seeded subsample, through the same imager geometry
    rng = numpy.random.default_rng(55)
    sel = numpy.sort(rng.choice(n, min(nsub, n), replace=False))
    img = orc.image_geometry(N, w['cellsize'], len(w['image_frequency']), npol, w['image_frequency'][0],
                             w['image_bandwidth'])
    _, ocf = orc.create_pswf_cf(1, npol, 8, 8, w['oversampling'], w['support'])
    vis64 = w['vis'][torch.as_tensor(sel, device=w['vis'].device)].cpu().numpy()
    wt = numpy.ones(vis64.shape)
    sub = arl.DeviceVisibility(torch.as_tensor(w['uvw'][sel], device=device),
                               torch.as_tensor(w['frequency'][sel], device=device),
                               torch.as_tensor(vis64, device=device).to(torch.complex64),
                               torch.ones(vis64.shape, dtype=torch.float32, device=device))
    del imager
    torch.cuda.empty_cache()
    simg = arl.WStackImager(sub, im, w['vis_slices'], gcfcf=gcfcf, precision='fp32c')
    simg.grid()
    gax = orc.grid_axes(img, nw=simg.vis_slices)
    gax['w'] = simg.w_axis
    cax = orc.cf_axes(img, w['oversampling'], w['support'])
    maps = orc.convolution_mapping(w['uvw'][sel], w['frequency'][sel], gax, cax)
    cells_i, vals, _ = orc.grid_sparse(vis64, wt, maps, ocf, gax['shape'])
    flat = simg.grid_t.reshape(-1)
    got = flat[torch.as_tensor(cells_i, device=device)].to(torch.complex128).cpu().numpy()
    out = simg.predict(model)
    idx = torch.as_tensor(orc.window_index(maps, gax['shape'], w['support']), device=device)
    win = simg.grid_t.reshape(-1)[idx].to(torch.complex128).cpu().numpy()
    d_ref = orc.degrid_windows(win, maps, ocf)
    err = {'rows': int(sel.size), 'grid': _err(got, vals),
           'degrid': _err(out.to(torch.complex128).cpu().numpy(), d_ref)}
    del simg, sub, dvis, idx, flat, out
    torch.cuda.empty_cache()
    e64 = _wstack_fp64_errors(arl, torch, w, im, gcfcf, model, img32, vis32, device)
    del img32, vis32
    torch.cuda.empty_cache()
    return {'workload': '%s: %d rows x %d pol, %d w-stack slices of %d^2, PSWF S=%d O=%d, FP32C' %
                        (name, n, npol, P, N, w['support'], w['oversampling']),
            'nvis': n, 'invert_ms': t_inv, 'predict_ms': t_pred, 'value': n / ((t_inv + t_pred) / 1e3),
            'unit': 'vis/s (invert + predict)', 'invert_vis_s': n / (t_inv / 1e3),
            'predict_vis_s': n / (t_pred / 1e3), 'stages_ms': st, 'roofline_stages': roof,
            'peak_gbs': peak, 'peak_source': peak_kind + ' (MEASURED_PEAKS.json hbm_gbs)',
            'err_vs_oracle_fp32c': err, 'err_vs_fp64_fp32c': e64, 'steps': steps, 'warmup': warmup,
            'l2': 'rows and grids exceed L2 (no flush needed)'}


def wstack_stages(torch, imager, stream):
    """One staged pass of the imager: plan, grid, transforms + w-screens into
    the image (g2i), w-screens + transforms of the model (i2g), degrid."""
    nat = importlib.import_module('algorithm-reference-library_gb300._native')
    e = _events(torch, 6)
    e[0].record(stream)
    imager.plan()
    e[1].record(stream)
    imager.grid()
    e[2].record(stream)
    imager.grid_to_image()
    e[3].record(stream)
    nat.call('arlgpu_wstack_image_to_grid', nat.ptr(imager.model), nat.ptr(imager.gcf_t), nat.ptr(imager.wmean),
             imager.cellsize, ctypes.byref(imager.gd), nat.PRECISIONS[imager.precision], nat.ptr(imager.grid_t),
             nat.stream_ptr())
    e[4].record(stream)
    nat.call('arlgpu_degrid_planned', imager.n, nat.PRECISIONS[imager.precision], nat.ptr(imager.cf_t),
             ctypes.byref(imager.cd), nat.ptr(imager.grid_t), ctypes.byref(imager.gd), nat.ptr(imager.out),
             nat.ptr(imager.ws), imager.ws.numel(), nat.stream_ptr())
    e[5].record(stream)
    torch.cuda.synchronize()
    names = ('plan', 'grid', 'g2i', 'i2g', 'degrid')
    return {k: round(e[i].elapsed_time(e[i + 1]), 3) for i, k in enumerate(names)}


def wstack_profile_case(args, torch):
    """A w-stack invert small enough for a multi-pass ncu capture of its
    transform passes: 2,000,000 seeded rows (uv uniform over the disk the grid
    holds, w uniform in +/-2000 wavelengths) onto 4 slices of 4096^2, PSWF
    S = 8, O = 16, FP32C."""
    arl = importlib.import_module('algorithm-reference-library_gb300')
    dev = torch.device('cuda', 0)
    rng = numpy.random.default_rng(3)
    N, cell, O, S, K, n = 4096, 5e-5, 16, 8, 4, 2_000_000
    im = arl.create_image(npixel=N, cellsize=cell, frequency=numpy.array([1e8]), channel_bandwidth=numpy.array([1e6]),
                          phasecentre=arl.PhaseCentre(0.0, -45.0))
    gcfcf = arl.create_pswf_convolutionfunction(im, oversampling=O, support=S)
    lim = (N // 2 - S // 2 - 2) / (N * cell)
    r = lim * numpy.sqrt(rng.uniform(size=n))
    th = rng.uniform(0, 2 * numpy.pi, n)
    uvw = numpy.stack([r * numpy.cos(th), r * numpy.sin(th), rng.uniform(-2000, 2000, n)], axis=1)
    dvis = arl.DeviceVisibility(torch.as_tensor(uvw, device=dev), torch.full((n,), 1e8, dtype=torch.float64, device=dev),
                                torch.ones((n, 1), dtype=torch.complex64, device=dev),
                                torch.ones((n, 1), dtype=torch.float32, device=dev))
    imager = arl.WStackImager(dvis, im, K, gcfcf=gcfcf, precision='fp32c')
    for _ in range(args.warmup + args.steps):
        img, _ = imager.invert()
    torch.cuda.synchronize()
    return {'case': 'w-stack invert, %d rows, %d slices of %d^2, FP32C' % (n, K, N), 'calls': args.warmup + args.steps,
            'image_max': float(img.abs().max()), 'device_gb': torch.cuda.max_memory_allocated() / 1e9}


def arm_transform(args, torch):
    """ms per call of the FP32C inverse transform (grid correction and sumwt
    normalisation fused) on two random N^2 planes: the double-single FFT
    (tuning dsfft=1) and cuFFT complex128 (dsfft=0).  The grid (8 B/cell) and
    the FFT scratch (16 B/cell) exceed L2 from N = 2048."""
    arl = importlib.import_module('algorithm-reference-library_gb300')
    dv = arl.device
    dev = torch.device('cuda', 0)
    N, nb = args.transform, 2
    g = torch.Generator(device='cpu').manual_seed(N)
    shape = (1, nb, 1, N, N)
    grid = torch.complex(torch.randn(shape, generator=g), torch.randn(shape, generator=g)).to(dev)
    gcf = (1.0 + torch.rand((1, nb, N, N), generator=g, dtype=torch.float64)).to(dev)
    sumwt = torch.ones((1, nb), dtype=torch.float64, device=dev)
    im = arl.create_image(npixel=64, cellsize=1e-3, frequency=numpy.array([1e8]), channel_bandwidth=numpy.array([1e6]),
                          phasecentre=arl.PhaseCentre(0.0, -45.0))
    gd = dv.grid_desc(arl.kernels._grid_wcs(im, 1, 1e15), shape)
    buf = torch.empty(nb * N * N, dtype=torch.complex128, device=dev)
    re = torch.empty((1, nb, N, N), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream()
    old = arl.tune.get_tuning()['dsfft']
    out = {}
    for ds in (1, 0):
        arl.tune.set_tuning(dsfft=ds)
        for _ in range(args.warmup):
            dv.fft_grid_to_image(grid, gd, gcf, 'fp32c', sumwt=sumwt, buf=buf)
        torch.cuda.synchronize()
        e = _events(torch, 2)
        e[0].record(stream)
        for _ in range(args.steps):
            dv.fft_grid_to_image(grid, gd, gcf, 'fp32c', sumwt=sumwt, buf=buf)
        e[1].record(stream)
        torch.cuda.synchronize()
        out[ds] = e[0].elapsed_time(e[1]) / args.steps
    arl.tune.set_tuning(dsfft=old)
    cells = nb * N * N
    return {'metric': 'ms per FP32C inverse 2-D transform with grid correction (%d planes of %d^2)' % (nb, N),
            'value': out[1], 'unit': 'ms', 'higher_is_better': False, 'steps': args.steps, 'warmup': args.warmup,
            'n_gpus': 1, 'dtype': 'f32 pairs (double-single)', 'data': 'synthetic (random grid)',
            'config': {'workload': 'transform %dx%d^2' % (nb, N)},
            'cufft_complex128_ms': out[0], 'speedup_vs_complex128': out[0] / out[1],
            'bytes_per_cell': {'grid_in': 8, 'gcf_in': 8, 'image_out': 8, 'ds_scratch_rw': 64},
            'gcells_per_s': cells / (out[1] * 1e-3) / 1e9}


def arm_reference(args, torch, world, rank):
    """The reference's CPU algorithm (the oracle's faithful per-row loops; the
    reference itself is Python that needs astropy, which is not installed) on
    all host cores: one process per core, each on its own seeded row sample."""
    if rank != 0:
        return None
    sim = importlib.import_module('algorithm-reference-library_gb300.simulation')
    from oracle import arl_oracle as orc
    w = sim.make_workload(args.workload, max_rows=400000)
    w['name'] = args.workload
    img = orc.image_geometry(w['npixel'], w['cellsize'], len(w['freqs']), w['npol'], w['freqs'][0],
                             w['channel_bandwidth'])
    if w['kernel'] == 'wproj':
        _, cf = orc.create_awterm_cf(img, nw=w['nwplanes'], wstep=w['wstep'], oversampling=w['oversampling'],
                                     support=w['support'])
        cf = orc.crop_cf_planes(cf, w['plane_support'])
    else:
        _, cf = orc.create_pswf_cf(len(w['freqs']), w['npol'], w['npixel'], w['npixel'], w['oversampling'],
                                   w['support'])
    procs = os.cpu_count() or 1
    budget = 4.0
    cb = CpuBaseline(w, cf, procs)
    for _ in range(args.warmup):
        cb.rate(1.0, 2000)
    rates = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        rate, rows = cb.rate(budget, 20000)
        rates.append(rate)
    wall = time.perf_counter() - t0
    cb.close()
    value = statistics.mean(rates)
    return {'metric': METRIC, 'value': value, 'unit': 'vis/s', 'impl': 'reference', 'n_gpus': world,
            'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': wall / args.steps * 1e3,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'c128',
            'data': 'synthetic (seeded)',
            'config': {'workload': workload_label(w), 'nvis_sampled_per_process': 20000},
            'cpu_baseline': {'value': value, 'unit': 'vis/s', 'cores': procs, 'kind': 'port',
                             'sample': 'per step, each of %d processes runs the oracle\'s per-row complex128 grid '
                                       'and degrid loops for %.0f s on its own seeded 20000-row sample; %s' %
                                       (procs, budget, cpu_model())},
            'e2e': {'value': value, 'unit': 'vis/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}


def profile_case(args, torch):
    """Small untimed case for ncu captures (one GPU): warmup + steps plan /
    grid / degrid calls on a row subsample, with the library's default
    kernel variants or those that --tuning names."""
    arl = importlib.import_module('algorithm-reference-library_gb300')
    sim = importlib.import_module('algorithm-reference-library_gb300.simulation')
    device = torch.device('cuda', 0)
    w = sim.make_workload(args.workload, max_rows=args.profile_rows, device=device)
    w['name'] = args.workload
    for kv in args.tuning:
        key, val = kv.split('=', 1)
        arl.tune.set_tuning(**{key: int(val)})
    ctx = build_context(arl, torch, w, 'fp32c', device)
    st = torch.cuda.current_stream()
    for _ in range(args.warmup + args.steps):
        run_step(arl, ctx, st)
    torch.cuda.synchronize()
    print(json.dumps({'profile_case': args.workload, 'rows': ctx['n'], 'steps': args.warmup + args.steps,
                      'tuning': arl.tune.get_tuning()}))


def main():
    args = parse()
    import torch
    if args.profile_rows:
        profile_case(args, torch)
        return
    if args.transform:
        print(json.dumps(arm_transform(args, torch)), flush=True)
        return
    if args.wstack_profile:
        print(json.dumps(wstack_profile_case(args, torch)), flush=True)
        return
    world, rank, local = dist_setup(torch)
    if args.impl == 'reference':
        line = arm_reference(args, torch, world, rank)
    elif args.workload in ('C3', 'C5'):
        line = arm_wstack(args, torch, world, rank, local)
    else:
        line = arm_gb300(args, torch, world, rank, local)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as tdist
        tdist.destroy_process_group()


if __name__ == '__main__':
    main()
