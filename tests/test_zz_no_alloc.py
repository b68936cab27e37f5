"""arlgpu_grid_noalloc: the gridder for callers that cannot allocate device
memory when they grid (device memory owned by another framework's pool,
real-time code that allocates only at start-up).  Called through the C ABI
and checked against arlgpu_grid, which grids the same rows with a
caller-provided workspace.  The shared scratch array keeps the previous
call's plan, so the check runs after a call on a different case (more rows,
other uv values, a larger grid with more bins), twice in a row, and as a
CUDA graph recorded once and replayed.

Kept in a file that pytest collects last, so a failure here cannot stop the
rest of the suite from running first."""
import ctypes

import numpy
import pytest
import torch

pytestmark = pytest.mark.gpu

MAX_ROWS = 1 << 19


@pytest.fixture(scope='module')
def case(arl):
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    rng = numpy.random.default_rng(99)
    N, cell, O, S, n = 256, 2e-3, 8, 8, 50000
    im = arl.create_image(npixel=N, cellsize=cell, frequency=numpy.array([1e8, 1.1e8]),
                          channel_bandwidth=numpy.array([1e7]), phasecentre=arl.PhaseCentre(0.0, -45.0))
    _, cf = arl.create_pswf_convolutionfunction(im, oversampling=O, support=S)
    dev = torch.device('cuda')
    lim = (N // 2 - S // 2 - 2) / (N * cell)
    uvw = numpy.stack([rng.uniform(-lim, lim, n), rng.uniform(-lim, lim, n), rng.uniform(-50, 50, n)], axis=1)
    freq = rng.choice([1e8, 1.1e8], n)
    t = dict(uvw=torch.as_tensor(uvw, device=dev), freq=torch.as_tensor(freq, device=dev),
             vis=torch.as_tensor(rng.normal(size=(n, 1)) + 1j * rng.normal(size=(n, 1)), device=dev).to(
                 torch.complex64),
             wt=torch.as_tensor(rng.uniform(0.5, 2, (n, 1)), device=dev).to(torch.float32))
    gd = arl.device.grid_desc(arl.kernels._grid_wcs(im, 1, 1e15), (2, 1, 1, N, N))
    cf_t, cs, ps, psup = arl.device.device_cf(cf, 'fp32c', dev)
    cd = arl.device.cf_desc(cf.grid_wcs, cf.data.shape, cs, ps, psup, table=cf_t)
    return arl, t, gd, cd, cf_t, n


@pytest.fixture(scope='module')
def other_case(arl):
    """A different call for the shared scratch: 400,000 rows with other uv
    values on a 512^2 grid (a larger plan with more bins than `case`)."""
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    rng = numpy.random.default_rng(7)
    N, cell, O, S, n = 512, 1e-3, 8, 8, 400000
    im = arl.create_image(npixel=N, cellsize=cell, frequency=numpy.array([1e8, 1.1e8]),
                          channel_bandwidth=numpy.array([1e7]), phasecentre=arl.PhaseCentre(0.0, -45.0))
    _, cf = arl.create_pswf_convolutionfunction(im, oversampling=O, support=S)
    dev = torch.device('cuda')
    lim = (N // 2 - S // 2 - 2) / (N * cell)
    uvw = numpy.stack([rng.uniform(-lim, lim, n), rng.uniform(-lim, lim, n), rng.uniform(-50, 50, n)], axis=1)
    freq = rng.choice([1e8, 1.1e8], n)
    t = dict(uvw=torch.as_tensor(uvw, device=dev), freq=torch.as_tensor(freq, device=dev),
             vis=torch.as_tensor(rng.normal(size=(n, 1)) + 1j * rng.normal(size=(n, 1)), device=dev).to(
                 torch.complex64),
             wt=torch.as_tensor(rng.uniform(0.5, 2, (n, 1)), device=dev).to(torch.float32))
    gd = arl.device.grid_desc(arl.kernels._grid_wcs(im, 1, 1e15), (2, 1, 1, N, N))
    cf_t, cs, ps, psup = arl.device.device_cf(cf, 'fp32c', dev)
    cd = arl.device.cf_desc(cf.grid_wcs, cf.data.shape, cs, ps, psup, table=cf_t)
    return arl, t, gd, cd, cf_t, n


def _grid(arl, t, gd, cd, cf_t, n, noalloc):
    nat = arl._native
    lib = nat.load()
    dev = t['uvw'].device
    grid = torch.full((gd.nchan, gd.npol, gd.nw, gd.ny, gd.nx), 7.0, dtype=torch.complex64, device=dev)
    sumwt = torch.full((gd.nchan, gd.npol), 7.0, dtype=torch.float64, device=dev)
    nbad = torch.full((1,), 7, dtype=torch.int64, device=dev)
    args = (nat.ptr(t['uvw']), nat.ptr(t['freq']), nat.ptr(t['vis']), nat.ptr(t['wt']), n, nat.FP32C,
            nat.ptr(cf_t), ctypes.byref(cd), nat.ptr(grid), ctypes.byref(gd), nat.ptr(sumwt), nat.ptr(nbad))
    if noalloc:
        st = lib.arlgpu_grid_noalloc(*args, nat.stream_ptr())
    else:
        ws = torch.empty(arl.device.plan_bytes(n, gd, cd), dtype=torch.uint8, device=dev)
        st = lib.arlgpu_grid(*args, nat.ptr(ws), ws.numel(), nat.stream_ptr())
    nat.check(st)
    torch.cuda.synchronize()
    return grid.to(torch.complex128).cpu().numpy(), sumwt.cpu().numpy(), int(nbad.item())


def test_noalloc_matches_workspace_gridder_twice(case, other_case):
    arl, t, gd, cd, cf_t, n = case
    ref, ref_sw, ref_bad = _grid(arl, t, gd, cd, cf_t, n, noalloc=False)
    assert ref_bad == 0
    # Leave a different, larger plan in the shared scratch first (and check
    # that call too): a part of the plan the next call failed to rewrite would
    # then hold wrong values.
    o_ref, o_sw, _ = _grid(*other_case, noalloc=False)
    o_got, o_sw2, o_bad = _grid(*other_case, noalloc=True)
    assert o_bad == 0
    assert numpy.max(numpy.abs(o_got - o_ref)) / numpy.max(numpy.abs(o_ref)) < 1e-5
    assert numpy.allclose(o_sw2, o_sw, rtol=1e-12)
    for _ in range(2):
        got, sw, bad = _grid(arl, t, gd, cd, cf_t, n, noalloc=True)
        assert bad == 0
        # same FP32C tolerance as the other gridder tests; sums differ only by
        # the order of the atomic additions
        assert numpy.max(numpy.abs(got - ref)) / numpy.max(numpy.abs(ref)) < 1e-5
        assert numpy.allclose(sw, ref_sw, rtol=1e-12)


def test_noalloc_replays_in_a_cuda_graph(case, other_case):
    """Recorded once under stream capture (no allocation may happen there)
    and replayed twice, with another case gridded in between: each replay
    rebuilds its plan in the shared scratch and gives the workspace result."""
    arl, t, gd, cd, cf_t, n = case
    nat = arl._native
    lib = nat.load()
    dev = t['uvw'].device
    ref, ref_sw, _ = _grid(arl, t, gd, cd, cf_t, n, noalloc=False)
    grid = torch.empty((gd.nchan, gd.npol, gd.nw, gd.ny, gd.nx), dtype=torch.complex64, device=dev)
    sumwt = torch.empty((gd.nchan, gd.npol), dtype=torch.float64, device=dev)
    nbad = torch.empty((1,), dtype=torch.int64, device=dev)

    def call():
        nat.check(lib.arlgpu_grid_noalloc(nat.ptr(t['uvw']), nat.ptr(t['freq']), nat.ptr(t['vis']), nat.ptr(t['wt']),
                                          n, nat.FP32C, nat.ptr(cf_t), ctypes.byref(cd), nat.ptr(grid),
                                          ctypes.byref(gd), nat.ptr(sumwt), nat.ptr(nbad), nat.stream_ptr()))

    side = torch.cuda.Stream(device=dev)
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        call()  # scratch address and kernel attributes set up before capture
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        call()
    for _ in range(2):
        _grid(*other_case, noalloc=True)  # another plan left in the scratch
        grid.fill_(7.0)
        sumwt.fill_(7.0)
        nbad.fill_(7)
        g.replay()
        torch.cuda.synchronize()
        got = grid.to(torch.complex128).cpu().numpy()
        assert int(nbad.item()) == 0
        assert numpy.max(numpy.abs(got - ref)) / numpy.max(numpy.abs(ref)) < 1e-5
        assert numpy.allclose(sumwt.cpu().numpy(), ref_sw, rtol=1e-12)


def test_noalloc_rejects_oversize_calls(case):
    arl, t, gd, cd, cf_t, n = case
    nat = arl._native
    lib = nat.load()
    # Rejected on the host before any GPU work: the pointers are never read.
    st = lib.arlgpu_grid_noalloc(nat.ptr(t['uvw']), nat.ptr(t['freq']), nat.ptr(t['vis']), nat.ptr(t['wt']),
                                 MAX_ROWS + 1, nat.FP32C, nat.ptr(cf_t), ctypes.byref(cd), None, ctypes.byref(gd),
                                 None, None, nat.stream_ptr())
    assert st == nat.ERR_WORKSPACE
    assert b'at most' in lib.arlgpu_last_error()
