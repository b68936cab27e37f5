"""The C ABI's argument checks, which return before any CUDA call: bad
descriptors, sizes, pointers and workspaces give the documented status codes
and a message through arlgpu_last_error (ARL's own path raises
AssertionError / ValueError for the same inputs).  No GPU needed."""
import ctypes

import numpy
import pytest

OK, INVALID, UNSUPPORTED, WORKSPACE = 0, 1, 4, 5
FP32C, FP64 = 0, 1


@pytest.fixture(scope='module')
def nat(arl):
    try:
        arl._native.load()
    except OSError as e:  # pragma: no cover - the library is built by build()
        pytest.skip('libarlgpu.so not loadable here: %s' % e)
    return arl._native


@pytest.fixture()
def descs(arl):
    """Valid (GridDesc, CfDesc) of a 128^2, 1-channel, 1-pol grid and an O = 8,
    S = 8 kernel with one plane (pol stride 0)."""
    im = arl.create_image(npixel=128, cellsize=1e-3, frequency=numpy.array([1e8]),
                          channel_bandwidth=numpy.array([1e6]), phasecentre=arl.PhaseCentre(0.0, -45.0))
    gd = arl.create_griddata_from_image(im)
    cf = arl.create_convolutionfunction_from_image(im, oversampling=8, support=8)
    g = arl.device.grid_desc(gd.grid_wcs, gd.data.shape)
    c = arl.device.cf_desc(cf.grid_wcs, cf.data.shape, 0, 0)
    return g, c


def ws_bytes(nat, nvis, g, c):
    n = ctypes.c_size_t(0)
    st = nat.load().arlgpu_plan_workspace_bytes(nvis, ctypes.byref(g), ctypes.byref(c), ctypes.byref(n))
    return st, n.value


def last_error(nat):
    return nat.load().arlgpu_last_error().decode()


def test_workspace_bytes_grow_with_rows(nat, descs):
    g, c = descs
    st0, b0 = ws_bytes(nat, 0, g, c)
    st1, b1 = ws_bytes(nat, 1000, g, c)
    st2, b2 = ws_bytes(nat, 2000, g, c)
    assert st0 == st1 == st2 == OK
    assert 0 < b0 < b1 < b2
    # keys, row maps, sorted ids and sorted maps: 40 B per row, each array 256-byte aligned
    assert abs((b2 - b1) - 1000 * 40) <= 4 * 256


@pytest.mark.parametrize('field,value,status,words', [
    ('nx', 1, INVALID, 'grid shape'),
    ('nchan', 0, INVALID, 'grid shape'),
    ('npol', 5, UNSUPPORTED, 'npol'),
])
def test_bad_grid_descriptor(nat, descs, field, value, status, words):
    g, c = descs
    setattr(g, field, value)
    st, _ = ws_bytes(nat, 10, g, c)
    assert st == status
    assert words in last_error(nat)


@pytest.mark.parametrize('field,value,status,words', [
    ('support', 7, UNSUPPORTED, 'even'),
    ('support', 66, UNSUPPORTED, 'support > 64'),
    ('oversampling', 0, UNSUPPORTED, 'oversampling'),
    ('nz', 0, UNSUPPORTED, 'nz'),
    ('npol', 2, INVALID, 'cf npol'),
])
def test_bad_cf_descriptor(nat, descs, field, value, status, words):
    g, c = descs
    setattr(c, field, value)
    if field == 'npol':
        c.pol_stride = 1  # two distinct pol blocks against a one-pol grid
    st, _ = ws_bytes(nat, 10, g, c)
    assert st == status
    assert words in last_error(nat)


def test_plan_build_rejects_bad_rows_and_workspace(nat, descs):
    g, c = descs
    lib = nat.load()
    _, need = ws_bytes(nat, 100, g, c)
    buf = ctypes.create_string_buffer(16)
    ptr = ctypes.cast(buf, ctypes.c_void_p)
    # negative row count
    assert lib.arlgpu_plan_build(ptr, ptr, -1, ctypes.byref(g), ctypes.byref(c), ptr, need, None, None) == INVALID
    assert 'nvis' in last_error(nat)
    # rows without uvw / frequency
    assert lib.arlgpu_plan_build(None, None, 100, ctypes.byref(g), ctypes.byref(c), ptr, need, None, None) == INVALID
    # workspace too small (checked before any device access)
    assert lib.arlgpu_plan_build(ptr, ptr, 100, ctypes.byref(g), ctypes.byref(c), ptr, need - 1, None, None) == WORKSPACE
    assert 'workspace' in last_error(nat)
    # workspace off a 16-byte boundary (the row maps move as 128-bit accesses)
    big = ctypes.create_string_buffer(need + 64)
    base = ctypes.addressof(big)
    odd = ctypes.c_void_p(base + (16 - base % 16) % 16 + 4)
    assert lib.arlgpu_plan_build(ptr, ptr, 100, ctypes.byref(g), ctypes.byref(c), odd, need, None, None) == INVALID
    assert '16-byte' in last_error(nat)
    # bad precision on the gridding entry point
    assert lib.arlgpu_grid_planned(ptr, ptr, 100, 7, ptr, ctypes.byref(c), ptr, ctypes.byref(g), None, ptr, need,
                                   None) == INVALID
    assert 'precision' in last_error(nat)
    # null output grid
    assert lib.arlgpu_grid_planned(ptr, ptr, 100, FP32C, ptr, ctypes.byref(c), None, ctypes.byref(g), None, ptr, need,
                                   None) == INVALID


def test_tuning_keys(nat):
    lib = nat.load()
    v = ctypes.c_int(-1)
    for key in ('grid_kernel', 'degrid_kernel', 'subgrid', 'chunk', 'persistent', 'dsfft', 'small_rows',
                'small_rows_degrid', 'lanes_per_row'):
        assert lib.arlgpu_get_tuning(key.encode(), ctypes.byref(v)) == OK
        old = v.value
        assert lib.arlgpu_set_tuning(key.encode(), old) == OK  # current values are valid
    assert lib.arlgpu_set_tuning(b'no_such_key', 1) == INVALID
    assert lib.arlgpu_set_tuning(b'small_rows', 3) == INVALID
    assert lib.arlgpu_set_tuning(b'lanes_per_row', 4) == INVALID
    assert lib.arlgpu_set_tuning(b'persistent', 3) == INVALID
    assert lib.arlgpu_get_tuning(b'no_such_key', ctypes.byref(v)) != OK


def test_noalloc_rejects_too_many_rows_or_bins(nat, descs):
    """arlgpu_grid_noalloc checks its row limit and its bin limit on their own,
    on the host, before any device access: a call with few rows but more than
    65,536 plan bins fails like a call with too many rows."""
    g, c = descs
    lib = nat.load()
    buf = ctypes.create_string_buffer(16)
    ptr = ctypes.cast(buf, ctypes.c_void_p)

    def call(nvis, gd):
        return lib.arlgpu_grid_noalloc(ptr, ptr, ptr, ptr, nvis, FP32C, ptr, ctypes.byref(c), ptr, ctypes.byref(gd),
                                       ptr, None, None)

    assert call((1 << 19) + 1, g) == WORKSPACE
    assert 'rows' in last_error(nat)
    # 1024^2 grid: 26 x 26 uv-tiles of 40 pixels per (channel, w-plane); 100
    # channels make 67,600 bins
    big = type(g).from_buffer_copy(g)
    big.nx = big.ny = 1024
    big.nchan = 100
    assert call(10, big) == WORKSPACE
    assert 'bins' in last_error(nat)
    big.nchan = 90  # 60,840 bins: accepted by both checks, fails only later
    st = call(-1, big)
    assert st == INVALID and 'nvis' in last_error(nat)
