"""Oracle pins: the reference's own known-answer values.

Values, locations and tolerances come from
``tests/processing_components/test_griddata_kernels.py`` (template: 512 x 512,
cellsize 0.0005 rad, :33-35) and ``tests/processing_library/test_convolutional_gridding.py``.
"""
import numpy
import pytest


def test_pswf_oversampled_peak(oracle):
    # test_griddata_kernels.py:60-79
    _, cf = oracle.create_pswf_cf(1, 1, 512, 512, oversampling=8, support=6)
    loc = numpy.unravel_index(numpy.argmax(numpy.abs(cf)), cf.shape)
    assert numpy.abs(cf[loc] - 0.1871722034219655) < 1e-7
    assert loc == (0, 0, 0, 4, 4, 3, 3)


def test_pswf_no_oversampling_peak(oracle):
    # test_griddata_kernels.py:82-101
    _, cf = oracle.create_pswf_cf(1, 1, 512, 512, oversampling=1, support=6)
    loc = numpy.unravel_index(numpy.argmax(numpy.abs(cf)), cf.shape)
    assert numpy.abs(cf[loc] - 0.18712109669890536) < 1e-7
    assert loc == (0, 0, 0, 0, 0, 3, 3)


def test_box_peak(oracle):
    # test_griddata_kernels.py:45-58
    _, cf = oracle.create_box_cf(1, 1, 512, 512)
    loc = numpy.unravel_index(numpy.argmax(numpy.abs(cf)), cf.shape)
    assert numpy.abs(cf[loc] - 1.0) < 1e-15
    assert loc == (0, 0, 0, 0, 0, 2, 2)


@pytest.fixture(scope='module')
def wterm(oracle):
    # test_griddata_kernels.py:104-139: nw=201, wstep=8, O=8, S=60.  Only the
    # centre plane (100) and a few others are needed; planes are independent
    # apart from the normalisation, which uses the centre plane.
    img = oracle.image_geometry(512, 0.0005)
    return oracle.create_awterm_cf(img, nw=201, wstep=8.0, oversampling=8, support=60, planes=[0, 37, 100, 163, 200])


def test_wterm_peak(wterm):
    _, cf = wterm
    loc = numpy.unravel_index(numpy.argmax(numpy.abs(cf)), cf.shape)
    assert loc == (0, 0, 100, 4, 4, 30, 30)
    assert numpy.abs(cf[loc] - (0.18704481681878257 - 0j)) < 1e-7


def test_wterm_clipped_peak(oracle, wterm):
    # apply_bounding_box_convolutionfunction(cf, 1e-3): peak moves to (..., 27, 27)
    # (test_griddata_kernels.py:122-139).  The box is computed on the planes held.
    _, cf = wterm
    clipped, _, _ = oracle.apply_bounding_box(cf, 31.0, 31.0, 1e-3)
    loc = numpy.unravel_index(numpy.argmax(numpy.abs(clipped)), clipped.shape)
    assert loc == (0, 0, 100, 4, 4, 27, 27)
    assert numpy.abs(clipped[loc] - (0.18704481681878257 - 0j)) < 1e-7


def test_wterm_symmetry(oracle):
    # test_griddata_kernels.py:257-296 (nw=110, wstep=8, O=8, S=60)
    img = oracle.image_geometry(512, 0.0005)
    _, cf = oracle.create_awterm_cf(img, nw=110, wstep=8.0, oversampling=8, support=60, planes=[25, 45, 55, 85])
    loc = numpy.unravel_index(numpy.argmax(numpy.abs(cf)), cf.shape)
    assert loc == (0, 0, 55, 4, 4, 30, 30)
    assert numpy.abs(cf[loc] - (0.18704481681878257 - 0j)) < 1e-12
    for z in (55, 45):
        assert numpy.abs(cf[0, 0, z, 4, 4, 25, 25] - cf[0, 0, z, 4, 4, 35, 35]) < 1e-15
        assert numpy.abs(cf[0, 0, z, 4, 4, 25, 25] - cf[0, 0, z, 4, 4, 25, 35]) < 1e-15
    assert numpy.abs(cf[0, 0, 45, 4, 4, 25, 25] - cf[0, 0, 45, 4, 4, 35, 25]) < 1e-15
    assert numpy.abs(cf[0, 0, 25, 4, 4, 25, 25] - numpy.conjugate(cf[0, 0, 85, 4, 4, 25, 25])) < 1e-15
    assert numpy.abs(cf[0, 0, 25, 4, 4, 25, 25] - numpy.conjugate(cf[0, 0, 85, 4, 4, 35, 35])) < 1e-15


def test_coordinates_and_w_beam(oracle):
    # test_convolutional_gridding.py:193-216
    for n in (4, 5, 6, 7, 8, 9, 1000, 1001, 1002, 1003):
        c = oracle.coordinates(n)
        assert c[0] >= -0.5 and c[-1] < 0.5
        assert numpy.abs(c[n // 2]) < 1e-15
    assert numpy.abs(oracle.w_beam(5, 0.1, 0)[0, 0] - 1.0) < 1e-15


def test_grdsf_edges(oracle):
    g, t = oracle.grdsf(numpy.array([0.0, 0.5, 0.75, 1.0, 1.2]))
    assert g[-1] == 0.0 and t[-1] == 0.0
    assert numpy.abs(t[3]) < 1e-15
    assert numpy.all(g[:4] > 0)
