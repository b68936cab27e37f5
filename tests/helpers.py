"""Shared comparison rules for the GPU parity tests.

Tolerances are max-norm error over max-norm of the reference result:
  * grids, visibilities, kernels: FP64 1e-12, FP32C 1e-5;
  * outputs that pass through an FFT: FP64 1e-10 (cuFFT and NumPy's pocketfft
    sum in different orders; measured ~2e-12);
  * grid-corrected images in FP32C: 1e-5 where the grid correction is <= 100
    (76% of a PSWF-corrected image) and 1e-3 over the whole image.  Towards
    the field edge the PSWF correction grows to ~6e4, and it multiplies the
    white FP32 rounding noise of complex64 taps and grid cells (which, unlike
    the signal, is not tapered): relative to the image peak the error there is
    ~1e-8 x gcf for a noise-like sky, so no FP32 kernel stays within 1e-5 at
    the edge.  Measured on the GPU (largest whole-image errors of the suite):
    2e-4 to 7.4e-4 on 128^2 .. 256^2 test images, 3e-6 to 9e-6 on the
    1024^2 .. 8192^2 workloads; test_fp32c_edge_error_is_storage_rounding
    shows that complex64 taps alone, or a complex64 grid alone, give the same
    edge error to the FP64 path.
"""
import numpy

INNER_GCF = 100.0


def rel(a, b):
    a = numpy.asarray(a)
    b = numpy.asarray(b)
    return float(numpy.max(numpy.abs(a - b)) / max(numpy.max(numpy.abs(b)), 1e-300))


def image_errors(got, want, gcf):
    """(full-image, inner-region) max-norm relative errors; the inner region is
    where the grid correction is <= INNER_GCF."""
    got = numpy.asarray(got)
    want = numpy.asarray(want)
    g = numpy.broadcast_to(numpy.asarray(gcf), want.shape)
    mx = max(numpy.max(numpy.abs(want)), 1e-300)
    err = numpy.abs(got - want)
    inner = g <= INNER_GCF
    return float(err.max() / mx), float(err[inner].max() / mx)


def assert_image(got, want, gcf, precision):
    full, inner = image_errors(got, want, gcf)
    if precision == 'fp64':
        assert full < 1e-10, full
    else:
        assert inner < 1e-5, (inner, full)
        assert full < 1e-3, (inner, full)
