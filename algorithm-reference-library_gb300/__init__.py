"""GB300-native implementation of ARL's convolutional gridding / degridding
imaging path (grid / degrid, PSWF and w-kernel convolution functions, the FFT
stages of invert_2d / predict_2d, and w-stacking).

The directory name is not a Python identifier; import it with
``importlib.import_module('algorithm-reference-library_gb300')``.

Compute runs only in ``libarlgpu.so`` (hand-written sm_103a CUDA behind the C
ABI in ``include/arlgpu.h``); the Python layer mirrors ARL's functions and data
models so existing callers switch by changing imports.
"""
from . import _native  # noqa: F401
from .data_models import (BlockVisibility, ConvolutionFunction, GridData, Image, PhaseCentre,  # noqa: F401
                          PolarisationFrame, QA, Visibility, copy_image, copy_visibility, create_empty_image_like,
                          create_image, create_image_from_array, create_visibility_from_rows)
from .device import default_precision, set_default_precision  # noqa: F401
from .gridding import (DeviceVisibility, convolution_mapping, degrid_visibility_from_griddata,  # noqa: F401
                       fft_griddata_to_image, fft_image_to_griddata, grid_visibility_to_griddata)
from .imaging import (imaging_context, imaging_contexts, invert_2d, invert_list_serial_workflow,  # noqa: F401
                      invert_wstack, invert_wstack_single, normalize_sumwt, predict_2d, predict_list_serial_workflow,
                      predict_wstack, predict_wstack_single, phaserotate_visibility, shift_vis_to_image,
                      vis_null_iter, vis_wslice_iter)
from . import autograd, simulation, tune  # noqa: F401
from .kernels import (apply_bounding_box_convolutionfunction, calculate_bounding_box_convolutionfunction,  # noqa: F401
                      copy_convolutionfunction, copy_griddata, create_awterm_convolutionfunction,
                      create_box_convolutionfunction, create_convolutionfunction_from_image,
                      create_griddata_from_image, create_griddata_on_device, create_pswf_convolutionfunction,
                      set_plane_support, support_schedule)
from .wcs import WCS  # noqa: F401
from .wstack import WStackImager  # noqa: F401
from .weighting import (grid_weight_to_griddata, griddata_merge_weights, griddata_reweight,  # noqa: F401
                        weight_visibility)
from .coalesce import (convert_blockvisibility_to_visibility, convert_visibility_to_blockvisibility,  # noqa: F401
                       decoalesce_visibility)
from .data_models import GainTable, ReceptorFrame, Skycomponent, copy_blockvisibility  # noqa: F401
from .calibration import apply_gaintable, vis_timeslice_iter  # noqa: F401
from .skycomponents import predict_skycomponent_visibility  # noqa: F401
from .deconvolution import (deconvolve_cube, hogbom, hogbom_complex, msclean, msmfsclean,  # noqa: F401
                            calculate_image_frequency_moments, calculate_image_from_frequency_moments)

__version__ = '0.1.0'
