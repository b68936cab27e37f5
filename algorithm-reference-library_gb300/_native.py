"""ctypes binding of libarlgpu.so (declared in include/arlgpu.h).

The library is the only compute path: if it is missing or no CUDA device is
present, every entry point raises; nothing falls back to the CPU.
"""
import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, 'libarlgpu.so')

OK, ERR_INVALID, ERR_CUDA, ERR_OUT_OF_GRID, ERR_UNSUPPORTED, ERR_WORKSPACE, ERR_CUFFT = range(7)
FP32C, FP64 = 0, 1
PRECISIONS = {'fp32c': FP32C, 'fp64': FP64}

# Entry points declared in include/arlgpu.h, with their ctypes signatures.
_i32, _i64, _f64, _vp, _sz = ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p, ctypes.c_size_t


class Axis(ctypes.Structure):
    _fields_ = [('crval', _f64), ('crpix', _f64), ('cdelt', _f64)]


class GridDesc(ctypes.Structure):
    _fields_ = [('nchan', _i32), ('npol', _i32), ('nw', _i32), ('ny', _i32), ('nx', _i32),
                ('u', Axis), ('v', Axis), ('w', Axis), ('f', Axis)]


class CfDesc(ctypes.Structure):
    _fields_ = [('nchan', _i32), ('npol', _i32), ('nz', _i32), ('oversampling', _i32), ('support', _i32),
                ('chan_stride', _i64), ('pol_stride', _i64), ('du', Axis), ('dv', Axis), ('z', Axis),
                ('plane_support', _vp), ('tap_absmax', _f64)]


_P = ctypes.POINTER
SIGNATURES = {
    'arlgpu_version': (ctypes.c_char_p, []),
    'arlgpu_last_error': (ctypes.c_char_p, []),
    'arlgpu_convolution_mapping': (ctypes.c_int, [_vp, _vp, _i64, _P(GridDesc), _P(CfDesc), _vp, _vp, _vp, _vp,
                                                  _vp, _vp, _vp, _P(_i64), _vp]),
    'arlgpu_plan_workspace_bytes': (ctypes.c_int, [_i64, _P(GridDesc), _P(CfDesc), _P(_sz)]),
    'arlgpu_grid': (ctypes.c_int, [_vp, _vp, _vp, _vp, _i64, ctypes.c_int, _vp, _P(CfDesc), _vp, _P(GridDesc),
                                   _vp, _vp, _vp, _sz, _vp]),
    'arlgpu_kernel_launches': (ctypes.c_ulonglong, []),
    'arlgpu_grid_noalloc': (ctypes.c_int, [_vp, _vp, _vp, _vp, _i64, ctypes.c_int, _vp, _P(CfDesc), _vp,
                                           _P(GridDesc), _vp, _vp, _vp]),
    'arlgpu_set_tuning': (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int]),
    'arlgpu_get_tuning': (ctypes.c_int, [ctypes.c_char_p, _P(ctypes.c_int)]),
    'arlgpu_plan_build': (ctypes.c_int, [_vp, _vp, _i64, _P(GridDesc), _P(CfDesc), _vp, _sz, _vp, _vp]),
    'arlgpu_grid_planned': (ctypes.c_int, [_vp, _vp, _i64, ctypes.c_int, _vp, _P(CfDesc), _vp, _P(GridDesc), _vp,
                                           _vp, _sz, _vp]),
    'arlgpu_degrid_planned': (ctypes.c_int, [_i64, ctypes.c_int, _vp, _P(CfDesc), _vp, _P(GridDesc), _vp, _vp, _sz,
                                             _vp]),
    'arlgpu_plan_flags': (ctypes.c_int, [_i64, _P(GridDesc), _P(CfDesc), _vp, _sz, _P(ctypes.c_uint32), _vp]),
    'arlgpu_plan_plane_mean_w': (ctypes.c_int, [_vp, _i64, _P(GridDesc), _P(CfDesc), _vp, _sz, _vp, _vp]),
    'arlgpu_wstack_grid_to_image': (ctypes.c_int, [_vp, _P(GridDesc), ctypes.c_int, _vp, _vp, _f64, _vp, _vp, _vp,
                                                   _vp]),
    'arlgpu_grid_weights': (ctypes.c_int, [_vp, _vp, _vp, _i64, ctypes.c_int, _P(CfDesc), _vp, _P(GridDesc), _vp,
                                           _vp, _vp]),
    'arlgpu_reweight': (ctypes.c_int, [_vp, _vp, _vp, _i64, ctypes.c_int, _P(CfDesc), _vp, _P(GridDesc), _vp]),
    'arlgpu_convert_blocks': (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _i32, _i32, _i32, _i32, ctypes.c_int, _vp,
                                             _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    'arlgpu_decoalesce': (ctypes.c_int, [_vp, _i64, _vp, _i32, _i32, _i32, _i32, ctypes.c_int, _vp, _vp, _vp]),
    'arlgpu_dft_predict': (ctypes.c_int, [_vp, _vp, _i64, _vp, _vp, _i32, _i32, _i32, ctypes.c_int, _vp, _vp]),
    'arlgpu_dft_adjoint': (ctypes.c_int, [_vp, _i64, _vp, _i32, _i32, ctypes.c_int, _vp, _vp, _vp]),
    'arlgpu_hogbom': (ctypes.c_int, [_vp, _vp, _vp, _i32, _i32, _i32, _i32, _f64, _f64, _i32, _f64, _f64, _f64,
                                     _vp, _vp, _P(_i32), _vp]),
    'arlgpu_hogbom_complex': (ctypes.c_int, [_vp, _vp, _vp, _vp, _i32, _i32, _i32, _i32, _f64, _f64, _i32, _f64,
                                             _f64, _f64, _vp, _vp, _vp, _vp, _P(_i32), _vp]),
    'arlgpu_msclean_setup_bytes': (ctypes.c_int, [_i32, _i32, _i32, _i32, _i32, _P(_sz)]),
    'arlgpu_scale_stack': (ctypes.c_int, [_vp, _i32, _i32, _i32, _vp, _vp]),
    'arlgpu_scale_convolve_bytes': (ctypes.c_int, [_i32, _i32, _i32, _P(_sz)]),
    'arlgpu_scale_convolve': (ctypes.c_int, [_vp, _i32, _i32, _i32, _vp, _i32, _i32, _f64, _vp, _vp, _sz, _vp]),
    'arlgpu_msmfsclean': (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _i32, _i32, _i32, _i32, _i32, _i32, _f64,
                                         _f64, _i32, _i32, _vp, _P(_i32), _vp]),
    'arlgpu_msclean_setup': (ctypes.c_int, [_vp, _i32, _i32, _vp, _i32, _i32, _vp, _vp, _i32, _vp, _vp, _vp, _vp,
                                            _vp, _vp, _vp, _sz, _vp]),
    'arlgpu_msclean': (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _i32, _i32, _i32, _i32, _i32, _f64, _f64, _i32, _vp,
                                      _P(_i32), _vp]),
    'arlgpu_wstack_fftbuf_bytes': (ctypes.c_int, [_P(GridDesc), _P(ctypes.c_size_t)]),
    'arlgpu_wstack_image_to_grid': (ctypes.c_int, [_vp, _vp, _vp, _f64, _P(GridDesc), ctypes.c_int, _vp, _vp]),
    'arlgpu_degrid': (ctypes.c_int, [_vp, _vp, _i64, ctypes.c_int, _vp, _P(CfDesc), _vp, _P(GridDesc), _vp, _vp,
                                     _vp, _sz, _vp]),
    'arlgpu_fft_grid_to_image': (ctypes.c_int, [_vp, _P(GridDesc), ctypes.c_int, _vp, _vp, _vp, _vp, _vp, _vp]),
    'arlgpu_fft_image_to_grid': (ctypes.c_int, [_vp, _vp, _P(GridDesc), ctypes.c_int, _vp, _vp]),
    'arlgpu_make_pswf': (ctypes.c_int, [_i32, _i32, _i32, _i32, _vp, _vp, _vp]),
    'arlgpu_make_wkernels': (ctypes.c_int, [_i32, _f64, _i32, _i32, _i32, _i32, _f64, _i32, _vp, _vp]),
    'arlgpu_apply_gains': (ctypes.c_int, [_vp, _i64, _i32, ctypes.c_int, _vp, _vp, _vp, ctypes.c_int, _vp]),
    'arlgpu_apply_gaintable': (ctypes.c_int, [_vp, _i32, _i32, _i32, ctypes.c_int, _vp, _vp, _vp, ctypes.c_int,
                                              _vp]),
    'arlgpu_gain_chi2': (ctypes.c_int, [_vp, _vp, _vp, _i64, _i32, ctypes.c_int, _vp, _vp, _vp, _i32, _vp, _vp,
                                        _vp, _vp]),
    'arlgpu_phaserotate': (ctypes.c_int, [_vp, _vp, _i64, _i32, ctypes.c_int, _f64, _f64, ctypes.c_int, _vp]),
}


class ArlGpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__('arlgpu error %d: %s' % (code, msg))
        self.code = code


_lib = None
_lock = threading.Lock()


def load(path=LIB_PATH):
    """Load libarlgpu.so and bind the C ABI (raises if it was never built)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise RuntimeError('libarlgpu.so is not built (%s); run __graft_entry__.build() or '
                               'python algorithm-reference-library_gb300/build.py' % path)
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(status):
    if status != OK:
        msg = load().arlgpu_last_error()
        raise ArlGpuError(status, msg.decode() if msg else '')


def call(name, *args):
    check(getattr(load(), name)(*args))


def ptr(t):
    """Device pointer of a torch tensor (or None).  The caller must hold a
    reference to the tensor until the library call that uses the pointer has
    returned: a tensor dropped earlier can have its memory handed to the next
    allocation before the call's kernels are even queued."""
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def stream_ptr(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)
