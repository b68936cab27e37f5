"""The C ABI: libarlgpu.so loads and exports every entry point include/arlgpu.h
declares, and the ctypes mirrors of its structs have the C layout.  No GPU call."""
import ctypes
import os
import re
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, 'include', 'arlgpu.h')


def declared():
    src = open(HEADER).read()
    return sorted(set(re.findall(r'\b(arlgpu_[a-z0-9_]+)\s*\(', src)))


@pytest.fixture(scope='module')
def lib(arl):
    path = arl._native.LIB_PATH
    if not os.path.exists(path):
        if not shutil.which('nvcc') and not os.path.exists('/usr/local/cuda/bin/nvcc'):
            pytest.skip('libarlgpu.so not built and nvcc unavailable')
        import importlib
        importlib.import_module('algorithm-reference-library_gb300.build').build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = declared()
    for must in ('arlgpu_grid', 'arlgpu_degrid', 'arlgpu_convolution_mapping', 'arlgpu_fft_grid_to_image',
                 'arlgpu_fft_image_to_grid', 'arlgpu_make_pswf', 'arlgpu_make_wkernels'):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(arl):
    assert set(declared()) <= set(arl._native.SIGNATURES)


def test_version_string(lib):
    lib.arlgpu_version.restype = ctypes.c_char_p
    assert lib.arlgpu_version().startswith(b'arlgpu')


def test_struct_layout_matches_c(arl):
    gcc = shutil.which('gcc')
    if not gcc:
        pytest.skip('gcc unavailable')
    prog = r'''
#include <stdio.h>
#include <stddef.h>
#include "arlgpu.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(arlgpu_axis), sizeof(arlgpu_grid_desc),
         offsetof(arlgpu_grid_desc, u), offsetof(arlgpu_grid_desc, f), sizeof(arlgpu_cf_desc),
         offsetof(arlgpu_cf_desc, chan_stride), offsetof(arlgpu_cf_desc, plane_support),
         offsetof(arlgpu_cf_desc, tap_absmax));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, 'l.c')
        open(c, 'w').write(prog)
        exe = os.path.join(d, 'l')
        subprocess.check_call([gcc, c, '-I', os.path.join(ROOT, 'include'), '-o', exe])
        got = [int(x) for x in subprocess.check_output([exe]).split()]
    n = arl._native
    want = [ctypes.sizeof(n.Axis), ctypes.sizeof(n.GridDesc), n.GridDesc.u.offset, n.GridDesc.f.offset,
            ctypes.sizeof(n.CfDesc), n.CfDesc.chan_stride.offset, n.CfDesc.plane_support.offset,
            n.CfDesc.tap_absmax.offset]
    assert got == want


def test_fails_loudly_without_cuda(arl):
    import torch
    if torch.cuda.is_available():
        pytest.skip('a CUDA device is present')
    with pytest.raises(RuntimeError):
        arl.device.require_cuda()
