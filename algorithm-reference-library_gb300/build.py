"""Build libarlgpu.so (sm_103a) in-tree with nvcc: one object per .cu, compiled
in parallel, linked against the CUDA runtime and cuFFT."""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libarlgpu.so')
INCLUDE = os.path.normpath(os.path.join(HERE, '..', 'include'))

ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-O3', '-std=c++17', '-lineinfo', '-Xcompiler', '-fPIC', '--expt-relaxed-constexpr', '-I' + INCLUDE]


def nvcc():
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found')


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith('.cu'))


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(verbose=False, force=False, extra_flags=()):
    """Compile every csrc/*.cu and link libarlgpu.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(('.cuh', '.h'))]
    headers.append(os.path.join(INCLUDE, 'arlgpu.h'))
    srcs = sources()
    objs = [os.path.join(BUILD, os.path.basename(s)[:-3] + '.o') for s in srcs]

    def compile_one(src, obj):
        if not force and _newer(obj, [src] + headers):
            return None
        cmd = [cc, '-c', src, '-o', obj] + ARCH + FLAGS + list(extra_flags)
        if verbose:
            print(' '.join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('nvcc failed for %s:\n%s%s' % (src, r.stdout, r.stderr))
        return r.stderr

    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        for msg in ex.map(compile_one, srcs, objs):
            if verbose and msg:
                print(msg, file=sys.stderr)
    if force or not _newer(LIB, objs):
        cmd = [cc, '-shared', '-o', LIB] + objs + ARCH + ['-lcufft', '-lcudart']
        if verbose:
            print(' '.join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('link failed:\n%s%s' % (r.stdout, r.stderr))
    return LIB


if __name__ == '__main__':
    print(build(verbose=True, force='--force' in sys.argv))
