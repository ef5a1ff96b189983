"""Build libfastpm_gb300.so in place (nvcc, sm_103a, one translation unit per
source file compiled in parallel, then linked).  No cmake, no torch extension
machinery: the library is plain C ABI and is loaded with ctypes."""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
REPO = os.path.dirname(PKG)
SOURCES = ['fft.cu', 'particles.cu', 'power.cu', 'trace.cu', 'adjoint.cu']
LIB = os.path.join(PKG, 'libfastpm_gb300.so')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '--expt-relaxed-constexpr',
         '-I' + os.path.join(REPO, 'include')]


def nvcc():
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found')


def build(verbose=False, extra=(), lib=None):
    outdir = os.path.join(PKG, '_build')
    os.makedirs(outdir, exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(outdir, src.replace('.cu', '.o'))
        cmd = [cc, '-c', os.path.join(HERE, src), '-o', obj] + ARCH + FLAGS + list(extra)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('nvcc failed for %s:\n%s\n%s' % (src, ' '.join(cmd), r.stderr))
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    out = lib or LIB
    tmp = out + '.tmp'
    cmd = [cc, '-shared', '-o', tmp] + objs + ARCH + ['-lcudart']
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('link failed:\n%s\n%s' % (' '.join(cmd), r.stderr))
    os.replace(tmp, out)
    return out


if __name__ == '__main__':
    extra = sys.argv[1:]
    print(build(verbose=True, extra=extra))
