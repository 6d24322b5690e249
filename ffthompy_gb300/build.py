"""Build libffthompy_gb300.so in-tree with nvcc (sm_103a only).

Each translation unit of ffthompy_gb300/csrc is compiled in parallel, then
linked into ffthompy_gb300/_lib/libffthompy_gb300.so with the CUDA runtime
linked statically, so the library needs only libcuda at run time.
Usage: python -m ffthompy_gb300.build [--force]
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
LIBDIR = os.path.join(HERE, '_lib')
OBJDIR = os.path.join(LIBDIR, 'obj')
LIBNAME = 'libffthompy_gb300.so'
LIBPATH = os.path.join(LIBDIR, LIBNAME)
SOURCES = ['fhp_engine_f64.cu', 'fhp_engine_f32.cu', 'fhp_capi.cu', 'fhp_lineplan.cpp',
           'fhp_noalloc.cu', 'fhp_coef.cu']
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']


def _nvcc():
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found: the CUDA toolkit is required to build ffthompy_gb300')


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(os.path.dirname(HERE), 'include', 'ffthompy_gb300.h'))
    return max(os.path.getmtime(f) for f in files)


def _compile(src):
    nvcc = _nvcc()
    obj = os.path.join(OBJDIR, os.path.splitext(src)[0] + '.o')
    cmd = [nvcc, '-std=c++17', '-O3', '-lineinfo', '-Xcompiler', '-fPIC', *ARCH,
           '-Xptxas', '-v' if os.environ.get('FHP_PTXAS_VERBOSE') else '-O3',
           '-c', os.path.join(CSRC, src), '-o', obj]
    if src.endswith('.cpp'):
        cmd = [nvcc, '-std=c++17', '-O3', '-Xcompiler', '-fPIC', '-x', 'c++',
               '-c', os.path.join(CSRC, src), '-o', obj]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError('nvcc failed for %s:\n%s\n%s' % (src, p.stdout, p.stderr))
    return obj, p.stderr


def build(force=False, verbose=False):
    """Compile and link; returns the path of the shared library."""
    if not force and os.path.exists(LIBPATH) and os.path.getmtime(LIBPATH) >= _deps():
        return LIBPATH
    os.makedirs(OBJDIR, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(_compile, SOURCES))
    if verbose:
        for _, log in results:
            if log:
                print(log)
    tmp = LIBPATH + '.tmp'
    cmd = [_nvcc(), '-shared', *ARCH, '-o', tmp] + [o for o, _ in results] + ['-cudart', 'static']
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError('link failed:\n%s\n%s' % (p.stdout, p.stderr))
    os.replace(tmp, LIBPATH)
    return LIBPATH


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose='-v' in sys.argv))
