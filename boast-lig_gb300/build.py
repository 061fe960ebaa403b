"""Build libconv_gb300.so (sm_103a) in-tree with nvcc.

Each translation unit under csrc/ is compiled in parallel to an object file
under _build/, then linked into ``libconv_gb300.so`` beside this file and
archived into ``libconv_gb300.a`` (the same objects, for callers that link
statically: a Fortran program links it with -lcudart -lstdc++).  The filter
header is regenerated first (deterministic; unchanged files are not
rewritten).  Only one -gencode is emitted: sm_103a.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libconv_gb300.so')
LIBA = os.path.join(HERE, 'libconv_gb300.a')
NVCC = os.environ.get('NVCC', '/usr/local/cuda/bin/nvcc')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '-Xcompiler', '-Wall',
         '--expt-relaxed-constexpr', '-I', CSRC, '-I', os.path.join(HERE, '..', 'include')]


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith('.cu'))


def _deps_newer(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    heads = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(('.cuh', '.h'))]
    heads += [os.path.join(HERE, '..', 'include', h)
              for h in ('libconv_gb300.h', 'libconv_fortran.h')]
    return any(os.path.getmtime(p) > t for p in [src] + heads if os.path.exists(p))


def _compile(src):
    obj = os.path.join(BUILD, os.path.basename(src)[:-3] + '.o')
    if _deps_newer(obj, src):
        cmd = [NVCC] + ARCH + FLAGS + ['-c', src, '-o', obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose=False):
    """Compile every CUDA source and link the shared library; returns its path."""
    subprocess.run([sys.executable, os.path.join(HERE, 'gen_filters.py')], check=True)
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(_compile, srcs))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [NVCC] + ARCH + ['-shared', '-o', LIB + '.tmp'] + objs + ['-lcudart']
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(LIB + '.tmp', LIB)
    if not os.path.exists(LIBA) or any(os.path.getmtime(o) > os.path.getmtime(LIBA) for o in objs):
        if os.path.exists(LIBA + '.tmp'):
            os.remove(LIBA + '.tmp')
        r = subprocess.run(['ar', 'rcs', LIBA + '.tmp'] + objs, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"archive failed:\n{r.stdout}\n{r.stderr}")
        os.replace(LIBA + '.tmp', LIBA)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == '__main__':
    build(verbose=True)
