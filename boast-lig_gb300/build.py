"""Build libconv_gb300.so (sm_103a) in-tree with nvcc.

Each translation unit under csrc/ is compiled in parallel to an object file
under _build/, then linked into ``libconv_gb300.so`` beside this file and
archived into ``libconv_gb300.a`` (the same objects, for callers that link
statically: a Fortran program links it with -lcudart -lstdc++).  The filter
header is regenerated first (deterministic; unchanged files are not
rewritten).  Only one -gencode is emitted: sm_103a.

``libconv_gb300_boast.so`` (plain C, gcc) exports the host-pointer compute
entry points under the same names with the generated procedures' void
prototypes (``include/libconv_boast.h``, written from the main header): a
caller built against those prototypes links it instead of the main library.
Each shim resolves its target through a dlopen handle of libconv_gb300.so
beside it; the main library binds its own internal calls locally
(-Bsymbolic-functions), so a shim loaded first never intercepts them.
"""
import concurrent.futures as cf
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libconv_gb300.so')
LIBA = os.path.join(HERE, 'libconv_gb300.a')
LIBB = os.path.join(HERE, 'libconv_gb300_boast.so')
INCLUDE = os.path.join(HERE, '..', 'include')
BOAST_HEADER = os.path.join(INCLUDE, 'libconv_boast.h')
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
    if (not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs)
            or os.path.getmtime(__file__) > os.path.getmtime(LIB)):   # the link recipe changed
        cmd = [NVCC] + ARCH + ['-shared', '-Xlinker', '-Bsymbolic-functions', '-o', LIB + '.tmp'] + \
            objs + ['-lcudart']
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
    build_boast_shims()
    if verbose:
        print(f"built {LIB}")
    return LIB


def _host_entries():
    """(name, [(type, arg)]) of every host-pointer compute entry point of the
    main header: int-returning, no stream argument, not the libconv_* library
    calls, not the size / cost queries."""
    text = open(os.path.join(INCLUDE, 'libconv_gb300.h')).read()
    text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
    out = []
    for name, args in re.findall(r'\bint\s+(\w+)\s*\(([^;{]*?)\)\s*;', text, flags=re.S):
        if (name.endswith(('_dev', '_cost', '_size', '_sizes', '_noalloc')) or name.startswith('libconv')
                or 'void *stream' in args):
            continue
        params = []
        for a in ' '.join(args.split()).split(','):
            a = a.strip()
            m = re.match(r'(.*?)(\w+)$', a)
            params.append((m.group(1).strip(), m.group(2)))
        out.append((name, params))
    return out


def boast_header_text():
    """include/libconv_boast.h: the void prototypes of the shim library."""
    lines = ['/* Generated from libconv_gb300.h by boast-lig_gb300/build.py: the host-pointer',
             ' * compute entry points with the void prototypes of the generated procedures',
             ' * (scalars by value, arrays by pointer, no status), exported by',
             ' * libconv_gb300_boast.so.  A failure is reported on stderr and aborts the',
             ' * process; libconv_gb300.h gives the same procedures with an int status.',
             ' * Include one of the two headers, not both. */',
             '#ifndef LIBCONV_BOAST_H', '#define LIBCONV_BOAST_H', '', '#ifdef __cplusplus',
             'extern "C" {', '#endif', '']
    for name, params in _host_entries():
        lines.append(f'void {name}(' + ', '.join(f'{t} {a}'.replace('* ', '*') for t, a in params) + ');')
    lines += ['', '#ifdef __cplusplus', '}', '#endif', '#endif /* LIBCONV_BOAST_H */', '']
    return '\n'.join(lines)


def _shim_source():
    src = ['/* Generated by boast-lig_gb300/build.py: void shims over libconv_gb300.so. */',
           '#define _GNU_SOURCE', '#include <dlfcn.h>', '#include <stdio.h>', '#include <stdlib.h>',
           '#include <string.h>', '',
           'static void *target(const char *name) {',
           '    static void *handle;',
           '    void *h = __atomic_load_n(&handle, __ATOMIC_ACQUIRE);',
           '    if (!h) {',
           '        Dl_info info;',
           '        char path[4096];',
           '        if (!dladdr((void *)&target, &info) || !info.dli_fname ||',
           '            strlen(info.dli_fname) + 32 > sizeof path) {',
           '            fprintf(stderr, "libconv_gb300_boast: cannot locate itself\\n");',
           '            abort();',
           '        }',
           '        strcpy(path, info.dli_fname);',
           '        char *slash = strrchr(path, \'/\');',
           '        strcpy(slash ? slash + 1 : path, "libconv_gb300.so");',
           '        h = dlopen(path, RTLD_NOW | RTLD_LOCAL);',
           '        if (!h) {',
           '            fprintf(stderr, "libconv_gb300_boast: %s\\n", dlerror());',
           '            abort();',
           '        }',
           '        __atomic_store_n(&handle, h, __ATOMIC_RELEASE);',
           '    }',
           '    void *f = dlsym(h, name);',
           '    if (!f) {',
           '        fprintf(stderr, "libconv_gb300_boast: %s not found\\n", name);',
           '        abort();',
           '    }',
           '    return f;',
           '}', '',
           'static void report(const char *name, int status) {',
           '    const char *(*msg)(void) = (const char *(*)(void))target("libconv_gb300_last_error");',
           '    fprintf(stderr, "libconv_gb300: %s failed with status %d: %s\\n", name, status, msg());',
           '    abort();',
           '}', '']
    for name, params in _host_entries():
        decl = ', '.join(f'{t} {a}' for t, a in params)
        types = ', '.join(t for t, _ in params)
        names = ', '.join(a for _, a in params)
        src += [f'void {name}({decl}) {{',
                f'    static int (*f)({types});',
                f'    int (*g)({types}) = __atomic_load_n(&f, __ATOMIC_ACQUIRE);',
                f'    if (!g) {{',
                f'        g = (int (*)({types}))target("{name}");',
                f'        __atomic_store_n(&f, g, __ATOMIC_RELEASE);',
                f'    }}',
                f'    int rc = g({names});',
                f'    if (rc) report("{name}", rc);',
                f'}}', '']
    return '\n'.join(src)


def build_boast_shims():
    """Write include/libconv_boast.h (if changed) and build the void shim library."""
    text = boast_header_text()
    if not os.path.exists(BOAST_HEADER) or open(BOAST_HEADER).read() != text:
        with open(BOAST_HEADER, 'w') as f:
            f.write(text)
    os.makedirs(BUILD, exist_ok=True)
    csrc = os.path.join(BUILD, 'boast_shims.c')
    code = _shim_source()
    if not os.path.exists(csrc) or open(csrc).read() != code:
        with open(csrc, 'w') as f:
            f.write(code)
    if not os.path.exists(LIBB) or os.path.getmtime(csrc) > os.path.getmtime(LIBB):
        r = subprocess.run(['gcc', '-O2', '-std=c11', '-Wall', '-shared', '-fPIC', '-o', LIBB + '.tmp', csrc,
                            '-ldl'], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"shim build failed:\n{r.stdout}\n{r.stderr}")
        os.replace(LIBB + '.tmp', LIBB)
    return LIBB


if __name__ == '__main__':
    build(verbose=True)
