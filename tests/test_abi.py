"""C-ABI library checks that need no GPU: it loads, exports every symbol the
header declares, validates arguments before touching the device, and its
cost model follows the reference formula (GenericConvolution2.rb:1269-1276,
1525-1558, 1850-1932)."""
import ctypes
import os

import numpy as np
import pytest


def test_library_exports_every_declared_symbol(pkg):
    L = pkg.lib()
    names = pkg.declared_symbols()
    assert len(names) >= 37
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    import subprocess
    nm = subprocess.run(['nm', '-D', '--defined-only', pkg.LIB_PATH], capture_output=True, text=True)
    if nm.returncode == 0:
        exported = {l.split()[2] for l in nm.stdout.splitlines()
                    if ' T ' in l and not l.split()[2].startswith('_Z')}
        assert exported == set(names), exported ^ set(names)
    assert pkg.lib().libconv_gb300_version().decode().startswith('libconv-gb300')


def test_status_strings(pkg):
    L = pkg.lib()
    for code in (0, -1, -2, -3, -4, -5, -6):
        assert L.libconv_gb300_strerror(code).decode() != 'unknown status'


@pytest.mark.parametrize('bc,nx,ny,status', [
    (7, 8, 8, -2),       # unknown BC
    (1, 8, 8, -3),       # grow needs ny >= n + 15
    (-1, 8, 8, -3),      # shrink needs nx >= n + 15
    (0, 0, 8, -1),       # bad leading size
])
def test_argument_validation_before_device(pkg, bc, nx, ny, status):
    x = np.zeros(1024)
    y = np.zeros(1024)
    with pytest.raises(pkg.LibconvError) as e:
        pkg.Kernel('d_s0s0_1d_sym8_md').run(1, 0, [8], bc, [nx], [ny], 1, x, y, 1.0, 0.0, 0.0)
    assert e.value.status == status
    assert pkg.last_error() != ''


def test_kinetic_rejects_grow(pkg):
    x = np.zeros(512)
    with pytest.raises(pkg.LibconvError) as e:
        pkg.Kernel('d_kin').run(3, [8, 8, 8], [1, 0, 0], x, x.copy(), x.copy(), x.copy(),
                                [1.0, 1.0, 1.0], 0.0, 0.0)
    assert e.value.status == -2


def test_mode_setting(pkg):
    pkg.set_mode(pkg.MODE_FP64)
    with pytest.raises(pkg.LibconvError):
        pkg.set_mode(99)


@pytest.mark.parametrize('value,mode', [(None, 0), ('tc_exact', 1), ('tc_bf16x3', 2), ('3', 3),
                                        ('fp64', 0), ('no-such-mode', 0), ('7', 0)])
def test_initial_mode_from_environment(pkg, value, mode):
    """A fresh process (and each of its threads) starts in the mode that
    LIBCONV_GB300_MODE names, FP64 when it is unset or names no mode."""
    import subprocess
    import sys
    env = dict(os.environ)
    env.pop('LIBCONV_GB300_MODE', None)
    if value is not None:
        env['LIBCONV_GB300_MODE'] = value
    code = ('import ctypes, sys, threading\n'
            'L = ctypes.CDLL(sys.argv[1])\n'
            'out = [L.libconv_gb300_get_mode()]\n'
            't = threading.Thread(target=lambda: out.append(L.libconv_gb300_get_mode()))\n'
            't.start(); t.join()\n'
            'print(out[0], out[1])\n')
    r = subprocess.run([sys.executable, '-c', code, pkg.LIB_PATH], capture_output=True, text=True,
                       env=env, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.split() == [str(mode), str(mode)]


def test_cost_model(pkg):
    n = [124, 132, 130]
    N = int(np.prod(n))
    # 1D: n[idim] * filter.cost * prod(other n) * narr
    assert pkg.cost('d_s0s0_1d_sym8_md_cost', 3, 1, n, 0, 2) == 32 * N * 2
    assert pkg.cost('d_s0s0_1d_sym8_d2_cost', 3, 0, n, 0, 1) == 58 * N
    assert pkg.cost('d_s0s1_1d_sym8_cost', 3, 0, [62, 66, 65], 0, 1) == 62 * 64 * 66 * 65
    # 3D periodic MagicFilter: 3 sweeps of 32 flop per point
    assert pkg.cost('d_sfrf_cost', 3, n, [0, 0, 0], 1) == 96 * N
    # grow: sizes grow sweep by sweep
    g = [v + 15 for v in n]
    want = 32 * (n[0] * n[1] * n[2] + n[1] * g[0] * n[2] + n[2] * g[0] * g[1])
    assert pkg.cost('d_sfrf_cost', 3, n, [1, 1, 1], 1) == want
    assert pkg.cost('d_kin_cost', 3, n, [0, 0, 0]) == 174 * N
    # wavelets: n pairs * 64 * (2n)(2n) per sweep
    m = [62, 66, 65]
    assert pkg.cost('d_dwt_sym8_cost', 3, m, [0, 0, 0]) == 3 * 64 * 4 * int(np.prod(m))


def test_declared_signatures_match_binding(pkg):
    """Every 1D / 3D operator the header declares has a host and a _dev
    export bound with the argument count of its reference procedure."""
    declared = set(pkg.declared_symbols())
    for name, args in pkg.SIGNATURES.items():
        assert name in declared and name + '_dev' in declared
    assert len(pkg.SIGNATURES['d_s0s0_1d_sym8_md']) == 12   # d,idim,n,bc,nx,ny,narr,x,y,a,a_x,a_y
    assert len(pkg.SIGNATURES['d_s0s1_1d_sym8']) == 11      # ... a, a_y
    assert len(pkg.SIGNATURES['d_sfrf_ld_narr']) == 10      # d,n,bc,nx,ny,narr,x,y,w1,w2
    assert len(pkg.SIGNATURES['d_kin']) == 10               # d,n,bc,x,y,w1,w2,a,a_x,a_y


def test_hamiltonian_sizes_and_validation(pkg):
    """Host logic of the local Hamiltonian (no device call): the fine grid
    grows by 14 and the real-space grid by 15 more along a free axis, and
    grow/shrink boundaries are refused (the pipeline chooses them itself)."""
    nsig, nreal, nwork = pkg.hamiltonian_sizes([5, 4, 6], [2, 0, 2])
    assert nsig == 8 * 5 * 4 * 6
    assert nreal == (10 + 14 + 15) * 8 * (12 + 14 + 15)
    nf = (10 + 14) * 8 * (12 + 14)
    assert nwork >= 2 * nf + nreal
    assert pkg.hamiltonian_sizes([3, 3, 3], [0, 0, 0])[1] == 6 ** 3
    for bad in ([1, 0, 0], [0, -1, 0], [0, 0, 7]):
        with pytest.raises(pkg.LibconvError) as e:
            pkg.hamiltonian_sizes([4, 4, 4], bad)
        assert e.value.status == -2
    with pytest.raises(pkg.LibconvError) as e:
        pkg.hamiltonian_sizes([4, 0, 4], [0, 0, 0])
    assert e.value.status == -1


def test_fortran_names_ids_and_sizes(pkg):
    """Fortran-facing layer, host-only parts: filter / boundary ids and names
    with blank-padded CHARACTER arguments, the size queries in the order the
    pipeline calls them (libconv.f90:248-256), and the status word."""
    F = pkg.Fortran()
    ids = {nm: F.filter_id(nm) for nm in ('SYM8_LP', 'SYM8_MD', 'SYM8_MI', 'SYM8_D1', 'SYM8_D2',
                                          'SYMICOMB8')}
    assert sorted(ids.values()) == [1, 2, 3, 4, 5, 6] and F.status() == 0
    assert F.filter_id('sym8_md  ') == ids['SYM8_MD']          # case and trailing blanks
    assert F.filter_id('SYM8_IMD') == ids['SYM8_MI']
    assert F.filter_name(ids['SYM8_D2']) == 'SYM8_D2'
    assert F.filter_id('NOPE') == 0 and F.status() == -1
    assert [F.bc_id(c) for c in 'PGSF'] == [0, 1, -1, 2]
    assert F.bc_id('fg') == 1 and F.bc_name(-1) == 'S'
    assert F.bc_id('X') == 0 and F.status() == -2
    n = [48, 40, 32]
    lp, md = ids['SYM8_LP'], ids['SYM8_MD']
    grow, shrink = [1] * 3, [-1] * 3
    ns0 = F.sizes('get_s1s0_output_size', 3, n, lp, grow)
    assert ns0 == [v + 7 for v in n]                           # pairs: 2n + 14 points
    assert F.sizes('get_s1s0_input_size', 3, n, lp, grow) == n
    assert F.sizes('get_s0s1_input_size', 3, n, lp, shrink) == [v + 7 for v in n]
    npsir = F.sizes('get_s0s0_md_output_size', 3, [2 * v for v in ns0], md, grow)
    assert npsir == [2 * v + 15 for v in ns0]
    assert F.sizes('get_s0s0_md_work_size', 3, [2 * v for v in ns0], md, grow, work=True) >= \
        2 * int(np.prod(npsir))
    assert F.sizes('get_s0s0_1ds_output_size', 3, n, ids['SYM8_D2'], [2] * 3) == n
    with pytest.raises(pkg.LibconvError):
        F.sizes('get_s0s1_input_size', 3, n, md, shrink)       # not a wavelet filter
    # tp must be 8; nothing reaches the device
    st = F.call('s0s0_md', md, 4, 3, n, [0] * 3, n, n, 1, 1.0, 0.0, 0.0, np.zeros(1), np.zeros(1),
                np.zeros(1), check=False)
    assert st == -1 and 'tp' in pkg.last_error()


def test_static_library_links_a_fortran_style_caller(pkg, tmp_path):
    """libconv_gb300.a links into a program that calls the Fortran-facing
    procedures the way gfortran would (symbols with a trailing underscore,
    arguments by reference, hidden CHARACTER lengths).  Only the link is
    checked here (no GPU); the program asks for the filter id and sizes,
    which need no device."""
    import os
    import shutil
    import subprocess
    lib_a = os.path.join(os.path.dirname(pkg.LIB_PATH), 'libconv_gb300.a')
    cc = shutil.which('gcc')
    if not cc or not os.path.exists(lib_a):
        pytest.skip('gcc or libconv_gb300.a missing')
    src = tmp_path / 'caller.c'
    src.write_text(r'''
#include <stdio.h>
#include <stddef.h>
void get_filter_id_(const char *, int *, size_t);
void get_s1s0_output_size_(const int *, const int *, const int *, const int *, int *);
void libconv_status_(int *);
void s0s0_md_(const int *, const int *, const int *, const int *, const int *, const int *,
              const int *, const int *, const double *, const double *, const double *,
              const double *, double *, double *);
int main(int argc, char **argv) {
    int fil = 0, st = -99, d = 3, n[3] = {4, 5, 6}, bc[3] = {1, 1, 1}, ns0[3];
    get_filter_id_("SYM8_LP ", &fil, 8);
    get_s1s0_output_size_(&d, n, &fil, bc, ns0);
    libconv_status_(&st);
    printf("%d %d %d %d %d\n", fil, st, ns0[0], ns0[1], ns0[2]);
    if (argc > 5) s0s0_md_(0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0);   /* referenced only */
    return 0;
}
''')
    cuda_lib = '/usr/local/cuda/lib64'
    exe = tmp_path / 'caller'
    r = subprocess.run([cc, str(src), lib_a, '-L' + cuda_lib, '-lcudart', '-lstdc++', '-lm',
                        '-lpthread', '-ldl', '-o', str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    run = subprocess.run([str(exe)], capture_output=True, text=True,
                         env={**os.environ, 'LD_LIBRARY_PATH': cuda_lib})
    assert run.returncode == 0, run.stderr
    assert run.stdout.split() == ['1', '0', '11', '12', '13']


def _build_module():
    import importlib.util
    import os
    import sys
    here = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), 'boast-lig_gb300')
    spec = importlib.util.spec_from_file_location('lcg_build_module', os.path.join(here, 'build.py'))
    mod = importlib.util.module_from_spec(spec)
    sys.modules['lcg_build_module'] = mod
    spec.loader.exec_module(mod)
    return mod


def _prototypes(path, ret):
    import re
    text = re.sub(r'/\*.*?\*/', '', open(path).read(), flags=re.S)
    return {n: ' '.join(a.split()).replace('* ', '*')
            for n, a in re.findall(r'\b' + ret + r'\s+(\w+)\s*\(([^;{]*?)\)\s*;', text, flags=re.S)}


def test_boast_void_shims(pkg, tmp_path):
    """libconv_gb300_boast.so exports every procedure of include/libconv_boast.h
    (the generated procedures' void prototypes), each declared with the same
    parameters in libconv_gb300.h; the header is the one the build writes;
    the main library binds its own entry points locally, so shims loaded
    first cannot intercept its internal calls (the Fortran layer calls the C
    entry points); a C caller built against the void prototypes links."""
    import os
    import shutil
    import subprocess
    B = _build_module()
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), 'include')
    boast_h = os.path.join(inc, 'libconv_boast.h')
    assert open(boast_h).read() == B.boast_header_text()
    void_protos = _prototypes(boast_h, 'void')
    int_protos = _prototypes(os.path.join(inc, 'libconv_gb300.h'), 'int')
    assert len(void_protos) >= 20
    for n, args in void_protos.items():
        assert int_protos.get(n) == args, n
    shim = os.path.join(os.path.dirname(pkg.LIB_PATH), 'libconv_gb300_boast.so')
    assert os.path.exists(shim)
    nm = subprocess.run(['nm', '-D', '--defined-only', shim], capture_output=True, text=True)
    if nm.returncode == 0:
        exported = {l.split()[2] for l in nm.stdout.splitlines() if ' T ' in l}
        assert exported == set(void_protos), exported ^ set(void_protos)
    re_out = subprocess.run(['readelf', '-rW', pkg.LIB_PATH], capture_output=True, text=True)
    if re_out.returncode == 0:
        for line in re_out.stdout.splitlines():
            f = line.split()
            assert not (len(f) >= 5 and f[4] in void_protos), line
    cc = shutil.which('gcc')
    if not cc:
        pytest.skip('gcc missing')
    src = tmp_path / 'boast_caller.c'
    src.write_text('#include "libconv_boast.h"\n#include <stdio.h>\n'
                   'int main(int argc, char **argv) {\n'
                   '    if (argc > 5) d_s0s0_1d_sym8_md(0, 0, 0, 0, 0, 0, 0, 0, 0, 0.0, 0.0, 0.0);\n'
                   '    if (argc > 5) d_kin(0, 0, 0, 0, 0, 0, 0, 0, 0.0, 0.0);\n'
                   '    printf("linked\\n");\n    return 0;\n}\n')
    exe = tmp_path / 'boast_caller'
    r = subprocess.run([cc, '-I', inc, str(src), '-L', os.path.dirname(shim), '-l:libconv_gb300_boast.so',
                        '-o', str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
