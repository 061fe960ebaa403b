"""ctypes binding of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Loads ``liblibconv_oracle.so`` (the C restatement of the reference arithmetic,
see libconv_oracle.h) and, when built, ``_ref/libmf_ref.so`` (the reference's
own benchmark/convolutions-c/MagicFilter.c).  Arrays are numpy float64 buffers
addressed as flat Fortran-ordered memory, exactly as the reference routines
address them.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline use this module.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_int = ctypes.c_int
_dbl = ctypes.c_double

_SIGS = {
    'oracle_magicfilter_per_ref': [_int, _int, _D, _D],
    'oracle_magicfilter_per_t_ref': [_int, _int, _D, _D],
    'oracle_magicfilter_free_ref': [_int, _int, _D, _D],
    'oracle_magicfilter_free_t_ref': [_int, _int, _D, _D],
    'oracle_kinetic_per_ref': [_int, _int, _int, _D, _D, _D, _dbl],
    'oracle_kinetic_per_ref_ekin': [_int, _int, _int, _D, _D, _D, _D],
    'oracle_synthesis_per_ref': [_int, _int, _D, _D],
    'oracle_synthesis_free_ref': [_int, _int, _D, _D],
    'oracle_analysis_per_ref': [_int, _int, _D, _D],
    'oracle_analysis_free_ref': [_int, _int, _D, _D],
}
_CONV1D = [_int, _int, _I, _int, _I, _I, _int, _D, _D, _dbl, _dbl, _dbl]
_WAV1D = [_int, _int, _I, _int, _I, _I, _int, _D, _D, _dbl, _dbl]
for _n in ('md', 'imd', 'd1'):
    _SIGS[f'oracle_d_s0s0_1d_sym8_{_n}'] = _CONV1D
_SIGS['oracle_d_s0s0_1d_sym8_d2_dotin'] = _CONV1D + [_D]
for _n in ('oracle_d_s0s1_1d_sym8', 'oracle_d_s1s0_1d_sym8',
           'oracle_d_s0s1_1d_symicomb8', 'oracle_d_s1s0_1d_symicomb8'):
    _SIGS[_n] = _WAV1D
_SIGS['oracle_d_sfrf_ld_narr'] = [_int, _I, _I, _I, _I, _int, _D, _D, _D, _D]
_SIGS['oracle_d_rfsf_ld_narr'] = _SIGS['oracle_d_sfrf_ld_narr']
_SIGS['oracle_d_kin'] = [_int, _I, _I, _D, _D, _D, _D, _D, _dbl, _dbl]
_SIGS['oracle_d_dwt_sym8'] = [_int, _I, _I, _D, _D, _D, _D]
_SIGS['oracle_d_idwt_sym8'] = _SIGS['oracle_d_dwt_sym8']
_SIGS['oracle_hamiltonian'] = [_I, _I, _D, _D, _D, _D, _D, _D, _D]
_SIGS['oracle_poisson_broker'] = [_int, _int, _I, _int, _D, _D, _dbl]
_SIGS['oracle_div_u_i'] = [_int, _int, _int, _int, _D, _D, _int, _D, _D]
_SIGS['oracle_nabla_u'] = [_int, _int, _int, _int, _D, _D, _int, _D]
_SIGS['oracle_nabla_u_and_square'] = [_int, _int, _int, _int, _D, _D, _D, _int, _D]
_SIGS['oracle_nabla_u_square'] = [_int, _int, _int, _int, _D, _D, _int, _D]
_SIGS['oracle_nabla_u_epsilon'] = [_int, _int, _int, _int, _D, _D, _int, _D, _D]
_SIGS['oracle_update_rhopol'] = [_int, _int, _int, _int, _D, _int, _D, _dbl, _D, _D, _D]
_SIGS['oracle_div_u_i_ref'] = [_int, _int, _int, _int, _D, _D, _int, _D]


def build(ref=None, ref_dir=None):
    """Compile the oracle, and the reference's MagicFilter.c when the
    reference tree is given (ref_dir, else $LIBCONV_REFERENCE_DIR; no default:
    without it the reference build is skipped).  Returns True when the
    reference build was made."""
    subprocess.run(['make', '-s', '-C', HERE, 'all'], check=True)
    ref_dir = ref_dir or os.environ.get('LIBCONV_REFERENCE_DIR')
    if not ref_dir:
        return False
    want_ref = ref if ref is not None else os.path.isdir(ref_dir)
    if want_ref and os.path.isfile(os.path.join(ref_dir, 'benchmark/convolutions-c/MagicFilter.c')):
        subprocess.run(['make', '-s', '-C', HERE, 'ref', f'REF_DIR={ref_dir}'], check=True)
        return True
    return False


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, 'liblibconv_oracle.so')
        if not os.path.exists(path):
            build(ref=False)
        L = ctypes.CDLL(path)
        for name, args in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = None if name.endswith(('_per_ref', '_per_t_ref', '_free_ref', '_free_t_ref', '_ref_ekin')) or name == 'oracle_kinetic_per_ref' else ctypes.c_int
        _LIB = L
    return _LIB


_TIMING = None


def timing_lib():
    """The CPU baseline timing build (liblibconv_timing.so: the restatement at
    -O3 with OpenMP step drivers), or None when it is not built."""
    global _TIMING
    if _TIMING is None:
        path = os.path.join(HERE, 'liblibconv_timing.so')
        if not os.path.exists(path):
            return None
        T = ctypes.CDLL(path)
        T.timing_mfkin_step.argtypes = [_int, _I, _D, _D, _D, _D, _int]
        T.timing_mfkin_step.restype = ctypes.c_double
        T.timing_wavelet_step.argtypes = [_int, _I, _D, _D, _D, _int]
        T.timing_wavelet_step.restype = ctypes.c_double
        T.timing_max_threads.argtypes = []
        T.timing_max_threads.restype = _int
        _TIMING = T
    return _TIMING


def ref_lib():
    """The reference's own MagicFilter.c, or None when it was not built."""
    global _REF
    if _REF is None:
        path = os.path.join(HERE, '_ref', 'libmf_ref.so')
        if not os.path.exists(path):
            return None
        R = ctypes.CDLL(path)
        U = ctypes.POINTER(ctypes.c_uint)
        for name in ('magicfilter1d_naive_', 'magicfilter1d_t_naive_'):
            getattr(R, name).argtypes = [U, U, _D, _D]
            getattr(R, name).restype = None
        _REF = R
    return _REF


def dp(a):
    """double* of a contiguous float64 array (None -> NULL)."""
    if a is None:
        return None
    assert a.dtype == np.float64 and (a.flags.c_contiguous or a.flags.f_contiguous)
    return a.ctypes.data_as(_D)


def ip(v):
    if v is None:
        return None
    arr = (ctypes.c_int * len(v))(*[int(t) for t in v])
    return arr


def call(name, *args):
    """Call an oracle routine; numpy arrays and int lists are converted."""
    fn = getattr(lib(), name)
    conv = []
    for a, t in zip(args, fn.argtypes):
        if isinstance(a, np.ndarray):
            conv.append(dp(a))
        elif t is _I:
            conv.append(ip(a))
        elif t is _D and isinstance(a, ctypes.Array):
            conv.append(ctypes.cast(a, _D))
        else:
            conv.append(a)
    return fn(*conv)


def ref_magicfilter(n, ndat, x, transposed_filter=False):
    """Run the reference MagicFilter.c naive kernel: x(0:n-1,ndat) -> y(ndat,0:n-1)."""
    R = ref_lib()
    if R is None:
        raise RuntimeError('reference MagicFilter.c was not built (oracle/_ref)')
    y = np.zeros(n * ndat)
    fn = R.magicfilter1d_t_naive_ if transposed_filter else R.magicfilter1d_naive_
    cn, cd = ctypes.c_uint(n), ctypes.c_uint(ndat)
    fn(ctypes.byref(cn), ctypes.byref(cd), dp(np.ascontiguousarray(x, dtype=np.float64)), dp(y))
    return y
