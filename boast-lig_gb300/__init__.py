"""libconv-gb300 host side: ctypes binding of the sm_103a C-ABI library.

The binding mirrors how the reference drives its generated kernels: a BOAST
``CKernel`` is run as ``k.run(*args)`` with the procedure's own argument list
and returns a stats hash ``{:duration, :reference_return}``
(BOAST runtime, called e.g. at BigDFT/MagicFilter1d2.rb:55-58 and
BigDFT/Kinetic1d-nb.ipynb cells 15-16).  ``Kernel(name).run(...)`` here takes
the same arguments in the same order (numpy arrays in place of NArrays) and
returns ``{'duration': seconds, 'reference_return': {...}}``; a non-zero status
raises ``LibconvError``.  ``run_dev`` is the device-pointer form (torch CUDA
tensors or raw integer addresses plus an optional stream).

There is no CPU fallback: if the CUDA library is missing the import of the
kernel fails loudly.
"""
import ctypes
import os
import re
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, 'libconv_gb300.so')
HEADER = os.path.join(HERE, '..', 'include', 'libconv_gb300.h')
FORTRAN_HEADER = os.path.join(HERE, '..', 'include', 'libconv_fortran.h')

BC_SHRINK, BC_PERIODIC, BC_GROW, BC_FREE = -1, 0, 1, 2
MODE_FP64 = 0
MODE_TC_EXACT = 1
MODE_TC_BF16X3 = 2
MODE_TC_TF32X3 = 3

_I = ctypes.POINTER(ctypes.c_int)
_D = ctypes.POINTER(ctypes.c_double)
_L = ctypes.POINTER(ctypes.c_longlong)
_int, _dbl, _vp = ctypes.c_int, ctypes.c_double, ctypes.c_void_p

_CONV1D = [_int, _int, _I, _int, _I, _I, _int, _vp, _vp, _dbl, _dbl, _dbl]
_WAV1D = [_int, _int, _I, _int, _I, _I, _int, _vp, _vp, _dbl, _dbl]
_MDT = [_int, _I, _I, _I, _I, _int, _vp, _vp, _vp, _vp]
_WMD = [_int, _I, _I, _vp, _vp, _vp, _vp]
_KIN = [_int, _I, _I, _vp, _vp, _vp, _vp, _D, _dbl, _dbl]
_KINN = [_int, _I, _I, _int, _vp, _vp, _vp, _vp, _D, _dbl, _dbl]
_WMDN = [_int, _I, _I, _int, _vp, _vp, _vp, _vp]

SIGNATURES = {
    'd_s0s0_1d_sym8_md': _CONV1D, 'd_s0s0_1d_sym8_imd': _CONV1D, 'd_s0s0_1d_sym8_d1': _CONV1D,
    'd_s0s0_1d_sym8_d2_dotin': _CONV1D + [_vp],
    'd_s0s1_1d_sym8': _WAV1D, 'd_s1s0_1d_sym8': _WAV1D,
    'd_s0s1_1d_symicomb8': _WAV1D, 'd_s1s0_1d_symicomb8': _WAV1D,
    'd_sfrf_ld_narr': _MDT, 'd_rfsf_ld_narr': _MDT,
    'd_kin': _KIN, 'd_kin_ekin': _KIN + [_vp], 'd_kin_narr': _KINN, 'd_dwt_sym8': _WMD, 'd_idwt_sym8': _WMD,
    'd_dwt_sym8_narr': _WMDN, 'd_idwt_sym8_narr': _WMDN,
}
COST_SIGNATURES = {
    'd_s0s0_1d_sym8_md_cost': [_int, _int, _I, _int, _int, _L],
    'd_s0s0_1d_sym8_d2_cost': [_int, _int, _I, _int, _int, _L],
    'd_s0s1_1d_sym8_cost': [_int, _int, _I, _int, _int, _L],
    'd_sfrf_cost': [_int, _I, _I, _int, _L],
    'd_kin_cost': [_int, _I, _I, _L],
    'd_dwt_sym8_cost': [_int, _I, _I, _L],
}

_lib = None


class LibconvError(RuntimeError):
    def __init__(self, status, name, detail):
        super().__init__(f"{name} returned {status}: {detail}")
        self.status = status


def lib():
    """The loaded CUDA library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run __graft_entry__.build() first")
        L = ctypes.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            for suffix, extra in (('', []), ('_dev', [_vp])):
                fn = getattr(L, name + suffix)
                fn.argtypes = args + extra
                fn.restype = _int
        for name, args in COST_SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = _int
        for name in ('libconv_gb300_version', 'libconv_gb300_strerror', 'libconv_gb300_last_error'):
            getattr(L, name).restype = ctypes.c_char_p
        L.libconv_gb300_strerror.argtypes = [_int]
        L.libconv_gb300_set_mode.argtypes = [_int]
        L.libconv_gb300_set_mode.restype = _int
        L.libconv_gb300_get_mode.restype = _int
        L.libconv_gb300_check.argtypes = [_vp]
        L.libconv_gb300_check.restype = _int
        _lib = L
    return _lib


def declared_symbols():
    """Every function name declared in include/libconv_gb300.h and
    include/libconv_fortran.h."""
    text = open(HEADER).read() + open(FORTRAN_HEADER).read()
    text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
    return sorted(set(re.findall(r'\b(?:int|const char \*|void)\s*\**\s*(\w+)\s*\(', text)))


def last_error():
    return lib().libconv_gb300_last_error().decode()


def get_mode():
    return lib().libconv_gb300_get_mode()


class mode:
    """Context manager: run the enclosed calls (this thread) in a compute mode."""

    def __init__(self, m):
        self.m = m

    def __enter__(self):
        self.old = get_mode()
        set_mode(self.m)
        return self

    def __exit__(self, *exc):
        set_mode(self.old)


def check(stream=None):
    """Synchronise and raise if a device-side wait of a *_dev call timed out."""
    s = stream
    if s is not None and not isinstance(s, int):
        s = s.cuda_stream if hasattr(s, 'cuda_stream') else int(s)
    st = lib().libconv_gb300_check(ctypes.c_void_p(s) if s else None)
    if st:
        raise LibconvError(st, 'libconv_gb300_check', last_error())


def set_mode(mode):
    st = lib().libconv_gb300_set_mode(int(mode))
    if st:
        raise LibconvError(st, 'libconv_gb300_set_mode', last_error())


def _ints(v):
    if v is None:
        return None
    v = [int(t) for t in (v if hasattr(v, '__len__') else [v])]
    return (ctypes.c_int * len(v))(*v)


def _host_ptr(a, writable):
    if a is None:
        return None
    if not isinstance(a, np.ndarray) or a.dtype != np.float64:
        raise TypeError('host arrays must be numpy float64')
    if not (a.flags.c_contiguous or a.flags.f_contiguous):
        raise TypeError('host arrays must be contiguous')
    if writable and not a.flags.writeable:
        raise TypeError('output array is read-only')
    return ctypes.c_void_p(a.ctypes.data)


def _dev_ptr(t):
    if t is None:
        return None
    if isinstance(t, int):
        return ctypes.c_void_p(t)
    if hasattr(t, 'data_ptr'):
        if not t.is_cuda or str(t.dtype) != 'torch.float64' or not t.is_contiguous():
            raise TypeError('device arrays must be contiguous float64 CUDA tensors')
        return ctypes.c_void_p(t.data_ptr())
    raise TypeError(f'unsupported device array {type(t)}')


class Kernel:
    """One exported procedure, run the way BOAST runs a generated kernel."""

    def __init__(self, name):
        if name not in SIGNATURES:
            raise KeyError(name)
        self.name = name
        self.argtypes = SIGNATURES[name]
        L = lib()
        self._host = getattr(L, name)
        self._dev = getattr(L, name + '_dev')

    def _convert(self, args, ptr):
        if len(args) != len(self.argtypes):
            raise TypeError(f"{self.name} takes {len(self.argtypes)} arguments, got {len(args)}")
        out, dot = [], None
        for i, (a, t) in enumerate(zip(args, self.argtypes)):
            if t is _I:
                out.append(_ints(a))
            elif t is _D:
                vals = [float(v) for v in a]
                out.append(ctypes.cast((ctypes.c_double * len(vals))(*vals), _D))
            elif t is _vp:
                if self.name.endswith('dotin') and i == len(self.argtypes) - 1:
                    dot = a
                    out.append(None)
                else:
                    out.append(ptr(a))
            else:
                out.append(a)
        return out, dot

    def run(self, *args):
        """Host-pointer call; returns {'duration', 'reference_return'}."""
        conv, _ = self._convert(args, lambda a: _host_ptr(a, True))
        dot = ctypes.c_double(0.0)
        if self.name.endswith('dotin'):
            conv[-1] = ctypes.cast(ctypes.pointer(dot), ctypes.c_void_p)
        t0 = time.perf_counter()
        st = self._host(*conv)
        dt = time.perf_counter() - t0
        if st:
            raise LibconvError(st, self.name, last_error())
        ret = {'dot_in': dot.value} if self.name.endswith('dotin') else {}
        return {'duration': dt, 'reference_return': ret}

    def run_dev(self, *args, stream=None):
        """Device-pointer call (enqueue only); dot_in is a device pointer."""
        conv, dot = self._convert(args, _dev_ptr)
        if self.name.endswith('dotin'):
            conv[-1] = _dev_ptr(dot)
        s = stream
        if s is not None and not isinstance(s, int):
            s = s.cuda_stream if hasattr(s, 'cuda_stream') else int(s)
        st = self._dev(*conv, ctypes.c_void_p(s) if s else None)
        if st:
            raise LibconvError(st, self.name + '_dev', last_error())


def cost(name, *args):
    """Reference flop model of an operator (``<name>_cost`` export)."""
    fn = getattr(lib(), name)
    out = ctypes.c_longlong(0)
    conv = [(_ints(a) if t is _I else a) for a, t in zip(args, fn.argtypes[:-1])]
    st = fn(*conv, ctypes.byref(out))
    if st:
        raise LibconvError(st, name, last_error())
    return out.value


# ---- local Hamiltonian of one orbital ---------------------------------------------
def _ham_lib():
    L = lib()
    if not getattr(L, '_ham_bound', False):
        L.libconv_hamiltonian_sizes.argtypes = [_I, _I, _L, _L, _L]
        L.libconv_hamiltonian.argtypes = [_I, _I, _D, _vp, _vp, _vp, _vp, _D, _D]
        L.libconv_hamiltonian_dev.argtypes = [_I, _I, _D, _vp, _vp, _vp, _vp, _vp, _vp, _vp]
        L.libconv_hamiltonian_narr_sizes.argtypes = [_I, _I, _int, _L, _L, _L]
        L.libconv_hamiltonian_narr.argtypes = [_I, _I, _D, _int, _vp, _vp, _vp, _vp, _vp]
        L.libconv_hamiltonian_narr_dev.argtypes = [_I, _I, _D, _int, _vp, _vp, _vp, _vp, _vp, _vp,
                                                   _vp]
        for f in (L.libconv_hamiltonian_sizes, L.libconv_hamiltonian, L.libconv_hamiltonian_dev,
                  L.libconv_hamiltonian_narr_sizes, L.libconv_hamiltonian_narr,
                  L.libconv_hamiltonian_narr_dev):
            f.restype = _int
        L._ham_bound = True
    return L


def _dbls(v):
    v = [float(t) for t in v]
    return ctypes.cast((ctypes.c_double * len(v))(*v), _D)


def hamiltonian_sizes(n, bc, norb=1):
    """(nsig, nreal, nwork): elements of psig/hpsig and of the real-space grid
    (pot, rho) per orbital, and of the device workspace of the local
    Hamiltonian over norb orbitals."""
    L = _ham_lib()
    out = [ctypes.c_longlong(0) for _ in range(3)]
    st = L.libconv_hamiltonian_narr_sizes(_ints(n), _ints(bc), int(norb),
                                          *[ctypes.byref(o) for o in out])
    if st:
        raise LibconvError(st, 'libconv_hamiltonian_narr_sizes', last_error())
    return tuple(o.value for o in out)


def hamiltonian_narr(n, bc, a_kin, norb, psig, pot, rho=None, hpsig=None, energies=None):
    """libconv_hamiltonian_narr on host arrays: norb orbitals back to back in
    psig, one potential.  Returns (hpsig, energies[norb, 4]) with rows
    [ekin_x, ekin_y, ekin_z, epot]; rho, when given, is updated in place.
    hpsig / energies may be given (e.g. page-locked arrays, which let the
    library overlap the copies of chunks of orbitals with their sweeps)."""
    nsig, nreal, _ = hamiltonian_sizes(n, bc, norb)
    if psig.size != norb * nsig or pot.size != nreal or (rho is not None and rho.size != nreal):
        raise ValueError(f'psig needs {norb * nsig} and pot/rho {nreal} elements')
    if hpsig is None:
        hpsig = np.zeros(norb * nsig)
    elif hpsig.size != norb * nsig:
        raise ValueError(f'hpsig needs {norb * nsig} elements')
    en = np.zeros((norb, 4)) if energies is None else energies
    if en.size != 4 * norb:
        raise ValueError(f'energies needs {4 * norb} elements')
    st = _ham_lib().libconv_hamiltonian_narr(
        _ints(n), _ints(bc), _dbls(a_kin), int(norb), _host_ptr(psig, False),
        _host_ptr(pot, False), _host_ptr(rho, True), _host_ptr(hpsig, True), _host_ptr(en, True))
    if st:
        raise LibconvError(st, 'libconv_hamiltonian_narr', last_error())
    return hpsig, en


def hamiltonian(n, bc, a_kin, psig, pot, rho=None):
    """Local Hamiltonian of one orbital on host arrays (libconv_hamiltonian,
    the pipeline of BigDFT/libconv.f90:248-294).  Returns (hpsig, ekin[3],
    epot); rho, when given, is updated in place with psir**2."""
    nsig, nreal, _ = hamiltonian_sizes(n, bc)
    if psig.size != nsig or pot.size != nreal or (rho is not None and rho.size != nreal):
        raise ValueError(f'psig needs {nsig} and pot/rho {nreal} elements')
    hpsig = np.zeros(nsig)
    ek = (ctypes.c_double * 3)()
    ep = ctypes.c_double(0.0)
    st = _ham_lib().libconv_hamiltonian(
        _ints(n), _ints(bc), _dbls(a_kin), _host_ptr(psig, False), _host_ptr(pot, False),
        _host_ptr(rho, True), _host_ptr(hpsig, True), ctypes.cast(ek, _D), ctypes.pointer(ep))
    if st:
        raise LibconvError(st, 'libconv_hamiltonian', last_error())
    return hpsig, np.array(ek[:]), ep.value


class Hamiltonian:
    """Device form (libconv_hamiltonian_narr_dev) over norb orbitals with its
    workspace: call with float64 CUDA tensors (psig, hpsig: norb * nsig);
    returns the device tensor of shape (norb, 4), rows [ekin_x, ekin_y,
    ekin_z, epot], enqueued on `stream` (no synchronisation)."""

    def __init__(self, n, bc, a_kin, norb=1, device='cuda'):
        import torch
        self.n, self.bc, self.a_kin = list(n), list(bc), [float(v) for v in a_kin]
        self.norb = int(norb)
        self.nsig, self.nreal, nwork = hamiltonian_sizes(n, bc, self.norb)
        self.work = torch.empty(nwork, dtype=torch.float64, device=device)
        self.energies = torch.zeros(self.norb, 4, dtype=torch.float64, device=device)

    # kernel launches of one call: 15 sweeps, in the exact tensor-core mode 13
    # line-exponent passes (one shared by the three kinetic sweeps), the
    # potential kernel and its reduction, and the three kinetic-energy reductions
    LAUNCHES = {'exact': 33, 'other': 20}

    def __call__(self, psig, pot, hpsig, rho=None, stream=None, energies=None):
        """energies: optional device tensor of norb * 4 doubles to receive the
        energies instead of the object's own buffer."""
        en = self.energies if energies is None else energies
        ns = self.norb * self.nsig
        if en.numel() != 4 * self.norb:
            raise ValueError(f'energies needs {4 * self.norb} elements')
        if psig.numel() != ns or hpsig.numel() != ns or pot.numel() != self.nreal:
            raise ValueError(f'psig/hpsig need {ns} and pot {self.nreal} elements')
        if rho is not None and rho.numel() != self.nreal:
            raise ValueError(f'rho needs {self.nreal} elements')
        st = _ham_lib().libconv_hamiltonian_narr_dev(
            _ints(self.n), _ints(self.bc), _dbls(self.a_kin), self.norb, _dev_ptr(psig),
            _dev_ptr(pot), _dev_ptr(rho), _dev_ptr(hpsig), _dev_ptr(en), _dev_ptr(self.work),
            _stream_ptr(stream))
        if st:
            raise LibconvError(st, 'libconv_hamiltonian_narr_dev', last_error())
        return en


# ---- Fortran-facing libconv procedures (include/libconv_fortran.h) ----------------
class Fortran:
    """Calls the Fortran-facing procedures the way gfortran does: every
    argument by reference (ints, doubles, int arrays, float64 arrays), and
    CHARACTER arguments with their hidden length at the end.  Raises on a
    non-zero libconv_status."""

    def __init__(self):
        self.L = lib()

    @staticmethod
    def _ref(v):
        if isinstance(v, np.ndarray):
            return ctypes.c_void_p(v.ctypes.data)
        if isinstance(v, (list, tuple)):
            return ctypes.cast((ctypes.c_int * len(v))(*[int(t) for t in v]), ctypes.c_void_p)
        if isinstance(v, float):
            return ctypes.cast(ctypes.pointer(ctypes.c_double(v)), ctypes.c_void_p)
        if isinstance(v, int):
            return ctypes.cast(ctypes.pointer(ctypes.c_int(v)), ctypes.c_void_p)
        if v is None:
            return None
        raise TypeError(f'unsupported Fortran argument {type(v)}')

    def status(self):
        st = ctypes.c_int(0)
        self.L.libconv_status_(ctypes.byref(st))
        return st.value

    def call(self, name, *args, check=True):
        fn = getattr(self.L, name + '_')
        fn.restype = None
        fn(*[self._ref(a) for a in args])
        st = self.status()
        if check and st:
            raise LibconvError(st, name, last_error())
        return st

    def filter_id(self, name):
        fid = ctypes.c_int(0)
        b = name.encode()
        self.L.get_filter_id_(ctypes.c_char_p(b), ctypes.byref(fid), ctypes.c_size_t(len(b)))
        return fid.value

    def bc_id(self, name):
        bid = ctypes.c_int(0)
        b = name.encode()
        self.L.get_bc_id_(ctypes.c_char_p(b), ctypes.byref(bid), ctypes.c_size_t(len(b)))
        return bid.value

    def filter_name(self, fid, length=16):
        buf = ctypes.create_string_buffer(length)
        self.L.get_filter_name_(ctypes.byref(ctypes.c_int(fid)), buf, ctypes.c_size_t(length))
        return buf.raw.decode().rstrip()

    def bc_name(self, bid, length=4):
        buf = ctypes.create_string_buffer(length)
        self.L.get_bc_name_(ctypes.byref(ctypes.c_int(bid)), buf, ctypes.c_size_t(length))
        return buf.raw.decode().rstrip()

    def sizes(self, name, d, n, fil, bc, work=False):
        out = (ctypes.c_int * (1 if work else d))()
        getattr(self.L, name + '_')(self._ref(d), self._ref(list(n)), self._ref(fil),
                                    self._ref(list(bc)), out)
        st = self.status()
        if st:
            raise LibconvError(st, name, last_error())
        return out[0] if work else list(out)


# ---- Poisson finite-difference operators (BigDFT/Poisson.rb) ----------------------
BC_NPERIODIC = -2


class Poisson:
    """Host-array calls of the Poisson operators (Poisson_broker, div_u_i,
    nabla_u, nabla_u_and_square, nabla_u_square, nabla_u_epsilon,
    update_rhopol); arrays are float64, Fortran order, flat."""

    _SIG = {
        'Poisson_broker': [_int, _int, _I, _int, _vp, _vp, _dbl],
        'div_u_i': [_int, _int, _int, _int, _vp, _vp, _int, _D, _vp],
        'nabla_u': [_int, _int, _int, _int, _vp, _vp, _int, _D],
        'nabla_u_and_square': [_int, _int, _int, _int, _vp, _vp, _vp, _int, _D],
        'nabla_u_square': [_int, _int, _int, _int, _vp, _vp, _int, _D],
        'nabla_u_epsilon': [_int, _int, _int, _int, _vp, _vp, _int, _D, _vp],
        'update_rhopol': [_int, _int, _int, _int, _vp, _int, _D, _dbl, _vp, _vp, _vp],
    }

    def __init__(self):
        L = lib()
        for name, args in self._SIG.items():
            getattr(L, name).argtypes = args
            getattr(L, name).restype = _int
        self.L = L

    def _call(self, name, *args):
        conv = []
        for a, t in zip(args, self._SIG[name]):
            if t is _I:
                conv.append(_ints(a))
            elif t is _D:
                conv.append(_dbls(a))
            elif t is _vp:
                conv.append(_host_ptr(a, True) if a is not None else None)
            else:
                conv.append(a)
        st = getattr(self.L, name)(*conv)
        if st:
            raise LibconvError(st, name, last_error())

    def broker(self, nord, idim, nn, bc, u, a):
        du = np.zeros(int(np.prod(nn)))
        self._call('Poisson_broker', nord, idim, nn, bc, u, du, float(a))
        return du

    def div_u_i(self, geocode, n, u, nord, h, cc=False):
        N = int(np.prod(n))
        du = np.zeros(N)
        c = np.zeros(N) if cc else None
        self._call('div_u_i', geocode, *n, u, du, nord, h, c)
        return (du, c) if cc else du

    def nabla_u(self, geocode, n, u, nord, h):
        du = np.zeros(3 * int(np.prod(n)))
        self._call('nabla_u', geocode, *n, u, du, nord, h)
        return du

    def nabla_u_and_square(self, geocode, n, u, nord, h):
        N = int(np.prod(n))
        du, ddu = np.zeros(3 * N), np.zeros(N)
        self._call('nabla_u_and_square', geocode, *n, u, du, ddu, nord, h)
        return du, ddu

    def nabla_u_square(self, geocode, n, u, nord, h):
        ddu = np.zeros(int(np.prod(n)))
        self._call('nabla_u_square', geocode, *n, u, ddu, nord, h)
        return ddu

    def nabla_u_epsilon(self, geocode, n, u, nord, h, eps):
        du = np.zeros(3 * int(np.prod(n)))
        self._call('nabla_u_epsilon', geocode, *n, u, du, nord, h, eps)
        return du

    def update_rhopol(self, geocode, n, u, nord, h, eta, dlogeps, rhopol):
        """rhopol is updated in place; returns rhores2."""
        r2 = np.zeros(1)
        self._call('update_rhopol', geocode, *n, u, nord, h, float(eta), dlogeps, rhopol, r2)
        return float(r2[0])


# ---- batched operators over many uneven grids ------------------------------------
BATCH_OP_MF, BATCH_OP_KIN = 0, 1
ENGINE_FP64_Q64, ENGINE_FP64_Q32, ENGINE_TC = 0, 1, 2


def _stream_ptr(stream):
    s = stream
    if s is not None and not isinstance(s, int):
        s = s.cuda_stream if hasattr(s, 'cuda_stream') else int(s)
    return ctypes.c_void_p(s) if s else None


def _batch_lib():
    L = lib()
    if not getattr(L, '_batch_bound', False):
        P = ctypes.POINTER(ctypes.c_void_p)
        L.libconv_batch_create.argtypes = [P, _int, _I, _I, _I, _D, _dbl]
        L.libconv_batch_sizes.argtypes = [_vp, _L, _L, _L]
        L.libconv_batch_offsets.argtypes = [_vp, _L, _L, _L]
        L.libconv_batch_set_config.argtypes = [_vp, _int, _int, _I]
        L.libconv_batch_get_config.argtypes = [_vp, _int, _I, _I, _I]
        L.libconv_batch_tune.argtypes = [_vp, _vp, _vp, _vp, _vp]
        L.libconv_batch_run.argtypes = [_vp, _vp, _vp, _vp, _vp]
        L.libconv_batch_destroy.argtypes = [_vp]
        for n in ('create', 'sizes', 'offsets', 'set_config', 'get_config', 'tune', 'run', 'destroy'):
            getattr(L, 'libconv_batch_' + n).restype = _int
        L._batch_bound = True
    return L


class Batch:
    """MagicFilter3D and/or Kinetic3D over many grids of different sizes in
    one persistent launch per sweep stage, replayed as a CUDA graph
    (``libconv_batch_*``).  Buffers are packed float64 CUDA tensors."""

    def __init__(self, dims, mf_bc=None, kin_bc=None, kin_a=None, kin_ax=0.0):
        L = _batch_lib()
        dims = [int(v) for d in dims for v in d]
        self.ngrids = len(dims) // 3
        self._h = ctypes.c_void_p()
        a = None
        if kin_a is not None:
            a = ctypes.cast((ctypes.c_double * 3)(*[float(v) for v in kin_a]), _D)
        st = L.libconv_batch_create(ctypes.byref(self._h), self.ngrids, _ints(dims), _ints(mf_bc),
                                    _ints(kin_bc), a, float(kin_ax))
        if st:
            raise LibconvError(st, 'libconv_batch_create', last_error())

    def _check(self, st, name):
        if st:
            raise LibconvError(st, name, last_error())

    def sizes(self):
        v = [ctypes.c_longlong() for _ in range(3)]
        self._check(_batch_lib().libconv_batch_sizes(self._h, *[ctypes.byref(t) for t in v]),
                    'libconv_batch_sizes')
        return tuple(t.value for t in v)

    def offsets(self):
        arrs = [(ctypes.c_longlong * (self.ngrids + 1))() for _ in range(3)]
        self._check(_batch_lib().libconv_batch_offsets(self._h, *[ctypes.cast(a, _L) for a in arrs]),
                    'libconv_batch_offsets')
        return tuple(list(a) for a in arrs)

    def set_config(self, op, engine, order):
        self._check(_batch_lib().libconv_batch_set_config(self._h, op, engine, _ints(order)),
                    'libconv_batch_set_config')

    def get_config(self, op):
        e, t = ctypes.c_int(), ctypes.c_int()
        o = (ctypes.c_int * 3)()
        self._check(_batch_lib().libconv_batch_get_config(self._h, op, ctypes.byref(e),
                                                          ctypes.cast(o, _I), ctypes.byref(t)),
                    'libconv_batch_get_config')
        return e.value, list(o), bool(t.value)

    def tune(self, x, y_mf=None, y_kin=None, stream=None):
        self._check(_batch_lib().libconv_batch_tune(self._h, _dev_ptr(x), _dev_ptr(y_mf),
                                                    _dev_ptr(y_kin), _stream_ptr(stream)),
                    'libconv_batch_tune')

    def run(self, x, y_mf=None, y_kin=None, stream=None):
        self._check(_batch_lib().libconv_batch_run(self._h, _dev_ptr(x), _dev_ptr(y_mf),
                                                   _dev_ptr(y_kin), _stream_ptr(stream)),
                    'libconv_batch_run')

    def close(self):
        if self._h:
            _batch_lib().libconv_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
