#!/usr/bin/env python3
"""Benchmark of the separable Daubechies-16 convolution operators.

Default workload (mfkin128): FP64 3D MagicFilter + Kinetic on 128^3 periodic
grids.  One step = the hot path over one batch of grids held in HBM: for every
grid x of the batch, psi_r = MagicFilter3D(x) (three rotated sweeps) and
T x = Kinetic3D(x) (h = 0.45 bohr per axis, three accumulating sweeps), both
from the same x.  Metric: grid points per second (points of x processed by
both operators), whole job.  Inputs are seeded Gaussian-filtered noise
(sigma = 2 points, unit RMS); the batch (default 32 grids, 537 MB per array)
is larger than the 126 MB L2, so every step streams from HBM.

Workload wavelet96: 3D wavelet synthesis of 8 subbands of 48^3 (coarse
uniform [-1, 1], details uniform [-1, 1] x 1e-3) into 96^3, then analysis
back; metric: 96^3 grid points per second through both transforms.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload mfkin128|wavelet96|orbitals512|precond256|hamiltonian48|poisson256]
                  [--mode tc_exact|fp64|tc_bf16x3|tc_tf32x3]

Workload orbitals512: 512 orbitals with axes uniform in {24..72} (seed 7),
Gaussian envelope times unit-RMS noise; MagicFilter3D free grow and
Kinetic3D free per orbital, batched (one persistent launch per sweep stage,
CUDA graph, autotuned); the line also times the same work as per-orbital
calls of the single-grid entry points.

Workload precond256: 256 shifted kinetic systems (T - eps) x = b on 48^3
periodic grids (h = 0.4, eps uniform in [-1, -0.1], Gaussian-filtered
noise right-hand sides with ||b|| = 1); metric: solves/s to ||r|| <= 1e-8 of
flexible CG with the learned preconditioner, plain CG timed beside it.

Workload hamiltonian48: the local Hamiltonian of orbitals on a 48^3 coarse
grid with free boundaries (libconv_hamiltonian_dev: idwt grow, MagicFilter
grow, potential and density, inverse MagicFilter shrink, kinetic with the
energies, dwt shrink), 32 orbitals per step; metric: orbitals/s.

Workload poisson256: the Poisson test's div_u_i with cc on 256^3 (nord 16,
geocode 3, h = 0.1, u uniform [0, 1)); metric: grid points per second.

Modes: tc_exact (default) runs the tensor-core exact-digit sweeps (FP64
accuracy); fp64 the FP64 FMA sweeps; tc_bf16x3 / tc_tf32x3 the split-precision
tensor-core sweeps, whose line carries each operator's max relative error
against the tc_exact output of the same step.

--impl reference times the CPU implementation of the same operators (the
C oracle: a restatement of the reference's Fortran/generated loops) on all
host cores, one grid per thread, and prints the same JSON line.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

HGRID = 0.45
UNIT = 'grid pts/s'


def peaks():
    p = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    d = json.load(open(p)) if os.path.exists(p) else {}
    return {'hbm': d.get('hbm_gbs', 6800.0), 'bf16': d.get('bf16_tflops', 1900.0),
            'source': 'measured' if d else 'fallback'}


class Ranks:
    """One process per GPU (torchrun): rank, world size and local GPU from the
    environment, a process group when world > 1 (NCCL on GPUs, gloo for the
    CPU tests), and the barrier / max / sum the runs need.  Nothing on the
    data path is collective: the ranks only agree on times and totals."""

    def __init__(self, backend='nccl'):
        import torch
        self.world = int(os.environ.get('WORLD_SIZE', '1'))
        self.rank = int(os.environ.get('RANK', '0'))
        self.local = int(os.environ.get('LOCAL_RANK', '0'))
        if backend == 'nccl':
            torch.cuda.set_device(self.local)
            self.device = torch.device('cuda', self.local)
        else:
            self.device = torch.device('cpu')
        if self.world > 1:
            import torch.distributed as dist
            if backend == 'nccl':
                dist.init_process_group('nccl', device_id=self.device)
            else:
                dist.init_process_group(backend)

    def barrier(self):
        if self.world > 1:
            import torch.distributed as dist
            dist.barrier()

    def _reduce(self, v, op):
        import torch
        import torch.distributed as dist
        t = torch.tensor([float(v)], dtype=torch.float64, device=self.device)
        dist.all_reduce(t, op=op)
        return t.item()

    def max(self, v):
        if self.world == 1:
            return float(v)
        import torch.distributed as dist
        return self._reduce(v, dist.ReduceOp.MAX)

    def sum(self, v):
        if self.world == 1:
            return float(v)
        import torch.distributed as dist
        return self._reduce(v, dist.ReduceOp.SUM)

    def close(self):
        if self.world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


def shard_balanced(sizes, rank, world):
    """Indices of the items rank takes: items in decreasing size dealt round
    robin (ties by index), so each rank's total is within one item of the
    others'."""
    order = sorted(range(len(sizes)), key=lambda g: (-sizes[g], g))
    return [g for i, g in enumerate(order) if i % world == rank]


def package():
    import __graft_entry__ as ge
    return ge.package()


# ----------------------------------------------------------------------------- workloads
class MfKin128:
    """MagicFilter3D + Kinetic3D on 128^3 periodic grids."""
    name = 'mfkin128'
    metric = 'grid pts/s, FP64 3D MagicFilter + Kinetic (128^3 periodic)'
    n = [128, 128, 128]
    n_in = 128 ** 3
    n_out = 128 ** 3
    ops = ('magicfilter3d', 'kinetic3d')
    a = [-0.5 / HGRID ** 2] * 3
    launches = 6                                     # 3 sweeps per operator
    # exact tensor-core mode: one shared line-exponent pass over x for the three kinetic
    # sweeps; the first MagicFilter sweep takes its tile windows' exponents itself and hands
    # the next sweep its line exponents, which hands them on to the third
    exact_prepasses = 1
    # the whole step's algorithmic bytes per grid point: as separate sweeps (MagicFilter 3 x 16;
    # kinetic 16 + 24 + 24, its y and z sweeps reading x beside their partial sum) and with x
    # read once and both outputs written once (the floor of any fusion of the two operators)
    step_bytes = {'sweeps': 48.0 + 64.0, 'fused': 24.0}
    desc = ('{B} grids of 128^3 periodic per GPU per step: MagicFilter3D (d_sfrf_ld_narr) + '
            'Kinetic3D (d_kin_narr, h=0.45)')

    def base(self, count):
        package()
        from boast_lig_gb300 import inputs
        return [inputs.gaussian_filtered_noise(1000 + i, tuple(self.n)).ravel(order='F')
                for i in range(count)]

    def fill(self, hx, B, rank, base):
        N = self.n_in
        for b in range(B):
            hx[b * N:(b + 1) * N] = base[(b + rank) % len(base)] * (1.0 + 1e-3 * b)

    def dev_ops(self, pkg, B, bufs):
        n, a = self.n, self.a
        mf, kin = pkg.Kernel('d_sfrf_ld_narr'), pkg.Kernel('d_kin_narr')
        x, o0, o1, w1, w2 = bufs['x'], bufs['o0'], bufs['o1'], bufs['w1'], bufs['w2']
        return [lambda sp: mf.run_dev(3, n, [0, 0, 0], n, n, B, x, o0, w1, w2, stream=sp),
                lambda sp: kin.run_dev(3, n, [0, 0, 0], B, x, o1, w1, w2, a, 0.0, 0.0, stream=sp)]

    def host_step(self, pkg, B, hx, ho0, ho1):
        n, a, hw = self.n, self.a, np.zeros(1)
        pkg.Kernel('d_sfrf_ld_narr').run(3, n, [0, 0, 0], n, n, B, hx, ho0, hw, hw)
        pkg.Kernel('d_kin_narr').run(3, n, [0, 0, 0], B, hx, ho1, hw, hw, a, 0.0, 0.0)

    e2e_note = ('d_sfrf_ld_narr (narr=B) + d_kin_narr (narr=B), host pointers (pinned), '
                'H2D of x and D2H of psi_r and T x inside every call (the library pipelines '
                'chunks of grids: copies overlap the sweeps)')

    def cpu_work(self, O, x, bufs):
        y, tx, w1, w2 = bufs
        n = self.n
        O.call('oracle_d_sfrf_ld_narr', 3, n, [0, 0, 0], n, n, 1, x, y, w1, w2)
        O.call('oracle_d_kin', 3, n, [0, 0, 0], x, tx, w1, w2, np.array(self.a), 0.0, 0.0)

    def timing_step(self, T, O, B, x, o0, o1, threads):
        """One step over B grids in the oracle's OpenMP timing build (seconds)."""
        return T.timing_mfkin_step(B, O.ip(self.n), O.dp(x), O.dp(o0), O.dp(o1),
                                   O.dp(np.array(self.a)), threads)

    # roofline: dominant kernel = the kinetic sweep (29 taps), 3 launches per
    # step over all grids; algorithmic bytes per grid point 64/3 per launch
    # (16 B first sweep, 24 B the two accumulating sweeps)
    dom = 1
    dom_bytes_per_pt = 64.0 / 3.0
    dom_flops_per_pt = 58 + 1 + 2.0 / 3.0
    dom_kernel = {'tc_exact': 'sweep_tc_kernel<KCONV,29,EXACT> (kinetic sweep, all grids per launch)',
                  'tc_bf16x3': 'sweep_tc_kernel<KCONV,29,BF16X3> (kinetic sweep)',
                  'tc_tf32x3': 'sweep_tc_kernel<KCONV,29,TF32X3> (kinetic sweep)',
                  'fp64': 'sweep_fp64_kernel<KCONV,29> (kinetic sweep, all grids per launch)'}
    traffic_file = {'tc_exact': 'kinetic_sweep_tc_traffic.json', 'fp64': 'kinetic_sweep_fp64_traffic.json'}
    kb = 48                                          # K per 16-output MMA block (29 taps)
    pairs_exact = 36


class Wavelet96:
    """idwt 8 x 48^3 -> 96^3, then dwt back (periodic)."""
    name = 'wavelet96'
    metric = 'grid pts/s, 3D wavelet synthesis + analysis (8 x 48^3 <-> 96^3 periodic)'
    n = [48, 48, 48]
    n_in = 96 ** 3
    n_out = 96 ** 3
    ops = ('idwt3d', 'dwt3d')
    launches = 6
    exact_prepasses = 6                              # one line-exponent pass per sweep
    desc = ('{B} grids per GPU per step: d_idwt_sym8_narr (8 subbands of 48^3 -> 96^3) then '
            'd_dwt_sym8_narr (96^3 -> 8 x 48^3)')

    def base(self, count):
        package()
        from boast_lig_gb300 import inputs
        out = []
        for i in range(count):
            c = inputs.uniform(2000 + i, self.n_in).reshape(96, 96, 96)
            c[48:, :, :] *= 1e-3
            c[:, 48:, :] *= 1e-3
            c[:, :, 48:] *= 1e-3
            out.append(np.ascontiguousarray(c).ravel())
        return out

    fill = MfKin128.fill

    def dev_ops(self, pkg, B, bufs):
        n = self.n
        iw, dw = pkg.Kernel('d_idwt_sym8_narr'), pkg.Kernel('d_dwt_sym8_narr')
        x, o0, o1, w1, w2 = bufs['x'], bufs['o0'], bufs['o1'], bufs['w1'], bufs['w2']
        return [lambda sp: iw.run_dev(3, n, [0, 0, 0], B, x, o0, w1, w2, stream=sp),
                lambda sp: dw.run_dev(3, n, [0, 0, 0], B, o0, o1, w1, w2, stream=sp)]

    def host_step(self, pkg, B, hx, ho0, ho1):
        n, hw = self.n, np.zeros(1)
        pkg.Kernel('d_idwt_sym8_narr').run(3, n, [0, 0, 0], B, hx, ho0, hw, hw)
        pkg.Kernel('d_dwt_sym8_narr').run(3, n, [0, 0, 0], B, ho0, ho1, hw, hw)

    e2e_note = ('d_idwt_sym8_narr then d_dwt_sym8_narr (narr=B), host pointers (pinned): '
                'H2D of the subbands and D2H of the 96^3 grids in the first call, H2D of '
                'the 96^3 grids and D2H of the subbands in the second')

    def cpu_work(self, O, x, bufs):
        y, back, w1, w2 = bufs
        n = self.n
        O.call('oracle_d_idwt_sym8', 3, n, [0, 0, 0], x, y, w1, w2)
        O.call('oracle_d_dwt_sym8', 3, n, [0, 0, 0], y, back, w1, w2)

    def timing_step(self, T, O, B, x, o0, o1, threads):
        return T.timing_wavelet_step(B, O.ip(self.n), O.dp(x), O.dp(o0), O.dp(o1), threads)

    # roofline: every sweep moves 16 B per 96^3 point; dominant = the synthesis
    dom = 0
    dom_bytes_per_pt = 16.0
    dom_flops_per_pt = 32.0
    dom_kernel = {'tc_exact': 'sweep_tc_kernel<KREC,8,EXACT> (synthesis sweep)',
                  'tc_bf16x3': 'sweep_tc_kernel<KREC,8,BF16X3> (synthesis sweep)',
                  'tc_tf32x3': 'sweep_tc_kernel<KREC,8,TF32X3> (synthesis sweep)',
                  'fp64': 'sweep_fp64_kernel<KREC,8> (synthesis sweep)'}
    traffic_file = {}
    kb = 32
    pairs_exact = 28


class Orbitals512:
    """512 orbitals of uneven sizes: MagicFilter3D free grow + Kinetic3D free."""
    name = 'orbitals512'
    metric = ('grid pts/s, 512 uneven orbitals (axes U{24..72}): MagicFilter3D free grow + '
              'Kinetic3D free, batched')
    count = 512
    a = [-0.5 / HGRID ** 2] * 3

    def dims(self):
        package()
        from boast_lig_gb300 import inputs
        return [[int(v) for v in d] for d in inputs.orbital_dims(7, self.count)]

    def base(self, count=None):
        package()
        from boast_lig_gb300 import inputs
        return [inputs.orbital(1000 + g, d, h=HGRID).ravel(order='F')
                for g, d in enumerate(self.dims())]

    def cpu_work(self, O, x, bufs, d):
        ny = [v + 15 for v in d]
        y, tx, w1, w2 = bufs
        O.call('oracle_d_sfrf_ld_narr', 3, d, [1, 1, 1], d, ny, 1, x, y, w1, w2)
        O.call('oracle_d_kin', 3, d, [2, 2, 2], x, tx, w1, w2, np.array(self.a), 0.0, 0.0)


class Precond256:
    """256 shifted kinetic solves (T - eps) x = b on 48^3 periodic grids."""
    name = 'precond256'
    n = 48
    h = 0.4
    nsys = 256
    tol = 1e-8
    weights = 'precond_n48_h0.40.npz'

    @property
    def metric(self):
        return (f'solves/s to ||r|| <= 1e-8, {self.nsys} x 48^3 periodic (T - eps) x = b, flexible '
                'CG with the learned preconditioner')

    def systems(self):
        package()
        from boast_lig_gb300 import train_precond
        return train_precond.test_systems(self.n, self.nsys, seed=11)


class Hamiltonian48:
    """Local Hamiltonian of orbitals on a 48^3 coarse grid, free boundaries."""
    name = 'hamiltonian48'
    metric = ('orbitals/s, local Hamiltonian (idwt grow, MagicFilter grow, potential, inverse '
              'MagicFilter shrink, kinetic + energies, dwt shrink), 48^3 coarse points, free BC')
    n = [48, 48, 48]
    bc = [2, 2, 2]
    h = 0.4
    a = [-0.5 / 0.4 ** 2] * 3

    def orbital(self, seed):
        """Wavelet coefficients of one orbital: unit-RMS Gaussian-filtered noise
        in the scaling subband, details 1e-3 of it (as the wavelet96 input)."""
        package()
        from boast_lig_gb300 import inputs
        c = inputs.gaussian_filtered_noise(seed, (96, 96, 96))
        c[48:, :, :] *= 1e-3
        c[:, 48:, :] *= 1e-3
        c[:, :, 48:] *= 1e-3
        return np.ascontiguousarray(c).ravel(order='F')

    def potential(self, nreal):
        """A smooth attractive well plus a seeded perturbation, on the real-space grid."""
        g = int(round(nreal ** (1 / 3)))
        r = (np.arange(g) - (g - 1) / 2.0) / g
        X, Y, Z = np.meshgrid(r, r, r, indexing='ij')
        v = -1.0 / np.sqrt(X ** 2 + Y ** 2 + Z ** 2 + 0.05)
        rng = np.random.default_rng(17)
        v = v + 0.01 * rng.standard_normal(v.shape)
        return np.ascontiguousarray(v).ravel(order='F')

    def cpu_work(self, O, x, pot, bufs):
        hpsig, ek, ep = bufs
        O.call('oracle_hamiltonian', self.n, self.bc, np.array(self.a), x, pot, None, hpsig, ek, ep)


class Poisson256:
    """div_u_i with cc on the Poisson test's 256^3 grid (Poisson_test.rb:5-19)."""
    name = 'poisson256'
    metric = ('grid pts/s, Poisson div_u_i with cc (16th-order finite differences, 256^3, '
              'geocode 3: y non-periodic, h = 0.1)')
    n = [256, 256, 256]
    geocode = 3
    nord = 16
    h = [0.1, 0.1, 0.1]
    # per point: six derivative sweeps (read 8, write 8 B) and the cc kernel
    # (read u 24, du 8, five derivatives 40; write cc 8, du 8)
    bytes_per_pt = 6 * 16 + 88
    sweep_bytes_per_pt = 16


def cpu_cg(O, n, h, eps, b, tol, maxit=3000):
    """Plain (Jacobi) CG on the host with the oracle's kinetic operator; returns
    the iteration count."""
    N = b.size
    a = np.array([-0.5 / h ** 2] * 3)
    w1, w2, Ap = np.zeros(N), np.zeros(N), np.zeros(N)
    x, r = np.zeros(N), b.copy()
    p = r.copy()
    rr = float(r @ r)
    bn = np.sqrt(rr)
    for it in range(1, maxit + 1):
        O.call('oracle_d_kin', 3, [n] * 3, [0, 0, 0], p, Ap, w1, w2, a, -eps, 0.0)
        al = rr / float(p @ Ap)
        x += al * p
        r -= al * Ap
        rr_new = float(r @ r)
        if np.sqrt(rr_new) <= tol * bn:
            return it
        p = r + (rr_new / rr) * p
        rr = rr_new
    return maxit + 1


def cpu_solves(W, seconds):
    """Plain CG solves of the benchmark systems on all host threads for about
    `seconds`; returns (solves, time, threads)."""
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import oracle as O
    O.lib()
    b, eps = W.systems()
    th = cpu_threads()
    done = [0] * th
    t0 = time.perf_counter()

    def work(t):
        s = t
        while time.perf_counter() - t0 < seconds:
            cpu_cg(O, W.n, W.h, float(eps[s % W.nsys]), b[s % W.nsys], W.tol)
            done[t] += 1
            s += th

    ts = [threading.Thread(target=work, args=(t,)) for t in range(th)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    return sum(done), time.perf_counter() - t0, th


WORKLOADS = {'mfkin128': MfKin128(), 'wavelet96': Wavelet96(), 'orbitals512': Orbitals512(),
             'precond256': Precond256(), 'hamiltonian48': Hamiltonian48(),
             'poisson256': Poisson256()}


def gpu_uuid(dev):
    """'GPU-<uuid>' of CUDA device dev (the name NVML and nvidia-smi -i
    accept whatever devices CUDA_VISIBLE_DEVICES hides or renumbers), or None."""
    try:
        import torch
        u = getattr(torch.cuda.get_device_properties(dev), 'uuid', None)
        return None if u is None else 'GPU-' + str(u)
    except Exception:
        return None


class NvmlClocks:
    """Read-only NVML sampler (ctypes on the driver's libnvidia-ml): the SM
    clock and the clock-event reasons of one GPU every `period` seconds in a
    background thread, so that a timed region shorter than nvidia-smi's
    sampling interval still gets a clock record.  Settings are only read."""
    SM = 1                                             # NVML_CLOCK_SM
    BITS = {0x8: 'hw_slowdown', 0x40: 'hw_thermal_slowdown', 0x20: 'sw_thermal_slowdown',
            0x4: 'sw_power_cap'}

    def __init__(self, dev, period=0.005):
        import ctypes
        import threading
        self.ok = False
        self.samples = []
        self.period = period
        self.stop_ev = threading.Event()
        self.th = None
        try:
            L = ctypes.CDLL('libnvidia-ml.so.1')
            if L.nvmlInit_v2() != 0:
                return
            h = ctypes.c_void_p()
            uid = gpu_uuid(dev)
            if uid is not None:
                if L.nvmlDeviceGetHandleByUUID(ctypes.c_char_p(uid.encode()), ctypes.byref(h)) != 0:
                    return
            elif L.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(dev), ctypes.byref(h)) != 0:
                return
            reasons = getattr(L, 'nvmlDeviceGetCurrentClocksEventReasons', None) or \
                L.nvmlDeviceGetCurrentClocksThrottleReasons
            mx = ctypes.c_uint(0)
            L.nvmlDeviceGetMaxClockInfo(h, self.SM, ctypes.byref(mx))
            self.L, self.h, self.reasons, self.max_mhz = L, h, reasons, mx.value
            self.ok = True
        except (OSError, AttributeError):
            self.ok = False

    def _run(self):
        import ctypes
        mhz, bits = ctypes.c_uint(0), ctypes.c_ulonglong(0)
        while not self.stop_ev.is_set():
            if (self.L.nvmlDeviceGetClockInfo(self.h, self.SM, ctypes.byref(mhz)) == 0 and
                    self.reasons(self.h, ctypes.byref(bits)) == 0):
                self.samples.append((mhz.value, bits.value))
            self.stop_ev.wait(self.period)

    def start(self):
        if self.ok:
            import threading
            self.th = threading.Thread(target=self._run, daemon=True)
            self.th.start()

    def stop(self):
        if not self.th:
            return None
        self.stop_ev.set()
        self.th.join()
        if not self.samples:
            return None
        reasons = sorted({n for _, b in self.samples for bit, n in self.BITS.items() if b & bit})
        return {'sm_mhz': float(np.median([m for m, _ in self.samples])),
                'sm_max_mhz': float(self.max_mhz) if self.max_mhz else None,
                'reasons': reasons, 'samples': len(self.samples)}


class Clocks:
    """Clock record of the timed region: NVML sampled every 5 ms when the
    driver's library loads, with nvidia-smi (200 ms) running beside it."""
    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
         'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
         'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, dev):
        self.dev = dev
        self.p = None
        self.out = os.path.join('/tmp', f'lcg_clocks_{os.getpid()}.csv')
        self.nvml = NvmlClocks(dev)

    def start(self):
        self.nvml.start()
        try:
            self.p = subprocess.Popen(['nvidia-smi', '-i', gpu_uuid(self.dev) or str(self.dev),
                                       f'--query-gpu={self.Q}',
                                       '--format=csv,noheader,nounits', '-lms', '200'],
                                      stdout=open(self.out, 'w'), stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        fast = self.nvml.stop()
        smi = None
        if self.p is not None:
            time.sleep(0.25)
            self.p.terminate()
            self.p.wait()
            rows = []
            for line in open(self.out):
                f = [t.strip() for t in line.split(',')]
                if len(f) >= 9:
                    rows.append(f)
            if rows:
                sm = [float(r[1]) for r in rows if r[1].replace('.', '').isdigit()]
                mx = [float(r[2]) for r in rows if r[2].replace('.', '').isdigit()]
                names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
                reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i] == 'Active'})
                smi = {'sm_mhz': float(np.median(sm)) if sm else None,
                       'sm_max_mhz': max(mx) if mx else None, 'reasons': reasons, 'samples': len(rows)}
        if fast:
            if smi:   # a reason either sampler saw counts
                fast['reasons'] = sorted(set(fast['reasons']) | set(smi['reasons']))
                fast['nvidia_smi'] = smi
            fast['source'] = 'NVML every 5 ms during the timed region (nvidia-smi every 200 ms beside it)'
            return fast
        return smi


# ----------------------------------------------------------------------------- CPU
def cpu_run(W, grids, threads, steps, warmup):
    """The workload's oracle operators, one grid per host thread (ctypes
    releases the GIL).  Returns the per-step times and the points per step."""
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import oracle as O
    O.lib()
    N = max(W.n_in, W.n_out)
    bufs = [[np.zeros(N) for _ in range(4)] for _ in range(threads)]

    def work(t):
        W.cpu_work(O, grids[t % len(grids)], bufs[t])

    times = []
    for s in range(warmup + steps):
        th = [threading.Thread(target=work, args=(t,)) for t in range(threads)]
        t0 = time.perf_counter()
        for t in th:
            t.start()
        for t in th:
            t.join()
        dt = time.perf_counter() - t0
        if s >= warmup:
            times.append(dt)
    return times, threads * W.n_in


def cpu_run_orbitals(W, xs, dims, threads, seconds):
    """Oracle MF free grow + kinetic free over orbitals taken round robin by
    host threads until about `seconds` have passed; returns (points, time)."""
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import oracle as O
    O.lib()
    big = max(int(np.prod([v + 15 for v in d])) for d in dims)
    bufs = [[np.zeros(big) for _ in range(4)] for _ in range(threads)]
    done = [0] * threads
    t0 = time.perf_counter()

    def work(t):
        g = t
        while time.perf_counter() - t0 < seconds and g < len(xs):
            W.cpu_work(O, xs[g], bufs[t], dims[g])
            done[t] += xs[g].size
            g += threads

    th = [threading.Thread(target=work, args=(t,)) for t in range(threads)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    return sum(done), time.perf_counter() - t0


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def fp64_peak(pkg, local):
    """Measured FP64 FMA throughput of this GPU (libconv_gb300_fp64_peak: 8
    independent FMA chains per thread, CUDA events), best of 3 launches of
    about 0.4 s, with the SM clock sampled meanwhile."""
    import ctypes
    L = pkg.lib()
    f = L.libconv_gb300_fp64_peak
    f.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]
    f.restype = ctypes.c_int
    v = ctypes.c_double(0.0)
    best = 0.0
    ck = Clocks(local)
    ck.start()
    for _ in range(3):
        if f(100000, ctypes.byref(v), None) != 0:
            return None
        best = max(best, v.value)
    c = ck.stop()
    return {'tflops': best, 'sm_mhz': c['sm_mhz'] if c else None,
            'how': 'libconv_gb300_fp64_peak: 8 independent FMA chains x 100000 steps per thread, '
                   '8 x SMs blocks of 256 threads, CUDA events, best of 3'}


def cpu_model():
    """CPU model name of this host (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(['lscpu'], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith('Model name:'):
                return line.split(':', 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open('/proc/cpuinfo'):
            if line.lower().startswith('model name'):
                return line.split(':', 1)[1].strip()
    except OSError:
        pass
    return 'unknown'


def cpu_timed(W, B, hx, repeats=5, seconds=None):
    """The oracle restatement's -O3 OpenMP timing build on the workload's own
    batch: all host threads over the B grids of hx (one grid per thread at a
    time), and one thread on one grid; each the minimum of at least `repeats`
    timed runs after one untimed run, the reference's protocol
    (GenericConvolution2.rb:1248-1252).  None when the timing build is
    missing."""
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import oracle as O
    T = O.timing_lib()
    if T is None or not hasattr(W, 'timing_step'):
        return None
    th = cpu_threads()
    N = max(W.n_in, W.n_out)
    o0, o1 = np.zeros(B * N), np.zeros(B * N)
    x = np.ascontiguousarray(hx[:B * W.n_in])
    W.timing_step(T, O, B, x, o0, o1, th)
    t_all = [W.timing_step(T, O, B, x, o0, o1, th) for _ in range(repeats)]
    x1 = np.ascontiguousarray(hx[:W.n_in])
    W.timing_step(T, O, 1, x1, o0, o1, 1)
    t_one = [W.timing_step(T, O, 1, x1, o0, o1, 1) for _ in range(repeats)]
    if min(t_all) <= 0 or min(t_one) <= 0:
        return None
    v_all, v_one = B * W.n_in / min(t_all), W.n_in / min(t_one)
    return {'value': v_all, 'unit': UNIT, 'cores': th, 'kind': 'port',
            'threads_all': {'threads': th, 'value': v_all, 'grids': B,
                            'min_s': min(t_all), 'median_s': float(np.median(t_all))},
            'threads_1': {'threads': 1, 'value': v_one, 'grids': 1, 'min_s': min(t_one),
                          'median_s': float(np.median(t_one))},
            'repeats': repeats, 'cpu_model': cpu_model(),
            'build': 'oracle restatement, gcc -O3 -fopenmp (oracle/Makefile liblibconv_timing.so)',
            'sample': f'the bench batch ({B} grids of the {W.name} operators) on {th} threads, and '
                      f'one grid on 1 thread; min of {repeats} runs each after a warm-up run'}


def cpu_baseline_sample(W, grids):
    """Bounded sample (~10 s): all host threads, one grid each, repeated."""
    th = cpu_threads()
    times, pts = cpu_run(W, grids, th, 1, 0)
    reps = max(1, min(10, int(10.0 / max(times[0], 1e-3))))
    times2, _ = cpu_run(W, grids, th, reps, 0)
    t = float(np.median(times + times2))
    return {'value': pts / t, 'unit': UNIT, 'cores': th, 'kind': 'port',
            'sample': f'{th} grids (one per thread) x {1 + reps} repetitions of the '
                      f'{W.name} operators, C oracle, median step {t:.3f} s'}


def run_reference_orbitals(args, W):
    dims = W.dims()
    xs = W.base()
    th = cpu_threads()
    vals = []
    for _ in range(max(args.steps, 1)):
        pts, t = cpu_run_orbitals(W, xs, dims, th, 10.0)
        vals.append(pts / t)
    v = float(np.median(vals))
    line = {'impl': 'reference', 'metric': W.metric, 'value': v, 'unit': UNIT,
            'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': sum(x.size for x in xs) / v * 1e3, 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic (seeded)',
            'config': {'workload': f'512 orbitals, oracle MF free grow + kinetic free, {th} host '
                                   'threads taking orbitals round robin, ~10 s sample per step'},
            'cpu_baseline': {'value': v, 'unit': UNIT, 'cores': th, 'kind': 'port',
                             'sample': 'orbitals processed in ~10 s per step, C oracle'},
            'e2e': {'value': v, 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)


def run_reference_precond(args, W):
    vals = []
    for _ in range(max(args.steps, 1)):
        k, t, th = cpu_solves(W, 10.0)
        vals.append(k / t)
    v = float(np.median(vals))
    unit = 'solves/s'
    line = {'impl': 'reference', 'metric': W.metric.replace('flexible CG with the learned '
                                                            'preconditioner', 'plain CG on the host'),
            'value': v, 'unit': unit, 'n_gpus': args.gpus, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': 1e3 / v, 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic (seeded)',
            'config': {'workload': f'plain CG (C oracle kinetic, numpy vector updates) on the '
                                   f'256 benchmark systems, {th} host threads, ~10 s per step'},
            'cpu_baseline': {'value': v, 'unit': unit, 'cores': th, 'kind': 'port',
                             'sample': 'systems solved in ~10 s per step'},
            'e2e': {'value': v, 'unit': unit, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)


def cpu_hamiltonian(W, xs, pot, seconds):
    """oracle_hamiltonian on orbitals taken round robin by all host threads
    for about `seconds` (every thread finishes the orbital it started);
    returns (orbitals, time, threads)."""
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import oracle as O
    O.lib()
    th = cpu_threads()
    bufs = [(np.zeros(xs[0].size), np.zeros(3), np.zeros(1)) for _ in range(th)]
    done = [0] * th
    t0 = time.perf_counter()

    def work(t):
        g = t
        while True:
            W.cpu_work(O, xs[g % len(xs)], pot, bufs[t])
            done[t] += 1
            g += th
            if time.perf_counter() - t0 >= seconds:
                break

    ts = [threading.Thread(target=work, args=(t,)) for t in range(th)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    return sum(done), time.perf_counter() - t0, th


def run_reference_hamiltonian(args, W):
    package()
    xs = [W.orbital(3000 + i) for i in range(4)]
    pot = W.potential(int(np.prod([2 * v + 29 for v in W.n])))
    vals = []
    for _ in range(max(args.steps, 1)):
        k, t, th = cpu_hamiltonian(W, xs, pot, 10.0)
        vals.append(k / t)
    v = float(np.median(vals))
    unit = 'orbitals/s'
    line = {'impl': 'reference', 'metric': W.metric, 'value': v, 'unit': unit,
            'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': 1e3 / v, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic (seeded)',
            'config': {'workload': f'oracle_hamiltonian (C restatement of the composed '
                                   f'reference dispatchers), {th} host threads taking orbitals '
                                   'round robin, ~10 s per step', 'grid': W.n, 'bc': 'free'},
            'cpu_baseline': {'value': v, 'unit': unit, 'cores': th, 'kind': 'port',
                             'sample': 'orbitals processed in ~10 s per step'},
            'e2e': {'value': v, 'unit': unit, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)


def cpu_poisson(W, seconds, n=(128, 128, 128)):
    """oracle_div_u_i with cc on one 128^3 grid per host thread, repeated for
    about `seconds`; returns (points, time, threads)."""
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import oracle as O
    O.lib()
    th = cpu_threads()
    N = int(np.prod(n))
    rng = np.random.default_rng(5)
    us = [rng.uniform(0, 1, 3 * N) for _ in range(2)]
    bufs = [(np.zeros(N), np.zeros(N)) for _ in range(th)]
    done = [0] * th
    h = np.array(W.h)
    t0 = time.perf_counter()

    def work(t):
        while True:
            du, cc = bufs[t]
            O.call('oracle_div_u_i', W.geocode, *n, us[t % 2], du, W.nord, h, cc)
            done[t] += N
            if time.perf_counter() - t0 >= seconds:
                break

    ts = [threading.Thread(target=work, args=(t,)) for t in range(th)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    return sum(done), time.perf_counter() - t0, th


def run_reference_poisson(args, W):
    vals = []
    for _ in range(max(args.steps, 1)):
        pts, t, th = cpu_poisson(W, 10.0)
        vals.append(pts / t)
    v = float(np.median(vals))
    line = {'impl': 'reference', 'metric': W.metric, 'value': v, 'unit': UNIT,
            'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': int(np.prod(W.n)) / v * 1e3, 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic (seeded)',
            'config': {'workload': f'oracle_div_u_i with cc (C restatement of the generated '
                                   f'driver), one 128^3 grid per host thread, {th} threads, '
                                   '~10 s per step', 'grid': [128, 128, 128]},
            'cpu_baseline': {'value': v, 'unit': UNIT, 'cores': th, 'kind': 'port',
                             'sample': '128^3 grids processed in ~10 s per step'},
            'e2e': {'value': v, 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)


def reference_timed(args, W, grids, th):
    """Reference arm on the GPU arm's own configuration: every step runs the
    workload's operators over the same B grids (--grids) on all host threads
    in the oracle's -O3 OpenMP timing build; value from the fastest step (the
    reference's min-of-repeats protocol), the median beside it.  None when
    the timing build is missing."""
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import oracle as O
    T = O.timing_lib()
    if T is None or not hasattr(W, 'timing_step'):
        return None
    B = args.grids
    hx = np.zeros(B * W.n_in)
    W.fill(hx, B, 0, grids)
    N = max(W.n_in, W.n_out)
    o0, o1 = np.zeros(B * N), np.zeros(B * N)
    for _ in range(max(args.warmup, 1)):
        W.timing_step(T, O, B, hx, o0, o1, th)
    times = [W.timing_step(T, O, B, hx, o0, o1, th) for _ in range(args.steps)]
    x1 = np.ascontiguousarray(hx[:W.n_in])
    W.timing_step(T, O, 1, x1, o0, o1, 1)
    t_one = [W.timing_step(T, O, 1, x1, o0, o1, 1) for _ in range(max(5, min(args.steps, 5)))]
    t = min(times)
    v = B * W.n_in / t
    cb = {'value': v, 'unit': UNIT, 'cores': th, 'kind': 'port',
          'threads_all': {'threads': th, 'value': v, 'grids': B, 'min_s': t,
                          'median_s': float(np.median(times))},
          'threads_1': {'threads': 1, 'value': W.n_in / min(t_one), 'grids': 1,
                        'min_s': min(t_one), 'median_s': float(np.median(t_one))},
          'repeats': args.steps, 'cpu_model': cpu_model(),
          'build': 'oracle restatement, gcc -O3 -fopenmp (oracle/Makefile liblibconv_timing.so)',
          'sample': f'{args.steps} steps of the {B}-grid batch on {th} threads (min), one grid '
                    'on 1 thread'}
    return {'impl': 'reference', 'metric': W.metric, 'value': v, 'unit': UNIT,
            'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': t * 1e3, 'ms_per_step_median': float(np.median(times)) * 1e3,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
            'data': 'synthetic (seeded)',
            'config': {'workload': W.desc.format(B=B), 'grid': W.n, 'grids_per_gpu': B},
            'cpu_baseline': cb,
            'e2e': {'value': v, 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}


def run_reference(args):
    rank = int(os.environ.get('RANK', '0'))
    if rank != 0:
        return
    W = WORKLOADS[args.workload]
    if W.name == 'poisson256':
        return run_reference_poisson(args, W)
    if W.name == 'hamiltonian48':
        return run_reference_hamiltonian(args, W)
    if W.name == 'orbitals512':
        return run_reference_orbitals(args, W)
    if W.name == 'precond256':
        return run_reference_precond(args, W)
    grids = W.base(4)
    th = cpu_threads()
    line = reference_timed(args, W, grids, th)
    if line:
        print(json.dumps(line), flush=True)
        return
    times, pts = cpu_run(W, grids, th, args.steps, max(args.warmup, 1))
    t = float(np.median(times))
    v = pts / t
    line = {'impl': 'reference', 'metric': W.metric, 'value': v, 'unit': UNIT,
            'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': t * 1e3, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic (seeded)',
            'config': {'workload': f'{th} grids per step, one per host thread, {W.name} '
                                   'operators', 'grid': W.n},
            'cpu_baseline': {'value': v, 'unit': UNIT, 'cores': th, 'kind': 'port',
                             'sample': f'{args.steps} steps of {th} grids (one per thread), '
                                       'C oracle restating the reference loops'},
            'e2e': {'value': v, 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- GPU
MODES = {'fp64': 'MODE_FP64', 'tc_exact': 'MODE_TC_EXACT', 'tc_bf16x3': 'MODE_TC_BF16X3',
         'tc_tf32x3': 'MODE_TC_TF32X3'}


def run_orbitals(args, W):
    """Batched uneven orbitals: one graph launch per step (6 persistent sweep
    launches over all orbitals, tuned engine and sweep order), against the
    same operators called grid by grid through the single-grid entry points."""
    import torch
    pkg = package()
    R = Ranks()
    world, rank, local, dev = R.world, R.rank, R.local, R.device
    dims_all = W.dims()
    xs_all = W.base()
    # orbitals are partitioned across ranks, balanced by size (largest first)
    mine = shard_balanced([int(np.prod(d)) for d in dims_all], rank, world)
    dims = [dims_all[g] for g in mine]
    xs = [xs_all[g] for g in mine]
    pkg.set_mode(getattr(pkg, MODES[args.mode]))
    B = pkg.Batch(dims, mf_bc=[1, 1, 1], kin_bc=[2, 2, 2], kin_a=W.a)
    n_in, n_mf, n_kin = B.sizes()
    host_x = torch.from_numpy(np.concatenate(xs)).pin_memory()
    x = host_x.to(dev)
    y_mf = torch.empty(n_mf, dtype=torch.float64, device=dev)
    y_kin = torch.empty(n_kin, dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)
    t0 = time.perf_counter()
    if not args.no_tune:
        B.tune(x, y_mf, y_kin, stream=stream)
    tune_s = time.perf_counter() - t0
    for _ in range(max(args.warmup, 3)):
        B.run(x, y_mf, y_kin, stream=stream)
    pkg.check(stream)

    barrier = R.barrier

    clocks = Clocks(local)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    start.record(stream)
    for _ in range(args.steps):
        B.run(x, y_mf, y_kin, stream=stream)
    stop.record(stream)
    stop.synchronize()
    barrier()
    ck = clocks.stop()
    pkg.check(stream)
    ms = start.elapsed_time(stop)
    ms = R.max(ms)
    pts_step = R.sum(n_in)               # input points of all ranks' orbitals
    value = pts_step * args.steps / (ms / 1e3)

    # the same work grid by grid through the single-grid device entry points
    in_off, mf_off, kin_off = B.offsets()
    w1 = torch.empty(max(int(np.prod([v + 15 for v in d])) for d in dims), dtype=torch.float64,
                     device=dev)
    w2 = torch.empty_like(w1)
    mf_k, kin_k = pkg.Kernel('d_sfrf_ld_narr'), pkg.Kernel('d_kin')
    sp = stream.cuda_stream
    xp, mp, kp = x.data_ptr(), y_mf.data_ptr(), y_kin.data_ptr()

    def per_grid():
        for g, d in enumerate(dims):
            ny = [v + 15 for v in d]
            mf_k.run_dev(3, d, [1, 1, 1], d, ny, 1, xp + 8 * in_off[g], mp + 8 * mf_off[g], w1, w2,
                         stream=sp)
            kin_k.run_dev(3, d, [2, 2, 2], xp + 8 * in_off[g], kp + 8 * kin_off[g], w1, w2, W.a,
                          0.0, 0.0, stream=sp)

    per_grid()
    stream.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(2):
        per_grid()
    e1.record(stream)
    e1.synchronize()
    per_grid_ms = e0.elapsed_time(e1) / 2

    # e2e: pinned host orbitals in, both outputs back, every step
    host_mf = torch.empty(n_mf, dtype=torch.float64).pin_memory()
    host_kin = torch.empty(n_kin, dtype=torch.float64).pin_memory()

    def e2e_step():
        with torch.cuda.stream(stream):
            x.copy_(host_x, non_blocking=True)
            B.run(x, y_mf, y_kin, stream=stream)
            host_mf.copy_(y_mf, non_blocking=True)
            host_kin.copy_(y_kin, non_blocking=True)
        stream.synchronize()

    e2e_step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(max(2, min(args.steps, 5))):
        e2e_step()
    barrier()
    e_t = (time.perf_counter() - t0) / max(2, min(args.steps, 5))
    e2e = {'value': pts_step / e_t, 'unit': UNIT, 'h2d_bytes_per_step': 8 * n_in,
           'd2h_bytes_per_step': 8 * (n_mf + n_kin),
           'note': 'libconv_batch_run (graph) on the packed orbitals, H2D of x and D2H of '
                   'both outputs from pinned host memory inside the timed region'}

    # roofline of the step (6 batched sweeps): MF grow moves 8 (in + out) per
    # sweep over the growing sizes, the kinetic 16 + 24 + 24 B per point
    mf_bytes = 0
    for d in dims:
        a, b_, c = d
        A, Bq, C = a + 15, b_ + 15, c + 15
        mf_bytes += 8 * ((a * b_ * c + A * b_ * c) + (A * b_ * c + A * Bq * c) + (A * Bq * c + A * Bq * C))
    kin_bytes = 64 * n_in
    pk = peaks()
    achieved = (mf_bytes + kin_bytes) / (ms / args.steps / 1e3) / 1e9
    eng = {0: 'fp64 q64', 1: 'fp64 q32', 2: 'tensor core'}
    cfg = {'magicfilter3d': B.get_config(pkg.BATCH_OP_MF), 'kinetic3d': B.get_config(pkg.BATCH_OP_KIN)}
    # 3 sweeps per operator, each exact tensor-core sweep preceded by its
    # line-exponent pass
    launches = sum(3 * (2 if args.mode == 'tc_exact' and v[0] == 2 else 1) for v in cfg.values())
    line = {'metric': W.metric, 'value': value, 'unit': UNIT, 'n_gpus': world, 'steps': args.steps,
            'warmup': max(args.warmup, 3), 'ms_per_step': ms / args.steps, 'higher_is_better': True,
            'scaling': 'weak' if world == 1 else 'strong', 'vs_baseline': None,
            'dtype': 'f64' if args.mode in ('fp64', 'tc_exact') else args.mode,
            'data': 'synthetic (seeded orbitals: Gaussian envelope x unit-RMS noise, h=0.45)',
            'config': {'workload': f'{len(dims)} orbitals per GPU (axes U{{24..72}}, seed 7, '
                                   f'{n_in / 1e6:.1f} M points), MagicFilter3D free grow + '
                                   'Kinetic3D free, one libconv_batch_run (CUDA graph of 6 '
                                   'persistent sweeps, each exact tensor-core sweep after a '
                                   'line-exponent pass) per step', 'mode': args.mode,
                       'tuned': {k: {'engine': eng[v[0]], 'order': v[1]} for k, v in cfg.items()},
                       'tune_seconds': tune_s,
                       'per_grid_calls_ms_per_step': per_grid_ms,
                       'batched_speedup_vs_per_grid_calls': per_grid_ms / (ms / args.steps),
                       'l2': f'inputs larger than L2 ({8 * n_in / 1e6:.0f} MB in, '
                             f'{8 * n_mf / 1e6:.0f} MB MF out)'},
            'clocks': ck, 'e2e': e2e, 'gpu_launches': args.steps * launches,
            'roofline': {'bound': 'hbm', 'achieved': achieved, 'peak': pk['hbm'], 'unit': 'GB/s',
                         'frac': achieved / pk['hbm'], 'traffic': None,
                         'kernel': 'whole step: 6 batched sweeps (3 MF grow, 3 kinetic)',
                         'peak_source': pk['source']}}
    if rank == 0 and world == 1 and not args.no_cpu:
        th = cpu_threads()
        pts, t = cpu_run_orbitals(W, xs, dims, th, 10.0)
        line['cpu_baseline'] = {'value': pts / t, 'unit': UNIT, 'cores': th, 'kind': 'port',
                                'sample': f'{pts / 1e6:.1f} M orbital points in {t:.1f} s, '
                                          'C oracle, orbitals round robin over host threads'}
    if rank == 0 and getattr(args, 'emit', True):
        print(json.dumps(line), flush=True)
    B.close()
    R.close()
    return line


def run_precond(args, W):
    """Batched solves: one step = the 256 systems solved by flexible CG with
    the learned preconditioner (committed checkpoint) to ||r|| <= 1e-8;
    plain (Jacobi) CG on the same systems timed beside it."""
    import torch
    pkg = package()
    from boast_lig_gb300 import precond as P
    R = Ranks()
    world, rank, local, dev = R.world, R.rank, R.local, R.device
    pkg.set_mode(getattr(pkg, MODES[args.mode if args.mode in ('fp64', 'tc_exact') else 'tc_exact']))
    net = P.Net.load(os.path.join(P.WEIGHTS_DIR, W.weights), device=dev)
    b_np, eps_np = W.systems()
    n, h, nsys = W.n, [W.h] * 3, W.nsys
    host_b = torch.from_numpy(b_np.reshape(-1)).pin_memory()
    b = host_b.to(dev)
    eps = torch.from_numpy(eps_np).to(dev)
    x = torch.empty_like(b)
    stream = torch.cuda.Stream(device=dev)

    barrier = R.barrier

    def timed(m, steps):
        for _ in range(max(args.warmup, 3) if m is net else 1):
            P.solve(n, eps, b, x, h, tol=W.tol, maxit=3000, net=m, stream=stream)
        barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            info = {}
            it, res = P.solve(n, eps, b, x, h, tol=W.tol, maxit=3000, net=m, stream=stream,
                              info=info)
        e1.record(stream)
        e1.synchronize()
        barrier()
        return e0.elapsed_time(e1), it, res, info

    clocks = Clocks(local)
    clocks.start()
    ms, it, res, info = timed(net, args.steps)
    ck = clocks.stop()
    ms_plain, it_p, res_p, _ = timed(None, max(1, min(args.steps, 3)))
    steps_plain = max(1, min(args.steps, 3))
    ms = R.max(ms)
    value = nsys * world * args.steps / (ms / 1e3)
    plain = nsys * steps_plain / (ms_plain / 1e3)

    # e2e: right-hand sides from pinned host memory, solutions back, every step
    host_x = torch.empty(nsys * n ** 3, dtype=torch.float64).pin_memory()
    t0 = time.perf_counter()
    e_steps = max(2, min(args.steps, 5))
    for _ in range(e_steps):
        with torch.cuda.stream(stream):
            b.copy_(host_b, non_blocking=True)
        P.solve(n, eps, b, x, h, tol=W.tol, maxit=3000, net=net, stream=stream)
        with torch.cuda.stream(stream):
            host_x.copy_(x, non_blocking=True)
        stream.synchronize()
    e_t = (time.perf_counter() - t0) / e_steps
    e2e = {'value': nsys * world / e_t, 'unit': 'solves/s', 'h2d_bytes_per_step': 8 * b.numel(),
           'd2h_bytes_per_step': 8 * x.numel(),
           'note': 'libconv_cg_solve (learned) with b copied in and x copied out from pinned '
                   'host memory inside the timed region'}

    # dominant kernel: one 16 -> 16 channel convolution layer over the batch
    L = P._bind()
    wt, _, bias = net._packed
    a_in = torch.randn(nsys * n ** 3 * 16, device=dev).to(torch.bfloat16)
    a_out = torch.empty_like(a_in)
    sp = P._s(stream)
    for _ in range(3):
        L.libconv_cnn_conv(n, nsys, 0, 0, P._p(a_in), None, None, P._p(wt[1]), P._p(bias[1]),
                           P._p(a_out), None, None, 16, None, sp)
    c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    c0.record(stream)
    for _ in range(10):
        L.libconv_cnn_conv(n, nsys, 0, 0, P._p(a_in), None, None, P._p(wt[1]), P._p(bias[1]),
                           P._p(a_out), None, None, 16, None, sp)
    c1.record(stream)
    c1.synchronize()
    t_conv = c0.elapsed_time(c1) / 10 / 1e3
    flops = nsys * n ** 3 * 16 * 16 * 27 * 2
    pk = peaks()
    tflops = flops / t_conv / 1e12
    # algorithmic bytes: 16 BF16 channels read and written per point
    alg_bytes = nsys * n ** 3 * 64
    achieved = alg_bytes / t_conv / 1e9
    traffic = None
    tf = os.path.join(ROOT, 'profiles', 'precond_conv_tc_traffic.json')
    if os.path.exists(tf):
        with open(tf) as f:
            traffic = json.load(f)['dram_bytes_per_point'] * nsys * n ** 3
    line = {'metric': W.metric, 'value': value, 'unit': 'solves/s', 'n_gpus': world,
            'steps': args.steps, 'warmup': max(args.warmup, 3), 'ms_per_step': ms / args.steps,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
            'dtype': 'f64 solver (vectors, inner products, scalars); bf16 network, fp32 accumulate',
            'data': 'synthetic (seeded Gaussian-filtered noise right-hand sides, ||b|| = 1; eps '
                    'uniform in [-1, -0.1])',
            'config': {'workload': f'{nsys} systems of 48^3 periodic per GPU, h = 0.4, flexible '
                                   'CG with the 4-layer 16-channel 3^3 network '
                                   f'(weights/{W.weights}) to ||r|| <= 1e-8',
                       'kinetic_mode': pkg.get_mode(),
                       'iterations_mean': float(it.mean()), 'iterations_max': int(it.max()),
                       'fell_back': int((info['fell_back'] > 0).sum()),
                       'max_true_residual': float(res.max()),
                       'plain_cg_solves_per_s': plain, 'plain_cg_iterations_mean': float(it_p.mean()),
                       'plain_cg_iterations_max': int(it_p.max()),
                       'plain_cg_max_true_residual': float(res_p.max()),
                       'learned_over_plain': value / world / plain,
                       'l2': 'working set (7 vectors x 226 MB + activations) far above L2'},
            'clocks': ck, 'e2e': e2e, 'gpu_launches': args.steps * (15 * int(it.max()) + 12),
            'roofline': {'bound': 'hbm', 'achieved': achieved, 'peak': pk['hbm'],
                         'unit': 'GB/s', 'frac': achieved / pk['hbm'], 'traffic': traffic,
                         'tensor_tflops': tflops, 'tensor_frac': tflops / pk['bf16'],
                         'kernel': 'conv_tc_kernel<ACT,ACT_RELU,8> (16 -> 16 channels, 3^3, '
                                   'tcgen05 kind::f16 BF16, 256 x 48^3 points per launch)',
                         'peak_source': pk['source'], 'launch_ms': t_conv * 1e3}}
    if rank == 0 and world == 1 and not args.no_cpu:
        k, t, th = cpu_solves(W, 10.0)
        line['cpu_baseline'] = {'value': k / t, 'unit': 'solves/s', 'cores': th, 'kind': 'port',
                                'sample': f'{k} plain-CG solves in {t:.1f} s (C oracle kinetic), '
                                          'one system per host thread at a time'}
    if rank == 0 and getattr(args, 'emit', True):
        print(json.dumps(line), flush=True)
    R.close()
    return line


def run_hamiltonian(args, W):
    """Local Hamiltonian of B orbitals per GPU per step: rho zeroed, then one
    libconv_hamiltonian_dev call per orbital on one stream (rho accumulated
    over the orbitals, per-orbital energies kept on the device)."""
    import torch
    pkg = package()
    R = Ranks()
    world, rank, local, dev = R.world, R.rank, R.local, R.device
    pkg.set_mode(getattr(pkg, MODES[args.mode]))
    nsig, nreal, nwork = pkg.hamiltonian_sizes(W.n, W.bc)
    B = args.grids
    base = [W.orbital(3000 + i) for i in range(4)]
    host_x = torch.empty(B * nsig, dtype=torch.float64, pin_memory=True)
    hx = host_x.numpy()
    for b in range(B):
        hx[b * nsig:(b + 1) * nsig] = base[(b + rank) % 4] * (1.0 + 1e-3 * b)
    pot = W.potential(nreal)
    host_pot = torch.from_numpy(pot).pin_memory()
    dx, dpot = host_x.to(dev), host_pot.to(dev)
    dh = torch.empty_like(dx)
    drho = torch.zeros(nreal, dtype=torch.float64, device=dev)
    H = pkg.Hamiltonian(W.n, W.bc, W.a, norb=B, device=dev)
    stream = torch.cuda.Stream(device=dev)
    sp = stream.cuda_stream

    def step():
        with torch.cuda.stream(stream):
            drho.zero_()
        H(dx, dpot, dh, drho, stream=sp)

    for _ in range(max(args.warmup, 3)):
        step()
    stream.synchronize()
    pkg.check(sp)

    # the same work as one single-orbital call per orbital (no batching)
    H1 = pkg.Hamiltonian(W.n, W.bc, W.a, device=dev)
    E1 = torch.zeros(B, 4, dtype=torch.float64, device=dev)

    def step_single():
        with torch.cuda.stream(stream):
            drho.zero_()
        for b in range(B):
            sl = slice(b * nsig, (b + 1) * nsig)
            H1(dx[sl], dpot, dh[sl], drho, stream=sp, energies=E1[b])

    step_single()
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    step_single()
    s1.record(stream)
    s1.synchronize()
    ms_single = s0.elapsed_time(s1)
    del H1
    step()

    barrier = R.barrier

    clocks = Clocks(local)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    start.record(stream)
    for _ in range(args.steps):
        step()
    stop.record(stream)
    stop.synchronize()
    torch.cuda.synchronize()
    barrier()
    ck = clocks.stop()
    pkg.check(sp)
    ms = start.elapsed_time(stop)
    ms = R.max(ms)
    value = B * world * args.steps / (ms / 1e3)
    en = H.energies.cpu().numpy()

    # e2e: the host-pointer C-ABI, one call over the B orbitals (H2D of psig,
    # pot and rho, D2H of hpsig, rho and the energies inside every call)
    hpot = host_pot.numpy()
    hrho = torch.zeros(nreal, dtype=torch.float64, pin_memory=True).numpy()
    hh = torch.empty(B * nsig, dtype=torch.float64, pin_memory=True).numpy()
    hen = torch.empty(B * 4, dtype=torch.float64, pin_memory=True).numpy()
    pkg.hamiltonian_narr(W.n, W.bc, W.a, B, hx, hpot, hrho, hpsig=hh, energies=hen)
    barrier()
    e_steps = max(2, min(args.steps, 5))
    t0 = time.perf_counter()
    for _ in range(e_steps):
        hrho[:] = 0.0
        pkg.hamiltonian_narr(W.n, W.bc, W.a, B, hx, hpot, hrho, hpsig=hh, energies=hen)
    barrier()
    e_t = (time.perf_counter() - t0) / e_steps
    e2e = {'value': B * world / e_t, 'unit': 'orbitals/s',
           'h2d_bytes_per_step': (B * nsig + 2 * nreal) * 8,
           'd2h_bytes_per_step': (B * nsig + nreal + 4 * B) * 8,
           'note': 'libconv_hamiltonian_narr (host pointers, page-locked), one call over the '
                   'orbitals (the library pipelines chunks of orbitals)'}

    # pipeline roofline: the bytes every sweep reads and writes (the
    # composition as separate sweeps), per orbital, against the HBM peak
    n0 = [2 * v + 14 for v in W.n]
    nr = [v + 15 for v in n0]
    nf, nR = int(np.prod(n0)), int(np.prod(nr))
    sweep_bytes = 0
    for d0, d1 in ((W.n, n0), (n0, nr), (nr, n0), (n0, W.n)):
        dims = [2 * v for v in d0] if d0 is W.n else list(d0)
        out = [2 * v for v in d1] if d1 is W.n else list(d1)
        for i in range(3):
            cur_in = int(np.prod(dims))
            dims[i] = out[i]
            sweep_bytes += 8 * (cur_in + int(np.prod(dims)))
    sweep_bytes += 8 * nf * (2 + 3 + 3)      # kinetic: x each sweep, x2 twice, y RMW in the last
    sweep_bytes += 8 * nR * 4                # potential: psir RW, pot, rho RW
    pk = peaks()
    t_orb = ms / 1e3 / (args.steps * B)
    achieved = sweep_bytes / t_orb / 1e9
    min_bytes = 8 * (2 * nsig + 3 * nR)
    roof = {'bound': 'hbm', 'achieved': achieved, 'peak': pk['hbm'], 'unit': 'GB/s',
            'frac': achieved / pk['hbm'], 'traffic': None, 'peak_source': pk['source'],
            'kernel': 'whole pipeline (15 sweeps + potential) per orbital',
            'algorithmic_bytes_per_orbital': sweep_bytes,
            'compulsory_bytes_per_orbital': min_bytes,
            'compulsory_frac': min_bytes / t_orb / 1e9 / pk['hbm']}
    exact = args.mode in ('fp64', 'tc_exact')
    launches = H.LAUNCHES['exact' if args.mode == 'tc_exact' else 'other']   # per call
    line = {'metric': W.metric, 'value': value, 'unit': 'orbitals/s', 'n_gpus': world,
            'steps': args.steps, 'warmup': max(args.warmup, 3), 'ms_per_step': ms / args.steps,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
            'dtype': 'f64' if exact else ('f64 in HBM, ' + args.mode[3:] + ' split on tensor cores'),
            'data': 'synthetic (seeded)',
            'config': {'workload': f'{B} orbitals per GPU per step in one '
                                   'libconv_hamiltonian_narr_dev call, 48^3 coarse points (96^3 '
                                   'coefficients), free BC: 110^3 fine and 125^3 real-space '
                                   'points; one potential, rho accumulated',
                       'mode': args.mode, 'orbitals_per_gpu': B,
                       'single_orbital_calls_orbitals_per_s': B / (ms_single / 1e3),
                       'l2': f'inputs larger than L2 ({B * nsig * 8 / 1e6:.0f} MB of psig)',
                       'energies_orbital0': {'ekin': [float(v) for v in en[0, :3]],
                                             'epot': float(en[0, 3])}},
            'clocks': ck, 'e2e': e2e, 'gpu_launches': args.steps * launches,
            'roofline': roof}
    if rank == 0 and world == 1 and not args.no_cpu:
        k, t, th = cpu_hamiltonian(W, base, pot, 10.0)
        line['cpu_baseline'] = {'value': k / t, 'unit': 'orbitals/s', 'cores': th, 'kind': 'port',
                                'sample': f'{k} orbitals in {t:.1f} s, oracle_hamiltonian, one '
                                          'orbital per host thread'}
    if rank == 0:
        print(json.dumps(line), flush=True)
    R.close()


def run_poisson(args, W):
    """div_u_i with cc on one 256^3 field per GPU per step (device pointers,
    one stream), timed with CUDA events; e2e through the host-pointer call."""
    import ctypes
    import torch
    pkg = package()
    R = Ranks()
    world, rank, local, dev = R.world, R.rank, R.local, R.device
    pkg.set_mode(getattr(pkg, MODES[args.mode]))
    n = W.n
    N = int(np.prod(n))
    gen = torch.Generator().manual_seed(256 + rank)
    host_u = torch.rand(3 * N, generator=gen, dtype=torch.float64).pin_memory()
    du_ = host_u.to(dev)
    ddu = torch.empty(N, dtype=torch.float64, device=dev)
    dcc = torch.empty(N, dtype=torch.float64, device=dev)
    work = torch.empty(5 * N, dtype=torch.float64, device=dev)
    L = pkg.lib()
    f = L.div_u_i_dev
    f.argtypes = [ctypes.c_int] * 4 + [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                       ctypes.POINTER(ctypes.c_double)] + [ctypes.c_void_p] * 3
    f.restype = ctypes.c_int
    h = (ctypes.c_double * 3)(*W.h)
    stream = torch.cuda.Stream(device=dev)
    sp = ctypes.c_void_p(stream.cuda_stream)

    def step():
        st = f(W.geocode, *n, du_.data_ptr(), ddu.data_ptr(), W.nord, h, dcc.data_ptr(),
               work.data_ptr(), sp)
        if st:
            raise pkg.LibconvError(st, 'div_u_i_dev', pkg.last_error())

    for _ in range(max(args.warmup, 3)):
        step()
    stream.synchronize()
    pkg.check(stream)

    barrier = R.barrier

    clocks = Clocks(local)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    start.record(stream)
    for _ in range(args.steps):
        step()
    stop.record(stream)
    stop.synchronize()
    torch.cuda.synchronize()
    barrier()
    ck = clocks.stop()
    pkg.check(stream)
    ms = start.elapsed_time(stop)
    ms = R.max(ms)
    value = N * world * args.steps / (ms / 1e3)

    # one derivative sweep timed alone (the dominant kernel): d/dz of u0
    fb = L.Poisson_broker_dev
    fb.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p]
    fb.restype = ctypes.c_int
    nn = (ctypes.c_int * 3)(*n)
    reps = 10
    for _ in range(3):
        fb(W.nord, 2, nn, 0, du_.data_ptr(), ddu.data_ptr(), 10.0, sp)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fb(W.nord, 2, nn, 0, du_.data_ptr(), ddu.data_ptr(), 10.0, sp)
    e1.record(stream)
    e1.synchronize()
    t_sweep = e0.elapsed_time(e1) / reps / 1e3

    # e2e: the host-pointer div_u_i with cc (H2D of u, D2H of du and cc)
    hu = host_u.numpy()
    hdu = torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()
    hcc = torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()
    fh = L.div_u_i
    fh.argtypes = [ctypes.c_int] * 4 + [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                        ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]
    fh.restype = ctypes.c_int

    def host_step():
        st = fh(W.geocode, *n, hu.ctypes.data, hdu.ctypes.data, W.nord, h, hcc.ctypes.data)
        if st:
            raise pkg.LibconvError(st, 'div_u_i', pkg.last_error())

    host_step()
    barrier()
    e_steps = max(2, min(args.steps, 5))
    t0 = time.perf_counter()
    for _ in range(e_steps):
        host_step()
    barrier()
    e_t = (time.perf_counter() - t0) / e_steps
    e2e = {'value': N * world / e_t, 'unit': UNIT, 'h2d_bytes_per_step': 3 * N * 8,
           'd2h_bytes_per_step': 2 * N * 8, 'note': 'div_u_i (host pointers) with cc'}
    pk = peaks()
    achieved = W.sweep_bytes_per_pt * N / t_sweep / 1e9
    step_s = ms / 1e3 / args.steps
    roof = {'bound': 'hbm', 'achieved': achieved, 'peak': pk['hbm'], 'unit': 'GB/s',
            'frac': achieved / pk['hbm'], 'traffic': None, 'peak_source': pk['source'],
            'kernel': f'one periodic 17-tap derivative sweep along z ({args.mode}), timed alone',
            'algorithmic_bytes_per_point': W.sweep_bytes_per_pt,
            'step': {'algorithmic_bytes_per_point': W.bytes_per_pt,
                     'achieved_gbs': W.bytes_per_pt * N / step_s / 1e9,
                     'frac': W.bytes_per_pt * N / step_s / 1e9 / pk['hbm']}}
    # six sweeps, the edge kernels of the two sweeps along the non-periodic axis and the cc
    # kernel; in the exact mode those two sweeps also make a line-exponent pass (the four
    # periodic ones take their tile windows' exponents themselves)
    launches = {'tc_exact': 11, 'fp64': 9}.get(args.mode, 9)
    exact = args.mode in ('fp64', 'tc_exact')
    line = {'metric': W.metric, 'value': value, 'unit': UNIT, 'n_gpus': world, 'steps': args.steps,
            'warmup': max(args.warmup, 3), 'ms_per_step': ms / args.steps,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
            'dtype': 'f64' if exact else ('f64 in HBM, ' + args.mode[3:] + ' split on tensor cores'),
            'data': 'synthetic (seeded uniform [0,1), as the reference test)',
            'config': {'workload': 'div_u_i_dev with cc, 256^3, nord 16, geocode 3, h 0.1: six '
                                   'derivative sweeps and the cc kernel per step',
                       'mode': args.mode, 'grid': n,
                       'l2': f'inputs larger than L2 ({3 * N * 8 / 1e6:.0f} MB of u)',
                       'ms_sweep': t_sweep * 1e3},
            'clocks': ck, 'e2e': e2e, 'gpu_launches': args.steps * launches, 'roofline': roof}
    if rank == 0 and world == 1 and not args.no_cpu:
        pts, t, th = cpu_poisson(W, 10.0)
        line['cpu_baseline'] = {'value': pts / t, 'unit': UNIT, 'cores': th, 'kind': 'port',
                                'sample': f'{pts // (128 ** 3)} grids of 128^3 in {t:.1f} s, '
                                          'oracle_div_u_i with cc, one grid per host thread'}
    if rank == 0:
        print(json.dumps(line), flush=True)
    R.close()


def run_gpu(args):
    import torch
    pkg = package()
    W = WORKLOADS[args.workload]
    if W.name == 'poisson256':
        return run_poisson(args, W)
    if W.name == 'hamiltonian48':
        return run_hamiltonian(args, W)
    if W.name == 'orbitals512':
        return run_orbitals(args, W)
    if W.name == 'precond256':
        return run_precond(args, W)
    R = Ranks()
    world, rank, local, dev = R.world, R.rank, R.local, R.device
    B = args.grids
    Ni, No = W.n_in, W.n_out
    base = W.base(4)
    host_x = torch.empty(B * Ni, dtype=torch.float64, pin_memory=True)
    hx = host_x.numpy()
    W.fill(hx, B, rank, base)
    bufs = {'x': host_x.to(dev)}
    for k in ('o0', 'o1', 'w1', 'w2'):
        bufs[k] = torch.empty(B * max(Ni, No), dtype=torch.float64, device=dev)
    pkg.set_mode(getattr(pkg, MODES[args.mode]))
    ops = W.dev_ops(pkg, B, bufs)
    stream = torch.cuda.Stream(device=dev)
    sp = stream.cuda_stream

    def step(evs=None):
        for i, op in enumerate(ops):
            if evs:
                evs[i].record(stream)
            op(sp)
        if evs:
            evs[len(ops)].record(stream)

    for _ in range(max(args.warmup, 3)):
        step()
    stream.synchronize()
    pkg.check(sp)

    barrier = R.barrier

    clocks = Clocks(local)
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(len(ops) + 1)]
           for _ in range(args.steps)]
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    start.record(stream)
    for k in range(args.steps):
        step(evs[k])
    stop.record(stream)
    stop.synchronize()
    torch.cuda.synchronize()
    barrier()
    ck = clocks.stop()
    pkg.check(sp)
    ms = start.elapsed_time(stop)
    op_ms = [sum(e[i].elapsed_time(e[i + 1]) for e in evs) for i in range(len(ops))]
    ms = R.max(ms)
    pts_step = B * Ni * world
    value = pts_step * args.steps / (ms / 1e3)

    # split precision: each operator's max relative error against the
    # exact-digit (FP64-accurate) output of the same step
    accuracy = None
    if args.mode in ('tc_bf16x3', 'tc_tf32x3'):
        got = [bufs['o0'][:B * No].clone(), bufs['o1'][:B * No].clone()]
        pkg.set_mode(pkg.MODE_TC_EXACT)
        step()
        stream.synchronize()
        ref = [bufs['o0'][:B * No], bufs['o1'][:B * No]]
        accuracy = {'reference': 'tc_exact output of the same step (FP64-accurate)'}
        for name, g, r in zip(W.ops, got, ref):
            accuracy[name] = float((g - r).abs().max() / r.abs().max())
        pkg.set_mode(getattr(pkg, MODES[args.mode]))

    # the configuration's second operator shape: free-BC grow MagicFilter3D on
    # B grids of 64^3 (output 79^3), device-resident, timed on its own
    grow = None
    if W.name == 'mfkin128':
        gn, gy = [64] * 3, [79] * 3
        gx = torch.rand(B * 64 ** 3, dtype=torch.float64, device=dev) * 2 - 1
        gyb = torch.empty(B * 79 ** 3, dtype=torch.float64, device=dev)
        gw1, gw2 = torch.empty_like(gyb), torch.empty_like(gyb)
        gk = pkg.Kernel('d_sfrf_ld_narr')
        gop = lambda: gk.run_dev(3, gn, [1, 1, 1], gn, gy, B, gx, gyb, gw1, gw2, stream=sp)
        for _ in range(3):
            gop()
        g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        g0.record(stream)
        for _ in range(10):
            gop()
        g1.record(stream)
        g1.synchronize()
        pkg.check(sp)
        g_ms = g0.elapsed_time(g1) / 10
        grow = {'op': 'MagicFilter3D free grow (d_sfrf_ld_narr, bc grow on every axis)',
                'grids': B, 'in': '64^3', 'out': '79^3', 'ms': g_ms,
                'in_pts_per_s': B * 64 ** 3 / (g_ms / 1e3), 'out_pts_per_s': B * 79 ** 3 / (g_ms / 1e3)}

    # e2e: the public host-pointer C-ABI with pinned host buffers, copies inside
    ho0 = torch.empty(B * max(Ni, No), dtype=torch.float64, pin_memory=True).numpy()
    ho1 = torch.empty(B * max(Ni, No), dtype=torch.float64, pin_memory=True).numpy()
    W.host_step(pkg, B, hx, ho0, ho1)
    barrier()
    e_steps = max(2, min(args.steps, 5))
    t0 = time.perf_counter()
    for _ in range(e_steps):
        W.host_step(pkg, B, hx, ho0, ho1)
    torch.cuda.synchronize()
    barrier()
    e_t = (time.perf_counter() - t0) / e_steps
    if W.name == 'mfkin128':
        h2d, d2h = 2 * B * Ni * 8, 2 * B * No * 8
    else:
        h2d, d2h = B * (Ni + No) * 8, B * (Ni + No) * 8
    e2e = {'value': pts_step / e_t, 'unit': UNIT, 'h2d_bytes_per_step': h2d,
           'd2h_bytes_per_step': d2h, 'note': W.e2e_note}

    # roofline of the dominant kernel
    pk = peaks()
    launches_dom = 3 * args.steps
    t_launch = op_ms[W.dom] / 1e3 / launches_dom
    pts_launch = Ni * B
    achieved = W.dom_bytes_per_pt * pts_launch / t_launch / 1e9
    traffic = None
    tf = W.traffic_file.get(args.mode)
    if tf and os.path.exists(os.path.join(ROOT, 'profiles', tf)):
        tj = json.load(open(os.path.join(ROOT, 'profiles', tf)))
        traffic = tj['dram_bytes_per_point'] * pts_launch
    roof = {'bound': 'hbm', 'achieved': achieved, 'peak': pk['hbm'], 'unit': 'GB/s',
            'frac': achieved / pk['hbm'], 'traffic': traffic, 'kernel': W.dom_kernel[args.mode],
            'peak_source': pk['source'],
            'algorithmic_bytes_per_point': W.dom_bytes_per_pt}
    if getattr(W, 'step_bytes', None):
        roof['step'] = step_roofline(W.step_bytes, B * Ni, ms / 1e3 / args.steps, pk['hbm'])
    if args.mode != 'fp64':
        # MMA work per output point (not algorithmic flops): products x K x 2
        prods = {'tc_exact': W.pairs_exact, 'tc_bf16x3': 6, 'tc_tf32x3': 3}[args.mode]
        mma_tflops = prods * W.kb * 2 * pts_launch / t_launch / 1e12
        peak_t = pk['bf16'] / (2 if args.mode == 'tc_tf32x3' else 1)
        roof['tensor_pipe'] = {'mma_tflops': mma_tflops, 'peak_tflops': peak_t,
                               'frac': mma_tflops / peak_t,
                               'note': f'{prods} operand-plane products, K={W.kb} per 16 outputs'
                                       + ('; tf32 peak = half the measured bf16 peak'
                                          if args.mode == 'tc_tf32x3' else '')}
    fp = fp64_peak(pkg, local) if getattr(args, 'emit', True) else None
    if args.mode == 'fp64':
        ach = W.dom_flops_per_pt * pts_launch / t_launch / 1e12
        roof['fp64_pipe'] = {'achieved_tflops': ach,
                             'peak_tflops': fp['tflops'] if fp else None,
                             'frac': ach / fp['tflops'] if fp else None,
                             'peak_source': 'measured' if fp else None, 'peak': fp,
                             'note': 'plain FP64 FMA path: bound by the FP64 pipe, not HBM'}
    elif fp:
        roof['fp64_pipe_peak'] = fp
    exact = args.mode in ('fp64', 'tc_exact')
    line = {'metric': W.metric, 'value': value, 'unit': UNIT, 'n_gpus': world, 'steps': args.steps,
            'warmup': max(args.warmup, 3), 'ms_per_step': ms / args.steps, 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None,
            'dtype': 'f64' if exact else ('f64 in HBM, ' + args.mode[3:] + ' split on tensor cores'),
            'data': 'synthetic (seeded)',
            'config': {'workload': W.desc.format(B=B), 'grid': W.n, 'grids_per_gpu': B,
                       'mode': args.mode,
                       'l2': f'inputs larger than L2 ({B * Ni * 8 / 1e6:.0f} MB per array)',
                       **{f'ms_{o}': t / args.steps for o, t in zip(W.ops, op_ms)},
                       **({'grow_magicfilter_64': grow} if grow else {})},
            'clocks': ck, 'e2e': e2e,
            # exact tensor-core sweeps are preceded by line-exponent passes
            'gpu_launches': args.steps * (W.launches + (W.exact_prepasses if args.mode == 'tc_exact'
                                                        else 0)),
            'roofline': roof}
    if accuracy:
        line['accuracy_max_rel_error'] = accuracy
    if rank == 0 and world == 1 and not args.no_cpu:
        line['cpu_baseline'] = cpu_timed(W, B, hx) or cpu_baseline_sample(W, base)
    if W.name == 'mfkin128' and world == 1 and getattr(args, 'emit', True) and not args.no_sub:
        # free the headline buffers first: the sub-records allocate their own
        del bufs, ops
        torch.cuda.empty_cache()
        line['config'].update(sub_records(args))
    if rank == 0 and getattr(args, 'emit', True):
        print(json.dumps(line), flush=True)
    R.close()
    return line


def step_roofline(step_bytes, points, step_s, hbm_gbs):
    """The whole step against HBM for each byte count of step_bytes
    ({name: algorithmic bytes per point}): GB/s over `points` grid points per
    step of `step_s` seconds, and the fraction of `hbm_gbs`."""
    out = {}
    for name, v in step_bytes.items():
        gbs = v * points / step_s / 1e9
        out[name] = {'algorithmic_bytes_per_point': v, 'achieved_gbs': gbs, 'frac': gbs / hbm_gbs}
    return out


def sub_records(args):
    """The other configurations of the metric, measured in the same run after
    the headline (one GPU, each bounded to a few steps): the 96^3 wavelet
    round trip (throughput in the exact mode, and the split-precision
    schemes' max relative error per operator), the 512 uneven orbitals
    (batched graph throughput and the tuner's choice) and the 256 learned-
    preconditioner solves (learned and plain CG solves/s, their ratio and the
    largest true FP64 residual).  A failure is recorded, not raised."""
    import argparse as _ap
    out = {}

    def sub(workload, mode, steps):
        a = _ap.Namespace(**vars(args))
        a.workload, a.mode, a.steps, a.warmup = workload, mode, steps, 3
        a.no_cpu, a.emit, a.no_sub, a.grids = True, False, True, 32
        W = WORKLOADS[workload]
        if workload == 'orbitals512':
            return run_orbitals(a, W)
        if workload == 'precond256':
            return run_precond(a, W)
        return run_gpu(a)

    try:
        t0 = time.perf_counter()
        wl = sub('wavelet96', 'tc_exact', 5)
        rec = {'workload': wl['config']['workload'], 'gpts_per_s': wl['value'] / 1e9,
               'e2e_gpts_per_s': wl['e2e']['value'] / 1e9, 'ms_idwt3d': wl['config']['ms_idwt3d'],
               'ms_dwt3d': wl['config']['ms_dwt3d'], 'mode': 'tc_exact'}
        for m in ('tc_bf16x3', 'tc_tf32x3'):
            ws = sub('wavelet96', m, 2)
            rec[m] = {'gpts_per_s': ws['value'] / 1e9,
                      'max_rel_error': {k: v for k, v in ws['accuracy_max_rel_error'].items()
                                        if k != 'reference'}}
        rec['seconds'] = time.perf_counter() - t0
        out['wavelet96'] = rec
    except Exception as e:   # noqa: BLE001 -- recorded in the line
        out['wavelet96'] = {'error': repr(e)[:300]}
    try:
        t0 = time.perf_counter()
        ob = sub('orbitals512', 'tc_exact', 5)
        c = ob['config']
        out['orbitals512'] = {'workload': c['workload'], 'gpts_per_s': ob['value'] / 1e9,
                              'e2e_gpts_per_s': ob['e2e']['value'] / 1e9, 'tuned': c['tuned'],
                              'tune_seconds': c['tune_seconds'],
                              'batched_speedup_vs_per_grid_calls': c['batched_speedup_vs_per_grid_calls'],
                              'mode': 'tc_exact', 'seconds': time.perf_counter() - t0}
    except Exception as e:   # noqa: BLE001
        out['orbitals512'] = {'error': repr(e)[:300]}
    try:
        t0 = time.perf_counter()
        pc = sub('precond256', 'tc_exact', 3)
        c = pc['config']
        out['precond256'] = {'workload': c['workload'], 'learned_solves_per_s': pc['value'],
                             'plain_cg_solves_per_s': c['plain_cg_solves_per_s'],
                             'learned_over_plain': c['learned_over_plain'],
                             'max_true_residual': c['max_true_residual'],
                             'plain_cg_max_true_residual': c['plain_cg_max_true_residual'],
                             'iterations_mean': c['iterations_mean'],
                             'plain_cg_iterations_mean': c['plain_cg_iterations_mean'],
                             'e2e_solves_per_s': pc['e2e']['value'],
                             'tolerance': 1e-8, 'seconds': time.perf_counter() - t0}
    except Exception as e:   # noqa: BLE001
        out['precond256'] = {'error': repr(e)[:300]}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=10)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--workload', default='mfkin128', choices=list(WORKLOADS))
    ap.add_argument('--grids', type=int, default=32)
    ap.add_argument('--systems', type=int, default=None,
                    help='precond256: number of systems (default 256; smaller for profiling)')
    ap.add_argument('--no-cpu', action='store_true', help='skip the CPU baseline sample')
    ap.add_argument('--no-sub', action='store_true',
                    help='mfkin128: skip the other configurations (wavelet96, orbitals512, '
                         'precond256) recorded under config after the headline')
    ap.add_argument('--no-tune', action='store_true',
                    help='orbitals512: use the cached or default batch configuration')
    ap.add_argument('--mode', default='tc_exact', choices=list(MODES),
                    help='tc_exact: tensor-core exact-digit sweeps (FP64-accurate); fp64: FP64 '
                         'FMA; tc_bf16x3 / tc_tf32x3: split precision (error reported)')
    args = ap.parse_args()
    if args.systems:
        WORKLOADS['precond256'].nsys = args.systems
    if args.impl == 'reference':
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == '__main__':
    main()
