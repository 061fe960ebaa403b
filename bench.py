#!/usr/bin/env python3
"""Benchmark: FP64 3D MagicFilter + Kinetic on 128^3 periodic grids.

One step = the hot path over one batch of grids held in HBM: for every grid
x of the batch, psi_r = MagicFilter3D(x) (three rotated sweeps) and
T x = Kinetic3D(x) (h = 0.45 bohr per axis, three accumulating sweeps), both
from the same x.  Metric: grid points per second (points of x processed by
both operators), whole job.  Inputs are seeded Gaussian-filtered noise
(sigma = 2 points, unit RMS); the batch (default 32 grids, 537 MB per array)
is larger than the 126 MB L2, so every step streams from HBM.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

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

N_AXIS = 128
HGRID = 0.45
METRIC = 'grid pts/s, FP64 3D MagicFilter + Kinetic (128^3 periodic)'
UNIT = 'grid pts/s'


def peaks():
    p = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get('hbm_gbs', 6800.0), 'measured'
    return 6800.0, 'fallback'


def base_grids(count, n):
    import __graft_entry__ as ge
    ge.package()
    from boast_lig_gb300 import inputs
    return [inputs.gaussian_filtered_noise(1000 + i, (n, n, n)).ravel(order='F') for i in range(count)]


class Clocks:
    """nvidia-smi sampler running during the timed region."""
    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
         'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
         'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, dev):
        self.dev = dev
        self.p = None
        self.out = os.path.join('/tmp', f'lcg_clocks_{os.getpid()}.csv')

    def start(self):
        try:
            self.p = subprocess.Popen(['nvidia-smi', '-i', str(self.dev), f'--query-gpu={self.Q}',
                                       '--format=csv,noheader,nounits', '-lms', '200'],
                                      stdout=open(self.out, 'w'), stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        time.sleep(0.25)
        self.p.terminate()
        self.p.wait()
        rows = []
        for line in open(self.out):
            f = [t.strip() for t in line.split(',')]
            if len(f) >= 9:
                rows.append(f)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace('.', '').isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace('.', '').isdigit()]
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i] == 'Active'})
        return {'sm_mhz': float(np.median(sm)) if sm else None,
                'sm_max_mhz': max(mx) if mx else None, 'reasons': reasons, 'samples': len(rows)}


# ----------------------------------------------------------------------------- CPU
def cpu_run(grids, threads, steps, warmup):
    """Oracle MagicFilter3D + Kinetic3D, one grid per host thread (ctypes
    releases the GIL).  Returns seconds per step (min over steps)."""
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import oracle as O
    O.lib()
    n = [N_AXIS] * 3
    N = grids[0].size
    a = np.array([-0.5 / HGRID ** 2] * 3)
    bufs = [[np.zeros(N) for _ in range(4)] for _ in range(threads)]

    def work(t):
        x = grids[t % len(grids)]
        y, tx, w1, w2 = bufs[t]
        O.call('oracle_d_sfrf_ld_narr', 3, n, [0, 0, 0], n, n, 1, x, y, w1, w2)
        O.call('oracle_d_kin', 3, n, [0, 0, 0], x, tx, w1, w2, a, 0.0, 0.0)

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
    return times, threads * N


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_baseline_sample(grids):
    """Bounded sample (~10 s): all host threads, one 128^3 grid each, repeated."""
    th = cpu_threads()
    times, pts = cpu_run(grids, th, 1, 0)
    reps = max(1, min(10, int(10.0 / max(times[0], 1e-3))))
    times2, _ = cpu_run(grids, th, reps, 0)
    t = float(np.median(times + times2))
    return {'value': pts / t, 'unit': UNIT, 'cores': th, 'kind': 'port',
            'sample': f'{th} grids of 128^3 (one per thread) x {1 + reps} repetitions, '
                      f'MagicFilter3D + Kinetic3D, C oracle, median step {t:.3f} s'}


def run_reference(args):
    rank = int(os.environ.get('RANK', '0'))
    if rank != 0:
        return
    grids = base_grids(4, N_AXIS)
    th = cpu_threads()
    times, pts = cpu_run(grids, th, args.steps, max(args.warmup, 1))
    t = float(np.median(times))
    v = pts / t
    line = {'impl': 'reference', 'metric': METRIC, 'value': v, 'unit': UNIT, 'n_gpus': args.gpus,
            'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': t * 1e3,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
            'data': 'synthetic (seeded Gaussian-filtered noise)',
            'config': {'workload': f'{th} grids of 128^3 periodic per step, one per host thread, '
                                   'MagicFilter3D + Kinetic3D (h=0.45)', 'grid': [128, 128, 128]},
            'cpu_baseline': {'value': v, 'unit': UNIT, 'cores': th, 'kind': 'port',
                             'sample': f'{args.steps} steps of {th} grids (one per thread), '
                                       'C oracle restating the reference loops'},
            'e2e': {'value': v, 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- GPU
def run_gpu(args):
    import torch
    import __graft_entry__ as ge
    pkg = ge.package()
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    torch.cuda.set_device(local)
    dev = torch.device('cuda', local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl', device_id=dev)
    B = args.grids
    n = [N_AXIS] * 3
    N = N_AXIS ** 3
    base = base_grids(4, N_AXIS)
    host_x = torch.empty(B * N, dtype=torch.float64, pin_memory=True)
    hx = host_x.numpy()
    for b in range(B):
        hx[b * N:(b + 1) * N] = base[(b + rank) % 4] * (1.0 + 1e-3 * b)
    xd = host_x.to(dev)
    psir = torch.empty(B * N, dtype=torch.float64, device=dev)
    tx = torch.empty(B * N, dtype=torch.float64, device=dev)
    w1 = torch.empty(B * N, dtype=torch.float64, device=dev)
    w2 = torch.empty(B * N, dtype=torch.float64, device=dev)
    a = [-0.5 / HGRID ** 2] * 3
    tc = args.mode == 'tc_exact'
    pkg.set_mode(pkg.MODE_TC_EXACT if tc else pkg.MODE_FP64)
    mf = pkg.Kernel('d_sfrf_ld_narr')
    kin = pkg.Kernel('d_kin_narr')
    stream = torch.cuda.Stream(device=dev)
    sp = stream.cuda_stream
    base_ptr = xd.data_ptr()

    def step(evs=None):
        if evs:
            evs[0].record(stream)
        mf.run_dev(3, n, [0, 0, 0], n, n, B, xd, psir, w1, w2, stream=sp)
        if evs:
            evs[1].record(stream)
        kin.run_dev(3, n, [0, 0, 0], B, xd, tx, w1, w2, a, 0.0, 0.0, stream=sp)
        if evs:
            evs[2].record(stream)

    for _ in range(max(args.warmup, 3)):
        step()
    stream.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    clocks = Clocks(local)
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
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
    ms = start.elapsed_time(stop)
    mf_ms = sum(e[0].elapsed_time(e[1]) for e in evs)
    kin_ms = sum(e[1].elapsed_time(e[2]) for e in evs)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = t.item()
    pts_step = B * N * world
    value = pts_step * args.steps / (ms / 1e3)

    # e2e: the public host-pointer C-ABI with pinned host buffers, copies inside
    host_psir = torch.empty(B * N, dtype=torch.float64, pin_memory=True).numpy()
    host_tx = torch.empty(B * N, dtype=torch.float64, pin_memory=True).numpy()
    hw = np.zeros(1)

    def e2e_step():
        mf.run(3, n, [0, 0, 0], n, n, B, hx, host_psir, hw, hw)
        kin.run(3, n, [0, 0, 0], B, hx, host_tx, hw, hw, a, 0.0, 0.0)

    e2e_step()
    barrier()
    e_steps = max(2, min(args.steps, 5))
    t0 = time.perf_counter()
    for _ in range(e_steps):
        e2e_step()
    torch.cuda.synchronize()
    barrier()
    e_t = (time.perf_counter() - t0) / e_steps
    e2e = {'value': pts_step / e_t, 'unit': UNIT, 'h2d_bytes_per_step': 2 * B * N * 8,
           'd2h_bytes_per_step': 2 * B * N * 8,
           'note': 'd_sfrf_ld_narr (narr=B) + d_kin_narr (narr=B), host pointers (pinned), '
                   'H2D of x and D2H of psi_r and T x inside every call'}

    # roofline of the dominant kernel (kinetic sweep, 29 taps): 3 launches per
    # grid; algorithmic bytes per grid 64 B/pt (16 + 24 + 24)
    hbm, src = peaks()
    launches_kin = 3 * args.steps
    t_launch = kin_ms / 1e3 / launches_kin
    bytes_launch = 64.0 / 3.0 * N * B
    achieved = bytes_launch / t_launch / 1e9
    flops_launch = (58 + 1 + 2.0 / 3.0) * N * B  # 29 FMA, scale, x2 add (2 of 3 sweeps)
    traffic = None
    kname = ('sweep_tc_kernel<29> (kinetic sweep, all grids per launch)' if tc
             else 'sweep_fp64_kernel<KCONV,29> (kinetic sweep, all grids per launch)')
    tp = os.path.join(ROOT, 'profiles', ('kinetic_sweep_tc_traffic.json' if tc
                                         else 'kinetic_sweep_fp64_traffic.json'))
    if os.path.exists(tp):
        tj = json.load(open(tp))
        traffic = tj['dram_bytes_per_point'] * N * B
    roof = {'bound': 'hbm', 'achieved': achieved, 'peak': hbm, 'unit': 'GB/s',
            'frac': achieved / hbm, 'traffic': traffic, 'kernel': kname, 'peak_source': src}
    if tc:
        # tensor work per output: 28 digit pairs x K=48 x 2 flops (not algorithmic flops)
        bf = json.load(open(os.path.join(ROOT, 'MEASURED_PEAKS.json'))).get('bf16_tflops', 1900.0) \
            if os.path.exists(os.path.join(ROOT, 'MEASURED_PEAKS.json')) else 1900.0
        tflops = 36 * 48 * 2 * N * B / t_launch / 1e12
        roof['tensor_pipe'] = {'mma_tflops': tflops, 'peak_tflops': bf, 'frac': tflops / bf,
                               'note': 'exact FP16-digit MMAs (36 byte pairs, K=48 per 16 outputs)'}
    else:
        roof['fp64_pipe'] = {'achieved_tflops': flops_launch / t_launch / 1e12,
                             'nominal_peak_tflops': 1.25,
                             'note': 'plain FP64 FMA path: bound by the FP64 pipe, not HBM'}
    line = {'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': world, 'steps': args.steps,
            'warmup': max(args.warmup, 3), 'ms_per_step': ms / args.steps, 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
            'data': 'synthetic (seeded Gaussian-filtered noise, sigma=2, unit RMS)',
            'config': {'workload': f'{B} grids of 128^3 periodic per GPU per step: '
                                   'MagicFilter3D (d_sfrf_ld_narr) + Kinetic3D (d_kin_narr, h=0.45)',
                       'grid': n, 'grids_per_gpu': B, 'mode': args.mode,
                       'l2': 'inputs larger than L2 (537 MB per array)',
                       'ms_magicfilter3d': mf_ms / args.steps, 'ms_kinetic3d': kin_ms / args.steps},
            'clocks': ck, 'e2e': e2e, 'gpu_launches': args.steps * 6,
            'roofline': roof}
    if rank == 0 and world == 1 and not args.no_cpu:
        line['cpu_baseline'] = cpu_baseline_sample(base)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=10)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--grids', type=int, default=32)
    ap.add_argument('--no-cpu', action='store_true', help='skip the CPU baseline sample')
    ap.add_argument('--mode', default='tc_exact', choices=['tc_exact', 'fp64'],
                    help='tc_exact: tensor-core exact-digit sweeps (FP64-accurate); fp64: FP64 FMA')
    args = ap.parse_args()
    if args.impl == 'reference':
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == '__main__':
    main()
