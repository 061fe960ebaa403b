"""Multi-rank host logic of bench.py on CPU (two gloo ranks on 127.0.0.1):
the ranks agree on the slowest step time (max) and on totals (sum), each
rank fills its own distinct batch of grids, and the orbital partition is
disjoint, complete and balanced by size.  The runs use NCCL, one rank per
GPU; nothing on the data path is collective, so these are the only
cross-rank operations."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


SIZES = [int(v) for v in np.random.default_rng(7).integers(24, 73, size=(37, 3)).prod(axis=1)]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    R = bench.Ranks(backend='gloo')
    mx = R.max(10.0 + 3.5 * rank)               # per-rank step times in ms
    tot = R.sum(100 * (rank + 1))               # per-rank points
    R.barrier()
    mine = bench.shard_balanced(SIZES, R.rank, R.world)
    base = [np.full(8, float(i + 1)) for i in range(4)]
    hx = np.zeros(3 * 8)
    W = bench.WORKLOADS['mfkin128']
    W.n_in = 8                                  # a tiny stand-in grid for the fill check
    W.fill(hx, 3, R.rank, base)
    q.put((rank, mx, tot, mine, hx.tolist()))
    R.close()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted([q.get(timeout=120) for _ in procs])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, mx0, tot0, mine0, hx0), (r1, mx1, tot1, mine1, hx1) = out
    assert mx0 == mx1 == 13.5                    # the slowest rank's time
    assert tot0 == tot1 == 300
    assert sorted(mine0 + mine1) == list(range(len(SIZES)))
    s0, s1 = sum(SIZES[g] for g in mine0), sum(SIZES[g] for g in mine1)
    assert abs(s0 - s1) <= max(SIZES)
    assert hx0 != hx1                            # each rank works on its own grids


def test_reference_arm_other_ranks_exit_quietly(monkeypatch):
    """Under torchrun only rank 0 runs and prints the reference arm."""
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv('RANK', '1')
    args = type('A', (), {'workload': 'mfkin128', 'steps': 1, 'warmup': 1, 'gpus': 2})()
    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_reference(args)
    assert buf.getvalue() == ''
