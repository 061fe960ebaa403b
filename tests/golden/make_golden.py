#!/usr/bin/env python3
"""Generate golden vectors from the reference's own code.

The only part of the reference on this path that compiles as-is is
benchmark/convolutions-c/MagicFilter.c (magicfilter1d_naive_ and
magicfilter1d_t_naive_, periodic MagicFilter and its transposed-filter form).
``make -C oracle ref`` builds it from the reference tree into oracle/_ref/;
this script runs it on seeded inputs and stores the outputs here, so tests on
machines without the reference tree still check against the reference's bits.

Inputs are regenerated from (seed, size) with the package's SplitMix64
generator; the file stores the outputs and a checksum of the inputs.
"""
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, 'oracle'))

# (name, n, ndat, seed, transposed filter)
CASES = [
    ('mf_per_n32_ndat1024', 32, 1024, 1, False),     # the 1D MagicFilter workload of a 32^3 grid
    ('mf_per_t_n32_ndat1024', 32, 1024, 1, True),
    ('mf_per_n8_ndat3', 8, 3, 5, False),             # shortest line the C code wraps correctly
    ('mf_per_n16_ndat7', 16, 7, 6, True),
    ('mf_per_n64_ndat33', 64, 33, 7, False),
    ('mf_per_n128_ndat5', 128, 5, 8, True),
]


def x_of(n, ndat, seed):
    import __graft_entry__ as ge
    ge.package()
    from boast_lig_gb300 import inputs
    return inputs.uniform(seed, n * ndat)


def main():
    import oracle
    oracle.build(ref=True)
    out = {}
    for name, n, ndat, seed, t in CASES:
        x = x_of(n, ndat, seed)
        out[name] = oracle.ref_magicfilter(n, ndat, x, transposed_filter=t)
        out[name + '__xsha'] = np.frombuffer(hashlib.sha256(x.tobytes()).digest(), dtype=np.uint8)
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                     'magicfilter_ref_c.npz'), **out)


if __name__ == '__main__':
    main()
