#!/usr/bin/env python3
"""Extract the reference's finite-difference table as a golden fixture.

BigDFT/Poisson.rb:20-166 holds, as Fortran source inside a Ruby heredoc, the
coefficient table c1D(-m:m, -m:m) of the first derivatives of order nord in
{2, 4, 6, 8, 16} used by every Poisson operator.  This script reads that text
(no Ruby, no Fortran compiler: each entry is a quotient of two decimal
literals), evaluates each entry the way the Fortran does -- one IEEE
division of two exactly representable doubles -- and stores the tables in
poisson_fd_c1d.npz as float64 arrays fd<nord>[j + m, i] = c1D(i - m, j), so
the library's own table can be checked against the reference's bits on
machines without the reference tree.

    python tests/golden/make_poisson_golden.py path/to/BigDFT/Poisson.rb

(or with $LIBCONV_REFERENCE_DIR set to the reference tree).
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def literal(tok):
    """Value of one Fortran table entry such as '-25.d0/12.0' or '8.d0'."""
    tok = tok.replace('d0', '').replace('+', '').strip()
    if '/' in tok:
        a, b = tok.split('/')
        return float(a) / float(b)
    return float(tok)


def parse(text):
    body = text[text.find('select case(nord)'):text.find('end select')]
    parts = re.split(r'case\((\d+)\)', body)
    tables = {}
    for k in range(1, len(parts), 2):
        nord = int(parts[k])
        m = nord // 2
        t = np.full((nord + 1, nord + 1), np.nan)
        for mm in re.finditer(r'c1D\(-m:m,\s*(-?\d+)\)\s*=\s*\(/(.*?)/\)', parts[k + 1], re.S):
            j = int(mm.group(1))
            toks = [x for x in mm.group(2).replace('&', ' ').replace('\n', ' ').split(',')
                    if x.strip()]
            assert len(toks) == nord + 1, (nord, j, len(toks))
            t[j + m] = [literal(x) for x in toks]
        assert not np.isnan(t).any(), nord
        tables[f'fd{nord}'] = t
    return tables


def main():
    if len(sys.argv) > 1:
        src = sys.argv[1]
    elif os.environ.get('LIBCONV_REFERENCE_DIR'):
        src = os.path.join(os.environ['LIBCONV_REFERENCE_DIR'], 'BigDFT', 'Poisson.rb')
    else:
        sys.exit('usage: make_poisson_golden.py path/to/BigDFT/Poisson.rb '
                 '(or set LIBCONV_REFERENCE_DIR)')
    tables = parse(open(src).read())
    assert sorted(tables) == ['fd16', 'fd2', 'fd4', 'fd6', 'fd8'], sorted(tables)
    np.savez(os.path.join(HERE, 'poisson_fd_c1d.npz'), **tables)
    print('wrote', {k: v.shape for k, v in tables.items()})


if __name__ == '__main__':
    main()
