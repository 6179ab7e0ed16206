#!/usr/bin/env python3
"""Widths of the SA-1TDVP stage's synthetic singular values, fitted from the
two-site sweeps' singular-value log (a restatement of the reference's
bin/nls.py, which total_start runs before the SA stage, holstein/tdvp.h:341-358).

The log ("SVS", written by the C++ layer from kv_tdvp_svs; the reference's
svd_impl appends it at holstein/svd.h:390-402) holds, after a header
"Total Site = N", one record per two-site split: the number of kept singular
values, then log10(s_i s_{i-2} / s_{i-1}^2) for i >= 2.  The records of the
left-to-right and right-to-left passes are folded onto the N - 1 bonds the way
bin/nls.py folds them; each bond's values are histogrammed (50 bins) and the
quasi-Gaussian density below is least-squares fitted to the normalised counts
(scipy's curve_fit, width bounded to [0, inf)).  A bond with two values or
fewer gets 1.0.  The file written ("beta") has one fitted width per line; the
SA stage takes 1 / each as that bond's beta.

Run as a script in the directory holding SVS (it writes beta there), e.g.
installed on PATH under the name the drop-in layer calls, ``nls.py``.
"""
from __future__ import annotations

import sys

import numpy as np


def quasi_gauss(x, bet):
    """The fitted density of bin/nls.py (its qua_gau)."""
    from scipy.special import erfc

    x = np.asarray(x, dtype=float)
    r = np.exp(-0.25 * bet * x ** 2) * np.abs(x / 4.0 / bet)
    r = r + (np.ones(x.shape) / 2.0 / bet - x ** 2 / 4.0) * erfc(np.sqrt(bet) * np.abs(x) / 2.0) * 0.5 * np.sqrt(
        np.pi / bet)
    return r * np.exp(-bet * x ** 2 / 4.0) * bet ** 2


def read_svs(path: str) -> list:
    """Per-bond lists of second log-differences from an SVS log, folded as
    bin/nls.py folds them: the first 2N - 2 records are the first sweep
    (bonds 0..N-2 left to right, then back), later records wrap around."""
    with open(path) as f:
        lines = f.read().split("\n")
    n_site = int(lines[0].split()[3])
    period = 2 * n_site - 2
    per_bond: list = []
    rec = 0
    i = 1
    while i < len(lines):
        ln = lines[i] + "\n" if i < len(lines) - 1 else lines[i]
        i += 1
        if not (0 < len(ln) < 10):
            continue
        rec += 1
        n = max(int(ln) - 2, 0)
        vals = [float(v) for v in lines[i:i + n]]
        i += n
        if rec <= period:
            if rec < n_site:
                per_bond.append(vals)
            else:
                per_bond[period - rec] = per_bond[period - rec] + vals
        else:
            b = rec % period
            if b > n_site - 1:
                b = period - b
            dest = per_bond[b] if b < len(per_bond) else per_bond[b - 1]
            dest.extend(vals)
    return per_bond


def fit_widths(per_bond: list) -> list:
    """One fitted width per bond (1.0 where a bond has two values or fewer)."""
    from scipy.optimize import curve_fit

    out = []
    for v in per_bond:
        if len(v) > 2:
            counts, edges = np.histogram(v, 50)
            p, _ = curve_fit(quasi_gauss, edges[:-1], counts / len(v), bounds=(0, np.inf))
            out.append(float(p[0]))
        else:
            out.append(1.0)
    return out


def write_beta(path: str, widths: list):
    with open(path, "w") as f:
        for w in widths:
            f.write("{:21.15f}\n".format(w))


def betas(widths: list) -> list:
    """The SA stage's betaSet from fitted widths (holstein/tdvp.h:351-356)."""
    return [1.0 / float("{:21.15f}".format(w)) for w in widths]


def main(argv=None) -> int:
    argv = sys.argv[1:] if argv is None else argv
    svs = argv[0] if argv else "SVS"
    out = argv[1] if len(argv) > 1 else "beta"
    write_beta(out, fit_widths(read_svs(svs)))
    return 0


if __name__ == "__main__":
    sys.exit(main())
