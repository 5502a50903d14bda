"""ORACLE — test infrastructure, never the product.

CPU restatement of the reference's kernel parameter conversions (code/srcF.kernel):
SI_ker_lamu2kamu.F90:823-830 (lambda/mu kernels -> kappa/mu), SI_ker_lamu2vpvs.F90:823-830
(lambda/mu -> Vp/Vs) and SI_ker_vpvs2kamu.F90:823-831 (Vp/Vs -> kappa/mu), point by point in
single precision.  Every numpy float32 operation rounds once, as each Fortran SP operation
does, and the expressions keep the source's left-to-right order, so the result is the
reference's rounding.  Only the tests use it.  Parity is pinned only by the source text
(the reference ships no kernel files) and by the algebra the tests check: the kappa/mu
kernels are K_kappa = K_lambda (lambda + 2 mu / 3) / lambda and
K_mu' = K_mu - 2 mu K_lambda / (3 lambda), and lamu2vpvs followed by vpvs2kamu is lamu2kamu.
"""
from __future__ import annotations

import numpy as np

MODES = {"lamu2kamu": 1, "lamu2vpvs": 2, "vpvs2kamu": 3}


def convert(mode, lam, mu, ka, kb):
    """One kernel pair (ka: the first parameter's kernel, kb: the second's) at points with
    lambda, mu.  mode: 1, 2, 3 or a name of MODES.  Returns new (ka, kb), float32."""
    mode = MODES.get(mode, mode)
    f = np.float32
    l, m = np.asarray(lam, f), np.asarray(mu, f)
    a, b = np.asarray(ka, f).copy(), np.asarray(kb, f).copy()
    two, three, four = f(2.0), f(3.0), f(4.0)
    if mode == 1:
        a = a / l
        b = b / m / two
        b = (two * b - two * a / three) * m
        a = a * (l + two * m / three)
    elif mode == 2:
        a = a / l
        b = b / m / two
        b = two * (b - a) * two * m
        a = a * two * (l + two * m)
    elif mode == 3:
        a = a / (two * (l + two * m))
        b = b / m / four + a
        b = (two * b - two * a / three) * m
        a = a * (l + two * m / three)
    else:
        raise ValueError(mode)
    return a.astype(f), b.astype(f)
