"""The SI_ker_pair restatement (oracle/kpair_oracle.py) pinned by independent formulations:

* the one-pass filter equals scipy.signal.lfilter from rest, and the forward-backward filter
  equals lfilter on the zero-padded series (NOD samples in front, 2 (NOD + 1) behind) with
  the backward pass started, as the reference's filter starts every pass, from its first
  NOD inputs and zero outputs (lfiltic), to 1e-12;
* the single-precision scatter series equal an FP64 convolution of the FP32 strains (x1 =
  dt sum trR(m) trS(n-m), x2 = dt sum of the strain double contraction) to FP32 rounding;
* the single-precision window kernels equal their FP64 trapezoid integrals to FP32
  rounding."""
import numpy as np
import pytest

from oracle import kpair_oracle as KP
from oracle import oracle as O


def _coeffs():
    signal = pytest.importorskip("scipy.signal")
    b, a = signal.butter(2, [0.1, 0.4], btype="band")
    return signal, b, a


def test_one_pass_filter_is_lfilter():
    signal, b, a = _coeffs()
    x = np.random.default_rng(1).normal(size=(60, 3))
    got = KP.pair_filter(x, b, a, 1)
    want = signal.lfilter(b, a, x, axis=0)
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-12 * np.abs(want).max())


def test_forward_backward_filter_is_padded_lfilter():
    signal, b, a = _coeffs()
    nod = b.size - 1
    x = np.random.default_rng(2).normal(size=50)
    got = KP.pair_filter(x, b, a, 2)
    xp = np.concatenate([np.zeros(nod), x, np.zeros(2 * nod + 2)])
    y = signal.lfilter(b, a, xp)
    w = y[::-1]
    zi = signal.lfiltic(b, a, np.zeros(nod), w[nod - 1::-1])
    yb = np.concatenate([np.zeros(nod), signal.lfilter(b, a, w[nod:], zi=zi)[0]])
    want = yb[::-1][nod:nod + x.size]
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-12 * np.abs(want).max())


def _pair_case(knt=24, npts=7, seed=4):
    rng = np.random.default_rng(seed)
    lam = rng.uniform(2e10, 4e10, npts).astype(np.float32)
    mu = rng.uniform(1e10, 3e10, npts).astype(np.float32)
    rs = (rng.normal(size=(6, knt, npts)) * 1e5).astype(np.float32)
    ss = (rng.normal(size=(6, knt, npts)) * 1e5).astype(np.float32)
    return lam, mu, rs, ss


def test_scatter_is_the_convolution():
    lam, mu, rs, ss = _pair_case()
    dt = 0.05
    sa, sb = KP.scatter_pair(lam, mu, rs, ss, dt)
    er = O.stress2strain(lam, mu, rs).astype(np.float64)
    es = O.stress2strain(lam, mu, ss).astype(np.float64)
    knt = rs.shape[1]
    trr, trs = er[:3].sum(0), es[:3].sum(0)
    x1 = np.zeros_like(trr)
    x2 = np.zeros_like(trr)
    for n in range(1, knt + 1):
        for m in range(1, n):
            x1[n - 1] += trr[m - 1] * trs[n - m - 1]
            x2[n - 1] += (er[0, m - 1] * es[0, n - m - 1] + er[1, m - 1] * es[1, n - m - 1] +
                          er[2, m - 1] * es[2, n - m - 1] + 2 * er[3, m - 1] * es[3, n - m - 1] +
                          2 * er[4, m - 1] * es[4, n - m - 1] + 2 * er[5, m - 1] * es[5, n - m - 1])
    l64, m64 = lam.astype(np.float64), mu.astype(np.float64)
    want_a = x1 * dt * 2 * (l64 + 2 * m64)
    want_b = 2 * (x2 - x1) * dt * 2 * m64
    for got, want in ((sa, want_a), (sb, want_b)):
        assert np.abs(got[0]).max() == 0.0          # no lag before the first frame
        np.testing.assert_allclose(got, want, rtol=0, atol=2e-5 * np.abs(want).max())


def test_kernels_are_the_trapezoid_integrals():
    lam, mu, rs, ss = _pair_case(knt=30)
    dt, m0 = 0.05, 1.0e15
    sa, sb = KP.scatter_pair(lam, mu, rs, ss, dt)
    rng = np.random.default_rng(9)
    v = rng.normal(size=30).astype(np.float32)
    u = rng.normal(size=30).astype(np.float32)
    nt1, nt2 = 4, 25
    got = KP.kernel_pair(v, u, sa, sb, dt, nt1, nt2, m0)
    w = np.full(30, dt)
    w[nt1 - 1] = w[nt2 - 1] = 0.5 * dt
    sel = slice(nt1 - 1, nt2)
    v64, u64 = v.astype(np.float64), u.astype(np.float64)
    v0 = np.sum(w[sel] * v64[sel] ** 2) * m0
    u0 = np.sum(w[sel] * u64[sel] ** 2) * m0
    want = [np.sum((w * v64)[sel, None] * sa[sel], 0) / v0, np.sum((w * u64)[sel, None] * sa[sel], 0) / u0,
            np.sum((w * v64)[sel, None] * sb[sel], 0) / v0, np.sum((w * u64)[sel, None] * sb[sel], 0) / u0]
    for g, wv in zip(got, want):
        np.testing.assert_allclose(g, wv, rtol=0, atol=2e-5 * np.abs(wv).max())
