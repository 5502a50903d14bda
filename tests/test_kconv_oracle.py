"""The restatement of the kernel parameter conversions (oracle/kconv_oracle.py) against the
algebra of the parameter change: d ln lambda, d ln mu -> d ln kappa, d ln mu gives
K_kappa = K_lambda kappa / lambda and K_mu' = K_mu - 2 mu K_lambda / (3 lambda)
(kappa = lambda + 2 mu / 3), the Vp/Vs kernels K_Vp = 2 (lambda + 2 mu) K_lambda / lambda and
K_Vs = 2 K_mu - 4 mu K_lambda / lambda, and lamu2vpvs followed by vpvs2kamu is lamu2kamu."""
import numpy as np

from oracle import kconv_oracle as KC


def _case(n=2000, seed=3):
    rng = np.random.default_rng(seed)
    vp = rng.uniform(5.5e3, 8.0e3, n)
    vs = vp / rng.uniform(1.65, 1.85, n)
    rho = rng.uniform(2.5e3, 3.3e3, n)
    mu = (rho * vs * vs).astype(np.float32)
    lam = (rho * vp * vp - 2 * rho * vs * vs).astype(np.float32)
    ka = rng.normal(size=n).astype(np.float32) * np.float32(1e-9)
    kb = rng.normal(size=n).astype(np.float32) * np.float32(1e-9)
    return lam, mu, ka, kb


def _close(a, b, rtol=2e-6):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    scale = np.maximum(np.abs(a), np.abs(b)).max()
    np.testing.assert_allclose(a, b, rtol=0, atol=rtol * scale)


def test_kappa_mu_kernels():
    lam, mu, ka, kb = _case()
    L, M, A, B = (x.astype(np.float64) for x in (lam, mu, ka, kb))
    a, b = KC.convert("lamu2kamu", lam, mu, ka, kb)
    _close(a, A * (L + 2 * M / 3) / L)
    _close(b, B - 2 * M * A / (3 * L))


def test_vp_vs_kernels():
    lam, mu, ka, kb = _case()
    L, M, A, B = (x.astype(np.float64) for x in (lam, mu, ka, kb))
    a, b = KC.convert("lamu2vpvs", lam, mu, ka, kb)
    _close(a, 2 * (L + 2 * M) * A / L)
    _close(b, 2 * B - 4 * M * A / L)


def test_vpvs_to_kamu_composes():
    lam, mu, ka, kb = _case(seed=4)
    a1, b1 = KC.convert("lamu2kamu", lam, mu, ka, kb)
    a2, b2 = KC.convert("vpvs2kamu", lam, mu, *KC.convert("lamu2vpvs", lam, mu, ka, kb))
    _close(a2, a1, 1e-6)
    _close(b2, b1, 1e-6)


def test_single_precision_steps():
    """Each step rounds to float32: the result equals a float32 evaluation term by term."""
    lam, mu, ka, kb = _case(50)
    a, b = KC.convert(3, lam, mu, ka, kb)
    f = np.float32
    for i in range(50):
        l, m, x, y = f(lam[i]), f(mu[i]), f(ka[i]), f(kb[i])
        x = x / (f(2) * (l + f(2) * m))
        y = y / m / f(4) + x
        y = (f(2) * y - f(2) * x / f(3)) * m
        x = x * (l + f(2) * m / f(3))
        assert a[i] == x and b[i] == y
