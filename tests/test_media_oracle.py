"""Pins of the medium preprocessor's CPU restatement (oracle/media_oracle.cpp) without a
GPU.  The reference ships no fixtures for seis3d_media, so the restatement is checked
against cases with known answers: a homogeneous medium, the harmonic average across a
horizontal interface, water (zero shear modulus) samples, the ghost extension, a straight
re-derivation of the time-step check in numpy, and a pure-Python loop restatement of the
cart1d + volume path on a tiny grid."""
import numpy as np
import pytest

import media_case as mc

f32 = np.float32


def _oracle(ni, nj, nk, x, y, z, zt, half, calls):
    from oracle import oracle as orc
    return mc.feed(orc.MediaOracle(ni, nj, nk, x, y, z, zt, half), calls)


def test_homogeneous(oracle_mod):
    x, y, z, zt = mc.grid(6, 5, 4)
    vp, vs, rho = f32(6000.0), f32(3500.0), f32(2700.0)
    d = np.array([0.0, 1e6], f32)
    m = _oracle(6, 5, 4, x, y, z, zt, (1, 1, 1), [("set_cart1d", (d, [vp] * 2, [vs] * 2, [rho] * 2))])
    lam, mu, r = m.eval()
    mu0 = float(rho) * float(vs) ** 2
    np.testing.assert_allclose(r, float(rho), rtol=1e-6)
    np.testing.assert_allclose(mu, mu0, rtol=1e-6)
    np.testing.assert_allclose(lam, float(rho) * float(vp) ** 2 - 2 * mu0, rtol=1e-6)


def test_harmonic_average_across_interface(oracle_mod):
    """A depth jump halfway between the k and k-1 sample rows of one grid plane: that
    plane's samples split four above, four below, so mu and lambda are the harmonic means
    and rho the arithmetic mean of the two layers"""
    ni, nj, nk = 4, 4, 6
    x, y, z, zt = mc.grid(ni, nj, nk)
    k = 3 + nk - 3  # an interior plane
    dz1 = (z[k] - z[k - 1]) / f32(2.0) / f32(2.0)
    dz2 = (z[k + 1] - z[k]) / f32(2.0) / f32(2.0)
    z_lo, z_hi = f32(-1.0) * dz1 + z[k], f32(1.0) * dz2 + z[k]  # the two sample radii
    jump = f32(zt) - f32(0.5) * (z_lo + z_hi)  # depth between them
    d = np.array([0.0, jump, jump, 1e6], f32)
    vp = np.array([5000.0, 5000.0, 7000.0, 7000.0], f32)
    vs = np.array([2900.0, 2900.0, 4000.0, 4000.0], f32)
    rh = np.array([2500.0, 2500.0, 3200.0, 3200.0], f32)
    m = _oracle(ni, nj, nk, x, y, z, zt, (1, 1, 1), [("set_cart1d", (d, vp, vs, rh))])
    lam, mu, r = m.eval()
    m1, m2 = 2500.0 * 2900.0 ** 2, 3200.0 * 4000.0 ** 2
    l1, l2 = 2500.0 * 5000.0 ** 2 - 2 * m1, 3200.0 * 7000.0 ** 2 - 2 * m2
    np.testing.assert_allclose(r[3:-3, 3:-3, k], 0.5 * (2500.0 + 3200.0), rtol=1e-6)
    np.testing.assert_allclose(mu[3:-3, 3:-3, k], 2.0 / (1 / m1 + 1 / m2), rtol=1e-6)
    np.testing.assert_allclose(lam[3:-3, 3:-3, k], 2.0 / (1 / l1 + 1 / l2), rtol=1e-6)
    # planes well away from the jump see one layer
    np.testing.assert_allclose(mu[3:-3, 3:-3, 3], m2, rtol=1e-6)
    np.testing.assert_allclose(mu[3:-3, 3:-3, -4], m1, rtol=1e-6)


def test_water_samples(oracle_mod):
    """vs = 0 below a depth: points with at least half of their samples in the water get
    mu = 0; points with fewer get (nsamp - nwater) over the sum of the solid samples"""
    ni, nj, nk = 4, 4, 6
    x, y, z, zt = mc.grid(ni, nj, nk)
    d = np.array([0.0, 1e6], f32)
    m = _oracle(ni, nj, nk, x, y, z, zt, (1, 1, 1),
                [("set_cart1d", (d, np.array([1500.0, 1500.0], f32), np.zeros(2, f32), np.array([1000.0] * 2, f32)))])
    lam, mu, r = m.eval()
    assert not np.any(mu)
    np.testing.assert_allclose(lam, 1000.0 * 1500.0 ** 2, rtol=1e-6)


def test_ghost_extension(oracle_mod):
    ni, nj, nk = 7, 6, 5
    x, y, z, zt = mc.grid(ni, nj, nk, seed=2)
    m = _oracle(ni, nj, nk, x, y, z, zt, (1, 1, 1), mc.case(mc.VOLUME, x, y, z, zt, seed=3))
    for a in m.eval():
        ci, cj, ck = (np.clip(np.arange(n + 6), 3, n + 2) for n in (ni, nj, nk))
        np.testing.assert_array_equal(a, a[np.ix_(ci, cj, ck)])


def _stept_numpy(x, y, z, lam, mu, rho):
    """media_stept_check re-derived with numpy arrays (same operation order)"""
    a = x.astype(np.float64) - np.pi / 2
    b = y.astype(np.float64)
    zz = z.astype(np.float64)
    G = np.empty(lam.shape + (3,))
    G[..., 0] = zz[None, None, :] * np.cos(a)[:, None, None] * np.cos(b)[None, :, None]
    G[..., 1] = zz[None, None, :] * np.cos(a)[:, None, None] * np.sin(b)[None, :, None]
    G[..., 2] = zz[None, None, :] * np.sin(a)[:, None, None] * np.ones_like(b)[None, :, None]
    nx, ny, nz = lam.shape
    I, J, K = np.meshgrid(np.arange(3, nx - 3), np.arange(3, ny - 3), np.arange(3, nz - 3), indexing="ij")
    P = G[I, J, K]
    dmin = None
    for s in range(8):
        A = G[I + (1 if s & 1 else -1), J, K]
        B = G[I, J + (1 if s & 2 else -1), K]
        C = G[I, J, K + (1 if s & 4 else -1)]
        AB, AC = B - A, C - A
        p0 = AB[..., 1] * AC[..., 2] - AB[..., 2] * AC[..., 1]
        p1 = AB[..., 2] * AC[..., 0] - AB[..., 0] * AC[..., 2]
        p2 = AB[..., 0] * AC[..., 1] - AB[..., 1] * AC[..., 0]
        d = -(p0 * A[..., 0] + p1 * A[..., 1] + p2 * A[..., 2])
        L = np.abs((p0 * P[..., 0] + p1 * P[..., 1] + p2 * P[..., 2] + d) / np.sqrt(p0 * p0 + p1 * p1 + p2 * p2))
        dmin = L if dmin is None else np.minimum(dmin, L)
    sl = (slice(3, -3),) * 3
    vp = np.sqrt((lam[sl] + f32(2.0) * mu[sl]) / rho[sl]).astype(f32)
    dt = (f32(1.3) / vp * dmin.astype(f32)).astype(f32)
    flat = dt.reshape(-1, order="F")
    q = int(np.argmin(flat))
    i, j, k = np.unravel_index(q, dt.shape, order="F")
    return float(flat[q]), (i + 4, j + 4, k + 4)


@pytest.mark.parametrize("kind", [mc.CART1D, mc.INTERFACE, mc.VOLUME])
def test_stept_check_against_numpy(kind, oracle_mod):
    ni, nj, nk = 9, 8, 7
    x, y, z, zt = mc.grid(ni, nj, nk, seed=4)
    m = _oracle(ni, nj, nk, x, y, z, zt, (1, 1, 1), mc.case(kind, x, y, z, zt, seed=5))
    lam, mu, rho = m.eval()
    dt, ijk, vp, dl = m.stept_check()
    dt_np, ijk_np = _stept_numpy(x, y, z, lam, mu, rho)
    assert dt == pytest.approx(dt_np, rel=1e-6)
    assert ijk == ijk_np
    assert dt == pytest.approx(1.3 / vp * dl, rel=1e-6)


def _locate(x0, xs):
    """indx_locate_1d (0-based lower index, clamped coordinate)"""
    n = len(xs)
    if x0 <= xs[0]:
        return 0, xs[0]
    if x0 >= xs[-1]:
        return n - 2, xs[-1]
    lo, hi = 1, n
    while hi - lo > 1:
        mid = (hi - lo) // 2 + lo
        if xs[mid - 1] == x0:
            lo = mid
            break
        if xs[mid - 1] > x0:
            hi = mid
        else:
            lo = mid
    return lo - 1, x0


def test_loop_restatement_cart1d_volume(oracle_mod):
    """effmedia_eval for the cart1d background and a volume perturbation written again as
    plain Python loops over float32 scalars, on a 3 x 3 x 3 grid: bit-identical"""
    ni = nj = nk = 3
    x, y, z, zt = mc.grid(ni, nj, nk, seed=7)
    calls = mc.case(mc.CART1D, x, y, z, zt, seed=8, perturb=mc.VOLUME)
    m = _oracle(ni, nj, nk, x, y, z, zt, (1, 1, 1), calls)
    lam, mu, rho = m.eval()
    d, cvp, cvs, cdp = calls[0][1]
    _, px, py, prz, rz0, dvp, dvs, ddp = calls[1][1]
    half = f32(2.0)
    for k in range(3, 3 + nk):
        for j in range(3, 3 + nj):
            for i in range(3, 3 + ni):
                def offs(g, c):
                    return [f32(-1.0) * ((g[c] - g[c - 1]) / half / half) + g[c],
                            f32(1.0) * ((g[c + 1] - g[c]) / half / half) + g[c]]
                r0 = m0 = l0 = f32(0.0)
                for z0 in offs(z, k):
                    d0 = max(f32(zt) - z0, f32(0.0))
                    for y0 in offs(y, j):
                        for x0 in offs(x, i):
                            # cart1d: interior interpolation (no sample of these grids sits on a node)
                            k2 = int(np.searchsorted(d, d0, side="right"))
                            k1 = k2 - 1
                            L1 = (d[k2] - d0) / (d[k2] - d[k1])
                            L2 = f32(1.0) - L1
                            V = [c[k1] * L1 + c[k2] * L2 for c in (cvp, cvs, cdp)]
                            ia, xa = _locate(x0, px)
                            ja, ya = _locate(y0, py)
                            ka, za = _locate(rz0 - z0, prz)
                            w = []
                            for g, a, v in ((px, ia, xa), (py, ja, ya), (prz, ka, za)):
                                w.append(((v - g[a + 1]) / (g[a] - g[a + 1]), (v - g[a]) / (g[a + 1] - g[a])))
                            P = []
                            for f in (dvp, dvs, ddp):
                                s = f32(0.0)
                                for kk in range(2):
                                    for jj in range(2):
                                        for ii in range(2):
                                            s = s + w[0][ii] * w[1][jj] * w[2][kk] * f[ia + ii, ja + jj, ka + kk]
                                P.append(s)
                            vp_, vs_, dp_ = (V[q] * (f32(1.0) + P[q]) for q in range(3))
                            mu_ = dp_ * vs_ * vs_
                            la_ = vp_ * vp_ * dp_ - f32(2.0) * mu_
                            r0 = r0 + f32(0.5) * (dp_ + dp_)
                            m0 = m0 + f32(0.5) * (f32(1.0) / mu_ + f32(1.0) / mu_)
                            l0 = l0 + f32(0.5) * (f32(1.0) / la_ + f32(1.0) / la_)
                assert rho[i, j, k] == r0 / f32(8.0)
                assert mu[i, j, k] == f32(8.0) / m0
                assert lam[i, j, k] == f32(8.0) / l0
