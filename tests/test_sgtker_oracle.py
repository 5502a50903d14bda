"""The CPU restatement of the sensitivity-kernel accumulation (SI_ker_sta.F90
stress2strain :1185-1211, sgt2scatter3 :1257-1337, scatter2kernel :1375-1431) against
independent numpy formulations: Hooke's law inverted, the convolution theorem's
np.convolve, and the trapezoid rule."""
import numpy as np
import pytest


def _media(rng, npts):
    vp = rng.uniform(5800.0, 8000.0, npts)
    vs = vp / 1.73
    rho = rng.uniform(2600.0, 3300.0, npts)
    mu = (rho * vs * vs).astype(np.float32)
    lam = (rho * vp * vp - 2.0 * rho * vs * vs).astype(np.float32)
    return lam, mu


def _stress_from_strain(lam, mu, eps):
    """eps (6, knt, npts) tensor strains Exx Eyy Ezz Exy Exz Eyz -> Hooke stresses."""
    lam = lam.astype(np.float64)
    mu = mu.astype(np.float64)
    tr = eps[0] + eps[1] + eps[2]
    out = np.empty_like(eps)
    for q in range(3):
        out[q] = lam * tr + 2.0 * mu * eps[q]
    for q in range(3, 6):
        out[q] = 2.0 * mu * eps[q]
    return out


def test_stress2strain_inverts_hooke(oracle_mod):
    rng = np.random.default_rng(11)
    npts, knt = 57, 9
    lam, mu = _media(rng, npts)
    eps = rng.normal(size=(6, knt, npts)) * 1e-6
    sig = _stress_from_strain(lam, mu, eps).astype(np.float32)
    got = oracle_mod.stress2strain(lam, mu, sig)
    np.testing.assert_allclose(got, eps, rtol=0, atol=2e-6 * np.max(np.abs(eps)))


def _series(rng, npts, knt):
    t = np.arange(1, knt + 1)[:, None]
    f = rng.uniform(0.02, 0.08, size=(6, 1, npts))
    ph = rng.uniform(0, 2 * np.pi, size=(6, 1, npts))
    env = np.exp(-((t - knt / 2) / (knt / 5)) ** 2)
    return (1e5 * env * np.sin(2 * np.pi * f * t + ph)).astype(np.float32)


def _strains64(lam, mu, sgt, oracle_mod):
    return oracle_mod.stress2strain(lam, mu, sgt).astype(np.float64)


@pytest.mark.parametrize("param", [0, 1], ids=["vpvs", "lamu"])
def test_scatter_fp64_matches_convolution(param, oracle_mod):
    """param 0: Vp/Vs kernels (SI_ker_sta.F90:1297-1298); param 1: lambda/mu kernels
    (SI_ker_sta_lamu.F90:1299-1300), against numpy convolutions of the strains."""
    rng = np.random.default_rng(5)
    npts, knt, dt = 13, 140, 0.2
    lam, mu = _media(rng, npts)
    r = [_series(rng, npts, knt) for _ in range(3)]
    s = _series(rng, npts, knt)
    out = oracle_mod.sgt2scatter3(lam, mu, r, s, dt, mode=1, param=param)
    es = _strains64(lam, mu, s, oracle_mod)
    for comp, slot_b in ((0, 3), (1, 5), (2, 4)):
        er = _strains64(lam, mu, r[comp], oracle_mod)
        for p in range(npts):
            tr_r = er[0, :, p] + er[1, :, p] + er[2, :, p]
            tr_s = es[0, :, p] + es[1, :, p] + es[2, :, p]
            x1 = np.zeros(knt)
            x1[1:] = dt * np.convolve(tr_r, tr_s)[: knt - 1]
            full = sum(w * np.convolve(er[q, :, p], es[q, :, p]) for q, w in
                       ((0, 1.0), (1, 1.0), (2, 1.0), (3, 2.0), (4, 2.0), (5, 2.0)))
            x2 = np.zeros(knt)
            x2[1:] = dt * full[: knt - 1]
            if param == 1:
                ka = x1 * float(lam[p])
                kb = 2.0 * x2 * float(mu[p])
            else:
                ka = x1 * 2.0 * (float(lam[p]) + 2.0 * float(mu[p]))
                kb = (x2 - x1) * 4.0 * float(mu[p])
            scale = np.max(np.abs(ka)) + np.max(np.abs(kb))
            np.testing.assert_allclose(out[comp, :, p], ka, rtol=0, atol=1e-12 * scale)
            np.testing.assert_allclose(out[slot_b, :, p], kb, rtol=0, atol=1e-12 * scale)


def test_scatter_known_answer_constant_strain(oracle_mod):
    """Constant SGTs: x1(n) = dt (n-1) trR trS exactly, in both arithmetic modes."""
    npts, knt, dt = 3, 40, 0.25
    lam = np.full(npts, 3.0e10, np.float32)
    mu = np.full(npts, 3.0e10, np.float32)
    r = np.zeros((6, knt, npts), np.float32)
    s = np.zeros((6, knt, npts), np.float32)
    # uniaxial stresses chosen so the strains are powers of two: sigma = lam tr I + 2 mu eps
    eps_r = np.array([2.0 ** -20, 0.0, 0.0])
    eps_s = np.array([0.0, 0.0, 2.0 ** -21])
    for q in range(3):
        r[q] = 3.0e10 * eps_r.sum() + 2 * 3.0e10 * eps_r[q]
        s[q] = 3.0e10 * eps_s.sum() + 2 * 3.0e10 * eps_s[q]
    for mode in (0, 1):
        out = oracle_mod.sgt2scatter3(lam, mu, [None, None, r], s, dt, mode=mode)
        n = np.arange(1, knt + 1)
        x1 = dt * (n - 1) * eps_r.sum() * eps_s.sum()
        np.testing.assert_allclose(out[2, :, 0], x1 * 2.0 * (3.0e10 + 2 * 3.0e10), rtol=1e-6)
        # exx*exx etc.: only the trace cross terms survive (R has xx, S has zz): x2 = 0
        np.testing.assert_allclose(out[4, :, 0], -x1 * 4.0 * 3.0e10, rtol=1e-6)
        assert not np.any(out[[0, 1, 3, 5]])


def test_scatter_reference_fp32_close_to_fp64(oracle_mod):
    rng = np.random.default_rng(8)
    npts, knt, dt = 9, 300, 0.1
    lam, mu = _media(rng, npts)
    r = [_series(rng, npts, knt), None, _series(rng, npts, knt)]
    s = _series(rng, npts, knt)
    a = oracle_mod.sgt2scatter3(lam, mu, r, s, dt, nt1=5, nt2=290, mode=0)
    b = oracle_mod.sgt2scatter3(lam, mu, r, s, dt, nt1=5, nt2=290, mode=1)
    for slot in (0, 3, 2, 4):
        rel = np.linalg.norm(a[slot] - b[slot]) / np.linalg.norm(b[slot])
        assert rel < 2e-5, (slot, rel)
    assert not np.any(b[:, :4]) and not np.any(b[:, 290:])  # outside nt1..nt2 untouched
    assert not np.any(b[[1, 5]])                            # Y not flagged


@pytest.mark.parametrize("nt1,nt2", [(1, 200), (17, 150), (60, 60)])
def test_scatter2kernel_trapezoid(nt1, nt2, oracle_mod):
    rng = np.random.default_rng(nt1)
    npts, knt, dt, m0 = 21, 200, 0.05, 1.0e16
    ka = rng.normal(size=(knt, npts))
    kb = rng.normal(size=(knt, npts))
    v = rng.normal(size=knt).astype(np.float32)
    u = rng.normal(size=knt).astype(np.float32)
    got = oracle_mod.scatter2kernel(v, u, ka, kb, dt, nt1, nt2, m0, mode=1)
    w = np.full(knt, dt)
    w[nt1 - 1] = w[nt2 - 1] = 0.5 * dt
    sel = slice(nt1 - 1, nt2)
    v64, u64 = v.astype(np.float64), u.astype(np.float64)
    if nt1 == nt2:
        v0 = dt * v64[nt1 - 1] ** 2 * m0
        u0 = dt * u64[nt1 - 1] ** 2 * m0
        want = [dt * v64[nt1 - 1] * ka[nt1 - 1] / v0, dt * u64[nt1 - 1] * ka[nt1 - 1] / u0,
                dt * v64[nt1 - 1] * kb[nt1 - 1] / v0, dt * u64[nt1 - 1] * kb[nt1 - 1] / u0]
    else:
        v0 = np.sum(w[sel] * v64[sel] ** 2) * m0
        u0 = np.sum(w[sel] * u64[sel] ** 2) * m0
        want = [(w[sel] * v64[sel]) @ ka[sel] / v0, (w[sel] * u64[sel]) @ ka[sel] / u0,
                (w[sel] * v64[sel]) @ kb[sel] / v0, (w[sel] * u64[sel]) @ kb[sel] / u0]
    for g, ww in zip(got, want):
        np.testing.assert_allclose(g, ww, rtol=1e-12, atol=1e-12 * np.max(np.abs(ww)))
    ref = oracle_mod.scatter2kernel(v, u, ka.astype(np.float32).astype(np.float64),
                                    kb.astype(np.float32).astype(np.float64), dt, nt1, nt2, m0, mode=0)
    for g, ww in zip(ref, want):
        assert np.linalg.norm(g - ww) / np.linalg.norm(ww) < 1e-5


@pytest.mark.parametrize("mode", [1, 2])
def test_iir_against_lfilter(mode, oracle_mod):
    """filter/filtfilt restated against scipy.signal.lfilter on the reference's padded
    series (zero initial conditions; scipy's own filtfilt pads differently).  The restatement
    evaluates the difference equation in direct form I as the reference does, lfilter in
    transposed direct form II: the order-8 band-pass's poles near the unit circle amplify
    their different roundings to ~1e-11 of the signal, hence the tolerance."""
    signal = pytest.importorskip("scipy.signal")
    b, a = signal.butter(4, [0.05, 0.2], btype="band")
    rng = np.random.default_rng(mode)
    nt = 180
    x = rng.normal(size=(nt, 3))
    got = oracle_mod.iir(x, b, a, mode)
    nod = b.size - 1
    nf = 3 * nod
    for q in range(3):
        w = x[:, q]
        left = np.zeros(nf) if mode == 1 else 2 * w[0] - w[nf:0:-1]
        right = 2 * w[-1] - w[-2:-nf - 2:-1]
        xp = np.concatenate([left, w, right])
        y = signal.lfilter(b, a, xp)
        if mode == 2:
            y = signal.lfilter(b, a, y[::-1])[::-1]
        np.testing.assert_allclose(got[:, q], y[nf:nf + nt], rtol=0, atol=1e-9 * np.abs(y).max())
