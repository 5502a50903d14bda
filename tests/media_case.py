"""Seeded grids and models in the six background and two perturbation kinds of the medium
preprocessor, as the reference's readers leave them (radians, metres, m/s, kg/m^3), for the
media tests.  A case is a grid plus a list of set-up calls that `fwant_gb300.Media` and the
oracle's `MediaOracle` both accept."""
import numpy as np

R_EARTH = 6371.0e3
CART1D, INTERFACE, LAYERED, COMPOSITE, VOLUME, VERPOLY = 1, 2, 3, 4, 5, 6
f32 = np.float32


def grid(ni, nj, nk, seed=0, dh=1000.0, dz_top=500.0, dz_bot=1500.0):
    """theta, phi, r with three ghosts per side; r stretched from dz_top at the top to
    dz_bot at depth (seeded jitter); ztopo = r at the top interior plane."""
    rng = np.random.default_rng(seed)
    th0 = np.deg2rad(50.0)
    x = th0 + (np.arange(ni + 6) - (ni + 6) / 2 + 0.2 * rng.random(ni + 6)) * dh / R_EARTH
    y = np.deg2rad(100.0) + (np.arange(nj + 6) - (nj + 6) / 2) * dh / R_EARTH
    dz = np.linspace(dz_bot, dz_top, nk + 5) * (1 + 0.05 * rng.random(nk + 5))
    z = R_EARTH - 200.0 - np.concatenate([[0.0], np.cumsum(dz)])[::-1]
    x, y, z = (np.sort(a).astype(f32) for a in (x, y, z))
    return x, y, z, float(z[3 + nk - 1])


def _axis(g, n, pad, rng, jitter=True):
    """model axis of n points spanning the grid axis g with a margin"""
    lo, hi = float(g[0]), float(g[-1])
    span = hi - lo
    a = np.linspace(lo - pad * span, hi + pad * span, n)
    if jitter:
        a[1:-1] += (rng.random(n - 2) - 0.5) * 0.3 * (a[1] - a[0])
    return np.sort(a).astype(f32)


def _gardner(vp):
    return f32(1741.0) * (vp / f32(1000.0)) ** f32(0.25)


def case(kind, x, y, z, ztopo, seed=1, perturb=None):
    """[(method, args), ...] for a background `kind` and an optional perturbation kind"""
    rng = np.random.default_rng(seed)
    depth_max = float(ztopo - z[0]) * 1.3
    calls = []
    if kind == CART1D:
        d = np.sort(rng.uniform(0.0, depth_max, 10)).astype(f32)
        d[0] = 0.0
        d[5] = d[4]  # a discontinuity: two values at one depth
        vp = np.sort(rng.uniform(5800.0, 8000.0, 10)).astype(f32)
        calls.append(("set_cart1d", (d, vp, (vp / f32(1.73)).astype(f32), _gardner(vp))))
    elif kind in (INTERFACE, LAYERED, COMPOSITE):
        mx, my = _axis(x, 7, 0.2, rng), _axis(y, 6, 0.2, rng)
        nl = 4
        h = np.zeros((7, 6, nl), f32)
        base = np.array([0.15, 0.25, 0.2, 0.9]) * depth_max
        for n in range(nl):
            h[:, :, n] = base[n] * (1 + 0.3 * (rng.random((7, 6)) - 0.5))
        h[2, 3, 1] = 0.0  # a pinched-out layer
        if kind == INTERFACE:
            zi = np.zeros((7, 6, nl), f32)
            zi[:, :, 0] = f32(ztopo + 300.0)
            for n in range(1, nl):
                zi[:, :, n] = zi[:, :, n - 1] - h[:, :, n - 1]
            hh = np.zeros_like(zi)
            hh[:, :, :-1] = zi[:, :, :-1] - zi[:, :, 1:]
            vp = np.sort(rng.uniform(5000.0, 8000.0, 2 * nl)).astype(f32).reshape(nl, 2).T
            calls.append(("set_layers", (INTERFACE, mx, my, zi, hh, vp, (vp / f32(1.75)).astype(f32), _gardner(vp))))
        elif kind == LAYERED:
            vp = np.sort(rng.uniform(5000.0, 8000.0, 2 * nl)).astype(f32).reshape(nl, 2).T
            calls.append(("set_layers", (LAYERED, mx, my, None, h, vp, (vp / f32(1.75)).astype(f32), _gardner(vp))))
        else:
            vp = (np.sort(rng.uniform(5000.0, 8000.0, 2 * nl)).reshape(nl, 2).T[:, None, None, :]
                  * (1 + 0.05 * rng.random((2, 7, 6, nl)))).astype(f32)
            ex = np.array([1.0, 2.0, 0.5, 1.0], f32)
            calls.append(("set_layers", (COMPOSITE, mx, my, None, h, vp, (vp / f32(1.75)).astype(f32), _gardner(vp),
                                         ex, ex[::-1].copy(), np.ones(nl, f32))))
    elif kind == VOLUME:
        mx, my = _axis(x, 9, 0.1, rng), _axis(y, 8, 0.1, rng)
        rz = np.linspace(-2000.0, depth_max, 7).astype(f32)
        vp = (6000.0 + 2000.0 * rng.random((9, 8, 7))).astype(f32)
        calls.append(("set_volume", (0, mx, my, rz, f32(ztopo), vp, (vp / f32(1.73)).astype(f32), _gardner(vp))))
    elif kind == VERPOLY:
        calls.append(("set_verpoly", _verpoly(x, y, ztopo, depth_max, rng, 6000.0, 1.0e-2)))
    if perturb == VOLUME:
        mx, my = _axis(x, 11, 0.05, rng), _axis(y, 10, 0.05, rng)
        rz = np.linspace(-1000.0, depth_max, 9).astype(f32)
        dv = [(0.1 * (rng.random((11, 10, 9)) - 0.5)).astype(f32) for _ in range(3)]
        calls.append(("set_volume", (1, mx, my, rz, f32(ztopo), *dv)))
    elif perturb == VERPOLY:
        calls.append(("set_verpoly", _verpoly(x, y, ztopo, depth_max, rng, 0.02, 1.0e-6, perturbed=1)))
    return calls


def _verpoly(x, y, ztopo, depth_max, rng, c0, c1, perturbed=0):
    ni, nj, nk, npoly = 5, 4, 4, 2
    mx, my = _axis(x, ni, 0.1, rng, jitter=False), _axis(y, nj, 0.1, rng, jitter=False)
    rz = np.zeros((ni, nj, nk), f32)
    rz[:, :, 0] = -500.0
    for k in range(1, nk):
        rz[:, :, k] = rz[:, :, k - 1] + depth_max / nk * (0.7 + 0.6 * rng.random((ni, nj)))
    sgn = 1.0 if perturbed == 0 else -1.0
    c = np.zeros((ni, nj, nk, npoly), f32)
    c[..., 0] = c0 * (1 + sgn * 0.1 * rng.random((ni, nj, nk)))
    c[..., 1] = c1 * rng.random((ni, nj, nk))
    ex = np.array([0.0, 1.0], f32)
    cs = (c / f32(1.73)).astype(f32) if perturbed == 0 else c * f32(0.5)
    cr = (c * f32(0.3)).astype(f32) if perturbed == 0 else c * f32(0.25)
    return (perturbed, mx, my, rz, f32(ztopo), c, cs, cr, ex, ex.copy(), ex.copy())


def feed(obj, calls):
    for name, args in calls:
        getattr(obj, name)(*args)
    return obj
